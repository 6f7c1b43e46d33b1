// Residual stage of one block that allocates no device memory.
//
// Some callers cannot allocate device memory while they run the solver
// step: a host code that records the step into a CUDA graph it owns (a
// cudaMalloc in the middle would synchronise the device and break the
// capture), a serving loop that hands all HBM to an admission budget up
// front, or a plugin host whose allocator owns every byte of the device.
// ath_block_residual_noalloc serves them.  The caller passes its own device
// arrays for every input and output; the only extra memory the stage needs,
// the F.|A| face fluxes that pass from the face kernels to the residual
// assembly, lives in g_face_scratch below: a fixed array of
// ATH_NOALLOC_MAX_CELLS padded cells x 3 directions x 5 equations (15.7 MB
// of FP64), reserved on every GPU that loads this library until the process
// exits.
//
// The kernels are the same arithmetic as k_face / k_cell (physics.cuh, this
// unit is built with --fmad=false), indexed directly from the block's
// dimensions instead of work lists, so nothing else has to live on the
// device.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "aither_gb300.h"
#include "cuda_check.hpp"
#include "errors.hpp"
#include "kernels.cuh"

namespace ath {
namespace {

constexpr int64_t kScratchDoubles = 3LL * 5 * ATH_NOALLOC_MAX_CELLS;

// Shared by every call on a device; holds the last call's face fluxes.
// Every entry a call reads is written earlier in the same call, so nothing
// has to be cleared between calls.
__device__ __align__(256) double g_face_scratch[kScratchDoubles];

struct BlockArgs {
  int32_t ni, nj, nk, ng, NI, NJ;
  int64_t n;  // padded cells
  const double *W, *vol, *width[3], *fa[3];
  double *R, *lam, *dt, *ainv;
  double *flux;  // device address of g_face_scratch
};

__device__ __forceinline__ int64_t CellIdx(const BlockArgs &a, int i, int j, int k) {
  return (int64_t)(i + a.ng) + (int64_t)a.NI * ((j + a.ng) + (int64_t)a.NJ * (k + a.ng));
}

template <int D>
__global__ void k_face_blk(BlockArgs a, SolveDev sv) {
  const int ei = a.ni + (D == 0), ej = a.nj + (D == 1), ek = a.nk + (D == 2);
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)ei * ej * ek) return;
  const int i = (int)(t % ei);
  const int j = (int)((t / ei) % ej);
  const int k = (int)(t / ((int64_t)ei * ej));
  const int64_t c = CellIdx(a, i, j, k);
  const int64_t s = D == 0 ? 1 : (D == 1 ? (int64_t)a.NI : (int64_t)a.NI * a.NJ);
  const int64_t n = a.n;
  const Gas<double> g = GasOf<double>(sv);
  const Prim<double> wm2 = LoadW<double>(a.W, n, c - 2 * s);
  const Prim<double> wm1 = LoadW<double>(a.W, n, c - s);
  const Prim<double> w0 = LoadW<double>(a.W, n, c);
  const Prim<double> wp1 = LoadW<double>(a.W, n, c + s);
  const double *wd = a.width[D];
  const Prim<double> L =
      Muscl(wm2, wm1, w0, wd[c - 2 * s], wd[c - s], wd[c], sv.kappa, sv.limiter);
  const Prim<double> R =
      Muscl(wp1, w0, wm1, wd[c + s], wd[c], wd[c - s], sv.kappa, sv.limiter);
  const double *fa = a.fa[D];
  double f[5];
  RoeFlux(L, R, g, fa[c], fa[n + c], fa[2 * n + c], f);
  const double mag = fa[3 * n + c];
  double *out = a.flux + (int64_t)D * 5 * n;
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n + c] = f[v] * mag;
}

__global__ void k_cell_blk(BlockArgs a, SolveDev sv, double cfl) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)a.ni * a.nj * a.nk) return;
  const int i = (int)(t % a.ni);
  const int j = (int)((t / a.ni) % a.nj);
  const int k = (int)(t / ((int64_t)a.ni * a.nj));
  const int64_t c = CellIdx(a, i, j, k);
  const int64_t n = a.n;
  const int64_t st[3] = {1, (int64_t)a.NI, (int64_t)a.NI * a.NJ};
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double r = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double *F = a.flux + (int64_t)d * 5 * n + v * n;
      r = r - F[c];
      r = r + F[c + st[d]];
    }
    a.R[v * n + c] = r;
  }
  const Gas<double> g = GasOf<double>(sv);
  const Prim<double> w = LoadW<double>(a.W, n, c);
  double lam = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double *fa = a.fa[d];
    const int64_t u = c + st[d];
    lam = lam + InvCellSpecRad(w, g, fa[c], fa[n + c], fa[2 * n + c], fa[3 * n + c],
                               fa[u], fa[n + u], fa[2 * n + u], fa[3 * n + u]);
  }
  a.lam[c] = lam;
  const double vol = a.vol[c];
  const double dt = cfl * (vol / lam);
  a.dt[c] = dt;
  const double diag = lam * sv.relax + (vol * (1.0 + sv.zeta)) / (dt * sv.theta);
  a.ainv[c] = 1.0 / diag;
}

// Device address of g_face_scratch on the current device (host code may
// not use the symbol itself as a pointer).  Looked up with that device
// current on every call whose stream is not being captured, so the address
// follows a reset of the device's primary context; a call made during a
// stream capture uses the address of the device's last uncaptured call.
std::mutex g_mu;
double *g_scratch_addr[64] = {nullptr};

double *ScratchAddress(int device, cudaStream_t stream) {
  if (device < 0 || device >= 64) throw Error(ATH_ERR_ARG, "device id out of range");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  Check(cudaStreamIsCapturing(stream, &cap), "cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lk(g_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_face_scratch);
    if (e != cudaSuccess)
      throw Error(ATH_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(face scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[device] = static_cast<double *>(p);
  } else if (!g_scratch_addr[device]) {
    throw Error(ATH_ERR_ARG,
                "the first allocation-free call on a device must come before any stream capture");
  }
  return g_scratch_addr[device];
}

}  // namespace
}  // namespace ath

extern "C" int ath_block_residual_noalloc(const ath_block_dev *blk,
                                          const ath_solve_view *phys, double cfl,
                                          void *stream) {
  return ath::Guard([&] {
    if (!blk || !phys) throw ath::Error(ATH_ERR_ARG, "null argument");
    if (blk->ni < 1 || blk->nj < 1 || blk->nk < 1 || blk->ng < 2)
      throw ath::Error(ATH_ERR_ARG, "block needs at least one cell per direction and 2 ghost layers");
    if (!blk->W || !blk->vol || !blk->R || !blk->lam || !blk->dt || !blk->ainv)
      throw ath::Error(ATH_ERR_ARG, "null device array");
    for (int d = 0; d < 3; ++d)
      if (!blk->width[d] || !blk->farea[d]) throw ath::Error(ATH_ERR_ARG, "null device array");
    const int64_t NI = blk->ni + 2 * blk->ng, NJ = blk->nj + 2 * blk->ng,
                  NK = blk->nk + 2 * blk->ng;
    const int64_t n = NI * NJ * NK;
    if (n > ATH_NOALLOC_MAX_CELLS)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "block has " + std::to_string(n) +
                           " padded cells; the allocation-free residual takes at most " +
                           std::to_string((long long)ATH_NOALLOC_MAX_CELLS));
    if (phys->limiter < ATH_LIMITER_NONE || phys->limiter > ATH_LIMITER_VANALBADA)
      throw ath::Error(ATH_ERR_ARG, "unknown limiter");
    if (phys->recon != ATH_RECON_MUSCL || phys->flux != ATH_FLUX_ROE)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual implements MUSCL reconstruction with the Roe flux");
    // it forms the inviscid residual, radius and scalar diagonal of a
    // steady (local time step) solve; views it would silently get wrong
    // are refused
    if (phys->eqn != ATH_EQN_EULER)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual implements the Euler equations only");
    if (phys->turb != ATH_TURB_NONE)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual has no turbulence model");
    if (phys->solver != ATH_SOLVER_LUSGS && phys->solver != ATH_SOLVER_DPLUR)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual forms the scalar diagonal of lusgs/dplur, "
                       "not the block diagonal of blusgs/bdplur");
    if (phys->dt_global > 0.0)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual uses the local (CFL) time step, not a "
                       "global timeStep");
    if (phys->dual_cfl > 0.0)
      throw ath::Error(ATH_ERR_UNSUPPORTED,
                       "the allocation-free residual has no dual-time term");
    int device = 0;
    ath::Check(cudaGetDevice(&device), "cudaGetDevice");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ath::BlockArgs a{};
    a.ni = blk->ni;
    a.nj = blk->nj;
    a.nk = blk->nk;
    a.ng = blk->ng;
    a.NI = (int32_t)NI;
    a.NJ = (int32_t)NJ;
    a.n = n;
    a.W = blk->W;
    a.vol = blk->vol;
    for (int d = 0; d < 3; ++d) {
      a.width[d] = blk->width[d];
      a.fa[d] = blk->farea[d];
    }
    a.R = blk->R;
    a.lam = blk->lam;
    a.dt = blk->dt;
    a.ainv = blk->ainv;
    a.flux = ath::ScratchAddress(device, s);
    ath::SolveDev sv{};
    sv.gas_r = phys->gas_r;
    sv.gas_n = phys->gas_n;
    sv.gas_hf = phys->gas_hf;
    sv.kappa = phys->kappa;
    sv.theta = phys->theta;
    sv.zeta = phys->zeta;
    sv.relax = phys->relax;
    sv.limiter = phys->limiter;
    sv.recon = ATH_RECON_MUSCL;
    sv.flux = ATH_FLUX_ROE;
    ath::SetDerived(sv);
    const int64_t nf[3] = {(int64_t)(blk->ni + 1) * blk->nj * blk->nk,
                           (int64_t)blk->ni * (blk->nj + 1) * blk->nk,
                           (int64_t)blk->ni * blk->nj * (blk->nk + 1)};
    ath::k_face_blk<0><<<(unsigned)((nf[0] + 127) / 128), 128, 0, s>>>(a, sv);
    ath::k_face_blk<1><<<(unsigned)((nf[1] + 127) / 128), 128, 0, s>>>(a, sv);
    ath::k_face_blk<2><<<(unsigned)((nf[2] + 127) / 128), 128, 0, s>>>(a, sv);
    const int64_t nc = (int64_t)blk->ni * blk->nj * blk->nk;
    ath::k_cell_blk<<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(a, sv, cfl);
    ath::Check(cudaGetLastError(), "kernel launch");
  });
}
