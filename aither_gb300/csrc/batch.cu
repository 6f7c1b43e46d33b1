// Device batch: HBM pools for every block of every solve, the work lists
// that drive the kernels, and the iteration sequence (captured once as a
// CUDA graph and replayed).  Implements the ath_ctx / ath_batch part of the
// C ABI (include/aither_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "aither_gb300.h"
#include "cuda_check.hpp"
#include "errors.hpp"
#include "kernels.cuh"
#include "setup.hpp"


struct ath_ctx {
  int device = 0;
  size_t budget = 0;  // 0 = whatever the device has
  size_t used = 0;
  // stream-ordered pool of the context's batches: allocations and frees are
  // ordered on the owning batch's stream and the pool keeps freed memory for
  // reuse, so creating and destroying batches (serving admission and
  // retirement) never synchronises the device
  cudaMemPool_t pool = nullptr;
};

namespace ath {

namespace {

// Device allocation accounted against the context's HBM budget, stream
// ordered on the owning batch's stream from the context's pool.
class DevMem {
 public:
  DevMem(ath_ctx *ctx, cudaStream_t stream) : ctx_(ctx), stream_(stream) {}
  ~DevMem() { Release(); }
  template <typename T>
  T *Alloc(size_t count) {
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (ctx_->budget && ctx_->used + bytes > ctx_->budget)
      throw Error(ATH_ERR_NOMEM, "device memory budget exceeded");
    void *p = nullptr;
    Check(cudaMallocFromPoolAsync(&p, bytes, ctx_->pool, stream_), "cudaMallocFromPoolAsync");
    ctx_->used += bytes;
    ptrs_.push_back({p, bytes});
    return static_cast<T *>(p);
  }
  template <typename T>
  T *Upload(const std::vector<T> &v) {
    T *p = Alloc<T>(v.size());
    if (!v.empty()) {
      Check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream_),
            "upload");
      Check(cudaStreamSynchronize(stream_), "upload");  // the host vector may go
    }
    return p;
  }
  void Zero(void *p, int value, size_t bytes) {
    Check(cudaMemsetAsync(p, value, bytes, stream_), "memset");
  }
  void Free(void *p) {
    for (size_t i = 0; i < ptrs_.size(); ++i)
      if (ptrs_[i].first == p) {
        cudaFreeAsync(p, stream_);
        ctx_->used -= ptrs_[i].second;
        ptrs_.erase(ptrs_.begin() + (long)i);
        return;
      }
  }
  void Release() {
    for (auto &e : ptrs_) {
      cudaFreeAsync(e.first, stream_);
      ctx_->used -= e.second;
    }
    ptrs_.clear();
  }

 private:
  ath_ctx *ctx_;
  cudaStream_t stream_;
  std::vector<std::pair<void *, size_t>> ptrs_;
};

// solve groups whose hyperplane chains a sweep pass can run concurrently
constexpr int kSweepGroups = 4;

struct Lists {
  std::vector<int32_t> cells, cell_cta_block, cell_cta_pos0;
  std::vector<int32_t> faces[3], face_cta_block[3];
  std::vector<int2> sweep_items;  // (q index, block)
  std::vector<int32_t> step_off;
  // the items of plane s ordered by solve group (kSweepGroups groups of
  // solves balanced by cells): group g's are [gstep_off[s * (kSweepGroups
  // + 1) + g], ... + g + 1)
  std::vector<int32_t> gstep_off;
  // the same items per solve, then plane, for the persistent sweep
  std::vector<int2> cl_items;
  std::vector<int32_t> cl_step_off, solve_step0, solve_nsteps;
  int max_plane = 0;  // largest plane of one solve
  std::vector<int32_t> solve_cta0;
  std::vector<GhostOpDev> ops, conn_ops;
  std::vector<int32_t> op_solve;
  // nonreflecting surfaces: their cells grouped by surface, offsets
  std::vector<NrDev> nr;
  std::vector<int32_t> nr_off;
  // cells whose ghosts a nonreflecting pressure outlet fills (pool index,
  // block): their gradients of the previous residual are kept
  std::vector<int32_t> nrg_cells, nrg_block;
  // hyperplane-ordered sweep tables
  std::vector<int64_t> q0;        // per block: first q index
  std::vector<int32_t> qpos;      // per pool cell
  std::vector<int32_t> nbq;       // [6][nq]
  std::vector<double> face_lo, face_hi;  // [3][4][nq]
  std::vector<int32_t> ghost_cell, ghost_src;
  std::vector<double> dist_lo, dist_hi;  // [3][nq]
  // block-edge ghosts, viscous-wall ghosts: ops grouped by phase
  std::vector<GhostOpDev> edge_ops, vops, vedge_ops;
  std::vector<int32_t> edge_solve, vop_solve, vedge_solve;
  std::vector<int32_t> edge_phase_off, vedge_phase_off;
  // viscous-wall faces, ordered by solve, and each solve's first entry
  std::vector<WallFaceDev> wall_faces;
  std::vector<int32_t> solve_face0;
  // cells whose laminar viscosity is needed (viscous blocks, all but corners)
  std::vector<int32_t> aux_cells, aux_block;
  bool any_viscous = false;
};

}  // namespace

// Per-batch state that does not depend on the arithmetic type.
struct BatchCore {
  ath_ctx *ctx;
  const Setup *setup;
  int precision, flags;
  int nsolves = 0, nblocks = 0;
  int64_t ncell = 0, nq = 0;
  std::vector<int64_t> cell0;        // pool offset of each block
  std::vector<int64_t> solve_pos0;   // per block: loop-order offset inside its solve
  Lists L;
  int nsteps = 0;
  int kinds = 0;        // bit 0: scalar solves present, bit 1: block solves
  int skinds = 0;       // the same for the LU-SGS solves (hyperplane sweeps)
  int jkinds = 0;       // and for the DP-LUR solves (Jacobi sweeps)
  int max_sweeps = 1;   // largest matrixSweeps of the LU-SGS solves
  int max_jsweeps = 0;  // largest matrixSweeps of the DP-LUR solves
  int sweep_threads = 128;  // CTA size of the per-plane sweep kernels (autotuned)
  // sweep shape: mode 1 = persistent (one cluster of cl_size CTAs of
  // cl_threads per solve), 0 = one launch per hyperplane, 2 = the same with
  // a group of lanes per scalar cell (one per neighbour term); autotuned
  int sweep_mode = 0, cl_size = 1, cl_threads = 256;
  // sweep mode 4: planes of fewer than hy_items cells take lane groups
  // (CTAs of sweep_threads), larger ones a thread per cell (CTAs of 128)
  int hy_items = 1 << 15;
  // modes 0 and 2: the solves' hyperplane chains run as sweep_groups
  // concurrent chains (1, 2 or 4 merged solve groups), forked from the
  // batch's stream onto gstream and joined back after each pass
  int sweep_groups = 1;
  cudaStream_t gstream[kSweepGroups - 1] = {};
  cudaEvent_t gfork = nullptr, gjoin[kSweepGroups - 1] = {};
  int2 *d_cl_items = nullptr;
  int32_t *d_cl_step_off = nullptr, *d_solve_step0 = nullptr, *d_solve_nsteps = nullptr;
  SweepLists Lists() const {
    return SweepLists{d_cl_items, d_cl_step_off, d_solve_step0, d_solve_nsteps, nsolves};
  }
  // mode 3 = the persistent tile-queue sweep: tiles of at most tq_size cells
  // of one solve's hyperplane, per kind (scalar, block) and direction; the
  // lists of every candidate tile size are built at batch creation
  struct TqList {
    int4 *tiles = nullptr;
    int32_t *deps = nullptr;
    int *done = nullptr;
    int ntiles = 0;
  };
  int tq_size = 32;
  std::map<int, std::array<TqList, 4>> tq;  // tile size -> [kind * 2 + backward], built
                                            // on first use (outside graph capture)
  int tq_ctas[2] = {0, 0};                  // resident CTAs, scalar and block kernels
  int *d_tq_ticket = nullptr, *d_tq_status = nullptr;
  long long tq_spin_limit = 1LL << 24;      // polls of one wait (~1 s)
  int tq_wait_never = 0;                    // test mode: every wait polls a flag never set
  bool block_viscous = false;
  bool any_rans = false;  // SST solves present: k, omega pools allocated
  bool any_unsteady = false;  // time-accurate or nonreflecting solves: time levels kept
  int fkinds = 0;  // bit 0: solves without turbulence equations, bit 1: SST
  // every solve without turbulence equations reconstructs with MUSCL and
  // takes the Roe flux (the fast faces then run their MUSCL-Roe kernel)
  bool mr_only = true;
  int vkinds = 0;  // bit 0: laminar viscous solves, bit 1: SST
  cudaStream_t stream = nullptr;
  bool own_stream = true;  // false: a multigrid level on its finest batch's stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::unique_ptr<DevMem> mem;
  // device lists
  int32_t *d_cells = nullptr, *d_cell_cta_block = nullptr, *d_cell_cta_pos0 = nullptr;
  int32_t *d_faces[3] = {nullptr, nullptr, nullptr};
  int32_t *d_face_cta_block[3] = {nullptr, nullptr, nullptr};
  int2 *d_sweep = nullptr;
  int32_t *d_solve_cta0 = nullptr;
  GhostOpDev *d_ops = nullptr, *d_conn_ops = nullptr;
  NrDev *d_nr = nullptr;
  int32_t *d_nr_off = nullptr;
  int32_t *d_nrg_cells = nullptr, *d_nrg_block = nullptr;
  int n_nr_surf = 0;
  GhostOpDev *d_edge_ops = nullptr, *d_vops = nullptr, *d_vedge_ops = nullptr;
  int32_t *d_edge_solve = nullptr, *d_vop_solve = nullptr, *d_vedge_solve = nullptr;
  int32_t *d_aux_cells = nullptr, *d_aux_block = nullptr;
  int32_t *d_op_solve = nullptr;
  NormPartial *d_partials = nullptr;
  double *d_mres = nullptr;
  WallFaceDev *d_wall_faces = nullptr;
  int32_t *d_solve_face0 = nullptr;
  double *d_wbuf = nullptr;   // [6][wall faces]
  double *d_fring = nullptr;  // [ring_cap][nsolves][6] wall forces
  NormOut *d_ring = nullptr;
  SolveState *d_sstate = nullptr;
  uint64_t *d_now = nullptr;
  int ring_cap = 1024;
  int64_t *d_iter = nullptr;
  int64_t iter_host = 0;
  double *d_cfl = nullptr;
  BlockDev *d_blocks = nullptr;
  SolveDev *d_solves = nullptr;
  ath_bc_state *d_states = nullptr;
  cudaGraphExec_t graph = nullptr;
  int64_t launches_per_iter = 0;
  ath_stats stats{};
};

__global__ void k_cfl(const SolveDev *solves, int nsolves, const SolveState *sstate,
                      double *cfl) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsolves) return;
  const SolveDev sv = solves[s];
  // input::CalcCFL of the time step (src/input.cpp:647)
  const double it = (double)(sstate[s].iter / sv.nl_iters);
  cfl[s] = fmin(sv.cfl_start + it * sv.cfl_step, sv.cfl_max);
}

__global__ void k_norms(const NormPartial *partials, const double *mres_partials,
                        const int32_t *solve_cta0, int nsolves, NormOut *ring,
                        int ring_cap, int64_t *iter_counter, SolveDev *solves,
                        SolveState *sstate, double *cfl) {
  const int s = blockIdx.x;
  if (s >= nsolves) return;
  const int lane = threadIdx.x;
  const int c0 = solve_cta0[s], c1 = solve_cta0[s + 1];
  double l2[kNvMax] = {0, 0, 0, 0, 0, 0, 0};
  double mx = 0.0, mres = 0.0;
  int64_t mpos = INT64_MAX;
  int bad = 0;
  for (int c = c0 + lane; c < c1; c += 32) {
    if (mres_partials) mres += mres_partials[c];
    const NormPartial p = partials[c];
#pragma unroll
    for (int v = 0; v < kNvMax; ++v) l2[v] += p.l2[v];
    if (p.linf > mx || (p.linf == mx && p.linf_pos < mpos)) {
      mx = p.linf;
      mpos = p.linf_pos;
    }
    bad |= p.bad;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int v = 0; v < kNvMax; ++v) l2[v] += __shfl_down_sync(0xffffffffu, l2[v], off);
    const double om = __shfl_down_sync(0xffffffffu, mx, off);
    const int64_t op = __shfl_down_sync(0xffffffffu, mpos, off);
    if (om > mx || (om == mx && op < mpos)) {
      mx = om;
      mpos = op;
    }
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
    mres += __shfl_down_sync(0xffffffffu, mres, off);
  }
  const int64_t it = *iter_counter;
  __syncwarp();
  if (lane == 0) {
    const SolveDev sv = solves[s];
    NormOut o;
    for (int v = 0; v < 7; ++v) o.l2[v] = sqrt(l2[v]);
    o.linf = mx;
    o.linf_pos = mpos;
    o.bad = sv.active ? bad : 2;
    o.pad = 0;
    o.cfl = cfl[s];
    // src/mgSolution.cpp:196-206 divides by the padded size, src/main.cpp:271
    // by cells x equations
    const double nv = sv.rans ? (double)kNvMax : (double)kNv;
    o.matrix_resid = mres_partials ? sqrt((mres / sv.padded_values) / (sv.cells * nv)) : 0.0;
    ring[(it % ring_cap) * nsolves + s] = o;
    if (sv.active) {
      // retirement: the drop of the total L2 against the solve's first
      // iteration (the reference normalises its residual history by the
      // first iteration's norms, src/main.cpp:254-271)
      SolveState &ss = sstate[s];
      double tot = 0.0;
      for (int v = 0; v < 7; ++v) tot += o.l2[v] * o.l2[v];
      tot = sqrt(tot);
      uint64_t now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (ss.iter == 0) {
        ss.l2_first = tot;
        ss.t_first_ns = now;
      }
      ss.iter += 1;
      ss.l2_last = tot;
      const bool reached = ss.target > 0.0 && tot <= ss.target * ss.l2_first;
      if (bad || reached) {
        solves[s].active = 0;
        ss.retire_iter = ss.iter;
        ss.t_retire_ns = now;
        ss.converged = bad ? -1 : 1;
      }
    }
  }
}

__global__ void k_iter_advance(int64_t *iter_counter) { *iter_counter += 1; }

__global__ void k_clock(uint64_t *out) {
  uint64_t now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  *out = now;
}

__global__ void k_wallsum(const double *wbuf, int nfaces, const int32_t *solve_face0,
                          int nsolves, double *fring, int ring_cap,
                          const int64_t *iter_counter) {
  const int s = blockIdx.x;
  if (s >= nsolves) return;
  const int lane = threadIdx.x;
  const int f0 = solve_face0[s], f1 = solve_face0[s + 1];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int f = f0 + lane; f < f1; f += 32)
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] += wbuf[(int64_t)q * nfaces + f];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], off);
  if (lane == 0) {
    const int64_t it = *iter_counter;
    double *o = fring + ((it % ring_cap) * nsolves + s) * 6;
#pragma unroll
    for (int q = 0; q < 6; ++q) o[q] = acc[q];
  }
}

// A coarse multigrid level follows its finest level's solves: the same
// CFL (input::CalcCFL of the iteration) and the same active flags
__global__ void k_mg_sync(const SolveDev *fine, const double *fine_cfl, SolveDev *coarse,
                          double *coarse_cfl, int nsolves) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsolves) return;
  coarse_cfl[s] = fine_cfl[s];
  coarse[s].active = fine[s].active;
}

// ---------------------------------------------------------------------------
class RunnerBase {
 public:
  virtual ~RunnerBase() = default;
  virtual void FillGhosts() = 0;
  virtual void Residual() = 0;
  virtual void Relax() = 0;
  virtual void Update() = 0;
  virtual void Iterate(int n) = 0;
  virtual void GetDU(int b, double *out) = 0;
  virtual void GetAinv(int b, double *out) = 0;
  virtual void GetAux(int b, double *out) = 0;
  virtual void GetVelGrad(int b, double *out) = 0;
  // block's current state into both time levels (a one-level restart)
  virtual void StoreTimeLevels(int b) = 0;
  // temperature and viscosity of a block's physical cells from its state
  virtual void RefreshAux(int b) = 0;
  virtual void Profile(int reps, double ms[8]) = 0;
  // drop the captured iteration graph (launch shapes changed)
  virtual void ResetGraph() = 0;
  // save (restore = false) or restore the iteration state: solution,
  // per-solve counters and flags, CFL, iteration counter
  virtual void Snapshot(bool restore) = 0;
  virtual void FreeSnapshot() = 0;
  virtual int MaxClusters(int kinds, int threads, int cluster) = 0;
  virtual int TqOccupancy(bool full, bool block) = 0;
};

template <typename T>
class Runner : public RunnerBase {
 public:
  explicit Runner(BatchCore &c) : c_(c) {
    DevMem &m = *c.mem;
    const int64_t n = c.ncell;
    P_.ncell = n;
    // FP64 batches with the fast option: contracted-FMA faces, cell, sweeps
    // and update (batch flag bit 1)
    P_.fast_fp64 = (std::is_same<T, double>::value && (c.flags & 2)) ? 1 : 0;
    P_.fkinds = c.fkinds;
    P_.W = m.Alloc<double>(5 * n);
    P_.R = m.Alloc<double>(5 * n);
    for (int d = 0; d < 3; ++d) P_.flux[d] = m.Alloc<double>(5 * n);
    if (c.L.any_viscous) {
      for (int d = 0; d < 3; ++d) {
        P_.vflux[d] = m.Alloc<T>(5 * n);
        c_.mem->Zero(P_.vflux[d], 0, 5 * n * sizeof(T));
      }
      P_.mu = m.Alloc<double>(n);
      c_.mem->Zero(P_.mu, 0, n * sizeof(double));
      P_.Taux = m.Alloc<double>(n);
      c_.mem->Zero(P_.Taux, 0, n * sizeof(double));
    }
    P_.lam = m.Alloc<double>(n);
    P_.dt = m.Alloc<double>(n);
    c_.mem->Zero(P_.R, 0, 5 * n * sizeof(double));
    c_.mem->Zero(P_.lam, 0, n * sizeof(double));
    // the nonreflecting boundaries' LODI relaxation of the first iteration
    // reads the time step before any has been formed: zero, as the
    // reference's zero-initialised per-cell time step
    c_.mem->Zero(P_.dt, 0, n * sizeof(double));
    // hyperplane-ordered sweep working set
    const int64_t nq = c.nq, ngh = (int64_t)c.L.ghost_cell.size();
    P_.nq = nq;
    P_.nghost = ngh;
    P_.Wq = m.Alloc<T>(5 * nq);
    P_.Rq = m.Alloc<T>(5 * nq);
    const int64_t aw = (c.kinds & 2) ? 25 : 1;  // width of the diagonal
    P_.Ainvq = m.Alloc<T>(aw * nq);
    P_.Aq = m.Alloc<T>(aw * nq);
    P_.dUq = m.Alloc<T>(5 * nq);
    P_.dUg = m.Alloc<T>(5 * std::max<int64_t>(ngh, 1));
    c_.mem->Zero(P_.Wq, 0, 5 * nq * sizeof(T));
    c_.mem->Zero(P_.Rq, 0, 5 * nq * sizeof(T));
    c_.mem->Zero(P_.Ainvq, 0, aw * nq * sizeof(T));
    c_.mem->Zero(P_.Aq, 0, aw * nq * sizeof(T));
    if (c.kinds & 2) {
      for (int d = 0; d < 3; ++d) {
        P_.fst[d] = m.Alloc<T>(10 * n);
        c_.mem->Zero(P_.fst[d], 0, 10 * n * sizeof(T));
        if (c.block_viscous) {
          P_.vst[d] = m.Alloc<T>(15 * n);
          c_.mem->Zero(P_.vst[d], 0, 15 * n * sizeof(T));
        }
      }
      P_.Joff = m.Alloc<T>(150 * nq);
      c_.mem->Zero(P_.Joff, 0, 150 * nq * sizeof(T));
      if (c.any_rans) {
        P_.Jtoff = m.Alloc<T>(24 * nq);
        c_.mem->Zero(P_.Jtoff, 0, 24 * nq * sizeof(T));
      }
    }
    if (c.block_viscous || c.any_rans) {
      // cell-averaged velocity gradients (block diagonal, SST sources, output)
      P_.vgq = m.Alloc<T>(9 * nq);
      c_.mem->Zero(P_.vgq, 0, 9 * nq * sizeof(T));
    }
    c_.mem->Zero(P_.dUq, 0, 5 * nq * sizeof(T));
    if (c.jkinds) {
      P_.dUq2 = m.Alloc<T>(5 * nq);
      c_.mem->Zero(P_.dUq2, 0, 5 * nq * sizeof(T));
    }
    c_.mem->Zero(P_.dUg, 0, 5 * std::max<int64_t>(ngh, 1) * sizeof(T));
    {
      std::vector<T> lo(c.L.face_lo.begin(), c.L.face_lo.end());
      std::vector<T> hi(c.L.face_hi.begin(), c.L.face_hi.end());
      P_.face_lo = m.Upload(lo);
      P_.face_hi = m.Upload(hi);
    }
    P_.nbq = m.Upload(c.L.nbq);
    {
      std::vector<T> dl(c.L.dist_lo.begin(), c.L.dist_lo.end());
      std::vector<T> dh(c.L.dist_hi.begin(), c.L.dist_hi.end());
      P_.dist_lo = m.Upload(dl);
      P_.dist_hi = m.Upload(dh);
    }
    P_.muq = m.Alloc<T>(c.L.any_viscous ? nq : 1);
    // per-cell neighbour terms of the FP64 scalar sweeps
    if (sizeof(T) == sizeof(double) && (c.kinds & 1)) P_.Npre = m.Alloc<T>(9 * nq);
    P_.qpos = m.Upload(c.L.qpos);
    P_.ghost_cell = m.Upload(c.L.ghost_cell);
    P_.ghost_src = m.Upload(c.L.ghost_src);
    for (int d = 0; d < 3; ++d) c_.mem->Zero(P_.flux[d], 0, 5 * n * sizeof(double));
    if (c.any_rans) AllocTurbulence(m, n, nq, ngh);
    if (!c.L.nrg_cells.empty()) {
      P_.nrg = m.Alloc<double>(12 * (size_t)n);
      c_.mem->Zero(P_.nrg, 0, 12 * (size_t)n * sizeof(double));
    }
    if (c.flags & 4) {
      // the residual's cell gradients kept for output
      P_.ogr = m.Alloc<double>(24 * (size_t)n);
      c_.mem->Zero(P_.ogr, 0, 24 * (size_t)n * sizeof(double));
    }
    if (c.n_nr_surf > 0) {
      P_.nr_mach = m.Alloc<double>(2 * (size_t)c.n_nr_surf);
      c_.mem->Zero(P_.nr_mach, 0, 2 * (size_t)c.n_nr_surf * sizeof(double));
    }
    if (c.any_unsteady) {
      P_.Un = m.Alloc<double>(7 * n);
      P_.Unm1 = m.Alloc<double>(7 * n);
      c_.mem->Zero(P_.Un, 0, 7 * n * sizeof(double));
      c_.mem->Zero(P_.Unm1, 0, 7 * n * sizeof(double));
      P_.Bq = m.Alloc<T>(5 * nq);
      P_.Btq = m.Alloc<T>(2 * nq);
      c_.mem->Zero(P_.Bq, 0, 5 * nq * sizeof(T));
      c_.mem->Zero(P_.Btq, 0, 2 * nq * sizeof(T));
    }
    // geometry and state
    std::vector<double> W(5 * n, 0.0), vol(n, 0.0), wid[3], fa[3];
    for (int d = 0; d < 3; ++d) {
      wid[d].assign(n, 0.0);
      fa[d].assign(4 * n, 0.0);
    }
    for (int bi = 0; bi < c.nblocks; ++bi) {
      const Block &b = c.setup->blocks[bi];
      const int64_t o = c.cell0[bi];
      const int64_t nc = b.NCell();
      for (int64_t x = 0; x < nc; ++x) {
        for (int v = 0; v < 5; ++v) W[v * n + o + x] = b.state0[x * b.nv + v];
        vol[o + x] = b.vol[x];
        for (int d = 0; d < 3; ++d) wid[d][o + x] = b.width[d * nc + x];
      }
      for (int d = 0; d < 3; ++d) {
        const int64_t nf = b.NFace(d);
        const int fi = b.NI + (d == 0), fj = b.NJ + (d == 1);
        for (int64_t f = 0; f < nf; ++f) {
          const int ii = (int)(f % fi);
          const int64_t r = f / fi;
          const int jj = (int)(r % fj);
          const int kk = (int)(r / fj);
          if (ii >= b.NI || jj >= b.NJ || kk >= b.NK) continue;
          const int64_t x = ii + (int64_t)b.NI * (jj + (int64_t)b.NJ * kk);
          for (int q = 0; q < 4; ++q) fa[d][q * n + o + x] = b.farea[d][q * nf + f];
        }
      }
    }
    Check(cudaMemcpyAsync(P_.W, W.data(), W.size() * 8, cudaMemcpyHostToDevice, c_.stream),
          "upload");
    Check(cudaStreamSynchronize(c_.stream), "upload");
    if (c.any_rans) {
      // k, omega of the initial state (0 outside RANS solves)
      std::vector<double> Wt(2 * n, 0.0);
      for (int bi = 0; bi < c.nblocks; ++bi) {
        const Block &b = c.setup->blocks[bi];
        if (b.nv < 7) continue;
        const int64_t o = c.cell0[bi];
        for (int64_t x = 0; x < b.NCell(); ++x) {
          Wt[o + x] = b.state0[x * b.nv + 5];
          Wt[n + o + x] = b.state0[x * b.nv + 6];
        }
      }
      Check(cudaMemcpyAsync(P_.Wt, Wt.data(), Wt.size() * 8, cudaMemcpyHostToDevice, c_.stream),
            "upload");
      Check(cudaStreamSynchronize(c_.stream), "upload");
    }
    if (c.L.any_viscous) {
      // wall distance (SST sources and wall omega, heat-flux walls)
      std::vector<double> wd(n, 0.0);
      for (int bi = 0; bi < c.nblocks; ++bi) {
        const Block &b = c.setup->blocks[bi];
        const int64_t o = c.cell0[bi];
        if (!b.wall_dist.empty())
          for (int64_t x = 0; x < b.NCell(); ++x) wd[o + x] = b.wall_dist[x];
      }
      P_.wd = m.Upload(wd);
    }
    P_.vol = m.Upload(vol);
    for (int d = 0; d < 3; ++d) {
      P_.width[d] = m.Upload(wid[d]);
      P_.fa[d] = m.Upload(fa[d]);
    }
    P_.blocks = c.d_blocks;
    P_.solves = c.d_solves;
    P_.states = c.d_states;
    P_.cfl = c.d_cfl;
    if (c.L.any_viscous) InitialViscosity(m);
    if constexpr (std::is_same<T, double>::value) {
      // FP64 batches: the geometry tables, formed once (the fast option's
      // forms, or the bit-exact ones)
      for (int d = 0; d < 3; ++d) {
        P_.fgeo[d] = m.Alloc<double>(4 * n);
        P_.cgeo[d] = m.Alloc<double>(4 * n);
        c_.mem->Zero(P_.fgeo[d], 0, 4 * n * sizeof(double));
        c_.mem->Zero(P_.cgeo[d], 0, 4 * n * sizeof(double));
      }
      const int nfc[3] = {(int)c.L.face_cta_block[0].size(), (int)c.L.face_cta_block[1].size(),
                          (int)c.L.face_cta_block[2].size()};
      if (P_.fast_fp64)
        LaunchFastGeomFp64(P_, c.d_faces, c.d_face_cta_block, nfc, c.d_cells,
                           c.d_cell_cta_block, (int)c.L.cell_cta_block.size(), c_.stream);
      else
        LaunchExactGeomFp64(P_, c.d_faces, c.d_face_cta_block, nfc, c.d_cells,
                            c.d_cell_cta_block, (int)c.L.cell_cta_block.size(), c_.stream);
      Check(cudaGetLastError(), "kernel launch");
    }
  }

  ~Runner() override {
    if (c_.graph) cudaGraphExecDestroy(c_.graph);
    c_.graph = nullptr;
  }

  const Pools<T> &P() const { return P_; }

  // k, omega and their residual, fluxes, radii, sweep arrays and the
  // per-face SST data (gradients, eddy viscosity, blending)
  void AllocTurbulence(DevMem &m, int64_t n, int64_t nq, int64_t ngh) {
    auto zero = [&](auto *p, size_t count) {
      c_.mem->Zero(p, 0, count * sizeof(*p));
      return p;
    };
    P_.Wt = zero(m.Alloc<double>(2 * n), 2 * n);
    P_.Rt = zero(m.Alloc<double>(2 * n), 2 * n);
    P_.lamt = zero(m.Alloc<double>(n), n);
    for (int d = 0; d < 3; ++d) {
      P_.fluxt[d] = zero(m.Alloc<double>(2 * n), 2 * n);
      P_.vfluxt[d] = zero(m.Alloc<T>(2 * n), 2 * n);
      P_.rst[d] = zero(m.Alloc<T>(19 * n), 19 * n);
    }
    const int64_t aw = (c_.kinds & 2) ? 4 : 1;
    P_.Rtq = zero(m.Alloc<T>(2 * nq), 2 * nq);
    P_.dUtq = zero(m.Alloc<T>(2 * nq), 2 * nq);
    if (c_.jkinds) P_.dUtq2 = zero(m.Alloc<T>(2 * nq), 2 * nq);
    const int64_t g = std::max<int64_t>(ngh, 1);
    P_.dUtg = zero(m.Alloc<T>(2 * g), 2 * g);
    P_.Ainvtq = zero(m.Alloc<T>(aw * nq), aw * nq);
    P_.Atq = zero(m.Alloc<T>(aw * nq), aw * nq);
    P_.mutq = zero(m.Alloc<T>(nq), nq);
    P_.f1q = zero(m.Alloc<T>(nq), nq);
    bool wilcox = false;
    for (const auto &sv : c_.setup->solves) wilcox = wilcox || sv.phys.turb == ATH_TURB_KW2006;
    if (wilcox) P_.nutq = zero(m.Alloc<T>(nq), nq);
    P_.f2q = zero(m.Alloc<T>(nq), nq);
  }

  // gridLevel::AuxillaryAndWidths (src/gridLevel.cpp:433): laminar
  // viscosity of the physical cells of the initial state (the wall ghost
  // omega of the first iteration reads it); only >= 0: that block's
  void InitialViscosity(DevMem &m, int only = -1) {
    std::vector<int32_t> cells, blk;
    for (int bi = 0; bi < c_.nblocks; ++bi) {
      if (only >= 0 && bi != only) continue;
      const Block &b = c_.setup->blocks[bi];
      if (c_.setup->solves[b.solve].phys.eqn == ATH_EQN_EULER) continue;
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i) {
            cells.push_back((int32_t)(c_.cell0[bi] + b.Cell(i, j, k)));
            blk.push_back(bi);
          }
    }
    if (cells.empty()) return;
    int32_t *dc = m.Upload(cells), *db = m.Upload(blk);
    Launch<T>::Aux(P_, dc, db, (int)cells.size(), c_.stream);
    Check(cudaStreamSynchronize(c_.stream), "sync");
    m.Free(dc);
    m.Free(db);
  }

  void StartIteration() {
    k_cfl<<<(c_.nsolves + 127) / 128, 128, 0, c_.stream>>>(c_.d_solves, c_.nsolves,
                                                            c_.d_sstate, c_.d_cfl);
  }
  void EdgePhases(const GhostOpDev *ops, const int32_t *solve,
                  const std::vector<int32_t> &off) {
    for (size_t ph = 0; ph + 1 < off.size(); ++ph)
      Launch<T>::Ghost(P_, ops + off[ph], off[ph + 1] - off[ph], solve + off[ph], c_.stream);
  }
  void FillGhosts() override {
    StartIteration();
    if (c_.any_unsteady)
      Launch<T>::StoreN(P_, c_.d_cells, c_.d_cell_cta_block, (int)c_.L.cell_cta_block.size(),
                        c_.d_sstate, -1, c_.stream);
    if (c_.n_nr_surf > 0) Launch<T>::NrMach(P_, c_.d_nr, c_.d_nr_off, c_.n_nr_surf, c_.stream);
    Launch<T>::Ghost(P_, c_.d_ops, (int)c_.L.ops.size(), c_.d_op_solve, c_.stream);
    EdgePhases(c_.d_edge_ops, c_.d_edge_solve, c_.L.edge_phase_off);
  }
  void Viscous() {
    if (!c_.L.any_viscous) return;
    Launch<T>::Ghost(P_, c_.d_vops, (int)c_.L.vops.size(), c_.d_vop_solve, c_.stream);
    EdgePhases(c_.d_vedge_ops, c_.d_vedge_solve, c_.L.vedge_phase_off);
    Launch<T>::Aux(P_, c_.d_aux_cells, c_.d_aux_block, (int)c_.L.aux_cells.size(), c_.stream);
    for (int d = 0; d < 3; ++d)
      Launch<T>::ViscFace(d, P_, c_.d_faces[d], c_.d_face_cta_block[d],
                          (int)c_.L.face_cta_block[d].size(), c_.vkinds, c_.stream);
    const int nw = (int)c_.L.wall_faces.size();
    if (nw > 0) {
      Launch<T>::Wall(P_, c_.d_wall_faces, nw, c_.d_wbuf, c_.stream);
      k_wallsum<<<c_.nsolves, 32, 0, c_.stream>>>(c_.d_wbuf, nw, c_.d_solve_face0, c_.nsolves,
                                                  c_.d_fring, c_.ring_cap, c_.d_iter);
    }
  }
  // gradients the nonreflecting outlets read at the next ghost fill, from
  // this residual's state and ghosts (viscous ghosts included)
  void NrGrads() {
    Launch<T>::NrGrads(P_, c_.d_nrg_cells, c_.d_nrg_block, (int)c_.L.nrg_cells.size(),
                       c_.stream);
    if (P_.ogr)
      Launch<T>::OutGrads(P_, c_.d_cells, c_.d_cell_cta_block, (int)c_.L.cell_cta_block.size(),
                          c_.fkinds, c_.stream);
  }
  void Residual() override {
    for (int d = 0; d < 3; ++d)
      Launch<T>::Face(d, P_, c_.d_faces[d], c_.d_face_cta_block[d],
                      (int)c_.L.face_cta_block[d].size(), FaceKinds(), c_.stream);
    Viscous();
    NrGrads();
    Launch<T>::Cell(P_, c_.d_cells, c_.d_cell_cta_block, (int)c_.L.cell_cta_block.size(),
                    c_.kinds, c_.stream);
    if (c_.kinds & 2)
      Launch<T>::OffJac(P_, c_.d_sweep, (int)c_.L.sweep_items.size(), c_.stream);
  }
  // face kernels to launch: the batch's solve kinds, plus bit 2 for the
  // fast FP64 faces (batch flag bit 1)
  // bit 2: the fast faces; bit 3: the solves without turbulence equations
  // are all MUSCL-Roe
  int FaceKinds() const {
    return c_.fkinds | ((c_.flags & 2) ? 4 : 0) | (c_.mr_only ? 8 : 0);
  }
  void SweepPass(int forward, int sweep) {
    const bool full = c_.max_sweeps > 1;
    if (c_.sweep_mode == 3) {
      auto &lists = c_.tq.at(c_.tq_size);
      for (int kind = 0; kind < 2; ++kind) {
        if (!(c_.skinds & (1 << kind))) continue;
        const BatchCore::TqList &t = lists[kind * 2 + (forward ? 0 : 1)];
        if (t.ntiles == 0) continue;
        Check(cudaMemsetAsync(t.done, 0, (size_t)(t.ntiles + 1) * sizeof(int), c_.stream),
              "memset");
        Check(cudaMemsetAsync(c_.d_tq_ticket, 0, sizeof(int), c_.stream), "memset");
        TileQueueDev Q{c_.d_cl_items, t.tiles,      t.deps,
                       t.done,        c_.d_tq_ticket, c_.d_tq_status,
                       t.ntiles,      c_.tq_wait_never, c_.tq_spin_limit};
        Launch<T>::SweepTq(P_, Q, forward, sweep, full, kind == 1, c_.tq_ctas[kind],
                           c_.stream);
      }
      return;
    }
    if (c_.sweep_mode == 1) {
      Launch<T>::SweepCl(P_, c_.Lists(), forward, sweep, full, c_.skinds, c_.cl_threads,
                         c_.cl_size, c_.stream);
      return;
    }
    // K concurrent chains: solve groups g0..g1 of kSweepGroups each, the
    // first on the batch's stream, the others forked and joined back
    const int K = c_.sweep_mode == 4 ? 1 : c_.sweep_groups;
    if (K > 1) {
      Check(cudaEventRecord(c_.gfork, c_.stream), "event");
      for (int g = 1; g < K; ++g) Check(cudaStreamWaitEvent(c_.gstream[g - 1], c_.gfork, 0), "event");
    }
    constexpr int W = kSweepGroups + 1;
    for (int g = 0; g < K; ++g) {
      cudaStream_t st = g == 0 ? c_.stream : c_.gstream[g - 1];
      const int g0 = g * kSweepGroups / K, g1 = (g + 1) * kSweepGroups / K;
      // a plane's launch is chained to the chain's previous launch only
      bool chained = false;
      for (int k = 0; k < c_.nsteps; ++k) {
        const int s = forward ? k : c_.nsteps - 1 - k;
        const int a = c_.L.gstep_off[(size_t)s * W + g0], b = c_.L.gstep_off[(size_t)s * W + g1];
        if (b <= a) continue;
        PlaneSweep(a, b - a, forward, sweep, full, chained, st);
        chained = true;
      }
    }
    if (K > 1) {
      for (int g = 1; g < K; ++g) {
        Check(cudaEventRecord(c_.gjoin[g - 1], c_.gstream[g - 1]), "event");
        Check(cudaStreamWaitEvent(c_.stream, c_.gjoin[g - 1], 0), "event");
      }
    }
  }
  // one hyperplane's launch in the batch's sweep shape (mode 0: a thread
  // per cell, 2: lane groups, 4: lane groups below hy_items cells)
  void PlaneSweep(int a, int n, int forward, int sweep, bool full, bool chained,
                  cudaStream_t st) {
    const bool group =
        c_.sweep_mode == 2 || (c_.sweep_mode == 4 && n < c_.hy_items);
    const int threads = (c_.sweep_mode == 4 && !group) ? 128 : c_.sweep_threads;
    Launch<T>::Sweep(P_, c_.d_sweep + a, n, forward, sweep, full, c_.skinds, threads, group,
                     chained, st);
  }
  void ZeroGhostUpdates() {
    if (P_.nghost <= 0) return;
    Check(cudaMemsetAsync(P_.dUg, 0, 5 * P_.nghost * sizeof(T), c_.stream), "memset");
    if (P_.dUtg)
      Check(cudaMemsetAsync(P_.dUtg, 0, 2 * P_.nghost * sizeof(T), c_.stream), "memset");
  }
  // dplur::Relax (src/linearSolver.cpp:501): x0 = A^-1 b, then per sweep a
  // ghost swap and one Jacobi pass over every cell at once, alternating
  // between the two update buffers; the final iterate ends in dUq
  void JacobiPhase() {
    const int n = (int)c_.L.sweep_items.size();
    Launch<T>::Init(P_, c_.d_sweep, n, 1, c_.stream);
    Pools<T> other = P_;
    other.dUq = P_.dUq2;
    other.dUtq = P_.dUtq2;
    for (int sw = 0; sw < c_.max_jsweeps; ++sw) {
      const bool even = sw % 2 == 0;
      const Pools<T> &src = even ? P_ : other;
      Launch<T>::ConnDu(src, c_.stream);
      Launch<T>::Jacobi(src, even ? P_.dUq2 : P_.dUq, even ? P_.dUtq2 : P_.dUtq, c_.d_sweep, n,
                        sw, c_.jkinds, c_.stream);
    }
    if (c_.max_jsweeps % 2 == 1)
      Launch<T>::JacobiCopy(P_, P_.dUq2, P_.dUtq2, c_.d_sweep, n, c_.stream);
  }
  // lusgs::Relax (src/linearSolver.cpp:430): dU ghost swap before every
  // pass and after the last one
  void SweepPhase() {
    if (c_.max_sweeps <= 1) {
      // x = 0 before the first sweep: only the connection ghosts are read
      // before being written
      ZeroGhostUpdates();
      SweepPass(1, 0);
      Launch<T>::ConnDu(P_, c_.stream);
      SweepPass(0, 0);
    } else {
      Launch<T>::Init(P_, c_.d_sweep, (int)c_.L.sweep_items.size(), 0, c_.stream);
      for (int sw = 0; sw < c_.max_sweeps; ++sw) {
        Launch<T>::ConnDu(P_, c_.stream);
        SweepPass(1, sw);
        Launch<T>::ConnDu(P_, c_.stream);
        SweepPass(0, sw);
      }
    }
  }
  // ---- multigrid (mgSolution::CycleAtLevel, src/mgSolution.cpp:160-207)
  // this batch is the finest level; mg_lv_[l] is level l's runner (its own
  // batch on this batch's stream), mg_link_[l] the transfer from level l to
  // l+1, with its coarse level's saved update and node buffer
  void MgAddLevel(Runner<T> *coarse, const MgLinkDev &link, T *du0, T *nodes) {
    if (mg_lv_.empty()) mg_lv_.push_back(this);
    mg_lv_.push_back(coarse);
    mg_link_.push_back(link);
    mg_du0_.push_back(du0);
    mg_nodes_.push_back(nodes);
  }
  void MgSetup(int cycle, int sweeps) {
    mg_cycle_ = cycle;
    mg_sweeps_ = sweeps;
  }
  Pools<T> &MutablePools() { return P_; }
  BatchCore &Core() { return c_; }
  // a coarse level's ghost fill (the CFL is the finest level's, copied)
  void LevelGhosts() {
    Launch<T>::Ghost(P_, c_.d_ops, (int)c_.L.ops.size(), c_.d_op_solve, c_.stream);
    EdgePhases(c_.d_edge_ops, c_.d_edge_solve, c_.L.edge_phase_off);
  }
  // Relax of one level with n sweeps from its current update (lusgs / dplur
  // ::Relax, src/linearSolver.cpp:430,501), ending with the ghost swap and
  // the per-cell matrix residual f - (A x - b) into MRq
  void RelaxN(int n) {
    if (c_.jkinds) {
      const int ni = (int)c_.L.sweep_items.size();
      Pools<T> other = P_;
      other.dUq = P_.dUq2;
      other.dUtq = P_.dUtq2;
      for (int sw = 0; sw < n; ++sw) {
        const bool even = sw % 2 == 0;
        const Pools<T> &src = even ? P_ : other;
        Launch<T>::ConnDu(src, c_.stream);
        Launch<T>::Jacobi(src, even ? P_.dUq2 : P_.dUq, even ? P_.dUtq2 : P_.dUtq, c_.d_sweep, ni,
                          sw, c_.jkinds, c_.stream);
      }
      if (n % 2 == 1) Launch<T>::JacobiCopy(P_, P_.dUq2, P_.dUtq2, c_.d_sweep, ni, c_.stream);
    }
    if (c_.skinds) {
      for (int sw = 0; sw < n; ++sw) {
        Launch<T>::ConnDu(P_, c_.stream);
        SweepPass(1, sw);
        Launch<T>::ConnDu(P_, c_.stream);
        SweepPass(0, sw);
      }
    }
    Launch<T>::ConnDu(P_, c_.stream);
    Launch<T>::MatRes(P_, c_.d_cells, c_.d_cell_cta_block, c_.d_mres,
                      (int)c_.L.cell_cta_block.size(), c_.kinds, c_.stream);
  }
  void MgCycle(int l) {
    Runner<T> &R = *mg_lv_[l];
    if (l + 1 == (int)mg_lv_.size()) {
      R.RelaxN(mg_sweeps_);
      return;
    }
    const int half = std::max(mg_sweeps_ / 2, 1);
    R.RelaxN(half);
    Runner<T> &C = *mg_lv_[l + 1];
    Pools<T> &CP = C.MutablePools();
    BatchCore &cc = C.Core();
    const MgLinkDev &k = mg_link_[l];
    cudaStream_t s = c_.stream;
    // gridLevel::Restriction (src/gridLevel.cpp:538): the state (into a
    // zeroed pool, ghosts refilled), the coarse residual, time step and
    // diagonal from it, the update with its ghost swap, and the forcing
    Check(cudaMemsetAsync(CP.W, 0, 5 * (size_t)CP.ncell * sizeof(double), s), "memset");
    Launch<T>::MgRestrictState(k, R.P_.W, R.P_.ncell, CP.W, CP.ncell, s);
    k_mg_sync<<<(cc.nsolves + 127) / 128, 128, 0, s>>>(c_.d_solves, c_.d_cfl, cc.d_solves,
                                                       cc.d_cfl, cc.nsolves);
    CP.mg_accum = ++mg_visits_[l + 1] > 1 ? 1 : 0;
    C.LevelGhosts();
    C.Residual();
    Launch<T>::MgRestrictQ(k, R.P_.dUq, R.P_.nq, CP.dUq, CP.nq, true, s);
    Launch<T>::ConnDu(CP, s);
    Launch<T>::MgRestrictQ(k, R.P_.MRq, R.P_.nq, CP.Fq, CP.nq, false, s);
    Launch<T>::MgForcing(CP, cc.d_cells, cc.d_cell_cta_block, (int)cc.L.cell_cta_block.size(),
                         cc.kinds, s);
    T *du0 = mg_du0_[l];
    Check(cudaMemcpyAsync(du0, CP.dUq, 5 * (size_t)CP.nq * sizeof(T), cudaMemcpyDeviceToDevice,
                          s),
          "copy");
    for (int n = 0; n < mg_cycle_; ++n) MgCycle(l + 1);
    Launch<T>::MgSubtract(CP.dUq, du0, CP.nq, s);
    Launch<T>::MgProlong(k, CP.dUq, CP.nq, mg_nodes_[l], R.P_.dUq, R.P_.nq, s);
    R.RelaxN(half);
  }
  // the finest level's relaxation with the coarse-grid corrections:
  // InitializeMatrixUpdate (A^-1 b or zero), then the cycle
  void MgRelax() {
    const int ni = (int)c_.L.sweep_items.size();
    if (c_.jkinds) Launch<T>::Init(P_, c_.d_sweep, ni, 1, c_.stream);
    if (c_.skinds) Launch<T>::Init(P_, c_.d_sweep, ni, 0, c_.stream);
    mg_visits_.assign(mg_lv_.size(), 0);
    MgCycle(0);
  }
  bool Multigrid() const { return !mg_lv_.empty(); }

  void Relax() override {
    if (Multigrid()) {
      MgRelax();
      return;
    }
    if (c_.jkinds) JacobiPhase();
    if (c_.skinds) SweepPhase();
    if (c_.flags & 1) {
      Launch<T>::ConnDu(P_, c_.stream);
      Launch<T>::MatRes(P_, c_.d_cells, c_.d_cell_cta_block, c_.d_mres,
                        (int)c_.L.cell_cta_block.size(), c_.kinds, c_.stream);
    }
  }
  void Update() override {
    Launch<T>::Update(P_, c_.d_cells, c_.d_cell_cta_block, c_.d_cell_cta_pos0,
                      c_.d_partials, (int)c_.L.cell_cta_block.size(), c_.d_sstate, c_.stream);
    k_norms<<<c_.nsolves, 32, 0, c_.stream>>>(c_.d_partials,
                                              (c_.flags & 1) ? c_.d_mres : nullptr,
                                              c_.d_solve_cta0, c_.nsolves, c_.d_ring,
                                              c_.ring_cap, c_.d_iter, c_.d_solves,
                                              c_.d_sstate, c_.d_cfl);
    k_iter_advance<<<1, 1, 0, c_.stream>>>(c_.d_iter);
  }
  void OneIteration() {
    FillGhosts();
    Residual();
    Relax();
    Update();
  }
  void Iterate(int n) override {
    if (!c_.graph) {
      cudaGraph_t g;
      Check(cudaStreamBeginCapture(c_.stream, cudaStreamCaptureModeThreadLocal),
            "begin capture");
      OneIteration();
      Check(cudaStreamEndCapture(c_.stream, &g), "end capture");
      // kernel launches of one iteration: the captured graph's kernel nodes
      size_t nn = 0;
      Check(cudaGraphGetNodes(g, nullptr, &nn), "graph nodes");
      std::vector<cudaGraphNode_t> nodes(nn);
      if (nn) Check(cudaGraphGetNodes(g, nodes.data(), &nn), "graph nodes");
      int64_t kernels = 0;
      for (auto nd : nodes) {
        cudaGraphNodeType t;
        Check(cudaGraphNodeGetType(nd, &t), "graph node type");
        kernels += t == cudaGraphNodeTypeKernel;
      }
      c_.launches_per_iter = kernels;
      Check(cudaGraphInstantiate(&c_.graph, g, 0), "graph instantiate");
      cudaGraphDestroy(g);
    }
    for (int i = 0; i < n; ++i) Check(cudaGraphLaunch(c_.graph, c_.stream), "graph launch");
  }
  void Profile(int reps, double ms[8]) override {
    cudaEvent_t e[9];
    for (auto &x : e) Check(cudaEventCreate(&x), "event");
    for (int q = 0; q < 8; ++q) ms[q] = 0.0;
    for (int r = 0; r < reps; ++r) {
      Check(cudaEventRecord(e[0], c_.stream), "event");
      FillGhosts();
      Check(cudaEventRecord(e[1], c_.stream), "event");
      for (int d = 0; d < 3; ++d) {
        Launch<T>::Face(d, P_, c_.d_faces[d], c_.d_face_cta_block[d],
                        (int)c_.L.face_cta_block[d].size(), FaceKinds(), c_.stream);
        Check(cudaEventRecord(e[2 + d], c_.stream), "event");
      }
      Viscous();
      NrGrads();
      Launch<T>::Cell(P_, c_.d_cells, c_.d_cell_cta_block, (int)c_.L.cell_cta_block.size(),
                      c_.kinds, c_.stream);
      if (c_.kinds & 2)
        Launch<T>::OffJac(P_, c_.d_sweep, (int)c_.L.sweep_items.size(), c_.stream);
      Check(cudaEventRecord(e[5], c_.stream), "event");
      // forward passes, then backward passes (one-sweep form; the timing
      // split of a multi-sweep relaxation puts each sweep's passes in turn);
      // DP-LUR sweeps count as forward passes
      float fwd = 0.f, bwd = 0.f;
      if (Multigrid()) {
        // the whole multigrid cycle counts as the forward passes
        Check(cudaEventRecord(e[6], c_.stream), "event");
        MgRelax();
        Check(cudaEventRecord(e[7], c_.stream), "event");
        Check(cudaEventSynchronize(e[7]), "sync");
        Check(cudaEventElapsedTime(&fwd, e[6], e[7]), "elapsed");
      } else if (c_.jkinds) {
        Check(cudaEventRecord(e[6], c_.stream), "event");
        JacobiPhase();
        Check(cudaEventRecord(e[7], c_.stream), "event");
        Check(cudaEventSynchronize(e[7]), "sync");
        float tj = 0.f;
        Check(cudaEventElapsedTime(&tj, e[6], e[7]), "elapsed");
        fwd += tj;
      }
      const bool lusgs = c_.skinds && !Multigrid();
      if (lusgs && c_.max_sweeps > 1)
        Launch<T>::Init(P_, c_.d_sweep, (int)c_.L.sweep_items.size(), 0, c_.stream);
      else if (lusgs)
        ZeroGhostUpdates();
      for (int sw = 0; sw < (lusgs ? c_.max_sweeps : 0); ++sw) {
        if (c_.max_sweeps > 1) Launch<T>::ConnDu(P_, c_.stream);
        Check(cudaEventRecord(e[6], c_.stream), "event");
        SweepPass(1, sw);
        Check(cudaEventRecord(e[7], c_.stream), "event");
        Launch<T>::ConnDu(P_, c_.stream);
        SweepPass(0, sw);
        Check(cudaEventRecord(e[8], c_.stream), "event");
        Check(cudaEventSynchronize(e[8]), "sync");
        float t1 = 0.f, t2 = 0.f;
        Check(cudaEventElapsedTime(&t1, e[6], e[7]), "elapsed");
        Check(cudaEventElapsedTime(&t2, e[7], e[8]), "elapsed");
        fwd += t1;
        bwd += t2;
      }
      Check(cudaEventRecord(e[6], c_.stream), "event");
      Update();
      c_.iter_host += 1;
      Check(cudaEventRecord(e[7], c_.stream), "event");
      Check(cudaEventSynchronize(e[7]), "sync");
      for (int q = 0; q < 5; ++q) {
        float t = 0.f;
        Check(cudaEventElapsedTime(&t, e[q], e[q + 1]), "elapsed");
        ms[q] += t;
      }
      float tu = 0.f;
      Check(cudaEventElapsedTime(&tu, e[6], e[7]), "elapsed");
      ms[5] += fwd;
      ms[6] += bwd;
      ms[7] += tu;
    }
    for (int q = 0; q < 8; ++q) ms[q] /= std::max(reps, 1);
    for (auto &x : e) cudaEventDestroy(x);
  }
  void ResetGraph() override {
    if (c_.graph) cudaGraphExecDestroy(c_.graph);
    c_.graph = nullptr;
  }
  int MaxClusters(int kinds, int threads, int cluster) override {
    return Launch<T>::MaxClusters(kinds, threads, cluster);
  }
  int TqOccupancy(bool full, bool block) override { return Launch<T>::TqOccupancy(full, block); }
  void Snapshot(bool restore) override {
    DevMem &m = *c_.mem;
    const size_t wbytes = 5 * (size_t)c_.ncell * sizeof(double);
    if (!snap_w_) {
      snap_w_ = m.Alloc<double>(5 * (size_t)c_.ncell);
      if (P_.Wt) snap_wt_ = m.Alloc<double>(2 * (size_t)c_.ncell);
      if (P_.Un) snap_un_ = m.Alloc<double>(14 * (size_t)c_.ncell);
      snap_ss_ = m.Alloc<SolveState>(c_.nsolves);
      snap_sv_ = m.Alloc<SolveDev>(c_.nsolves);
      snap_cfl_ = m.Alloc<double>(c_.nsolves);
      snap_it_ = m.Alloc<int64_t>(1);
    }
    auto cp = [&](void *dst, const void *src, size_t bytes) {
      Check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c_.stream), "snapshot");
    };
    if (!restore) {
      cp(snap_w_, P_.W, wbytes);
      if (P_.Wt) cp(snap_wt_, P_.Wt, wbytes / 5 * 2);
      if (P_.Un) {
        cp(snap_un_, P_.Un, wbytes / 5 * 7);
        cp(snap_un_ + 7 * (size_t)c_.ncell, P_.Unm1, wbytes / 5 * 7);
      }
      cp(snap_ss_, c_.d_sstate, c_.nsolves * sizeof(SolveState));
      cp(snap_sv_, c_.d_solves, c_.nsolves * sizeof(SolveDev));
      cp(snap_cfl_, c_.d_cfl, c_.nsolves * sizeof(double));
      cp(snap_it_, c_.d_iter, sizeof(int64_t));
      snap_iter_host_ = c_.iter_host;
    } else {
      cp(P_.W, snap_w_, wbytes);
      if (P_.Wt) cp(P_.Wt, snap_wt_, wbytes / 5 * 2);
      if (P_.Un) {
        cp(P_.Un, snap_un_, wbytes / 5 * 7);
        cp(P_.Unm1, snap_un_ + 7 * (size_t)c_.ncell, wbytes / 5 * 7);
      }
      cp(c_.d_sstate, snap_ss_, c_.nsolves * sizeof(SolveState));
      cp(c_.d_solves, snap_sv_, c_.nsolves * sizeof(SolveDev));
      cp(c_.d_cfl, snap_cfl_, c_.nsolves * sizeof(double));
      cp(c_.d_iter, snap_it_, sizeof(int64_t));
      c_.iter_host = snap_iter_host_;
    }
    Check(cudaStreamSynchronize(c_.stream), "sync");
  }
  void FreeSnapshot() override {
    if (!snap_w_) return;
    DevMem &m = *c_.mem;
    m.Free(snap_w_);
    if (snap_wt_) m.Free(snap_wt_);
    snap_wt_ = nullptr;
    if (snap_un_) m.Free(snap_un_);
    snap_un_ = nullptr;
    m.Free(snap_ss_);
    m.Free(snap_sv_);
    m.Free(snap_cfl_);
    m.Free(snap_it_);
    snap_w_ = nullptr;
  }
  void GetDU(int b, double *out) override {
    const int nv = c_.setup->blocks[b].nv;
    CopyOutQ(P_.dUq, 5, nv, 0, b, out);
    if (nv > 5) CopyOutQ(P_.dUtq, 2, nv, 5, b, out);
  }
  void GetAinv(int b, double *out) override { CopyOutQ(P_.Ainvq, 1, 1, 0, b, out); }
  void RefreshAux(int b) override { InitialViscosity(*c_.mem, b); }
  void StoreTimeLevels(int b) override {
    Launch<T>::StoreN(P_, c_.d_cells, c_.d_cell_cta_block, (int)c_.L.cell_cta_block.size(),
                      c_.d_sstate, b, c_.stream);
    Check(cudaGetLastError(), "kernel launch");
    Check(cudaStreamSynchronize(c_.stream), "sync");
  }
  void GetAux(int bi, double *out) override {
    const Block &b = c_.setup->blocks[bi];
    const auto &ph = c_.setup->solves[b.solve].phys;
    const size_t m = (size_t)b.ni * b.nj * b.nk;
    std::fill(out, out + 5 * m, 0.0);
    if (ph.eqn != ATH_EQN_EULER) {
      GatherPool(P_.Taux, bi, 5, 0, out);
      GatherPool(P_.mu, bi, 5, 1, out);
    } else {
      // idealGas::Temperature (src/eos.cpp:100) of the current state
      std::vector<double> w(5 * m);
      for (int v = 0; v < 5; ++v) GatherPool(P_.W + v * c_.ncell, bi, 5, v, w.data());
      for (size_t q = 0; q < m; ++q) out[5 * q] = w[5 * q + 4] / (0.0 + w[5 * q] * ph.gas_r);
    }
    if (ph.eqn == ATH_EQN_RANS) {
      CopyOutQ(P_.mutq, 1, 5, 2, bi, out);
      CopyOutQ(P_.f1q, 1, 5, 3, bi, out);
      CopyOutQ(P_.f2q, 1, 5, 4, bi, out);
    }
  }
  void GetVelGrad(int bi, double *out) override {
    const Block &b = c_.setup->blocks[bi];
    const auto &ph = c_.setup->solves[b.solve].phys;
    const bool have = ph.eqn == ATH_EQN_RANS ||
                      (ph.eqn != ATH_EQN_EULER && IsBlockSolver(ph.solver));
    if (!have || !P_.vgq)
      throw Error(ATH_ERR_UNSUPPORTED, "cell velocity gradients are kept for block LU-SGS "
                                       "viscous and SST solves only");
    CopyOutQ(P_.vgq, 9, 9, 0, bi, out);
  }

 private:
  template <typename U>
  void CopyOut(const U *pool, int w, int bi, double *out) {
    const Block &b = c_.setup->blocks[bi];
    const int64_t nc = b.NCell(), o = c_.cell0[bi], n = c_.ncell;
    std::vector<U> h(nc);
    size_t q = 0;
    std::vector<double> tmp((size_t)b.ni * b.nj * b.nk * w);
    for (int v = 0; v < w; ++v) {
      Check(cudaMemcpy(h.data(), pool + v * n + o, nc * sizeof(U), cudaMemcpyDeviceToHost),
            "download");
      q = 0;
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i) tmp[(q++) * w + v] = (double)h[b.Cell(i, j, k)];
    }
    std::memcpy(out, tmp.data(), tmp.size() * sizeof(double));
  }

  // one cell-indexed FP64 pool -> physical cells of block bi, AoS with
  // `stride` values per cell at `voff`, k slowest
  void GatherPool(const double *pool, int bi, int stride, int voff, double *out) {
    const Block &b = c_.setup->blocks[bi];
    const int64_t nc = b.NCell(), o = c_.cell0[bi];
    std::vector<double> h(nc);
    Check(cudaMemcpy(h.data(), pool + o, nc * sizeof(double), cudaMemcpyDeviceToHost),
          "download");
    size_t q = 0;
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i < b.ni; ++i) out[(q++) * stride + voff] = h[b.Cell(i, j, k)];
  }

  // q-ordered array of w values -> physical cells of block bi, AoS with
  // `stride` values per cell starting at `voff`, k slowest
  template <typename U>
  void CopyOutQ(const U *arr, int w, int stride, int voff, int bi, double *out) {
    const Block &b = c_.setup->blocks[bi];
    const int64_t cnt = (int64_t)b.ni * b.nj * b.nk, q0 = c_.L.q0[bi];
    std::vector<U> h(cnt);
    for (int v = 0; v < w; ++v) {
      Check(cudaMemcpy(h.data(), arr + v * c_.nq + q0, cnt * sizeof(U),
                       cudaMemcpyDeviceToHost),
            "download");
      size_t q = 0;
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i)
            out[(q++) * stride + voff + v] =
                (double)h[c_.L.qpos[c_.cell0[bi] + b.Cell(i, j, k)] - q0];
    }
  }

  BatchCore &c_;
  std::vector<Runner<T> *> mg_lv_;
  std::vector<MgLinkDev> mg_link_;
  std::vector<T *> mg_du0_, mg_nodes_;
  std::vector<int> mg_visits_;
  int mg_cycle_ = 1, mg_sweeps_ = 1;
  Pools<T> P_{};
  double *snap_w_ = nullptr, *snap_wt_ = nullptr, *snap_un_ = nullptr, *snap_cfl_ = nullptr;
  SolveState *snap_ss_ = nullptr;
  SolveDev *snap_sv_ = nullptr;
  int64_t *snap_it_ = nullptr, snap_iter_host_ = 0;
};

}  // namespace ath

struct ath_batch {
  ath::BatchCore core;
  std::unique_ptr<ath::RunnerBase> run;
  // coarser multigrid levels: batches of their own on this batch's stream,
  // driven by this batch's relaxation
  std::vector<ath_batch *> levels;
  double *W = nullptr, *R = nullptr, *dt = nullptr, *lam = nullptr;
  double *Wt = nullptr, *Rt = nullptr, *lamt = nullptr;  // RANS solves only
  double *Un = nullptr, *Unm1 = nullptr;  // time-accurate solves only
  double *ogr = nullptr;  // output gradients (flag ATH_BATCH_OUTPUT_GRADS)
};

namespace ath {
namespace {

void BuildLists(BatchCore &c) {
  const auto &st = *c.setup;
  auto &L = c.L;
  c.cell0.resize(c.nblocks);
  c.solve_pos0.resize(c.nblocks);
  int64_t off = 0;
  for (int b = 0; b < c.nblocks; ++b) {
    c.cell0[b] = off;
    off += st.blocks[b].NCell();
  }
  c.ncell = off;
  if (off >= (int64_t)INT32_MAX) throw Error(ATH_ERR_UNSUPPORTED, "batch too large");
  // physical cells, padded per block to whole CTAs
  L.solve_cta0.assign(c.nsolves + 1, 0);
  for (int s = 0; s < c.nsolves; ++s) {
    L.solve_cta0[s] = (int32_t)L.cell_cta_block.size();
    int64_t pos = 0;
    for (int b : st.solves[s].blocks) {
      const Block &bk = st.blocks[b];
      c.solve_pos0[b] = pos;
      const int64_t start = (int64_t)L.cells.size();
      for (int k = 0; k < bk.nk; ++k)
        for (int j = 0; j < bk.nj; ++j)
          for (int i = 0; i < bk.ni; ++i)
            L.cells.push_back((int32_t)(c.cell0[b] + bk.Cell(i, j, k)));
      const int64_t cnt = (int64_t)L.cells.size() - start;
      const int64_t ncta = (cnt + kCta - 1) / kCta;
      L.cells.resize(start + ncta * kCta, -1);
      for (int64_t t = 0; t < ncta; ++t) {
        L.cell_cta_block.push_back(b);
        L.cell_cta_pos0.push_back((int32_t)(pos + t * kCta));
      }
      pos += cnt;
    }
  }
  L.solve_cta0[c.nsolves] = (int32_t)L.cell_cta_block.size();
  // faces per direction
  for (int d = 0; d < 3; ++d) {
    for (int b = 0; b < c.nblocks; ++b) {
      const Block &bk = st.blocks[b];
      const int64_t start = (int64_t)L.faces[d].size();
      for (int k = 0; k < bk.nk + (d == 2); ++k)
        for (int j = 0; j < bk.nj + (d == 1); ++j)
          for (int i = 0; i < bk.ni + (d == 0); ++i)
            L.faces[d].push_back((int32_t)(c.cell0[b] + bk.Cell(i, j, k)));
      const int64_t cnt = (int64_t)L.faces[d].size() - start;
      const int64_t ncta = (cnt + kCta - 1) / kCta;
      L.faces[d].resize(start + ncta * kCta, -1);
      for (int64_t t = 0; t < ncta; ++t) L.face_cta_block[d].push_back(b);
    }
  }
  // hyperplane-ordered (q) numbering of the physical cells: block by block,
  // in each block the reference's visit order (plane, then k, then j)
  L.q0.assign(c.nblocks + 1, 0);
  for (int b = 0; b < c.nblocks; ++b)
    L.q0[b + 1] = L.q0[b] + (int64_t)st.blocks[b].ni * st.blocks[b].nj * st.blocks[b].nk;
  c.nq = L.q0[c.nblocks];
  L.qpos.assign(c.ncell, -1);
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &bk = st.blocks[b];
    for (size_t q = 0; q < bk.plane_cells.size(); ++q)
      L.qpos[c.cell0[b] + bk.plane_cells[q]] = (int32_t)(L.q0[b] + (int64_t)q);
  }
  // connection ghosts adjacent to a physical cell (layer 1): their W and dU
  // enter the off-diagonal sums
  std::vector<int32_t> ghost_slot(c.ncell, -1);
  for (int b = 0; b < c.nblocks; ++b) {
    for (const auto &op : st.blocks[b].ops) {
      if (op.layer != 1 || (op.type != ATH_BC_PERIODIC && op.type != ATH_BC_INTERBLOCK)) continue;
      const int64_t gcell = c.cell0[b] + op.dst;
      if (ghost_slot[gcell] >= 0) continue;
      ghost_slot[gcell] = (int32_t)L.ghost_cell.size();
      L.ghost_cell.push_back((int32_t)gcell);
      const int32_t src_q = L.qpos[c.cell0[op.src_block] + op.src];
      if (src_q < 0) throw Error(ATH_ERR_ARG, "connection donor is not a physical cell");
      L.ghost_src.push_back(src_q);
    }
  }
  const int64_t nq = c.nq;
  L.nbq.assign(6 * nq, -1);
  L.face_lo.assign(12 * nq, 0.0);
  L.face_hi.assign(12 * nq, 0.0);
  L.dist_lo.assign(3 * nq, 1.0);
  L.dist_hi.assign(3 * nq, 1.0);
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &bk = st.blocks[b];
    const int64_t st3[3] = {1, (int64_t)bk.NI, (int64_t)bk.NI * bk.NJ};
    const int nd[3] = {bk.ni, bk.nj, bk.nk};
    for (size_t ql = 0; ql < bk.plane_cells.size(); ++ql) {
      const int64_t q = L.q0[b] + (int64_t)ql;
      const int64_t cl = bk.plane_cells[ql];
      const int ijk[3] = {(int)(cl % bk.NI) - bk.ng, (int)((cl / bk.NI) % bk.NJ) - bk.ng,
                          (int)(cl / ((int64_t)bk.NI * bk.NJ)) - bk.ng};
      const uint8_t m = bk.nbr_mask[cl];
      for (int d = 0; d < 3; ++d) {
        for (int up = 0; up < 2; ++up) {
          const int64_t nbl = up ? cl + st3[d] : cl - st3[d];
          int32_t code = -1;
          if (m & (1u << (2 * d + up))) {
            const int nbi = ijk[d] + (up ? 1 : -1);
            if (nbi >= 0 && nbi < nd[d]) {
              code = L.qpos[c.cell0[b] + nbl];
            } else {
              const int32_t slot = ghost_slot[c.cell0[b] + nbl];
              if (slot < 0) throw Error(ATH_ERR_ARG, "connection ghost without a donor");
              code = -slot - 2;
            }
          }
          L.nbq[(int64_t)(3 * up + d) * nq + q] = code;
          // face between the cell and this neighbour
          int fi = ijk[0], fj = ijk[1], fk = ijk[2];
          if (up) (d == 0 ? fi : d == 1 ? fj : fk) += 1;
          const int64_t f = bk.Face(d, fi, fj, fk);
          const int64_t nf = bk.NFace(d);
          auto &dst = up ? L.face_hi : L.face_lo;
          for (int comp = 0; comp < 4; ++comp)
            dst[(int64_t)(d * 4 + comp) * nq + q] = bk.farea[d][comp * nf + f];
          // ProjC2CDist (src/procBlock.cpp:6316): centre above the face
          // minus centre below, along the face's unit normal
          const int64_t above = up ? nbl : cl, below = up ? cl : nbl;
          const int64_t ncb = bk.NCell();
          double dc[3];
          for (int comp = 0; comp < 3; ++comp)
            dc[comp] = bk.center[comp * ncb + above] - bk.center[comp * ncb + below];
          (up ? L.dist_hi : L.dist_lo)[(int64_t)d * nq + q] =
              dc[0] * bk.farea[d][f] + dc[1] * bk.farea[d][nf + f] +
              dc[2] * bk.farea[d][2 * nf + f];
        }
      }
    }
  }
  // hyperplane steps: step s holds plane s of every block that has one,
  // ordered by solve group.  The groups balance the solves' cells (largest
  // solve first into the lightest group)
  c.nsteps = 0;
  for (auto &b : st.blocks) c.nsteps = std::max(c.nsteps, (int)b.plane_offsets.size() - 1);
  std::vector<int> sgroup(c.nsolves, 0);
  {
    std::vector<int64_t> scells(c.nsolves, 0);
    for (int s = 0; s < c.nsolves; ++s)
      for (int b : st.solves[s].blocks)
        scells[s] += (int64_t)st.blocks[b].ni * st.blocks[b].nj * st.blocks[b].nk;
    std::vector<int> order(c.nsolves);
    for (int s = 0; s < c.nsolves; ++s) order[s] = s;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return scells[x] > scells[y]; });
    int64_t load[kSweepGroups] = {};
    for (int s : order) {
      int g = 0;
      for (int k = 1; k < kSweepGroups; ++k)
        if (load[k] < load[g]) g = k;
      sgroup[s] = g;
      load[g] += scells[s];
    }
  }
  L.step_off.assign(c.nsteps + 1, 0);
  L.gstep_off.assign((size_t)c.nsteps * (kSweepGroups + 1), 0);
  for (int s2 = 0; s2 < c.nsteps; ++s2) {
    L.step_off[s2] = (int32_t)L.sweep_items.size();
    for (int g = 0; g < kSweepGroups; ++g) {
      L.gstep_off[(size_t)s2 * (kSweepGroups + 1) + g] = (int32_t)L.sweep_items.size();
      for (int b = 0; b < c.nblocks; ++b) {
        const Block &bk = st.blocks[b];
        if (sgroup[bk.solve] != g || s2 + 1 >= (int)bk.plane_offsets.size()) continue;
        for (int q = bk.plane_offsets[s2]; q < bk.plane_offsets[s2 + 1]; ++q)
          L.sweep_items.push_back(make_int2((int)(L.q0[b] + q), b));
      }
    }
    L.gstep_off[(size_t)s2 * (kSweepGroups + 1) + kSweepGroups] =
        (int32_t)L.sweep_items.size();
  }
  L.step_off[c.nsteps] = (int32_t)L.sweep_items.size();
  for (int s = 0; s < c.nsolves; ++s) {
    int ns = 0;
    for (int b : st.solves[s].blocks)
      ns = std::max(ns, (int)st.blocks[b].plane_offsets.size() - 1);
    L.solve_step0.push_back((int32_t)L.cl_step_off.size());
    L.solve_nsteps.push_back(ns);
    for (int p = 0; p < ns; ++p) {
      L.cl_step_off.push_back((int32_t)L.cl_items.size());
      for (int b : st.solves[s].blocks) {
        const Block &bk = st.blocks[b];
        if (p + 1 >= (int)bk.plane_offsets.size()) continue;
        for (int q = bk.plane_offsets[p]; q < bk.plane_offsets[p + 1]; ++q)
          L.cl_items.push_back(make_int2((int)(L.q0[b] + q), b));
      }
      L.max_plane = std::max(L.max_plane, (int)L.cl_items.size() - L.cl_step_off.back());
    }
    L.cl_step_off.push_back((int32_t)L.cl_items.size());
  }
  // ghost operations with pool indices
  auto face_pool = [&](int b, int d, int64_t face) {
    const Block &bk = st.blocks[b];
    const int fi = bk.NI + (d == 0), fj = bk.NJ + (d == 1);
    const int ii = (int)(face % fi);
    const int64_t r = face / fi;
    const int jj = (int)(r % fj), kk = (int)(r / fj);
    return (int32_t)(c.cell0[b] + ii + (int64_t)bk.NI * (jj + (int64_t)bk.NJ * kk));
  };
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &bk = st.blocks[b];
    // nonreflecting surfaces of the block: batch-wide surface numbers
    const int nr_base = (int)L.nr_off.size();
    for (size_t i = 0; i < bk.nr_cells.size(); ++i) {
      const ath_nr_cell &x = bk.nr_cells[i];
      if (i == 0 || x.surf != bk.nr_cells[i - 1].surf) L.nr_off.push_back((int32_t)L.nr.size());
      NrDev e{};
      e.cell = (int32_t)(c.cell0[b] + x.cell);
      e.face = face_pool(b, x.dir, x.face);
      e.lower = x.lower;
      e.dir = x.dir;
      e.solve = bk.solve;
      L.nr.push_back(e);
    }
    for (const auto &op : bk.ops) {
      GhostOpDev g{};
      g.src2 = op.src2 >= 0 ? nr_base + (int32_t)op.src2 : -1;
      g.dst = (int32_t)(c.cell0[b] + op.dst);
      g.src = (int32_t)(c.cell0[op.src_block] + op.src);
      g.type = op.type;
      g.lower = op.lower;
      g.dir = op.dir;
      g.state = op.state;
      g.layer = op.layer;
      {
        const int d = op.dir;
        const int fi = bk.NI + (d == 0), fj = bk.NJ + (d == 1);
        const int ii = (int)(op.face % fi);
        const int64_t r = op.face / fi;
        const int jj = (int)(r % fj), kk = (int)(r / fj);
        g.face = (int32_t)(c.cell0[b] + ii + (int64_t)bk.NI * (jj + (int64_t)bk.NJ * kk));
      }
      L.ops.push_back(g);
      L.op_solve.push_back(bk.solve);
      if (op.type == ATH_BC_PRESSURE_OUTLET && op.state >= 0 &&
          st.solves[bk.solve].states[op.state].nonreflecting &&
          std::find(L.nrg_cells.begin(), L.nrg_cells.end(), g.src) == L.nrg_cells.end()) {
        L.nrg_cells.push_back(g.src);
        L.nrg_block.push_back(b);
      }
      if (op.type == ATH_BC_PERIODIC || op.type == ATH_BC_INTERBLOCK) L.conn_ops.push_back(g);
    }
  }
  if (!L.nr_off.empty()) L.nr_off.push_back((int32_t)L.nr.size());
  // block-edge and viscous-wall ghost ops, pool indices, grouped by phase
  auto convert = [&](int b, const ath_ghost_op &op) {
    const Block &bk = st.blocks[b];
    GhostOpDev g{};
    g.dst = (int32_t)(c.cell0[b] + op.dst);
    g.src = (int32_t)(c.cell0[op.src_block] + op.src);
    g.src2 = op.src2 >= 0 ? (int32_t)(c.cell0[b] + op.src2) : -1;
    g.type = op.type;
    g.lower = op.lower;
    g.dir = op.dir;
    g.state = op.state;
    g.layer = op.layer;
    const int d = op.dir;
    const int fi = bk.NI + (d == 0), fj = bk.NJ + (d == 1);
    const int ii = (int)(op.face % fi);
    const int64_t r = op.face / fi;
    const int jj = (int)(r % fj), kk = (int)(r / fj);
    g.face = (ii < bk.NI && jj < bk.NJ && kk < bk.NK)
                 ? (int32_t)(c.cell0[b] + ii + (int64_t)bk.NI * (jj + (int64_t)bk.NJ * kk))
                 : -1;
    return g;
  };
  int max_phase = 0;
  for (auto &bk : st.blocks) max_phase = std::max(max_phase, bk.ng * bk.ng);
  L.edge_phase_off.assign(max_phase + 1, 0);
  L.vedge_phase_off.assign(max_phase + 1, 0);
  for (int ph = 0; ph < max_phase; ++ph) {
    L.edge_phase_off[ph] = (int32_t)L.edge_ops.size();
    L.vedge_phase_off[ph] = (int32_t)L.vedge_ops.size();
    for (int b = 0; b < c.nblocks; ++b) {
      const Block &bk = st.blocks[b];
      for (const auto &op : bk.edge_ops)
        if (op.layer == ph) {
          L.edge_ops.push_back(convert(b, op));
          L.edge_solve.push_back(bk.solve);
        }
      for (const auto &op : bk.vedge_ops)
        if (op.layer == ph) {
          L.vedge_ops.push_back(convert(b, op));
          L.vedge_solve.push_back(bk.solve);
        }
    }
  }
  L.edge_phase_off[max_phase] = (int32_t)L.edge_ops.size();
  L.vedge_phase_off[max_phase] = (int32_t)L.vedge_ops.size();
  L.solve_face0.assign(c.nsolves + 1, 0);
  for (int s = 0; s < c.nsolves; ++s) {
    L.solve_face0[s] = (int32_t)L.wall_faces.size();
    for (int b : st.solves[s].blocks)
      for (const auto &op : st.blocks[b].vops) {
        if (op.layer != 1) continue;
        const GhostOpDev g = convert(b, op);
        L.wall_faces.push_back(WallFaceDev{g.face, g.dir, b, 0});
      }
  }
  L.solve_face0[c.nsolves] = (int32_t)L.wall_faces.size();
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &bk = st.blocks[b];
    for (const auto &op : bk.vops) {
      L.vops.push_back(convert(b, op));
      L.vop_solve.push_back(bk.solve);
    }
    if (st.solves[bk.solve].phys.eqn == ATH_EQN_EULER) continue;
    L.any_viscous = true;
    for (int k = -bk.ng; k < bk.nk + bk.ng; ++k)
      for (int j = -bk.ng; j < bk.nj + bk.ng; ++j)
        for (int i = -bk.ng; i < bk.ni + bk.ng; ++i) {
          const bool gi = i < 0 || i >= bk.ni, gj = j < 0 || j >= bk.nj, gk = k < 0 || k >= bk.nk;
          if (gi && gj && gk) continue;  // corner cells are never used
          L.aux_cells.push_back((int32_t)(c.cell0[b] + bk.Cell(i, j, k)));
          L.aux_block.push_back(b);
        }
  }
}

// Kernel launches of one iteration (the graph's nodes): cfl, ghost ops and
// edge phases, viscous ghosts, aux, faces, wall forces, cell, off-diagonal
// Jacobians, the relaxations' launches, update, norms, counter, and the
// optional matrix residual
// Tile-queue lists of one tile size: for each kind of LU-SGS solve (scalar,
// block) and each pass direction, the tiles in ticket order -- step by step
// (forward: plane 0 first; backward: each solve's last plane first), the
// solves of a step in turn, each solve's plane cut into runs of at most
// `size` cells of the solve-grouped item list -- and for every tile the
// tiles of the previous step that hold its cells' neighbours on the swept
// side (lower neighbours forward, upper ones backward; connection
// neighbours are read from ghost slots filled before the pass, so they add
// no dependency).
void BuildTileQueue(BatchCore &c, const Setup &st, DevMem &m, int size) {
  const int64_t nq = c.nq;
  std::array<BatchCore::TqList, 4> out;
  std::vector<int32_t> tile_of(nq, -1);
  for (int kind = 0; kind < 2; ++kind) {
    if (!(c.skinds & (1 << kind))) continue;
    std::vector<int> solves;
    int maxst = 0;
    for (int s = 0; s < c.nsolves; ++s) {
      const auto &ph = st.solves[s].phys;
      if (IsJacobiSolver(ph.solver) || (IsBlockSolver(ph.solver) ? 1 : 0) != kind) continue;
      solves.push_back(s);
      maxst = std::max(maxst, (int)c.L.solve_nsteps[s]);
    }
    for (int back = 0; back < 2; ++back) {
      std::vector<int4> tiles;
      std::vector<int32_t> deps;
      std::vector<int32_t> seen;
      for (int k = 0; k < maxst; ++k)
        for (int s : solves) {
          const int ns = c.L.solve_nsteps[s];
          if (k >= ns) continue;
          const int p = back ? ns - 1 - k : k;
          const int base = c.L.solve_step0[s];
          const int a = c.L.cl_step_off[base + p], b = c.L.cl_step_off[base + p + 1];
          for (int t0 = a; t0 < b; t0 += size) {
            const int t1 = std::min(b, t0 + size);
            const int id = (int)tiles.size();
            const int dep0 = (int)deps.size();
            seen.clear();
            for (int i = t0; i < t1; ++i) {
              const int64_t q = c.L.cl_items[i].x;
              for (int d = 0; d < 3; ++d) {
                const int32_t code = c.L.nbq[(int64_t)(3 * back + d) * nq + q];
                if (code < 0) continue;
                const int32_t dt = tile_of[code];
                if (dt < 0) throw Error(ATH_ERR_ARG, "tile queue: neighbour outside the swept order");
                if (std::find(seen.begin(), seen.end(), dt) == seen.end()) seen.push_back(dt);
              }
            }
            std::sort(seen.begin(), seen.end());
            deps.insert(deps.end(), seen.begin(), seen.end());
            tiles.push_back(make_int4(t0, t1, dep0, (int)deps.size() - dep0));
            for (int i = t0; i < t1; ++i) tile_of[c.L.cl_items[i].x] = id;
          }
        }
      BatchCore::TqList &tl = out[kind * 2 + back];
      tl.ntiles = (int)tiles.size();
      tl.tiles = m.Upload(tiles);
      tl.deps = m.Upload(deps);
      tl.done = m.Alloc<int>((size_t)tl.ntiles + 1);
      m.Zero(tl.done, 0, ((size_t)tl.ntiles + 1) * sizeof(int));
      for (const int4 &x : tiles)
        for (int i = x.x; i < x.y; ++i) tile_of[c.L.cl_items[i].x] = -1;
    }
  }
  c.tq[size] = out;
}

void EnsureTileQueue(BatchCore &c, int size) {
  if (!c.tq.count(size)) BuildTileQueue(c, *c.setup, *c.mem, size);
}

// Candidate tile sizes of the tile-queue sweep: whole rounds of a warp
// worker (10 cells of scalar solves, 5 with both triangles, 4 of block
// solves), one to eight rounds per tile.
std::vector<int> TileSizes(const BatchCore &c) {
  if (c.skinds == 1) return c.max_sweeps > 1 ? std::vector<int>{5, 10, 20, 40}
                                              : std::vector<int>{10, 20, 40, 80};
  if (c.skinds == 2) return {4, 8, 16, 32};
  return {8, 16, 32, 64};
}

void CountLaunches(BatchCore &c) {
  int edge_phases = 0, vedge_phases = 0;
  for (size_t ph = 0; ph + 1 < c.L.edge_phase_off.size(); ++ph) {
    edge_phases += c.L.edge_phase_off[ph + 1] > c.L.edge_phase_off[ph];
    vedge_phases += c.L.vedge_phase_off[ph + 1] > c.L.vedge_phase_off[ph];
  }
  const int nkinds = (c.kinds & 1) + ((c.kinds >> 1) & 1);
  const int nskinds = (c.skinds & 1) + ((c.skinds >> 1) & 1);
  const int njkinds = (c.jkinds & 1) + ((c.jkinds >> 1) & 1);
  const int nf = (c.fkinds & 1) + ((c.fkinds >> 1) & 1);
  const int nvf = (c.vkinds & 1) + ((c.vkinds >> 1) & 1);
  const int conn = c.L.ghost_cell.empty() ? 0 : 1;
  const int per_pass = (c.sweep_mode == 1 || c.sweep_mode == 3) ? 1 : c.nsteps;
  c.launches_per_iter = edge_phases +
                        (c.L.any_viscous ? (c.L.vops.empty() ? 0 : 1) + vedge_phases + 1 + 3 * nvf
                                         : 0) +
                        (c.L.wall_faces.empty() ? 0 : 2) +
                        1 + (c.L.ops.empty() ? 0 : 1) + 3 * nf + nkinds + ((c.kinds & 2) ? 1 : 0) +
                        (c.any_unsteady ? 1 : 0) + (c.n_nr_surf > 0 ? 1 : 0) +
                        (c.L.nrg_cells.empty() ? 0 : 1) +
                        (nskinds ? 2 * per_pass * c.max_sweeps * nskinds +
                                       (c.max_sweeps > 1 ? 1 + 2 * c.max_sweeps * conn : conn)
                                 : 0) +
                        (njkinds ? 1 + c.max_jsweeps * (conn + njkinds) + (c.max_jsweeps % 2)
                                 : 0) +
                        3 +
                        ((c.flags & 1) ? nkinds + conn : 0);
}

void CreateBatch(ath_batch *B, ath_ctx *ctx, const Setup &st, int precision, int flags,
                 cudaStream_t shared = nullptr);

// Releases a batch and its multigrid levels (also a partly built one).
void DestroyBatch(ath_batch *batch) {
  if (!batch) return;
  if (batch->core.ctx) cudaSetDevice(batch->core.ctx->device);
  if (batch->core.stream) cudaStreamSynchronize(batch->core.stream);
  for (auto *lv : batch->levels) DestroyBatch(lv);
  batch->levels.clear();
  batch->run.reset();
  batch->core.mem.reset();
  if (batch->core.ev0) cudaEventDestroy(batch->core.ev0);
  if (batch->core.ev1) cudaEventDestroy(batch->core.ev1);
  if (batch->core.stream && batch->core.own_stream) cudaStreamDestroy(batch->core.stream);
  for (auto x : batch->core.gstream)
    if (x) cudaStreamDestroy(x);
  if (batch->core.gfork) cudaEventDestroy(batch->core.gfork);
  for (auto x : batch->core.gjoin)
    if (x) cudaEventDestroy(x);
  delete batch;
}

// Transfer tables between level fine (setup sf, batch cf) and the next
// coarser level (sc, cc), in pool and q indices of the two batches
MgLinkDev BuildMgLink(const Setup &sf, const BatchCore &cf, const Setup &sc,
                      const BatchCore &cc, DevMem &m) {
  const int64_t ncq = cc.nq;
  std::vector<std::vector<int32_t>> members(ncq);  // fine gather entries per coarse q
  std::vector<int32_t> f_pool, f_q;
  std::vector<double> f_w;
  std::vector<int32_t> p_q, p_node0, p_sx, p_sxy;
  std::vector<double> coef;
  // nodes of the coarse blocks, block by block
  std::vector<int64_t> node0(sc.blocks.size() + 1, 0);
  for (size_t b = 0; b < sc.blocks.size(); ++b) {
    const Block &k = sc.blocks[b];
    node0[b + 1] = node0[b] + (int64_t)(k.ni + 1) * (k.nj + 1) * (k.nk + 1);
  }
  const int64_t nnode = node0.back();
  for (size_t bi = 0; bi < sf.blocks.size(); ++bi) {
    const Block &fb = sf.blocks[bi];
    if (fb.mg_coarse < 0) throw Error(ATH_ERR_UNSUPPORTED, "block without a coarser level");
    const Block &cb = sc.blocks[fb.mg_coarse];
    int64_t x = 0;
    for (int k = 0; k < fb.nk; ++k)
      for (int j = 0; j < fb.nj; ++j)
        for (int i = 0; i < fb.ni; ++i, ++x) {
          const int64_t fp = cf.cell0[bi] + fb.Cell(i, j, k);
          const int cci = fb.mg_cell[x];
          const int ci = cci % cb.ni, cj = (cci / cb.ni) % cb.nj, ck = cci / (cb.ni * cb.nj);
          const int64_t cp = cc.cell0[fb.mg_coarse] + cb.Cell(ci, cj, ck);
          const int32_t fq = cf.L.qpos[fp], cq = cc.L.qpos[cp];
          members[cq].push_back((int32_t)f_pool.size());
          f_pool.push_back((int32_t)fp);
          f_q.push_back(fq);
          f_w.push_back(fb.mg_volfac[x]);
          p_q.push_back(fq);
          p_node0.push_back((int32_t)(node0[fb.mg_coarse] + ci +
                                      (int64_t)(cb.ni + 1) * (cj + (int64_t)(cb.nj + 1) * ck)));
          p_sx.push_back(cb.ni + 1);
          p_sxy.push_back((cb.ni + 1) * (cb.nj + 1));
        }
  }
  const int64_t nf = (int64_t)f_pool.size();
  // prolongation coefficients [7][nfine], fine cells in the same order
  coef.assign(7 * nf, 0.0);
  {
    int64_t e = 0;
    for (size_t bi = 0; bi < sf.blocks.size(); ++bi) {
      const Block &fb = sf.blocks[bi];
      const int64_t n = (int64_t)fb.ni * fb.nj * fb.nk;
      for (int64_t x = 0; x < n; ++x, ++e)
        for (int a = 0; a < 7; ++a) coef[a * nf + e] = fb.mg_coef[7 * x + a];
    }
  }
  // gather lists in coarse q order; each coarse cell's entries in the fine
  // cells' k, j, i order
  std::vector<int32_t> off(ncq + 1, 0), c_pool(ncq, -1), c_q(ncq), gp, gq;
  std::vector<double> gw;
  for (int64_t q = 0; q < ncq; ++q) {
    off[q + 1] = off[q] + (int32_t)members[q].size();
    c_q[q] = (int32_t)q;
    for (int32_t e : members[q]) {
      gp.push_back(f_pool[e]);
      gq.push_back(f_q[e]);
      gw.push_back(f_w[e]);
    }
  }
  for (int64_t p = 0; p < cc.ncell; ++p)
    if (cc.L.qpos[p] >= 0) c_pool[cc.L.qpos[p]] = (int32_t)p;
  // node sums: the cells around each node in the cell loop's k, j, i order
  std::vector<int32_t> node_cells(8 * nnode, -1);
  std::vector<double> node_fac(nnode, 0.125);
  for (size_t b = 0; b < sc.blocks.size(); ++b) {
    const Block &k = sc.blocks[b];
    for (int nk = 0; nk <= k.nk; ++nk)
      for (int nj = 0; nj <= k.nj; ++nj)
        for (int ni = 0; ni <= k.ni; ++ni) {
          const int64_t nd =
              node0[b] + ni + (int64_t)(k.ni + 1) * (nj + (int64_t)(k.nj + 1) * nk);
          int e = 0;
          for (int dk = -1; dk <= 0; ++dk)
            for (int dj = -1; dj <= 0; ++dj)
              for (int di = -1; di <= 0; ++di, ++e) {
                const int ci = ni + di, cj = nj + dj, ck = nk + dk;
                if (ci < 0 || cj < 0 || ck < 0 || ci >= k.ni || cj >= k.nj || ck >= k.nk) continue;
                node_cells[8 * nd + e] = cc.L.qpos[cc.cell0[b] + k.Cell(ci, cj, ck)];
              }
          const int ei = ni == 0 || ni == k.ni, ej = nj == 0 || nj == k.nj,
                    ek = nk == 0 || nk == k.nk;
          node_fac[nd] = (ei && ej && ek) ? 1.0 : (ei + ej + ek == 2) ? 0.5 : 0.125;
        }
  }
  MgLinkDev d{};
  d.ncoarse = (int)ncq;
  d.nfine = (int)nf;
  d.nnode = (int)nnode;
  d.off = m.Upload(off);
  d.c_pool = m.Upload(c_pool);
  d.c_q = m.Upload(c_q);
  d.f_pool = m.Upload(gp);
  d.f_q = m.Upload(gq);
  d.f_w = m.Upload(gw);
  d.node_cells = m.Upload(node_cells);
  d.node_fac = m.Upload(node_fac);
  d.p_q = m.Upload(p_q);
  d.p_node0 = m.Upload(p_node0);
  d.p_sx = m.Upload(p_sx);
  d.p_sxy = m.Upload(p_sxy);
  d.p_coef = m.Upload(coef);
  return d;
}

// The coarser levels of a multigrid batch: every solve has the same levels,
// cycle and sweeps (one relaxation schedule for the batch)
template <typename T>
void WireMultigrid(ath_batch *B, const Setup &st) {
  BatchCore &c = B->core;
  const int nl = st.solves[0].phys.mg_levels;
  for (const auto &sv : st.solves)
    if (sv.phys.mg_levels != nl || sv.phys.mg_cycle != st.solves[0].phys.mg_cycle ||
        sv.phys.sweeps != st.solves[0].phys.sweeps ||
        sv.phys.solver != st.solves[0].phys.solver)
      throw Error(ATH_ERR_UNSUPPORTED,
                  "a multigrid batch needs the same multigrid levels, cycle, matrix solver and "
                  "sweeps in every solve");
  if ((int)st.levels.size() < nl - 1) throw Error(ATH_ERR_UNSUPPORTED, "multigrid levels missing");
  auto *fine = static_cast<Runner<T> *>(B->run.get());
  const int64_t nqf = c.nq;
  fine->MutablePools().MRq = c.mem->Alloc<T>(5 * (size_t)nqf);
  fine->MgSetup(st.solves[0].phys.mg_cycle, st.solves[0].phys.sweeps);
  const Setup *sf = &st;
  ath_batch *fb = B;
  for (int l = 1; l < nl; ++l) {
    const Setup &sc = *st.levels[l - 1];
    if (sc.solves.size() != st.solves.size())
      throw Error(ATH_ERR_UNSUPPORTED, "multigrid levels differ between the batch's solves");
    auto *lb = new ath_batch();
    B->levels.push_back(lb);
    CreateBatch(lb, c.ctx, sc, c.precision, c.flags, c.stream);
    auto *cr = static_cast<Runner<T> *>(lb->run.get());
    BatchCore &cc = lb->core;
    Pools<T> &cp = cr->MutablePools();
    cp.Fq = cc.mem->Alloc<T>(5 * (size_t)cc.nq);
    cp.MRq = cc.mem->Alloc<T>(5 * (size_t)cc.nq);
    cc.mem->Zero(cp.Fq, 0, 5 * (size_t)cc.nq * sizeof(T));
    const MgLinkDev link = BuildMgLink(*sf, fb->core, sc, cc, *c.mem);
    T *du0 = c.mem->Alloc<T>(5 * (size_t)cc.nq);
    T *nodes = c.mem->Alloc<T>(5 * (size_t)std::max(link.nnode, 1));
    fine->MgAddLevel(cr, link, du0, nodes);
    sf = &sc;
    fb = lb;
  }
  Check(cudaStreamSynchronize(c.stream), "sync");
}

void CreateBatch(ath_batch *B, ath_ctx *ctx, const Setup &st, int precision, int flags,
                 cudaStream_t shared) {
  auto &c = B->core;
  c.ctx = ctx;
  c.setup = &st;
  c.precision = precision;
  c.flags = flags;
  c.nsolves = (int)st.solves.size();
  c.nblocks = (int)st.blocks.size();
  for (const auto &b : st.blocks) {
    const bool rans = st.solves[b.solve].phys.eqn == ATH_EQN_RANS;
    if (b.nv != (rans ? 7 : 5) || b.ng < 1)
      throw Error(ATH_ERR_UNSUPPORTED, "block layout not supported by this build");
    if (rans) c.any_rans = true;
  }
  for (const auto &sv : st.solves) {
    const bool blk = IsBlockSolver(sv.phys.solver), jac = IsJacobiSolver(sv.phys.solver);
    c.kinds |= blk ? 2 : 1;
    if (jac) {
      c.jkinds |= blk ? 2 : 1;
      c.max_jsweeps = std::max(c.max_jsweeps, (int)sv.phys.sweeps);
    } else {
      c.skinds |= blk ? 2 : 1;
      c.max_sweeps = std::max(c.max_sweeps, (int)sv.phys.sweeps);
    }
    if (blk && sv.phys.eqn != ATH_EQN_EULER) c.block_viscous = true;
    const bool rans = sv.phys.eqn == ATH_EQN_RANS;
    c.fkinds |= rans ? 2 : 1;
    if (!rans && !(sv.phys.recon == ATH_RECON_MUSCL && sv.phys.flux == ATH_FLUX_ROE))
      c.mr_only = false;
    if (sv.phys.eqn != ATH_EQN_EULER) c.vkinds |= rans ? 2 : 1;
  }
  Check(cudaSetDevice(ctx->device), "cudaSetDevice");
  BuildLists(c);
  if (shared) {
    c.stream = shared;
    c.own_stream = false;
  } else {
    Check(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "stream");
  }
  for (auto &x : c.gstream) Check(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), "stream");
  Check(cudaEventCreateWithFlags(&c.gfork, cudaEventDisableTiming), "event");
  for (auto &x : c.gjoin) Check(cudaEventCreateWithFlags(&x, cudaEventDisableTiming), "event");
  c.mem.reset(new DevMem(ctx, c.stream));
  DevMem &m = *c.mem;
  std::vector<BlockDev> bd(c.nblocks);
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &k = st.blocks[b];
    bd[b] = BlockDev{k.ni, k.nj, k.nk, k.ng, k.NI, k.NJ, k.NK, k.solve, c.cell0[b]};
  }
  std::vector<SolveDev> sd(c.nsolves);
  std::vector<ath_bc_state> states;
  for (int s = 0; s < c.nsolves; ++s) {
    const auto &p = st.solves[s].phys;
    SolveDev x{};
    x.gas_r = p.gas_r;
    x.gas_n = p.gas_n;
    x.gas_hf = p.gas_hf;
    x.kappa = p.kappa;
    x.theta = p.theta;
    x.zeta = p.zeta;
    x.relax = p.relax;
    x.cfl_start = p.cfl_start;
    x.cfl_step = p.cfl_step;
    x.cfl_max = p.cfl_max;
    x.limiter = p.limiter;
    x.recon = p.recon;
    x.flux = p.flux;
    x.viscous = p.eqn != ATH_EQN_EULER;
    x.visc_scale = p.visc_scale;
    x.mu_c1 = p.mu_c1;
    x.mu_s = p.mu_s;
    x.mu_ref = p.mu_ref;
    x.t_ref = p.t_ref;
    x.k_c1 = p.k_c1;
    x.k_s = p.k_s;
    x.k_ref = p.k_ref;
    x.visc_coeff = p.visc_cfl_coeff;
    x.block = IsBlockSolver(p.solver);
    x.jacobi = IsJacobiSolver(p.solver);
    x.dt_global = p.dt_global;
    x.dual_cfl = p.dual_cfl;
    x.nl_iters = std::max(1, (int)p.nl_iters);
    x.multilevel = p.multilevel;
    x.unsteady = (p.multilevel || p.nl_iters > 1) ? 1 : 0;
    // the time-n state is kept for the time-accurate terms and for the
    // nonreflecting boundaries (every implicit solve stores it in the
    // reference, procBlock storeTimeN_; only these two read it)
    bool nonreflecting = false;
    for (const auto &bs : st.solves[s].states) nonreflecting = nonreflecting || bs.nonreflecting;
    x.store_n = (x.unsteady || nonreflecting) ? 1 : 0;
    if (x.store_n) c.any_unsteady = true;
    x.rans = p.eqn == ATH_EQN_RANS;
    x.wilcox = x.rans && p.turb == ATH_TURB_KW2006;
    x.sweeps = p.sweeps;
    x.active = 1;
    x.padded_values = 0.0;
    x.cells = 0.0;
    for (int b : st.solves[s].blocks) {
      x.padded_values += (double)st.blocks[b].NCell() * st.blocks[b].nv;
      x.cells += (double)st.blocks[b].ni * st.blocks[b].nj * st.blocks[b].nk;
    }
    x.nstates = (int32_t)st.solves[s].states.size();
    x.state0 = (int32_t)states.size();
    for (auto &q : st.solves[s].states) states.push_back(q);
    SetDerived(x);
    sd[s] = x;
  }
  c.d_blocks = m.Upload(bd);
  c.d_solves = m.Upload(sd);
  c.d_states = m.Upload(states);
  c.d_cfl = m.Alloc<double>(c.nsolves);
  c.d_iter = m.Alloc<int64_t>(1);
  c.mem->Zero(c.d_iter, 0, sizeof(int64_t));
  c.d_now = m.Alloc<uint64_t>(1);
  c.d_sstate = m.Alloc<SolveState>(c.nsolves);
  c.mem->Zero(c.d_sstate, 0, c.nsolves * sizeof(SolveState));
  c.d_cells = m.Upload(c.L.cells);
  c.d_cell_cta_block = m.Upload(c.L.cell_cta_block);
  c.d_cell_cta_pos0 = m.Upload(c.L.cell_cta_pos0);
  for (int d = 0; d < 3; ++d) {
    c.d_faces[d] = m.Upload(c.L.faces[d]);
    c.d_face_cta_block[d] = m.Upload(c.L.face_cta_block[d]);
  }
  c.d_sweep = m.Upload(c.L.sweep_items);
  c.d_cl_items = m.Upload(c.L.cl_items);
  c.d_cl_step_off = m.Upload(c.L.cl_step_off);
  if (c.skinds) {
    c.d_tq_ticket = m.Alloc<int>(1);
    c.d_tq_status = m.Alloc<int>(1);
    c.mem->Zero(c.d_tq_status, 0, sizeof(int));
  }
  c.d_solve_step0 = m.Upload(c.L.solve_step0);
  c.d_solve_nsteps = m.Upload(c.L.solve_nsteps);
  c.d_solve_cta0 = m.Upload(c.L.solve_cta0);
  c.d_ops = m.Upload(c.L.ops);
  if (!c.L.nr_off.empty()) {
    c.d_nr = m.Upload(c.L.nr);
    c.d_nr_off = m.Upload(c.L.nr_off);
    c.n_nr_surf = (int)c.L.nr_off.size() - 1;
  }
  if (!c.L.nrg_cells.empty()) {
    c.d_nrg_cells = m.Upload(c.L.nrg_cells);
    c.d_nrg_block = m.Upload(c.L.nrg_block);
  }
  c.d_conn_ops = m.Upload(c.L.conn_ops);
  c.d_op_solve = m.Upload(c.L.op_solve);
  c.d_edge_ops = m.Upload(c.L.edge_ops);
  c.d_edge_solve = m.Upload(c.L.edge_solve);
  c.d_vops = m.Upload(c.L.vops);
  c.d_vop_solve = m.Upload(c.L.vop_solve);
  c.d_vedge_ops = m.Upload(c.L.vedge_ops);
  c.d_vedge_solve = m.Upload(c.L.vedge_solve);
  c.d_aux_cells = m.Upload(c.L.aux_cells);
  c.d_aux_block = m.Upload(c.L.aux_block);
  c.d_partials = m.Alloc<NormPartial>(c.L.cell_cta_block.size());
  c.d_mres = m.Alloc<double>(c.L.cell_cta_block.size());
  c.d_ring = m.Alloc<NormOut>((size_t)c.ring_cap * c.nsolves);
  c.d_wall_faces = m.Upload(c.L.wall_faces);
  c.d_solve_face0 = m.Upload(c.L.solve_face0);
  c.d_wbuf = m.Alloc<double>(6 * std::max<size_t>(c.L.wall_faces.size(), 1));
  c.d_fring = m.Alloc<double>((size_t)c.ring_cap * c.nsolves * 6);
  c.mem->Zero(c.d_fring, 0, (size_t)c.ring_cap * c.nsolves * 6 * sizeof(double));
  Check(cudaEventCreate(&c.ev0), "event");
  Check(cudaEventCreate(&c.ev1), "event");
  if (precision == ATH_PREC_FP64) {
    auto *r = new Runner<double>(c);
    B->run.reset(r);
    B->W = r->P().W;
    B->R = r->P().R;
    B->dt = r->P().dt;
    B->lam = r->P().lam;
    B->Wt = r->P().Wt;
    B->Rt = r->P().Rt;
    B->lamt = r->P().lamt;
    B->Un = r->P().Un;
    B->Unm1 = r->P().Unm1;
    B->ogr = r->P().ogr;
  } else if (precision == ATH_PREC_MIXED) {
    auto *r = new Runner<float>(c);
    B->run.reset(r);
    B->W = r->P().W;
    B->R = r->P().R;
    B->dt = r->P().dt;
    B->lam = r->P().lam;
    B->Wt = r->P().Wt;
    B->Rt = r->P().Rt;
    B->lamt = r->P().lamt;
    B->Un = r->P().Un;
    B->Unm1 = r->P().Unm1;
    B->ogr = r->P().ogr;
  } else {
    throw Error(ATH_ERR_ARG, "unknown precision");
  }
  // multigrid: the coarser levels (only the finest batch builds them)
  if (!shared && !st.solves.empty() && st.solves[0].phys.mg_levels > 1) {
    if (precision == ATH_PREC_FP64) WireMultigrid<double>(B, st);
    else WireMultigrid<float>(B, st);
  } else if (!shared) {
    for (const auto &sv : st.solves)
      if (sv.phys.mg_levels > 1)
        throw Error(ATH_ERR_UNSUPPORTED,
                    "a multigrid batch needs the same multigrid levels in every solve");
  }
  // resident CTAs of the tile-queue sweep kernels (one wave of persistent
  // CTAs; more would only wait for tickets)
  if (c.skinds) {
    int sms = 0;
    Check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "attribute");
    c.tq_ctas[0] = std::max(1, B->run->TqOccupancy(c.max_sweeps > 1, false)) * sms;
    c.tq_ctas[1] = std::max(1, B->run->TqOccupancy(true, true)) * sms;
  }
  // default sweep shape: the persistent sweep with a cluster wide enough for
  // the largest plane (at most 8 CTAs of 256 threads), when launchable
  if (c.skinds) {
    const int lanes = (c.skinds & 2) ? 8 : 1;  // block sweeps: 8 lanes per cell
    const int want = std::min(8, std::max(1, (c.L.max_plane * lanes + 255) / 256));
    for (int cl = want; cl >= 1; --cl)
      if (B->run->MaxClusters(c.skinds, 256, cl) > 0) {
        c.sweep_mode = 1;
        c.cl_size = cl;
        c.cl_threads = 256;
        break;
      }
  }
  CountLaunches(c);
  // every stream-ordered allocation and fill of the batch is complete before
  // host calls touch its memory from other streams
  Check(cudaStreamSynchronize(c.stream), "sync");
}

// After a synchronised run: a tile-queue sweep wait that ran out (its
// kernels returned without finishing the pass) is reported, and the status
// word is cleared so the batch can run again.
void CheckSweepStatus(BatchCore &c) {
  if (!c.d_tq_status) return;
  int st = 0;
  Check(cudaMemcpyAsync(&st, c.d_tq_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream),
        "status download");
  Check(cudaStreamSynchronize(c.stream), "sync");
  if (st == 0) return;
  c.mem->Zero(c.d_tq_status, 0, sizeof(int));
  throw Error(ATH_ERR_TIMEOUT,
              "a tile-queue sweep wait gave up after its poll limit; the iteration's update is "
              "incomplete");
}

// Reads norms of iterations [it0, it0+n) from the ring into norms_h.
void ReadNorms(BatchCore &c, int64_t it0, int n, ath_norms *norms_h) {
  if (!norms_h || n <= 0) return;
  std::vector<NormOut> ring((size_t)c.ring_cap * c.nsolves);
  Check(cudaMemcpyAsync(ring.data(), c.d_ring, ring.size() * sizeof(NormOut),
                        cudaMemcpyDeviceToHost, c.stream),
        "norms download");
  std::vector<double> fring((size_t)c.ring_cap * c.nsolves * 6);
  Check(cudaMemcpyAsync(fring.data(), c.d_fring, fring.size() * sizeof(double),
                        cudaMemcpyDeviceToHost, c.stream),
        "forces download");
  Check(cudaStreamSynchronize(c.stream), "sync");
  const auto &st = *c.setup;
  for (int q = 0; q < n; ++q) {
    const int64_t it = it0 + q;
    for (int s = 0; s < c.nsolves; ++s) {
      const NormOut &o = ring[(it % c.ring_cap) * c.nsolves + s];
      ath_norms &d = norms_h[(size_t)q * c.nsolves + s];
      std::memset(&d, 0, sizeof(d));
      for (int v = 0; v < 7; ++v) d.l2[v] = o.l2[v];
      d.linf = o.linf;
      d.cfl = o.cfl;
      d.matrix_resid = o.matrix_resid;
      d.status = o.bad == 2 ? ATH_RETIRED : o.bad ? ATH_ERR_NONPHYSICAL : ATH_OK;
      for (int q2 = 0; q2 < 6; ++q2)
        d.force[q2] = fring[((it % c.ring_cap) * c.nsolves + s) * 6 + q2];
      d.linf_block = d.linf_i = d.linf_j = d.linf_k = d.linf_eqn = -1;
      if (o.linf_pos != INT64_MAX) {
        const int64_t cellpos = o.linf_pos / kNvMax;
        d.linf_eqn = (int32_t)(o.linf_pos % kNvMax) + 1;
        const auto &blocks = st.solves[s].blocks;
        for (size_t bi = 0; bi < blocks.size(); ++bi) {
          const Block &b = st.blocks[blocks[bi]];
          const int64_t p0 = c.solve_pos0[blocks[bi]];
          const int64_t cnt = (int64_t)b.ni * b.nj * b.nk;
          if (cellpos >= p0 && cellpos < p0 + cnt) {
            const int64_t l = cellpos - p0;
            d.linf_block = (int32_t)bi;
            d.linf_i = (int32_t)(l % b.ni);
            d.linf_j = (int32_t)((l / b.ni) % b.nj);
            d.linf_k = (int32_t)(l / ((int64_t)b.ni * b.nj));
          }
        }
      }
    }
  }
}

}  // namespace
}  // namespace ath

using ath::Check;
using ath::Guard;

extern "C" {

int ath_ctx_create(int device, size_t hbm_budget_bytes, ath_ctx **out) {
  return Guard([&] {
    if (!out) throw ath::Error(ATH_ERR_ARG, "null argument");
    int n = 0;
    Check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) throw ath::Error(ATH_ERR_ARG, "no such CUDA device");
    Check(cudaSetDevice(device), "cudaSetDevice");
    auto *c = new ath_ctx();
    c->device = device;
    c->budget = hbm_budget_bytes;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&c->pool, &props) != cudaSuccess) {
      delete c;
      throw ath::Error(ATH_ERR_CUDA, "cudaMemPoolCreate failed");
    }
    uint64_t keep = UINT64_MAX;  // freed memory stays in the pool for reuse
    cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    *out = c;
  });
}

int ath_ctx_destroy(ath_ctx *ctx) {
  if (!ctx) return ATH_OK;
  if (ctx->pool) {
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();  // every batch's frees have been ordered before
    cudaMemPoolDestroy(ctx->pool);
  }
  delete ctx;
  return ATH_OK;
}

int ath_batch_create(ath_ctx *ctx, const ath_setup *setup, int precision, int flags,
                     ath_batch **out) {
  return Guard([&] {
    if (!ctx || !setup || !out) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto *b = new ath_batch();
    try {
      ath::CreateBatch(b, ctx, setup->s, precision, flags);
    } catch (...) {
      ath::DestroyBatch(b);
      throw;
    }
    *out = b;
  });
}

int ath_batch_destroy(ath_batch *batch) {
  ath::DestroyBatch(batch);
  return ATH_OK;
}

int ath_batch_iterate(ath_batch *batch, int n, ath_norms *norms_h) {
  return Guard([&] {
    if (!batch || n < 0) throw ath::Error(ATH_ERR_ARG, "bad argument");
    auto &c = batch->core;
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    // the iteration graph is captured (when a shape change dropped it)
    // before the timed interval opens
    batch->run->Iterate(0);
    Check(cudaEventRecord(c.ev0, c.stream), "event");
    int done = 0;
    while (done < n) {
      const int chunk = std::min(n - done, c.ring_cap);
      const int64_t it0 = c.iter_host;
      batch->run->Iterate(chunk);
      c.iter_host += chunk;
      if (norms_h) ath::ReadNorms(c, it0, chunk, norms_h + (size_t)done * c.nsolves);
      done += chunk;
    }
    Check(cudaEventRecord(c.ev1, c.stream), "event");
    Check(cudaEventSynchronize(c.ev1), "sync");
    Check(cudaGetLastError(), "kernel launch");
    float ms = 0.f;
    Check(cudaEventElapsedTime(&ms, c.ev0, c.ev1), "elapsed");
    c.stats.device_ms = ms;
    c.stats.kernel_launches = (int64_t)n * c.launches_per_iter;
    ath::CheckSweepStatus(c);
  });
}

namespace {
void SolveInfo(ath::BatchCore &c, ath_converge_info *info) {
  std::vector<ath::SolveState> ss(c.nsolves);
  Check(cudaMemcpyAsync(ss.data(), c.d_sstate, ss.size() * sizeof(ath::SolveState),
                        cudaMemcpyDeviceToHost, c.stream),
        "solve state download");
  // device clock now, for solves still running
  ath::k_clock<<<1, 1, 0, c.stream>>>(c.d_now);
  uint64_t now = 0;
  Check(cudaMemcpyAsync(&now, c.d_now, sizeof(now), cudaMemcpyDeviceToHost, c.stream), "clock");
  Check(cudaStreamSynchronize(c.stream), "sync");
  for (int s = 0; s < c.nsolves; ++s) {
    ath_converge_info &o = info[s];
    const ath::SolveState &x = ss[s];
    o.iterations = x.iter;
    o.drop = x.l2_first > 0.0 ? x.l2_last / x.l2_first : 0.0;
    const uint64_t end = x.converged ? x.t_retire_ns : now;
    o.ms = x.iter > 0 ? (double)(end - x.t_first_ns) * 1e-6 : 0.0;
    o.converged = x.converged;
    o.pad = 0;
  }
}
}  // namespace

int ath_batch_set_target(ath_batch *batch, int solve, double drop, int active) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    auto &c = batch->core;
    if (solve < 0 || solve >= c.nsolves) throw ath::Error(ATH_ERR_ARG, "solve out of range");
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    Check(cudaMemcpyAsync(&c.d_sstate[solve].target, &drop, sizeof(double),
                          cudaMemcpyHostToDevice, c.stream),
          "target upload");
    const int32_t a = active ? 1 : 0;
    Check(cudaMemcpyAsync(&c.d_solves[solve].active, &a, sizeof(int32_t),
                          cudaMemcpyHostToDevice, c.stream),
          "active upload");
    if (active) {
      const int32_t z = 0;
      Check(cudaMemcpyAsync(&c.d_sstate[solve].converged, &z, sizeof(int32_t),
                            cudaMemcpyHostToDevice, c.stream),
            "state upload");
    }
    Check(cudaStreamSynchronize(c.stream), "sync");
  });
}

int ath_batch_solve_info(ath_batch *batch, ath_converge_info *info) {
  return Guard([&] {
    if (!batch || !info) throw ath::Error(ATH_ERR_ARG, "null argument");
    Check(cudaSetDevice(batch->core.ctx->device), "cudaSetDevice");
    SolveInfo(batch->core, info);
  });
}

int ath_batch_converge(ath_batch *batch, int max_iters, double drop, int check_every,
                       ath_converge_info *info) {
  return Guard([&] {
    if (!batch || max_iters < 0 || !(drop > 0.0) || check_every < 1)
      throw ath::Error(ATH_ERR_ARG, "bad argument");
    auto &c = batch->core;
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    for (int s = 0; s < c.nsolves; ++s)
      Check(cudaMemcpyAsync(&c.d_sstate[s].target, &drop, sizeof(double),
                            cudaMemcpyHostToDevice, c.stream),
            "target upload");
    std::vector<ath::SolveDev> sv(c.nsolves);
    int done = 0;
    batch->run->Iterate(0);  // capture the iteration graph outside the timed interval
    Check(cudaEventRecord(c.ev0, c.stream), "event");
    while (done < max_iters) {
      const int chunk = std::min(max_iters - done, std::min(check_every, c.ring_cap));
      batch->run->Iterate(chunk);
      c.iter_host += chunk;
      done += chunk;
      Check(cudaMemcpyAsync(sv.data(), c.d_solves, sv.size() * sizeof(ath::SolveDev),
                            cudaMemcpyDeviceToHost, c.stream),
            "solve flags download");
      Check(cudaStreamSynchronize(c.stream), "sync");
      bool any = false;
      for (auto &x : sv) any |= x.active != 0;
      if (!any) break;
    }
    Check(cudaEventRecord(c.ev1, c.stream), "event");
    Check(cudaEventSynchronize(c.ev1), "sync");
    Check(cudaGetLastError(), "kernel launch");
    float ms = 0.f;
    Check(cudaEventElapsedTime(&ms, c.ev0, c.ev1), "elapsed");
    c.stats.device_ms = ms;
    c.stats.kernel_launches = (int64_t)done * c.launches_per_iter;
    ath::CheckSweepStatus(c);
    if (info) SolveInfo(c, info);
  });
}

int ath_batch_autotune(ath_batch *batch, int reps, int *sweep_threads) {
  return Guard([&] {
    if (!batch || reps < 1) throw ath::Error(ATH_ERR_ARG, "bad argument");
    auto &c = batch->core;
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    auto &run = *batch->run;
    // candidates: one launch per hyperplane with CTAs of 32..256 threads (a
    // thread per scalar cell, or with scalar solves present a group of lanes
    // per cell), and the persistent sweep with clusters of 1..8 CTAs of 256
    // threads
    struct Shape {
      int mode, threads, cluster;
    };
    std::vector<Shape> cand = {{0, 32, 1}, {0, 64, 1}, {0, 128, 1}, {0, 256, 1}};
    if (c.skinds & 1)
      for (int t : {32, 64, 128, 256}) cand.push_back({2, t, 1});
    // lane groups on small planes, a thread per cell on planes of at least
    // 32768 cells
    if (c.skinds & 1) cand.push_back({4, 32, 32768});
    // lane groups with the solves' chains run as 2 or 4 concurrent chains
    if ((c.skinds & 1) && c.nsolves > 1)
      for (int t : {32, 64})
        for (int k : {2, 4}) cand.push_back({2, t, k});
    if (c.skinds)
      for (int cl : {1, 2, 4, 8})
        if (run.MaxClusters(c.skinds, 256, cl) > 0) cand.push_back({1, 256, cl});
    // the persistent tile-queue sweep with tiles of one to eight warp rounds
    if (c.skinds)
      for (int ts : ath::TileSizes(c)) cand.push_back({3, ts, 0});
    const Shape keep{c.sweep_mode,
                     c.sweep_mode == 1 ? c.cl_threads
                                       : (c.sweep_mode == 3 ? c.tq_size : c.sweep_threads),
                     c.sweep_mode == 4 ? c.hy_items
                                       : (c.sweep_mode == 1 ? c.cl_size : c.sweep_groups)};
    auto apply = [&](const Shape &sh) {
      c.sweep_mode = sh.mode;
      if (sh.mode == 1) {
        c.cl_threads = sh.threads;
        c.cl_size = sh.cluster;
      } else if (sh.mode == 4) {
        c.sweep_threads = sh.threads;
        c.hy_items = sh.cluster;
      } else if (sh.mode == 3) {
        ath::EnsureTileQueue(c, sh.threads);
        c.tq_size = sh.threads;
      } else {
        c.sweep_threads = sh.threads;
        c.sweep_groups = std::max(1, sh.cluster);
      }
    };
    run.Snapshot(false);
    float best = 1e30f;
    Shape best_sh = keep;
    for (const Shape &sh : cand) {
      apply(sh);
      run.ResetGraph();
      run.Iterate(1);  // capture and warm
      Check(cudaEventRecord(c.ev0, c.stream), "event");
      run.Iterate(reps);
      Check(cudaEventRecord(c.ev1, c.stream), "event");
      Check(cudaEventSynchronize(c.ev1), "sync");
      ath::CheckSweepStatus(c);
      float ms = 0.f;
      Check(cudaEventElapsedTime(&ms, c.ev0, c.ev1), "elapsed");
      if (ms < best) {
        best = ms;
        best_sh = sh;
      }
      run.Snapshot(true);
    }
    apply(best_sh);
    ath::CountLaunches(c);
    run.ResetGraph();
    run.FreeSnapshot();
    Check(cudaGetLastError(), "kernel launch");
    if (sweep_threads) *sweep_threads = best_sh.threads;
  });
}

int ath_batch_sweep_shape(ath_batch *batch, int *mode, int *threads, int *cluster) {
  if (!batch) return ATH_ERR_ARG;
  const auto &c = batch->core;
  if (mode) *mode = c.sweep_mode;
  if (threads)
    *threads = c.sweep_mode == 1 ? c.cl_threads : (c.sweep_mode == 3 ? c.tq_size : c.sweep_threads);
  if (cluster)
    *cluster = c.sweep_mode == 1 ? c.cl_size
               : c.sweep_mode == 4 ? c.hy_items
               : c.sweep_mode == 3 ? 0
                                   : c.sweep_groups;
  return ATH_OK;
}

int ath_batch_set_sweep_shape(ath_batch *batch, int mode, int threads, int cluster) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    auto &c = batch->core;
    if (mode == 0 || mode == 2) {
      if (threads != 32 && threads != 64 && threads != 128 && threads != 256)
        throw ath::Error(ATH_ERR_ARG, "per-plane sweeps take CTAs of 32, 64, 128 or 256 threads");
      if (mode == 2 && !(c.skinds & 1))
        throw ath::Error(ATH_ERR_ARG, "lane groups serve scalar solves only");
      if (cluster != 0 && cluster != 1 && cluster != 2 && cluster != 4)
        throw ath::Error(ATH_ERR_ARG, "per-plane sweeps run 1, 2 or 4 concurrent chains");
      c.sweep_threads = threads;
      c.sweep_groups = std::max(1, cluster);
    } else if (mode == 1) {
      if (threads != 256 || cluster < 1 || cluster > 8 ||
          batch->run->MaxClusters(c.skinds, 256, cluster) <= 0)
        throw ath::Error(ATH_ERR_ARG, "persistent sweep: 256 threads and a launchable cluster");
      c.cl_threads = threads;
      c.cl_size = cluster;
    } else if (mode == 4) {
      if (threads != 32 && threads != 64 && threads != 128 && threads != 256)
        throw ath::Error(ATH_ERR_ARG, "per-plane sweeps take CTAs of 32, 64, 128 or 256 threads");
      if (!(c.skinds & 1)) throw ath::Error(ATH_ERR_ARG, "lane groups serve scalar solves only");
      if (cluster < 1) throw ath::Error(ATH_ERR_ARG, "hybrid sweep: a threshold of cells >= 1");
      c.sweep_threads = threads;
      c.hy_items = cluster;
    } else if (mode == 3) {
      if (!c.skinds || threads < 1 || threads > 4096)
        throw ath::Error(ATH_ERR_ARG, "tile-queue sweep: LU-SGS solves and tiles of 1..4096 cells");
      ath::EnsureTileQueue(c, threads);
      c.tq_size = threads;
    } else {
      throw ath::Error(ATH_ERR_ARG, "unknown sweep mode");
    }
    c.sweep_mode = mode;
    ath::CountLaunches(c);
    batch->run->ResetGraph();
  });
}

int ath_batch_sweep_wait_test(ath_batch *batch, long long poll_limit, int wait_never) {
  return Guard([&] {
    if (!batch || poll_limit < 0) throw ath::Error(ATH_ERR_ARG, "bad argument");
    auto &c = batch->core;
    c.tq_spin_limit = poll_limit;
    c.tq_wait_never = wait_never ? 1 : 0;
    batch->run->ResetGraph();
  });
}

int ath_batch_fill_ghosts(ath_batch *batch) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    batch->run->FillGhosts();
    Check(cudaStreamSynchronize(batch->core.stream), "sync");
    Check(cudaGetLastError(), "kernel launch");
  });
}

int ath_batch_residual(ath_batch *batch) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    batch->run->Residual();
    Check(cudaStreamSynchronize(batch->core.stream), "sync");
    Check(cudaGetLastError(), "kernel launch");
  });
}

// The local time step and the inverted diagonal are produced by the
// residual stage's cell kernel (they need only the spectral radius, the
// volume and the CFL); these two stages exist for call-surface parity and
// have nothing left to do.
int ath_batch_timestep(ath_batch *batch) { return batch ? ATH_OK : ATH_ERR_ARG; }
int ath_batch_diag_invert(ath_batch *batch) { return batch ? ATH_OK : ATH_ERR_ARG; }

int ath_batch_relax(ath_batch *batch) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    batch->run->Relax();
    Check(cudaStreamSynchronize(batch->core.stream), "sync");
    Check(cudaGetLastError(), "kernel launch");
    ath::CheckSweepStatus(batch->core);
  });
}

int ath_batch_update(ath_batch *batch, ath_norms *norms_h) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null batch");
    auto &c = batch->core;
    const int64_t it0 = c.iter_host;
    batch->run->Update();
    c.iter_host += 1;
    Check(cudaStreamSynchronize(c.stream), "sync");
    Check(cudaGetLastError(), "kernel launch");
    ath::ReadNorms(c, it0, 1, norms_h);
  });
}

int ath_batch_field_width(ath_batch *batch, int block, int field) {
  if (!batch || block < 0 || block >= batch->core.nblocks) return ATH_ERR_ARG;
  switch (field) {
    case ATH_FIELD_STATE:
    case ATH_FIELD_STATE_GHOSTS:
    case ATH_FIELD_RESID:
    case ATH_FIELD_DU:
      return batch->core.setup->blocks[block].nv;
    case ATH_FIELD_DT:
    case ATH_FIELD_AINV:
      return 1;
    case ATH_FIELD_SPECRAD:
      return 2;
    case ATH_FIELD_AUX:
      return 5;
    case ATH_FIELD_VELGRAD:
      return 9;
    case ATH_FIELD_GRADS:
      return 24;
    case ATH_FIELD_WALLDIST:
      return 1;
    case ATH_FIELD_CONS_N:
    case ATH_FIELD_CONS_NM1:
      return batch->core.setup->blocks[block].nv;
    default:
      return ATH_ERR_ARG;
  }
}

int ath_batch_get_field(ath_batch *batch, int block, int field, double *out_h) {
  return Guard([&] {
    if (!batch || !out_h) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto &c = batch->core;
    if (block < 0 || block >= c.nblocks) throw ath::Error(ATH_ERR_ARG, "block out of range");
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    Check(cudaStreamSynchronize(c.stream), "sync");
    const ath::Block &b = c.setup->blocks[block];
    const int64_t nc = b.NCell(), o = c.cell0[block], n = c.ncell;
    const int nv = b.nv;
    // w values of an SoA pool -> AoS output with `stride` values per cell
    // from `voff`; physical cells (k slowest) or the padded block
    auto gather = [&](const double *pool, int w, int stride, int voff, bool ghosts) {
      std::vector<double> h(nc);
      for (int v = 0; v < w; ++v) {
        Check(cudaMemcpy(h.data(), pool + v * n + o, nc * 8, cudaMemcpyDeviceToHost),
              "download");
        if (ghosts) {
          for (int64_t x = 0; x < nc; ++x) out_h[x * stride + voff + v] = h[x];
        } else {
          size_t q = 0;
          for (int k = 0; k < b.nk; ++k)
            for (int j = 0; j < b.nj; ++j)
              for (int i = 0; i < b.ni; ++i)
                out_h[(q++) * stride + voff + v] = h[b.Cell(i, j, k)];
        }
      }
    };
    const bool turb = nv > 5;
    switch (field) {
      case ATH_FIELD_STATE:
      case ATH_FIELD_STATE_GHOSTS: {
        const bool gh = field == ATH_FIELD_STATE_GHOSTS;
        gather(batch->W, 5, nv, 0, gh);
        if (turb) gather(batch->Wt, 2, nv, 5, gh);
        break;
      }
      case ATH_FIELD_RESID:
        gather(batch->R, 5, nv, 0, false);
        if (turb) gather(batch->Rt, 2, nv, 5, false);
        break;
      case ATH_FIELD_DT: gather(batch->dt, 1, 1, 0, false); break;
      case ATH_FIELD_SPECRAD: {
        // spectral radius (flow, turbulence; 0 without turbulence equations)
        const size_t m = (size_t)b.ni * b.nj * b.nk;
        std::fill(out_h, out_h + 2 * m, 0.0);
        gather(batch->lam, 1, 2, 0, false);
        if (turb) gather(batch->lamt, 1, 2, 1, false);
        break;
      }
      case ATH_FIELD_DU: batch->run->GetDU(block, out_h); break;
      case ATH_FIELD_AINV: batch->run->GetAinv(block, out_h); break;
      case ATH_FIELD_AUX: batch->run->GetAux(block, out_h); break;
      case ATH_FIELD_VELGRAD: batch->run->GetVelGrad(block, out_h); break;
      case ATH_FIELD_GRADS:
        if (!batch->ogr)
          throw ath::Error(ATH_ERR_UNSUPPORTED, "the cell gradients are kept by batches created "
                                                "with ATH_BATCH_OUTPUT_GRADS");
        gather(batch->ogr, 24, 24, 0, false);
        break;
      case ATH_FIELD_WALLDIST: {
        size_t q = 0;
        for (int k = 0; k < b.nk; ++k)
          for (int j = 0; j < b.nj; ++j)
            for (int i = 0; i < b.ni; ++i) out_h[q++] = b.wall_dist[b.Cell(i, j, k)];
        break;
      }
      case ATH_FIELD_CONS_N:
      case ATH_FIELD_CONS_NM1: {
        const auto &ph = c.setup->solves[b.solve].phys;
        const bool nm1 = field == ATH_FIELD_CONS_NM1;
        if (!batch->Un || !(nm1 ? ph.multilevel : (ph.multilevel || ph.nl_iters > 1)))
          throw ath::Error(ATH_ERR_UNSUPPORTED, nm1 ? "time n-1 is kept for bdf2 solves only"
                                                    : "time n is kept for time-accurate "
                                                      "solves only");
        gather(nm1 ? batch->Unm1 : batch->Un, nv, nv, 0, false);
        break;
      }
      default: throw ath::Error(ATH_ERR_ARG, "unknown field");
    }
  });
}

int ath_batch_set_state(ath_batch *batch, int block, const double *prim_h) {
  return Guard([&] {
    if (!batch || !prim_h) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto &c = batch->core;
    if (block < 0 || block >= c.nblocks) throw ath::Error(ATH_ERR_ARG, "block out of range");
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    Check(cudaStreamSynchronize(c.stream), "sync");
    const ath::Block &b = c.setup->blocks[block];
    const int64_t nc = b.NCell(), o = c.cell0[block], n = c.ncell;
    const int nv = b.nv;
    std::vector<double> h(nc);
    for (int v = 0; v < nv; ++v) {
      double *pool = v < 5 ? batch->W + v * n + o : batch->Wt + (v - 5) * n + o;
      Check(cudaMemcpy(h.data(), pool, nc * 8, cudaMemcpyDeviceToHost), "download");
      size_t q = 0;
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i) h[b.Cell(i, j, k)] = prim_h[(q++) * nv + v];
      Check(cudaMemcpy(pool, h.data(), nc * 8, cudaMemcpyHostToDevice), "upload");
    }
    // a state loaded before the run (initial condition or restart) gets its
    // temperature and viscosity, as after ReadRestart in the reference
    // (gridLevel::AuxillaryAndWidths src/gridLevel.cpp:433); the lagged
    // eddy viscosity stays that of the initial condition
    batch->run->RefreshAux(block);
  });
}

int ath_batch_set_state_nm1(ath_batch *batch, int block, const double *cons_h) {
  return Guard([&] {
    if (!batch) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto &c = batch->core;
    if (block < 0 || block >= c.nblocks) throw ath::Error(ATH_ERR_ARG, "block out of range");
    const ath::Block &b = c.setup->blocks[block];
    if (!batch->Unm1 || !c.setup->solves[b.solve].phys.multilevel)
      throw ath::Error(ATH_ERR_UNSUPPORTED, "time n-1 is kept for bdf2 solves only");
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    Check(cudaStreamSynchronize(c.stream), "sync");
    if (cons_h) {
      const int64_t nc = b.NCell(), o = c.cell0[block], n = c.ncell;
      const int nv = b.nv;
      std::vector<double> h(nc);
      for (int v = 0; v < nv; ++v) {
        double *pool = batch->Unm1 + v * n + o;
        Check(cudaMemcpy(h.data(), pool, nc * 8, cudaMemcpyDeviceToHost), "download");
        size_t q = 0;
        for (int k = 0; k < b.nk; ++k)
          for (int j = 0; j < b.nj; ++j)
            for (int i = 0; i < b.ni; ++i) h[b.Cell(i, j, k)] = cons_h[(q++) * nv + v];
        Check(cudaMemcpy(pool, h.data(), nc * 8, cudaMemcpyHostToDevice), "upload");
      }
    } else {
      batch->run->StoreTimeLevels(block);
    }
    const int32_t one = 1;
    Check(cudaMemcpy(&c.d_sstate[b.solve].nm1_given, &one, sizeof(one), cudaMemcpyHostToDevice),
          "upload");
  });
}

int ath_batch_pool_cells(ath_batch *batch, int64_t *ncell) {
  if (!batch || !ncell) return ATH_ERR_ARG;
  *ncell = batch->core.ncell;
  return ATH_OK;
}

int ath_batch_pool_vars(ath_batch *batch, int *nv) {
  if (!batch || !nv) return ATH_ERR_ARG;
  *nv = batch->core.any_rans ? 7 : 5;
  return ATH_OK;
}

int ath_batch_copy_state(ath_batch *batch, double *host, int to_device) {
  return Guard([&] {
    if (!batch || !host) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto &c = batch->core;
    Check(cudaSetDevice(c.ctx->device), "cudaSetDevice");
    const size_t bytes = 5 * (size_t)c.ncell * sizeof(double);
    const size_t tbytes = c.any_rans ? 2 * (size_t)c.ncell * sizeof(double) : 0;
    double *ht = host + 5 * (size_t)c.ncell;
    if (to_device) {
      Check(cudaMemcpyAsync(batch->W, host, bytes, cudaMemcpyHostToDevice, c.stream), "H2D");
      if (tbytes)
        Check(cudaMemcpyAsync(batch->Wt, ht, tbytes, cudaMemcpyHostToDevice, c.stream), "H2D");
    } else {
      Check(cudaMemcpyAsync(host, batch->W, bytes, cudaMemcpyDeviceToHost, c.stream), "D2H");
      if (tbytes)
        Check(cudaMemcpyAsync(ht, batch->Wt, tbytes, cudaMemcpyDeviceToHost, c.stream), "D2H");
    }
    Check(cudaStreamSynchronize(c.stream), "sync");
  });
}

int ath_batch_profile(ath_batch *batch, int reps, double ms[8]) {
  return Guard([&] {
    if (!batch || !ms || reps <= 0) throw ath::Error(ATH_ERR_ARG, "bad argument");
    Check(cudaSetDevice(batch->core.ctx->device), "cudaSetDevice");
    batch->run->Profile(reps, ms);
    Check(cudaGetLastError(), "kernel launch");
  });
}

namespace {
// eight independent FMA chains per thread; the sum is stored only when it
// matches a value it never takes, so the chains stay live
__global__ void __launch_bounds__(256) k_fp64_peak(double seed, int iters, double *sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + (double)(threadIdx.x + k);
  const double m = 0.999999999, c = 1e-9;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0) sink[0] = s;
}
}  // namespace

int ath_ctx_fp64_peak(ath_ctx *ctx, int reps, double *tflops) {
  return Guard([&] {
    if (!ctx || !tflops || reps < 1) throw ath::Error(ATH_ERR_ARG, "bad argument");
    Check(cudaSetDevice(ctx->device), "cudaSetDevice");
    int sms = 0;
    Check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "attr");
    // owned resources released on every path; a private non-blocking stream
    // so the measurement does not serialise with batches on other streams
    struct Res {
      cudaStream_t s = nullptr;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      double *sink = nullptr;
      ~Res() {
        if (s) cudaStreamSynchronize(s);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (sink) cudaFreeAsync(sink, s);
        if (s) {
          cudaStreamSynchronize(s);
          cudaStreamDestroy(s);
        }
      }
    } r;
    Check(cudaStreamCreateWithFlags(&r.s, cudaStreamNonBlocking), "stream");
    Check(cudaEventCreate(&r.e0), "event");
    Check(cudaEventCreate(&r.e1), "event");
    Check(cudaMallocAsync(&r.sink, sizeof(double), r.s), "cudaMallocAsync");
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fp64_peak<<<blocks, threads, 0, r.s>>>(1.0, iters, r.sink);  // warm-up
    Check(cudaGetLastError(), "kernel launch");
    double best = 0.0;
    for (int k = 0; k < reps; ++k) {
      Check(cudaEventRecord(r.e0, r.s), "event");
      k_fp64_peak<<<blocks, threads, 0, r.s>>>(1.0 + k, iters, r.sink);
      Check(cudaGetLastError(), "kernel launch");
      Check(cudaEventRecord(r.e1, r.s), "event");
      Check(cudaEventSynchronize(r.e1), "sync");
      float ms = 0.f;
      Check(cudaEventElapsedTime(&ms, r.e0, r.e1), "elapsed");
      const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
      best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    *tflops = best;
  });
}

int ath_batch_flags(const ath_batch *batch, int *flags) {
  if (!batch || !flags) return ATH_ERR_ARG;
  *flags = batch->core.flags;
  return ATH_OK;
}

int ath_batch_stats(ath_batch *batch, ath_stats *out) {
  if (!batch || !out) return ATH_ERR_ARG;
  *out = batch->core.stats;
  return ATH_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Serving: a request loop over independent solves.  Each admitted request
// is a device-resident batch with its own stream, so the iterations of all
// admitted requests overlap on the device; admission is first come, first
// served, when a slot is free and the request's device memory (estimated
// before anything is allocated) fits the context's budget.  Requests retire
// on the device when their residual drop is reached (or nonphysical); the
// host then copies the final state out and frees the request's memory,
// which admits the next requests.  A request's result does not depend on
// what else is resident: the batches share no data.
namespace ath {
namespace {

double NowMs() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Device bytes of a batch of this setup, estimated from its cell counts
// (the per-cell sizes of the pools plus the work lists), with headroom.
size_t EstimateBatchBytes(const Setup &st, int precision) {
  double bytes = 64.0 * (1 << 20);
  const double ts = precision == ATH_PREC_FP64 ? 8.0 : 4.0;
  for (const auto &b : st.blocks) {
    const auto &ph = st.solves[b.solve].phys;
    const double n = (double)b.NCell();
    const double nq = (double)b.ni * b.nj * b.nk;
    const bool visc = ph.eqn != ATH_EQN_EULER, blk = IsBlockSolver(ph.solver);
    double pc = 8.0 * (5 + 5 + 15 + 1 + 1 + 1 + 3 + 12) + 4.0 * 6;  // pools, lists
    if (precision == ATH_PREC_FP64) pc += 8.0 * 24;  // geometry tables
    if (visc) pc += 15 * ts + 8;
    if (blk) pc += 30 * ts + (visc ? 45 * ts : 0);
    double qc = ts * (5 + 5 + 5 + 24 + 6 + 2 + 1) + 4.0 * 8;
    if (blk) qc += ts * (48 + (visc ? 9 : 0) + 150);  // + stored off-diagonal blocks
    if (!blk && precision == ATH_PREC_FP64) qc += 8.0 * 9;  // neighbour terms of the sweeps
    if (ph.eqn == ATH_EQN_RANS) {
      // k, omega, their residual, radius, wall distance, inviscid fluxes
      // (FP64); viscous fluxes and per-face SST data; sweep arrays
      pc += 8.0 * (2 + 2 + 1 + 1 + 6) + ts * (6 + 54);
      qc += ts * (2 + 2 + (blk ? 8 + 24 : 2) + 2);
    }
    bytes += n * pc + nq * qc;
  }
  return (size_t)(bytes * 1.25);
}

}  // namespace
}  // namespace ath

struct ath_server {
  struct Req {
    int64_t id = 0;
    ath_setup *setup = nullptr;
    ath_batch *batch = nullptr;
    size_t est = 0;
    int state = 0;  // 0 queued, 1 active, 2 done
    double t_submit = 0, t_admit = 0, t_done = 0;
    int64_t launched = 0;
    int32_t *flag_h = nullptr;  // its slot of the server's page-locked active flags
    int slot = -1;
    cudaEvent_t ev = nullptr;
    ath_converge_info info{};
    std::vector<std::vector<double>> result;  // final state per block
  };
  ath_ctx *ctx = nullptr;
  int precision = ATH_PREC_FP64, chunk = 50, max_active = 16;
  int64_t max_iters = 100000;
  double drop = 1e-6;
  int64_t next_id = 1;
  size_t capacity = 0;  // device bytes the server may hand out
  size_t reserved = 0;  // estimates of the admitted requests
  std::deque<Req *> queue;
  std::vector<Req *> active;
  std::map<int64_t, Req *> all;
  std::vector<int64_t> finished;  // done, not yet reported by poll
  // page-locked copies of the admitted solves' active flags, one slot per
  // active request, allocated once (admission and retirement reuse slots
  // rather than allocate and free page-locked memory)
  int32_t *flags_h = nullptr;
  std::vector<int> free_slots;
};

namespace ath {
namespace {


void LaunchChunk(ath_server *S, ath_server::Req *r) {
  auto &c = r->batch->core;
  const int n = (int)std::min<int64_t>(S->chunk, S->max_iters - r->launched);
  r->batch->run->Iterate(n);
  c.iter_host += n;
  r->launched += n;
  Check(cudaMemcpyAsync(r->flag_h, &c.d_solves[0].active, sizeof(int32_t),
                        cudaMemcpyDeviceToHost, c.stream),
        "flag download");
  Check(cudaEventRecord(r->ev, c.stream), "event");
}

void Finish(ath_server *S, ath_server::Req *r) {
  auto &c = r->batch->core;
  Check(cudaStreamSynchronize(c.stream), "sync");
  SolveInfo(c, &r->info);
  r->result.resize(c.nblocks);
  for (int b = 0; b < c.nblocks; ++b) {
    const Block &bk = c.setup->blocks[b];
    r->result[b].resize((size_t)bk.ni * bk.nj * bk.nk * bk.nv);
    const int rc = ath_batch_get_field(r->batch, b, ATH_FIELD_STATE, r->result[b].data());
    if (rc != ATH_OK) throw Error(rc, "result download");
  }
  ath_batch_destroy(r->batch);
  r->batch = nullptr;
  S->reserved -= r->est;
  cudaEventDestroy(r->ev);
  r->ev = nullptr;
  S->free_slots.push_back(r->slot);
  r->slot = -1;
  r->flag_h = nullptr;
  ath_setup_destroy(r->setup);
  r->setup = nullptr;
  r->state = 2;
  r->t_done = NowMs();
  S->finished.push_back(r->id);
}

bool Admit(ath_server *S, ath_server::Req *r) {
  if (S->reserved + r->est > S->capacity || S->free_slots.empty()) return false;
  ath_batch *b = nullptr;
  const int rc = ath_batch_create(S->ctx, r->setup, S->precision, 0, &b);
  if (rc == ATH_ERR_NOMEM) return false;
  if (rc != ATH_OK) throw Error(rc, std::string("admission: ") + ath_last_error());
  r->batch = b;
  S->reserved += r->est;
  const int rt = ath_batch_set_target(b, 0, S->drop, 1);
  if (rt != ATH_OK) throw Error(rt, "target");
  r->slot = S->free_slots.back();
  S->free_slots.pop_back();
  r->flag_h = S->flags_h + r->slot;
  *r->flag_h = 1;
  Check(cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming), "event");
  r->state = 1;
  r->t_admit = NowMs();
  LaunchChunk(S, r);
  return true;
}

}  // namespace
}  // namespace ath

extern "C" {

int ath_server_create(ath_ctx *ctx, int precision, double drop, int64_t max_iters,
                      int chunk, int max_active, ath_server **out) {
  return Guard([&] {
    if (!ctx || !out || !(drop > 0.0) || max_iters < 1 || chunk < 1 || chunk > 1024 ||
        max_active < 1)
      throw ath::Error(ATH_ERR_ARG, "bad argument");
    if (precision != ATH_PREC_FP64 && precision != ATH_PREC_MIXED)
      throw ath::Error(ATH_ERR_ARG, "unknown precision");
    auto *S = new ath_server();
    S->ctx = ctx;
    S->precision = precision;
    S->drop = drop;
    S->max_iters = max_iters;
    S->chunk = chunk;
    S->max_active = max_active;
    if (ctx->budget) {
      S->capacity = ctx->budget;
    } else {
      Check(cudaSetDevice(ctx->device), "cudaSetDevice");
      size_t fr = 0, tot = 0;
      Check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
      const size_t reserve = (size_t)1 << 30;
      S->capacity = fr > reserve ? fr - reserve : 0;
    }
    Check(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (cudaHostAlloc(&S->flags_h, sizeof(int32_t) * (size_t)max_active, cudaHostAllocDefault) !=
        cudaSuccess) {
      delete S;
      throw ath::Error(ATH_ERR_CUDA, "cudaHostAlloc of the active flags failed");
    }
    for (int q = max_active - 1; q >= 0; --q) S->free_slots.push_back(q);
    *out = S;
  });
}

int ath_server_submit(ath_server *S, const char *inp_path, int64_t *id) {
  return Guard([&] {
    if (!S || !inp_path || !id) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto *r = new ath_server::Req();
    r->t_submit = ath::NowMs();
    // the cells' geometry and wall distance are computed on the server's GPU
    const int rc = ath_setup_from_input_dev(inp_path, S->ctx->device, &r->setup);
    if (rc != ATH_OK) {
      delete r;
      throw ath::Error(rc, ath_last_error());
    }
    if (r->setup->s.solves.size() != 1) {
      ath_setup_destroy(r->setup);
      delete r;
      throw ath::Error(ATH_ERR_ARG, "a request is one solve");
    }
    r->est = ath::EstimateBatchBytes(r->setup->s, S->precision);
    r->id = S->next_id++;
    S->queue.push_back(r);
    S->all[r->id] = r;
    *id = r->id;
  });
}

int ath_server_step(ath_server *S, int *n_active, int *n_queued) {
  return Guard([&] {
    if (!S) throw ath::Error(ATH_ERR_ARG, "null server");
    Check(cudaSetDevice(S->ctx->device), "cudaSetDevice");
    // progress: every request whose last chunk finished either retires or
    // gets its next chunk
    for (size_t i = 0; i < S->active.size();) {
      auto *r = S->active[i];
      const cudaError_t q = cudaEventQuery(r->ev);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      Check(q, "event query");
      if (*r->flag_h == 0 || r->launched >= S->max_iters) {
        ath::Finish(S, r);
        S->active.erase(S->active.begin() + (long)i);
        continue;
      }
      ath::LaunchChunk(S, r);
      ++i;
    }
    // admission, first come first served
    while (!S->queue.empty() && (int)S->active.size() < S->max_active) {
      auto *r = S->queue.front();
      if (!ath::Admit(S, r)) break;
      S->queue.pop_front();
      S->active.push_back(r);
    }
    if (n_active) *n_active = (int)S->active.size();
    if (n_queued) *n_queued = (int)S->queue.size();
  });
}

int ath_server_poll(ath_server *S, ath_request_status *out, int max, int *n) {
  return Guard([&] {
    if (!S || !n || (max > 0 && !out)) throw ath::Error(ATH_ERR_ARG, "bad argument");
    int k = 0;
    while (k < max && !S->finished.empty()) {
      auto *r = S->all.at(S->finished.front());
      S->finished.erase(S->finished.begin());
      ath_request_status &o = out[k++];
      std::memset(&o, 0, sizeof(o));
      o.id = r->id;
      o.iterations = r->info.iterations;
      o.drop = r->info.drop;
      o.converged = r->info.converged;
      o.queue_ms = r->t_admit - r->t_submit;
      o.latency_ms = r->t_done - r->t_submit;
      o.device_ms = r->info.ms;
    }
    *n = k;
  });
}

int ath_server_fetch(ath_server *S, int64_t id, int block, double *prim_out) {
  return Guard([&] {
    if (!S || !prim_out) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto it = S->all.find(id);
    if (it == S->all.end() || it->second->state != 2) throw ath::Error(ATH_ERR_ARG, "not done");
    auto *r = it->second;
    if (block < 0 || block >= (int)r->result.size()) throw ath::Error(ATH_ERR_ARG, "block");
    std::memcpy(prim_out, r->result[block].data(), r->result[block].size() * sizeof(double));
  });
}

int ath_server_release(ath_server *S, int64_t id) {
  return Guard([&] {
    if (!S) throw ath::Error(ATH_ERR_ARG, "null server");
    auto it = S->all.find(id);
    if (it == S->all.end() || it->second->state != 2) throw ath::Error(ATH_ERR_ARG, "not done");
    delete it->second;
    S->all.erase(it);
  });
}

int ath_server_destroy(ath_server *S) {
  if (!S) return ATH_OK;
  for (auto &kv : S->all) {
    auto *r = kv.second;
    if (r->batch) {
      cudaStreamSynchronize(r->batch->core.stream);
      ath_batch_destroy(r->batch);
    }
    if (r->ev) cudaEventDestroy(r->ev);
    if (r->setup) ath_setup_destroy(r->setup);
    delete r;
  }
  if (S->flags_h) cudaFreeHost(S->flags_h);
  delete S;
  return ATH_OK;
}

}  // extern "C"
