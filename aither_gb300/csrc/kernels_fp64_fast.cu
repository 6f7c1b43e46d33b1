// The fast FP64 arithmetic of batch flag ATH_BATCH_FAST_FACES: the faces in
// their reduced-operation form, and the cell kernel, the scalar LU-SGS
// sweeps and the update.  Built with --fmad=true: products feeding sums
// contract to fused multiply-adds, one rounding instead of two and one FP64
// instruction instead of two.  Results are roundoff-equal to the
// reference's, not bit-equal; the bit-exact kernels stay in kernels_fp64.cu
// (--fmad=false).
#include "kernels_impl.cuh"

namespace ath {

// muscl_roe: every solve the kernel serves is MUSCL-Roe, and the kernel
// built for that alone (no other reconstruction or flux) runs
void LaunchFastFaceFp64(int d, const Pools<double> &P, const int32_t *list,
                        const int32_t *cta_block, int ncta, bool muscl_roe, cudaStream_t s) {
  if (ncta <= 0) return;
  if (muscl_roe) {
    if (d == 0) k_face<double, 0, false, true, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
    else if (d == 1) k_face<double, 1, false, true, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
    else k_face<double, 2, false, true, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
    return;
  }
  if (d == 0) k_face<double, 0, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  else if (d == 1) k_face<double, 1, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  else k_face<double, 2, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}

void LaunchFastCellFp64(const Pools<double> &P, const int32_t *list, const int32_t *cta_block,
                        int ncta, int kinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if ((kinds & 1) && (P.fkinds & 1))
    k_cell<double, false, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 1) && (P.fkinds & 2))
    k_cell<double, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 2) && (P.fkinds & 1))
    k_cell<double, true, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 2) && (P.fkinds & 2))
    k_cell<double, true, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}

void LaunchFastSweepFp64(const Pools<double> &P, const int2 *items, int n, int forward,
                         int sweep, bool full, int threads, bool group, bool chained,
                         cudaStream_t s) {
  if (n <= 0) return;
  if (group) {
    LaunchSweepGroup<double>(P, items, n, forward, sweep, full, threads, chained, s);
  } else {
    LaunchSweepCell<double>(P, items, n, forward, sweep, full, threads, chained, s);
  }
}

template <int D>
__global__ void __launch_bounds__(kCta) k_fast_fgeo(Pools<double> P, const int32_t *list,
                                                    const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const int64_t n = P.ncell, s = StrideOf(b, D);
  const double *wd = P.width[D];
  double dpL, dmL, dpR, dmR;
  MusclFastRatios(wd[c - 2 * s], wd[c - s], wd[c], wd[c + s], dpL, dmL, dpR, dmR);
  double *g = P.fgeo[D];
  g[c] = dpL;
  g[n + c] = dmL;
  g[2 * n + c] = dpR;
  g[3 * n + c] = dmR;
}

__global__ void __launch_bounds__(kCta) k_fast_cgeo(Pools<double> P, const int32_t *list,
                                                    const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double *fa = P.fa[d];
    const int64_t u = c + st[d];
    const double ax = fa[c] + fa[u], ay = fa[n + c] + fa[n + u], az = fa[2 * n + c] + fa[2 * n + u];
    const double rs = rsqrt(Dot(ax, ay, az, ax, ay, az));
    double *g = P.cgeo[d];
    g[c] = ax * rs;
    g[n + c] = ay * rs;
    g[2 * n + c] = az * rs;
    g[3 * n + c] = 0.5 * (fa[3 * n + c] + fa[3 * n + u]);
  }
}

void LaunchFastGeomFp64(const Pools<double> &P, const int32_t *const faces[3],
                        const int32_t *const face_cta_block[3], const int nface_cta[3],
                        const int32_t *cells, const int32_t *cell_cta_block, int ncell_cta,
                        cudaStream_t s) {
  if (nface_cta[0] > 0) k_fast_fgeo<0><<<nface_cta[0], kCta, 0, s>>>(P, faces[0], face_cta_block[0]);
  if (nface_cta[1] > 0) k_fast_fgeo<1><<<nface_cta[1], kCta, 0, s>>>(P, faces[1], face_cta_block[1]);
  if (nface_cta[2] > 0) k_fast_fgeo<2><<<nface_cta[2], kCta, 0, s>>>(P, faces[2], face_cta_block[2]);
  if (ncell_cta > 0) k_fast_cgeo<<<ncell_cta, kCta, 0, s>>>(P, cells, cell_cta_block);
}

void LaunchFastUpdateFp64(const Pools<double> &P, const int32_t *list, const int32_t *cta_block,
                          const int32_t *cta_pos0, NormPartial *partials, int ncta,
                          const SolveState *ss, cudaStream_t s) {
  if (ncta > 0)
    k_update<double><<<ncta, kCta, 0, s>>>(P, list, cta_block, cta_pos0, partials, ss);
}

}  // namespace ath
