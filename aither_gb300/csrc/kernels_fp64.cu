// FP64 instantiation of the per-iteration kernels.  Built with --fmad=false:
// every product and sum rounds separately, like the reference's host build,
// so FP64 results agree with the reference CPU code to a few ulps.
#include "kernels_impl.cuh"

namespace ath {

template struct Launch<double>;

// Geometry tables of bit-exact FP64 batches, formed with the expressions the
// kernels would evaluate per face and per cell (this unit's rounding): the
// faces' MUSCL width ratios (MusclRatios of both sides) and the cells'
// normalised average normals and areas (CellAvgNormal)
template <int D>
__global__ void __launch_bounds__(kCta) k_exact_fgeo(Pools<double> P, const int32_t *list,
                                                     const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const int64_t n = P.ncell, s = StrideOf(b, D);
  const double *wd = P.width[D];
  const double xm2 = wd[c - 2 * s], xm1 = wd[c - s], x0 = wd[c], xp1 = wd[c + s];
  double dpL, dmL, dpR, dmR;
  MusclRatios(xm2, xm1, x0, dpL, dmL);  // lower side: upwind2 c-2, upwind1 c-1, downwind c
  MusclRatios(xp1, x0, xm1, dpR, dmR);  // upper side: upwind2 c+1, upwind1 c, downwind c-1
  double *g = P.fgeo[D];
  g[c] = dpL;
  g[n + c] = dmL;
  g[2 * n + c] = dpR;
  g[3 * n + c] = dmR;
}

__global__ void __launch_bounds__(kCta) k_exact_cgeo(Pools<double> P, const int32_t *list,
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
    double ax, ay, az, fm;
    CellAvgNormal(fa[c], fa[n + c], fa[2 * n + c], fa[3 * n + c], fa[u], fa[n + u],
                  fa[2 * n + u], fa[3 * n + u], ax, ay, az, fm);
    double *g = P.cgeo[d];
    g[c] = ax;
    g[n + c] = ay;
    g[2 * n + c] = az;
    g[3 * n + c] = fm;
  }
}

void LaunchExactGeomFp64(const Pools<double> &P, const int32_t *const faces[3],
                         const int32_t *const face_cta_block[3], const int nface_cta[3],
                         const int32_t *cells, const int32_t *cell_cta_block, int ncell_cta,
                         cudaStream_t s) {
  if (nface_cta[0] > 0) k_exact_fgeo<0><<<nface_cta[0], kCta, 0, s>>>(P, faces[0], face_cta_block[0]);
  if (nface_cta[1] > 0) k_exact_fgeo<1><<<nface_cta[1], kCta, 0, s>>>(P, faces[1], face_cta_block[1]);
  if (nface_cta[2] > 0) k_exact_fgeo<2><<<nface_cta[2], kCta, 0, s>>>(P, faces[2], face_cta_block[2]);
  if (ncell_cta > 0) k_exact_cgeo<<<ncell_cta, kCta, 0, s>>>(P, cells, cell_cta_block);
}

}  // namespace ath
