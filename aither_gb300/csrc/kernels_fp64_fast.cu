// The fast FP64 arithmetic of batch flag ATH_BATCH_FAST_FACES: the faces in
// their reduced-operation form, and the cell kernel, the scalar LU-SGS
// sweeps and the update.  Built with --fmad=true: products feeding sums
// contract to fused multiply-adds, one rounding instead of two and one FP64
// instruction instead of two.  Results are roundoff-equal to the
// reference's, not bit-equal; the bit-exact kernels stay in kernels_fp64.cu
// (--fmad=false).
#include "kernels_impl.cuh"

namespace ath {

void LaunchFastFaceFp64(int d, const Pools<double> &P, const int32_t *list,
                        const int32_t *cta_block, int ncta, cudaStream_t s) {
  if (ncta <= 0) return;
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
  // without turbulence solves the kernels are built without their rows
  const bool turb = (P.fkinds & 2) != 0;
  if (group) {
    LaunchSweepGroup<double>(P, items, n, forward, sweep, full, threads, chained, s);
  } else {
    const unsigned grid = (unsigned)((n + threads - 1) / threads);
    if (full && turb) k_sweep<double, true, true><<<grid, threads, 0, s>>>(P, items, n, forward, sweep);
    else if (full) k_sweep<double, true, false><<<grid, threads, 0, s>>>(P, items, n, forward, sweep);
    else if (turb) k_sweep<double, false, true><<<grid, threads, 0, s>>>(P, items, n, forward, sweep);
    else k_sweep<double, false, false><<<grid, threads, 0, s>>>(P, items, n, forward, sweep);
  }
}

void LaunchFastUpdateFp64(const Pools<double> &P, const int32_t *list, const int32_t *cta_block,
                          const int32_t *cta_pos0, NormPartial *partials, int ncta,
                          const SolveState *ss, cudaStream_t s) {
  if (ncta > 0)
    k_update<double><<<ncta, kCta, 0, s>>>(P, list, cta_block, cta_pos0, partials, ss);
}

}  // namespace ath
