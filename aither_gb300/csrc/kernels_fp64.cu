// FP64 instantiation of the per-iteration kernels.  Built with --fmad=false:
// every product and sum rounds separately, like the reference's host build,
// so FP64 results agree with the reference CPU code to a few ulps.
#include "kernels_impl.cuh"

namespace ath {

template struct Launch<double>;

}  // namespace ath
