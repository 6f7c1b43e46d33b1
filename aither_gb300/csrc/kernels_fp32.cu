// FP32 instantiation of the reconstruction, flux, spectral-radius and sweep
// kernels for the mixed-precision path.  The residual assembly, the
// conserved-state update and the norms stay FP64 inside these kernels.
#include "kernels_impl.cuh"

namespace ath {

template struct Launch<float>;

}  // namespace ath
