// Step, init and exchange kernels for __half population storage.
#include "lbm_impl.cuh"

namespace lbmh {
LBM_INSTANTIATE(__half)
}  // namespace lbmh
