// Step, init and exchange kernels for double population storage.
#include "lbm_impl.cuh"

namespace lbmh {
LBM_INSTANTIATE(double)
}  // namespace lbmh
