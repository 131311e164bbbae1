// Step, init and exchange kernels for float population storage.
#include "lbm_impl.cuh"

namespace lbmh {
LBM_INSTANTIATE(float)
}  // namespace lbmh
