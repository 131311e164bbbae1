// Step, init and exchange kernels for __nv_bfloat16 population storage.
#include "lbm_impl.cuh"

namespace lbmh {
LBM_INSTANTIATE(__nv_bfloat16)
}  // namespace lbmh
