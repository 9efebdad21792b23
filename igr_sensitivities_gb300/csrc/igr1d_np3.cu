// 1D kernels instantiated for NP = 3 (p = 2).
#include "igr1d_launch_impl.cuh"

namespace igrgpu {
IGR1D_INSTANTIATE(3)
}  // namespace igrgpu
