// 1D kernels instantiated for NP = 2 (p = 1).
#include "igr1d_launch_impl.cuh"

namespace igrgpu {
IGR1D_INSTANTIATE(2)
}  // namespace igrgpu
