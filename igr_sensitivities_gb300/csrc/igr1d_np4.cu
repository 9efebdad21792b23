// 1D kernels instantiated for NP = 4 (p = 3).
#include "igr1d_launch_impl.cuh"

namespace igrgpu {
IGR1D_INSTANTIATE(4)
}  // namespace igrgpu
