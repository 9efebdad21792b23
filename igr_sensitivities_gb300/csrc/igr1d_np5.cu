// 1D kernels instantiated for NP = 5 (p = 4).
#include "igr1d_launch_impl.cuh"

namespace igrgpu {
IGR1D_INSTANTIATE(5)
}  // namespace igrgpu
