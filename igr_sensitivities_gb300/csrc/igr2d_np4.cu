// 2D kernels instantiated for NP = 4 (polynomial degree 3).
#include "igr2d_launch_impl.cuh"
namespace igrgpu {
IGR2D_INSTANTIATE(4)
}  // namespace igrgpu
