// 2D kernels instantiated for NP = 3 (polynomial degree 2).
#include "igr2d_launch_impl.cuh"
namespace igrgpu {
IGR2D_INSTANTIATE(3)
}  // namespace igrgpu
