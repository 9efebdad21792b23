// 2D kernels instantiated for NP = 2 (polynomial degree 1).
#include "igr2d_launch_impl.cuh"
namespace igrgpu {
IGR2D_INSTANTIATE(2)
}  // namespace igrgpu
