// 2D kernels instantiated for NP = 5 (polynomial degree 4).
#include "igr2d_launch_impl.cuh"
namespace igrgpu {
IGR2D_INSTANTIATE(5)
}  // namespace igrgpu
