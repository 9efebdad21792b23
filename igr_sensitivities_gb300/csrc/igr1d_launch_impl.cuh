// Definitions of the 1D launchers declared in igr1d_launch.h; included once
// per NP by igr1d_np<NP>.cu.
#pragma once
#include "igr1d_launch.h"
#include "igr1d_rev_kernels.cuh"
#include "igr1d_sens_kernels.cuh"

namespace igrgpu {

template <int NP> void launch_k1_forward(const Fwd1DArgs& a, int nb, cudaStream_t s) {
  k1_forward<NP><<<nb, T1, 0, s>>>(a);
}
template <int NP> void launch_k1_adjoint(const Adj1DArgs& a, int nb, cudaStream_t s) {
  k1_adjoint<NP><<<nb, T1, 0, s>>>(a);
}
template <int NP> void launch_k1_tangent(const Tan1DArgs& a, int nb, cudaStream_t s) {
  k1_tangent<NP><<<nb, T1, 0, s>>>(a);
}

#define IGR1D_INSTANTIATE(NP)                                                   \
  template void launch_k1_forward<NP>(const Fwd1DArgs&, int, cudaStream_t);    \
  template void launch_k1_adjoint<NP>(const Adj1DArgs&, int, cudaStream_t);    \
  template void launch_k1_tangent<NP>(const Tan1DArgs&, int, cudaStream_t);

}  // namespace igrgpu
