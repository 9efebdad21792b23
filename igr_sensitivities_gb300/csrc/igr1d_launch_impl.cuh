// Definitions of the 1D launchers declared in igr1d_launch.h; included once
// per NP by igr1d_np<NP>.cu.
#pragma once
#include "igr1d_launch.h"
#include "igr1d_rev_kernels.cuh"
#include "igr1d_ops_kernels.cuh"
#include "igr1d_pde_kernels.cuh"
#include "igr1d_sens_kernels.cuh"

namespace igrgpu {

// n_inst instances, a.cs CTAs each; cs > 1 launches thread-block clusters of
// cs CTAs (sizes above 8 need the non-portable opt-in). Returns the launch error.
template <class Args>
static cudaError_t launch_per_instance(void (*kernel)(Args), const Args& a, int n_inst, cudaStream_t s) {
  if (a.cs <= 1) {
    kernel<<<n_inst, T1, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (a.cs > 8) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n_inst * a.cs), 1, 1);
  cfg.blockDim = dim3(T1, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)a.cs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

template <int NP> cudaError_t launch_k1_forward(const Fwd1DArgs& a, int n_inst, cudaStream_t s) {
  return launch_per_instance<Fwd1DArgs>(k1_forward<NP>, a, n_inst, s);
}
template <int NP> cudaError_t launch_k1_adjoint(const Adj1DArgs& a, int n_inst, cudaStream_t s) {
  return launch_per_instance<Adj1DArgs>(k1_adjoint<NP>, a, n_inst, s);
}
template <int NP> cudaError_t launch_k1_tangent(const Tan1DArgs& a, int n_inst, cudaStream_t s) {
  return launch_per_instance<Tan1DArgs>(k1_tangent<NP>, a, n_inst, s);
}

template <int NP> cudaError_t launch_k1_pde_adjoint(const Pde1DArgs& a, int n_inst, cudaStream_t s) {
  return launch_per_instance<Pde1DArgs>(k1_pde_adjoint<NP>, a, n_inst, s);
}

template <int NP> cudaError_t launch_k1_ops(const Ops1DArgs& a, int n_inst, cudaStream_t s) {
  return launch_per_instance<Ops1DArgs>(k1_ops<NP>, a, n_inst, s);
}

#define IGR1D_INSTANTIATE(NP)                                                          \
  template cudaError_t launch_k1_forward<NP>(const Fwd1DArgs&, int, cudaStream_t);    \
  template cudaError_t launch_k1_adjoint<NP>(const Adj1DArgs&, int, cudaStream_t);    \
  template cudaError_t launch_k1_tangent<NP>(const Tan1DArgs&, int, cudaStream_t);    \
  template cudaError_t launch_k1_pde_adjoint<NP>(const Pde1DArgs&, int, cudaStream_t); \
  template cudaError_t launch_k1_ops<NP>(const Ops1DArgs&, int, cudaStream_t);

}  // namespace igrgpu
