// Host-side launchers of the 1D per-instance kernels, explicitly
// instantiated for NP = 2..5 in igr1d_np<NP>.cu (compiled in parallel).
#pragma once
#include <cuda_runtime.h>

namespace igrgpu {

struct Fwd1DArgs;
struct Adj1DArgs;
struct Tan1DArgs;
struct Pde1DArgs;
struct Ops1DArgs;

// One launch for n_inst instances (a.cs CTAs per instance); returns the launch status.
template <int NP> cudaError_t launch_k1_forward(const Fwd1DArgs& a, int n_inst, cudaStream_t s);
template <int NP> cudaError_t launch_k1_adjoint(const Adj1DArgs& a, int n_inst, cudaStream_t s);
template <int NP> cudaError_t launch_k1_tangent(const Tan1DArgs& a, int n_inst, cudaStream_t s);
template <int NP> cudaError_t launch_k1_pde_adjoint(const Pde1DArgs& a, int n_inst, cudaStream_t s);
template <int NP> cudaError_t launch_k1_ops(const Ops1DArgs& a, int n_inst, cudaStream_t s);

}  // namespace igrgpu
