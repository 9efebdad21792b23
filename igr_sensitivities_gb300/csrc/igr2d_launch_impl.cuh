// Definitions of the 2D launchers declared in igr2d_launch.h. Included once
// per NP by igr2d_np<NP>.cu, which instantiates them explicitly.
#pragma once
#include "igr2d_launch.h"
#include "igr2d_rev_kernels.cuh"
#include "igr2d_sens_kernels.cuh"
#include "igr2d_pde_kernels.cuh"
#include "igr2d_pcg_persist.cuh"

namespace igrgpu {

template <int NP> int threads2d() { return Tiling2D<NP>::NT; }
template <int NP> void tile_shape2d(int* tx, int* ty) { *tx = Tiling2D<NP>::TX; *ty = Tiling2D<NP>::TY; }

template <int NP> void launch_k2_setup(const SetupArgs2D& a, int nb, cudaStream_t s) {
  k2_setup<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_apply(int epi, const ApplyArgs2D& a, int nb, cudaStream_t s) {
  if (epi == EPI_CHEB) k2_apply<NP, EPI_CHEB><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else if (epi == EPI_JACOBI) k2_apply<NP, EPI_JACOBI><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else if (epi == EPI_PCG0) k2_apply<NP, EPI_PCG0><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else if (epi == EPI_PCG) k2_apply<NP, EPI_PCG><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else k2_apply<NP, EPI_RESID><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_hyp_rk(const HypArgs2D& a, int nb, cudaStream_t s) {
  k2_hyp_rk<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_hyp_rev(const HypRevArgs2D& a, int nb, cudaStream_t s) {
  k2_hyp_rev<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_apply_rev(int srev, const ApplyRevArgs2D& a, int nb, cudaStream_t s) {
  if (srev == SREV_CHEB) k2_apply_rev<NP, SREV_CHEB><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else if (srev == SREV_JACOBI) k2_apply_rev<NP, SREV_JACOBI><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else if (srev == SREV_PCG) k2_apply_rev<NP, SREV_PCG><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
  else k2_apply_rev<NP, SREV_NONE><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_setup_rev(const SetupRevArgs2D& a, int nb, cudaStream_t s) {
  k2_setup_rev<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}

template <int NP> void launch_k2_sens_rhs(const SensRhsArgs2D& a, int nb, cudaStream_t s) {
  k2_sens_rhs<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_sens_hyp_rk(const SensHypArgs2D& a, int nb, cudaStream_t s) {
  k2_sens_hyp_rk<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}

template <int NP> void launch_k2_pde_prep(const PdePrepArgs2D& a, int nb, cudaStream_t s) {
  k2_pde_prep<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_pde_b(const PdeBArgs2D& a, int nb, cudaStream_t s) {
  k2_pde_b<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}
template <int NP> void launch_k2_pde_rk(const PdeRkArgs2D& a, int nb, cudaStream_t s) {
  k2_pde_rk<NP><<<nb, Tiling2D<NP>::NT, 0, s>>>(a);
}

template <int NP> int pcg_persist_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k2_pcg_persist<NP>, Tiling2D<NP>::NT, 0) != cudaSuccess) return 0;
  return n;
}
template <int NP> cudaError_t launch_k2_pcg_persist(const PcgPersistArgs& a, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3(Tiling2D<NP>::NT, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k2_pcg_persist<NP>, a);
}

#define IGR2D_INSTANTIATE(NP)                                                                        \
  template int threads2d<NP>();                                                                      \
  template void tile_shape2d<NP>(int*, int*);                                                        \
  template void launch_k2_setup<NP>(const SetupArgs2D&, int, cudaStream_t);                          \
  template void launch_k2_apply<NP>(int, const ApplyArgs2D&, int, cudaStream_t);                     \
  template void launch_k2_hyp_rk<NP>(const HypArgs2D&, int, cudaStream_t);                           \
  template void launch_k2_hyp_rev<NP>(const HypRevArgs2D&, int, cudaStream_t);                       \
  template void launch_k2_apply_rev<NP>(int, const ApplyRevArgs2D&, int, cudaStream_t);              \
  template void launch_k2_setup_rev<NP>(const SetupRevArgs2D&, int, cudaStream_t);                    \
  template void launch_k2_sens_rhs<NP>(const SensRhsArgs2D&, int, cudaStream_t);                      \
  template void launch_k2_sens_hyp_rk<NP>(const SensHypArgs2D&, int, cudaStream_t);                   \
  template void launch_k2_pde_prep<NP>(const PdePrepArgs2D&, int, cudaStream_t);                       \
  template void launch_k2_pde_b<NP>(const PdeBArgs2D&, int, cudaStream_t);                             \
  template void launch_k2_pde_rk<NP>(const PdeRkArgs2D&, int, cudaStream_t);                           \
  template int pcg_persist_blocks_per_sm<NP>();                                                        \
  template cudaError_t launch_k2_pcg_persist<NP>(const PcgPersistArgs&, int, cudaStream_t);

}  // namespace igrgpu
