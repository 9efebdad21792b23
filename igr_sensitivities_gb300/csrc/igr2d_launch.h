// Host-side launchers of the 2D kernel templates. Each is explicitly
// instantiated for NP = 2..5 (p = 1..4) in igr2d_np<NP>.cu, so the engine
// only sees these declarations and the per-NP objects compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "igr_device.cuh"

namespace igrgpu {

struct SetupArgs2D;
struct ApplyArgs2D;
struct HypArgs2D;
struct HypRevArgs2D;
struct ApplyRevArgs2D;
struct SetupRevArgs2D;
struct SensRhsArgs2D;
struct SensHypArgs2D;
struct PdePrepArgs2D;
struct PdeBArgs2D;
struct PdeRkArgs2D;
struct PcgPersistArgs;

template <int NP> int threads2d();
template <int NP> void launch_k2_setup(const SetupArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_apply(int epi, const ApplyArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_hyp_rk(const HypArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_hyp_rev(const HypRevArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_apply_rev(int srev, const ApplyRevArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_setup_rev(const SetupRevArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_sens_rhs(const SensRhsArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_sens_hyp_rk(const SensHypArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_pde_prep(const PdePrepArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_pde_b(const PdeBArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void launch_k2_pde_rk(const PdeRkArgs2D& a, int nblocks, cudaStream_t s);
template <int NP> void tile_shape2d(int* tx, int* ty);
// Persistent PCG solve: resident CTAs per SM of k2_pcg_persist, and its
// cooperative launch on `grid` CTAs (every CTA resident, or the launch fails).
template <int NP> int pcg_persist_blocks_per_sm();
template <int NP> cudaError_t launch_k2_pcg_persist(const PcgPersistArgs& a, int grid, cudaStream_t s);

}  // namespace igrgpu
