// Pointwise kernels of the fixed-count Jacobi-preconditioned CG solve for
// Sigma (pcg_fixed!, elliptic.jl:329-347) and of its discrete reverse.
//
// The operator applications run in k2_apply (EPI_PCG0 / EPI_PCG) and
// k2_apply_rev (SREV_PCG); these kernels do the vector updates between them.
// The per-instance inner products reduce deterministically: block tree sum ->
// one partial per block -> the instance's last block to finish adds the
// instance's partials in a fixed order (InstSum). The results are therefore
// identical from run to run and independent of the batch composition.
//
// Scalars live on the device, one per instance: rz_k = r_k . M^-1 r_k and
// pAp_k = p_k . A p_k for every iteration, with alpha_k = rz_k / (pAp_k + 1e-30)
// and beta_k = rz_{k+1} / (rz_k + 1e-30) (the reference's 1e-30 guards,
// elliptic.jl:338, 343): the tape of the scalar recurrence. An FP64 divide
// is a software sequence of ~20 FP64 instructions on GB300, so the quotients
// are formed once per instance, by the block that completes their inner
// product (InstSum), and the node kernels read them.
//
// The pointwise kernels (k2_pcg_update, k2_pcg_rev_update) run one block per
// tile group (TILE_GROUP tiles of one instance): thread t takes node t of
// every tile of the group, so the block reduction's synchronisation is paid
// once per group. The forward update reduces each tile of the group in its
// own fixed tree and writes partials[tile]; the persistent PCG kernel forms
// the same tile partials. The reverse update reduces the group as one and
// group j of an instance writes partials[tile0 + j].
#pragma once
#include "igr2d_kernels.cuh"  // Tiling2D
#include "igr_device.cuh"

namespace igrgpu {

constexpr int PCG_THREADS = 256;

// Node n of element-local index idx within the tile; false if the element is
// outside the mesh (ragged last tile). The tile shape is the operator
// kernels' (Tiling2D<NP>), a compile-time constant, so the index arithmetic
// needs no run-time integer division.
template <int NP>
__device__ __forceinline__ bool tile_node(const Tile2D& tl, const Inst2D& I, int idx, long long* n) {
  constexpr int nn = NP * NP, tx = Tiling2D<NP>::TX;
  const int e = idx / nn, nd = idx - e * nn;
  const int ex = tl.ex0 + e % tx, ey = tl.ey0 + e / tx;
  if (ex >= I.nex || ey >= I.ney) return false;
  *n = I.off + (long long)nn * ((long long)ex + (long long)I.nex * ey) + nd;
  return true;
}

// Forward iteration k, after A p_k:  x_{k+1} = x_k + alpha_k p_k,
// r_{k+1} = r_k - alpha_k A p_k, rz_{k+1} = r_{k+1} . M^-1 r_{k+1}.
struct PcgUpdateArgs {
  const Tile2D* tiles; const TileGroup* groups; const Inst2D* inst;
  const double *x_in, *p, *ap, *r_in, *cinvM;
  double *x_out, *r_out;
  const double* al;         // per-instance alpha_k
  double* partials;         // per-tile partials of rz_{k+1}
  InstSum isum;             // rz_{k+1} and beta_k
};

// Number of tile groups of an instance.
__host__ __device__ __forceinline__ int inst_groups(const Inst2D& I) { return (I.ntiles + TILE_GROUP - 1) / TILE_GROUP; }

// Writes a group's partial (group j of the instance to partials[tile0 + j])
// and, when fused, lets the instance's last group complete the sum (the
// reverse update's inner product).
__device__ __forceinline__ void group_partial(const InstSum& isum, const TileGroup& g, const Inst2D& I, double tot,
                                              double* partials) {
  const int ng = inst_groups(I);
  inst_sum_last_block(isum, g.inst, ng, tot, partials, I.tile0 + (g.first - I.tile0) / TILE_GROUP, I.tile0, ng);
}

// The partial of one tile's r . M^-1 r: node idx of the tile (its index in
// tile_node's order) contributes r_idx (r_idx m_idx) in slot idx of a 256-slot
// fixed tree (slots past the tile's nodes hold 0). Both the update kernel and
// the persistent PCG kernel form it this way, so their sums agree bitwise.
template <int P2>
__device__ __forceinline__ void tile_tree(double* s, int tid, int nthreads) {
  static_assert(P2 >= 64, "shared-memory levels down to 32 slots");
#pragma unroll
  for (int w = P2 / 2; w >= 32; w >>= 1) {
    for (int v = tid; v < w; v += nthreads) s[v] += s[v + w];
    __syncthreads();
  }
  if (tid < 32) {
    const double x = warp_tree_tail<32>(s[tid]);
    if (tid == 0) s[0] = x;
  }
  __syncthreads();
}

// Thread 0 stores the group's tile partials (tile g.first + j to
// partials[g.first + j]); with isum.cnt set the instance's last group (the
// counter counts groups) sums the instance's tile partials and completes the
// InstSum.
__device__ __forceinline__ void group_tile_partials(const InstSum& a, const TileGroup& g, const Inst2D& I,
                                                    const double* vals, int stride, double* partials) {
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    for (int j = 0; j < g.count; ++j) partials[g.first + j] = vals[j * stride];
    if (a.cnt) {
      __threadfence();
      s_last = atomicAdd(a.cnt + g.inst, 1) == inst_groups(I) - 1;
    }
  }
  if (!a.cnt) return;
  __syncthreads();
  if (!s_last || threadIdx.x >= 32) return;
  __threadfence();
  const double sum = warp_sum_partials(partials + I.tile0, I.ntiles);
  if (threadIdx.x == 0) {
    inst_sum_finish(a, g.inst, sum);
    a.cnt[g.inst] = 0;
  }
}

template <int NP>
__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_update(PcgUpdateArgs a) {
  constexpr int P2 = PCG_THREADS, G = TILE_GROUP;
  constexpr int cnt = Tiling2D<NP>::TE * NP * NP;
  static_assert(cnt <= P2, "one node of each tile per thread");
  __shared__ double s_red[G][P2];
  const TileGroup g = a.groups[blockIdx.x];
  const Inst2D I = a.inst[g.inst];
  const double al = a.al[g.inst];
  const int idx = threadIdx.x;
  long long n[G];
  bool ok[G];
#pragma unroll
  for (int j = 0; j < G; ++j) ok[j] = idx < cnt && j < g.count && tile_node<NP>(a.tiles[g.first + j], I, idx, &n[j]);
  double p[G], ap[G], x[G], r[G], im[G];
#pragma unroll
  for (int j = 0; j < G; ++j)
    if (ok[j]) { p[j] = a.p[n[j]]; ap[j] = a.ap[n[j]]; x[j] = a.x_in[n[j]]; r[j] = a.r_in[n[j]]; im[j] = a.cinvM[n[j]]; }
#pragma unroll
  for (int j = 0; j < G; ++j) {
    double part = 0.0;
    if (ok[j]) {
      a.x_out[n[j]] = fma(al, p[j], x[j]);
      const double rn = fma(-al, ap[j], r[j]);
      a.r_out[n[j]] = rn;
      part = fma(rn, rn * im[j], 0.0);
    }
    s_red[j][idx] = part;
  }
  __syncthreads();
#pragma unroll
  for (int w = P2 / 2; w >= 32; w >>= 1) {
    if (idx < w) {
#pragma unroll
      for (int j = 0; j < G; ++j) s_red[j][idx] += s_red[j][idx + w];
    }
    __syncthreads();
  }
  // the last five levels of tile j's tree in warp j (the same pairs as tile_tree)
  static_assert(G * 32 <= P2, "a warp per tile of the group");
  if ((idx >> 5) < G) {
    const int j = idx >> 5;
    const double x = warp_tree_tail<32>(s_red[j][idx & 31]);
    if ((idx & 31) == 0) s_red[j][0] = x;
  }
  __syncthreads();
  group_tile_partials(a.isum, g, I, &s_red[0][0], P2, a.partials);
}

// ---------------------------------------------------------------------------
// Reverse of forward iteration it (run for it = n-1 .. 0), first half:
//   p_{it+1} = z_{it+1} + beta p_it        -> zb = pb, pb <- beta pb
//   beta = rz_{it+1} / (rz_it + eps)        -> rzb_{it+1} += betab / (rz_it + eps)
//   rz_{it+1} = r_{it+1} . z_{it+1}, z_{it+1} = M^-1 r_{it+1}
//                                           -> rb += rzb_{it+1} z + M^-1 zb', iMb += zb' r
//   ab = -(rb . A p_it) + (xb . p_it)       (reduced; stored through RZB, PAPB)
// beta_it is read from the forward tape; rzb1 = RZB + betab / (rz_it + eps),
// with betab = pb . p_it from the previous reverse apply, is formed by the
// block that completes betab in the previous reverse apply (RZB1; 0 on the
// first reverse iteration, where pb = rb = 0). The instance's last block
// completes ab and sets RZB = rzb_it (its part known so far) and PAPB = the
// adjoint of pAp_it (InstSum mode 1); k2_apply_rev<SREV_PCG> finishes the
// iteration.
// ---------------------------------------------------------------------------
struct PcgRevArgs {
  const Tile2D* tiles; const TileGroup* groups; const Inst2D* inst;
  int first;
  double *pb, *rb, *iMb;
  const double *r1, *cinvM, *ap, *p, *xb;
  const double *beta, *rzb1;       // per-instance beta_it (tape) and rzb_{it+1}
  double* partials;
  InstSum isum;                    // mode 1: RZB, PAPB
};

template <int NP>
__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_rev_update(PcgRevArgs a) {
  constexpr int P2 = PCG_THREADS, G = TILE_GROUP;
  __shared__ double s_red[P2];
  const TileGroup g = a.groups[blockIdx.x];
  const Inst2D I = a.inst[g.inst];
  const double beta = a.beta[g.inst], rzb1 = a.first ? 0.0 : a.rzb1[g.inst];
  constexpr int cnt = Tiling2D<NP>::TE * NP * NP;
  double part = 0.0;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n[G];
    bool ok[G];
#pragma unroll
    for (int j = 0; j < G; ++j) ok[j] = j < g.count && tile_node<NP>(a.tiles[g.first + j], I, idx, &n[j]);
    double pbv[G], rbv[G], imb[G], r1[G], im[G], ap[G], xb[G], p[G];
#pragma unroll
    for (int j = 0; j < G; ++j)
      if (ok[j]) {
        pbv[j] = a.first ? 0.0 : a.pb[n[j]];
        rbv[j] = a.first ? 0.0 : a.rb[n[j]];
        imb[j] = a.first ? 0.0 : a.iMb[n[j]];
        r1[j] = a.r1[n[j]]; im[j] = a.cinvM[n[j]]; ap[j] = a.ap[n[j]]; xb[j] = a.xb[n[j]]; p[j] = a.p[n[j]];
      }
#pragma unroll
    for (int j = 0; j < G; ++j)
      if (ok[j]) {
        a.pb[n[j]] = beta * pbv[j];
        const double zb = fma(rzb1, r1[j], pbv[j]);
        double rb = fma(rzb1, r1[j] * im[j], rbv[j]);
        rb = fma(zb, im[j], rb);
        a.rb[n[j]] = rb;
        a.iMb[n[j]] = a.first ? zb * r1[j] : fma(zb, r1[j], imb[j]);
        part = fma(xb[j], p[j], fma(-rb, ap[j], part));
      }
  }
  const double tot = block_sum<P2>(part, s_red);
  group_partial(a.isum, g, I, tot, a.partials);
}

template <int NP>
void launch_k2_pcg_update(const PcgUpdateArgs& a, int nblocks, cudaStream_t s) {
  k2_pcg_update<NP><<<nblocks, PCG_THREADS, 0, s>>>(a);
}
template <int NP>
void launch_k2_pcg_rev_update(const PcgRevArgs& a, int nblocks, cudaStream_t s) {
  k2_pcg_rev_update<NP><<<nblocks, PCG_THREADS, 0, s>>>(a);
}

// Per-instance sums in a separate launch (InstSum with cnt null): one
// 64-thread block per instance over the instance's tile partials, or its
// group partials when grouped, in warp_sum_partials' order with the 64 lane
// sums on both warps (half the dependent FP64 adds of one warp).
static __global__ void __launch_bounds__(64) k2_inst_sum(const Inst2D* inst, const double* partials, int grouped, InstSum a) {
  __shared__ double s_acc[64];
  const int i = blockIdx.x;
  const Inst2D I = inst[i];
  const double* p = partials + I.tile0;
  const int count = grouped ? inst_groups(I) : I.ntiles;
  double acc = 0.0;
#pragma unroll 8
  for (int k = threadIdx.x; k < count; k += 64) acc += __ldcg(p + k);
  s_acc[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = s_acc[threadIdx.x] + s_acc[threadIdx.x + 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (threadIdx.x == 0) inst_sum_finish(a, i, x);
  }
}

// Reverse of the PCG start (p_0 = z_0, rz_0 = r_0 . z_0, z_0 = M^-1 r_0):
//   rb += rzb_0 z_0 + M^-1 (pb + rzb_0 r_0),  iMb += (pb + rzb_0 r_0) r_0.
// rb then holds the adjoint of r_0 = b - A x_0 for the final reverse apply.
struct PcgRevFinalArgs {
  const Tile2D* tiles; const Inst2D* inst;
  const double *pb, *r0, *cinvM, *RZB;
  double *rb, *iMb;
};

template <int NP>
__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_rev_final(PcgRevFinalArgs a) {
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const double rzb0 = a.RZB[tl.inst];
  constexpr int cnt = Tiling2D<NP>::TE * NP * NP;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n;
    if (!tile_node<NP>(tl, I, idx, &n)) continue;
    const double r0 = a.r0[n], im = a.cinvM[n];
    const double z0b = fma(rzb0, r0, a.pb[n]);
    a.rb[n] = a.rb[n] + fma(rzb0, r0 * im, z0b * im);
    a.iMb[n] = fma(z0b, r0, a.iMb[n]);
  }
}

template <int NP>
void launch_k2_pcg_rev_final(const PcgRevFinalArgs& a, int nblocks, cudaStream_t s) {
  k2_pcg_rev_final<NP><<<nblocks, PCG_THREADS, 0, s>>>(a);
}

}  // namespace igrgpu
