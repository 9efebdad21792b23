// Pointwise kernels of the fixed-count Jacobi-preconditioned CG solve for
// Sigma (pcg_fixed!, elliptic.jl:329-347) and of its discrete reverse.
//
// The operator applications run in k2_apply (EPI_PCG0 / EPI_PCG) and
// k2_apply_rev (SREV_PCG); these kernels do the vector updates between them.
// Each block covers one tile of elements (the same tile list as the operator
// kernels), so the per-instance inner products reduce deterministically:
// block tree sum -> one partial per tile -> k2_tile_sum adds an instance's
// partials in tile order (a separate launch: ordering across blocks comes from
// the kernel boundary, with no fences or atomics). The results are therefore
// identical from run to run and independent of the batch composition.
//
// Scalars live on the device, one per instance: rz_k = r_k . M^-1 r_k and
// pAp_k = p_k . A p_k for every iteration, with alpha_k = rz_k / (pAp_k + 1e-30)
// and beta_k = rz_{k+1} / (rz_k + 1e-30) (the reference's 1e-30 guards,
// elliptic.jl:338, 343): the tape of the scalar recurrence. An FP64 divide
// is a software sequence of ~20 FP64 instructions on GB300, so the quotients
// are formed once per instance, by k2_tile_sum as soon as their inner product
// is complete, and the node kernels read them.
//
// The pointwise kernels (k2_pcg_update, k2_pcg_rev_update) run one block per
// tile group (TILE_GROUP tiles of one instance): thread t takes node t of
// every tile of the group, so the block reduction is paid once per group.
// The group's partial goes to the entry of its first tile and the other
// entries of the group get 0, so k2_tile_sum reads the same per-tile layout
// as after the operator kernels.
#pragma once
#include "igr_device.cuh"

namespace igrgpu {

constexpr int PCG_THREADS = 256;

// Node n of element-local index idx within the tile; false if the element is
// outside the mesh (ragged last tile).
__device__ __forceinline__ bool tile_node(const Tile2D& tl, const Inst2D& I, int np, int tx, int idx, long long* n) {
  const int nn = np * np;
  const int e = idx / nn, nd = idx - e * nn;
  const int ex = tl.ex0 + e % tx, ey = tl.ey0 + e / tx;
  if (ex >= I.nex || ey >= I.ney) return false;
  *n = I.off + (long long)nn * ((long long)ex + (long long)I.nex * ey) + nd;
  return true;
}

// Forward iteration k, after A p_k:  x_{k+1} = x_k + alpha_k p_k,
// r_{k+1} = r_k - alpha_k A p_k, rz_{k+1} = r_{k+1} . M^-1 r_{k+1}.
struct PcgUpdateArgs {
  const Tile2D* tiles; const TileGroup* groups; const Inst2D* inst; int np, tx, ty;
  const double *x_in, *p, *ap, *r_in, *cinvM;
  double *x_out, *r_out;
  const double* al;         // per-instance alpha_k
  double* partials;         // per-tile partials of rz_{k+1}
};

// Writes a group's partial: the group sum to its first tile, 0 to the others.
__device__ __forceinline__ void group_partial(const TileGroup& g, double tot, double* partials) {
  if ((int)threadIdx.x < g.count) partials[g.first + threadIdx.x] = threadIdx.x == 0 ? tot : 0.0;
}

__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_update(PcgUpdateArgs a) {
  constexpr int P2 = PCG_THREADS, G = TILE_GROUP;
  __shared__ double s_red[P2];
  const TileGroup g = a.groups[blockIdx.x];
  const Inst2D I = a.inst[g.inst];
  const double al = a.al[g.inst];
  const int cnt = a.tx * a.ty * a.np * a.np;
  double part = 0.0;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n[G];
    bool ok[G];
#pragma unroll
    for (int j = 0; j < G; ++j) ok[j] = j < g.count && tile_node(a.tiles[g.first + j], I, a.np, a.tx, idx, &n[j]);
    double p[G], ap[G], x[G], r[G], im[G];
#pragma unroll
    for (int j = 0; j < G; ++j)
      if (ok[j]) { p[j] = a.p[n[j]]; ap[j] = a.ap[n[j]]; x[j] = a.x_in[n[j]]; r[j] = a.r_in[n[j]]; im[j] = a.cinvM[n[j]]; }
#pragma unroll
    for (int j = 0; j < G; ++j)
      if (ok[j]) {
        a.x_out[n[j]] = fma(al, p[j], x[j]);
        const double rn = fma(-al, ap[j], r[j]);
        a.r_out[n[j]] = rn;
        part = fma(rn, rn * im[j], part);
      }
  }
  const double tot = block_sum<P2>(part, s_red);
  group_partial(g, tot, a.partials);
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
// k2_tile_sum that completes betab (RZB1; 0 on the first reverse iteration,
// where pb = rb = 0). The tile partials of ab go to partials; k2_tile_sum
// (PCG-reverse mode) then sets RZB = rzb_it (its part known so far) and
// PAPB = the adjoint of pAp_it, and k2_apply_rev<SREV_PCG> finishes the
// iteration.
// ---------------------------------------------------------------------------
struct PcgRevArgs {
  const Tile2D* tiles; const TileGroup* groups; const Inst2D* inst; int np, tx, ty;
  int first;
  double *pb, *rb, *iMb;
  const double *r1, *cinvM, *ap, *p, *xb;
  const double *beta, *rzb1;       // per-instance beta_it (tape) and rzb_{it+1}
  double* partials;
};

__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_rev_update(PcgRevArgs a) {
  constexpr int P2 = PCG_THREADS, G = TILE_GROUP;
  __shared__ double s_red[P2];
  const TileGroup g = a.groups[blockIdx.x];
  const Inst2D I = a.inst[g.inst];
  const double beta = a.beta[g.inst], rzb1 = a.first ? 0.0 : a.rzb1[g.inst];
  const int cnt = a.tx * a.ty * a.np * a.np;
  double part = 0.0;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n[G];
    bool ok[G];
#pragma unroll
    for (int j = 0; j < G; ++j) ok[j] = j < g.count && tile_node(a.tiles[g.first + j], I, a.np, a.tx, idx, &n[j]);
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
  group_partial(g, tot, a.partials);
}

// Per-instance sum of the tile partials (one block per instance, fixed
// order: thread t adds tiles t, t + 256, ..., then a block tree).
// mode 0: out[i] = sum; with quot set, also
//   quot[i] = (qnum ? qnum[i] : sum) / ((qden ? qden[i] : sum) + 1e-30)
// (alpha_k = rz_k / (pAp_k + eps) after pAp_k, beta_k = rz_{k+1} / (rz_k + eps)
// after rz_{k+1}).
// mode 1 (after k2_pcg_rev_update of iteration it): ab = sum,
//   RZB[i] = -betab rz_{it+1} / (rz_it + eps)^2 + ab / (pAp_it + eps),
//   PAPB[i] = -ab rz_it / (pAp_it + eps)^2, betab = BET[i] (0 when first).
// mode 2 (after k2_apply_rev<SREV_PCG> of iteration it + 1, it >= 0):
//   BET[i] = betab = sum, RZB1[i] = RZB[i] + betab / (rz_it + eps).
struct TileSumArgs {
  const Inst2D* inst; const double* partials;
  double* out;
  const double *qnum, *qden;
  double* quot;
  int mode, first, it, ni;
  const double *RZ, *PAP;
  double *BET, *RZB, *PAPB, *RZB1;
};

__global__ void __launch_bounds__(PCG_THREADS) k2_tile_sum(TileSumArgs a) {
  constexpr int P2 = PCG_THREADS;
  __shared__ double s_red[P2];
  const int i = blockIdx.x;
  const Inst2D I = a.inst[i];
  double acc = 0.0;
  for (int k = threadIdx.x; k < I.ntiles; k += blockDim.x) acc += a.partials[I.tile0 + k];
  const double tot = block_sum<P2>(acc, s_red);
  if (threadIdx.x != 0) return;
  if (a.mode == 0) {
    a.out[i] = tot;
    if (a.quot) a.quot[i] = (a.qnum ? a.qnum[i] : tot) / ((a.qden ? a.qden[i] : tot) + 1e-30);
    return;
  }
  const double rz0 = a.RZ[(long long)a.it * a.ni + i];
  const double e0 = rz0 + 1e-30;
  if (a.mode == 2) {
    a.BET[i] = tot;
    a.RZB1[i] = a.RZB[i] + tot / e0;
    return;
  }
  const double rz1 = a.RZ[(long long)(a.it + 1) * a.ni + i];
  const double betab = a.first ? 0.0 : a.BET[i];
  const double den = a.PAP[(long long)a.it * a.ni + i] + 1e-30;
  a.RZB[i] = -betab * rz1 / (e0 * e0) + tot / den;
  a.PAPB[i] = -tot * rz0 / (den * den);
}

// Reverse of the PCG start (p_0 = z_0, rz_0 = r_0 . z_0, z_0 = M^-1 r_0):
//   rb += rzb_0 z_0 + M^-1 (pb + rzb_0 r_0),  iMb += (pb + rzb_0 r_0) r_0.
// rb then holds the adjoint of r_0 = b - A x_0 for the final reverse apply.
struct PcgRevFinalArgs {
  const Tile2D* tiles; const Inst2D* inst; int np, tx, ty;
  const double *pb, *r0, *cinvM, *RZB;
  double *rb, *iMb;
};

__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_rev_final(PcgRevFinalArgs a) {
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const double rzb0 = a.RZB[tl.inst];
  const int cnt = a.tx * a.ty * a.np * a.np;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n;
    if (!tile_node(tl, I, a.np, a.tx, idx, &n)) continue;
    const double r0 = a.r0[n], im = a.cinvM[n];
    const double z0b = fma(rzb0, r0, a.pb[n]);
    a.rb[n] = a.rb[n] + fma(rzb0, r0 * im, z0b * im);
    a.iMb[n] = fma(z0b, r0, a.iMb[n]);
  }
}

}  // namespace igrgpu
