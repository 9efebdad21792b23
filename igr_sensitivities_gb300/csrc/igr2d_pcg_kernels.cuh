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
// pAp_k = p_k . A p_k for every iteration (the tape of the scalar
// recurrence); alpha_k = rz_k / (pAp_k + 1e-30) and
// beta_k = rz_{k+1} / (rz_k + 1e-30) are recomputed where needed, with the
// reference's 1e-30 guards (elliptic.jl:338, 343). An FP64 divide is a
// software sequence of ~20 FP64 instructions on GB300, so one thread of each
// block forms these quotients and the block reads them from shared memory.
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
  const Tile2D* tiles; const Inst2D* inst; int np, tx, ty;
  const double *x_in, *p, *ap, *r_in, *cinvM;
  double *x_out, *r_out;
  const double *rz, *pap;   // per-instance rz_k, pAp_k
  double* partials;         // per-tile partials of rz_{k+1}
};

__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_update(PcgUpdateArgs a) {
  constexpr int P2 = PCG_THREADS;
  __shared__ double s_red[P2];
  __shared__ double s_al;
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  if (threadIdx.x == 0) s_al = a.rz[tl.inst] / (a.pap[tl.inst] + 1e-30);
  __syncthreads();
  const double al = s_al;
  const int cnt = a.tx * a.ty * a.np * a.np;
  double part = 0.0;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n;
    if (!tile_node(tl, I, a.np, a.tx, idx, &n)) continue;
    a.x_out[n] = fma(al, a.p[n], a.x_in[n]);
    const double r = fma(-al, a.ap[n], a.r_in[n]);
    a.r_out[n] = r;
    part = fma(r, r * a.cinvM[n], part);
  }
  const double tot = block_sum<P2>(part, s_red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = tot;
}

// ---------------------------------------------------------------------------
// Reverse of forward iteration it (run for it = n-1 .. 0), first half:
//   p_{it+1} = z_{it+1} + beta p_it        -> zb = pb, pb <- beta pb
//   beta = rz_{it+1} / (rz_it + eps)        -> rzb_{it+1} += betab / (rz_it + eps)
//   rz_{it+1} = r_{it+1} . z_{it+1}, z_{it+1} = M^-1 r_{it+1}
//                                           -> rb += rzb_{it+1} z + M^-1 zb', iMb += zb' r
//   ab = -(rb . A p_it) + (xb . p_it)       (reduced; stored through RZB, PAPB)
// betab = pb . p_it arrives from the previous reverse apply (BET), or is 0 on
// the first reverse iteration, where pb = rb = 0. The tile partials of ab go
// to partials; k2_tile_sum (PCG-reverse mode) then sets RZB = rzb_it (its part
// known so far) and PAPB = the adjoint of pAp_it, and k2_apply_rev<SREV_PCG>
// finishes the iteration.
// ---------------------------------------------------------------------------
struct PcgRevArgs {
  const Tile2D* tiles; const Inst2D* inst; int np, tx, ty;
  int first, it, ni;
  double *pb, *rb, *iMb;
  const double *r1, *cinvM, *ap, *p, *xb;
  const double *RZ;                // taped scalars: RZ[k*ni+i]
  const double *BET, *RZB;         // per-instance adjoint scalars
  double* partials;
};

__global__ void __launch_bounds__(PCG_THREADS) k2_pcg_rev_update(PcgRevArgs a) {
  constexpr int P2 = PCG_THREADS;
  __shared__ double s_red[P2];
  __shared__ double s_sc[2];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const int i = tl.inst;
  if (threadIdx.x == 0) {
    const double rz0 = a.RZ[(long long)a.it * a.ni + i], rz1 = a.RZ[(long long)(a.it + 1) * a.ni + i];
    const double e0 = rz0 + 1e-30;
    const double betab = a.first ? 0.0 : a.BET[i];
    s_sc[0] = rz1 / e0;                                  // beta
    s_sc[1] = (a.first ? 0.0 : a.RZB[i]) + betab / e0;   // adjoint of rz_{it+1}
  }
  __syncthreads();
  const double beta = s_sc[0], rzb1 = s_sc[1];
  const int cnt = a.tx * a.ty * a.np * a.np;
  double part = 0.0;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    long long n;
    if (!tile_node(tl, I, a.np, a.tx, idx, &n)) continue;
    const double pbv = a.first ? 0.0 : a.pb[n];
    double rbv = a.first ? 0.0 : a.rb[n];
    const double r1 = a.r1[n], im = a.cinvM[n];
    a.pb[n] = beta * pbv;
    const double zb = fma(rzb1, r1, pbv);
    rbv = fma(rzb1, r1 * im, rbv);
    rbv = fma(zb, im, rbv);
    a.rb[n] = rbv;
    a.iMb[n] = a.first ? zb * r1 : fma(zb, r1, a.iMb[n]);
    part = fma(a.xb[n], a.p[n], fma(-rbv, a.ap[n], part));
  }
  const double tot = block_sum<P2>(part, s_red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = tot;
}

// Per-instance sum of the tile partials (one block per instance, fixed
// order: thread t adds tiles t, t + 256, ..., then a block tree).
// mode 0: out[i] = sum. mode 1 (after k2_pcg_rev_update of iteration it):
// ab = sum, RZB[i] = -betab rz_{it+1} / (rz_it + eps)^2 + ab / (pAp_it + eps),
// PAPB[i] = -ab rz_it / (pAp_it + eps)^2, betab = BET[i] (0 when first).
struct TileSumArgs {
  const Inst2D* inst; const double* partials;
  double* out;
  int mode, first, it, ni;
  const double *RZ, *PAP, *BET;
  double *RZB, *PAPB;
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
    return;
  }
  const double rz0 = a.RZ[(long long)a.it * a.ni + i], rz1 = a.RZ[(long long)(a.it + 1) * a.ni + i];
  const double e0 = rz0 + 1e-30;
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
