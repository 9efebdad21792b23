// Device-side types shared by the 2D and 1D kernel families.
//
// Layout in HBM: every field (state variable, coefficient, tape slot) is one
// contiguous FP64 array over all instances of a batch group, instance-major.
// Inside an instance the node order is the reference's Julia column-major
// order, (n_p, n_p, N_ex, N_ey) with the x-node fastest
// (IGR_adjoints_2d/mesh.jl:85-88): the NP*NP nodes of an element are
// contiguous (128 B for P3), so each element is one aligned block.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace igrgpu {

constexpr int MAXNP = 5;  // p <= 4

// DG basis constants (IGR_adjoints_2d/basis.jl:7-12), passed by value as a
// kernel parameter (constant bank, broadcast reads).
struct BasisDev {
  int np;
  double D[MAXNP][MAXNP];   // D[i][k] = l_k'(xi_i)
  double w[MAXNP];          // LGL weights
  double xi[MAXNP];         // LGL nodes (node coordinates for windowed objectives)
  double W2[MAXNP][MAXNP];  // w_i * D[i][k]^2 (diagonal of the stiffness term)
  double cheb_theta, cheb_delta, cheb_sigma;  // elliptic.jl:373-378
  double hw;                // -1 / (2 w_0): SIP face coefficient factor
  double iw0, iwL;          // 1 / w_0, 1 / w_L
};

// One problem instance of a batch (2D): mesh, physics parameters and where
// its nodes start in every field array.
struct Inst2D {
  long long off;    // first node of this instance in every field
  int nex, ney;
  double lx, ly, dx, dy, jx, jy;
  double gamma, alpha, dt;
  // reciprocals precomputed on the host (an FP64 divide costs ~9 FMA slots)
  double ijx, ijy, idx, idy, ialpha;
  int tile0, ntiles;  // this instance's tiles in the tile list (contiguous)
};

// One 1D instance (IGR_adjoints_1d/mesh.jl:21-33): its nodes start at `off`
// in every batch field; its private scratch (tapes, solver vectors) is
// `scr_fields` arrays of NP*ne doubles starting at `soff` in the scratch arena.
struct Inst1D {
  long long off, soff;
  int ne, n_steps;
  double L, dx, J, iJ, idx;  // dx = L / ne, J = dx / 2, iJ = 1/J, idx = 1/dx
  double gamma, alpha, dt;
  double t_end;  // tangent: final time of the `while t < T` stepping
  double h;      // continuous adjoint: the backward step min(dt, T)
};

// A tile of TX x TY elements of one instance; blocks map 1:1 onto tiles.
struct Tile2D { int inst, ex0, ey0, pad; };

// Up to TILE_GROUP consecutive tiles of one instance (tiles first ..
// first + count - 1), the unit of the pointwise PCG kernels: one block per
// group amortises the block reduction over several tiles. Groups start at
// the instance's first tile, so group sums do not depend on the batch.
constexpr int TILE_GROUP = 4;
struct TileGroup { int inst, first, count, pad; };

// Operator-level calls of the 1D package, one evaluation per instance (k1_ops).
enum : int {
  OP1_APPLY_SIP = 0,  // apply_sip!, elliptic.jl:32-116: y = A(rho, alpha) x
  OP1_IGR_RHS = 1,    // compute_igr_rhs!, elliptic.jl:126-154, and compute_sip_diagonal, :206-253
  OP1_SOLVE = 2,      // solve_elliptic!, elliptic.jl:451-467 (Sigma warm start in, solution out)
  OP1_HYP_RHS = 3,    // compute_hyperbolic_rhs!, hyperbolic.jl:23-83
  OP1_EULER_RHS = 4,  // compute_igr_euler_rhs!, forward.jl:24-33
  OP1_CG = 5          // cg_solve! / cg_fixed!, elliptic.jl:163-199 / 265-292, with apply_A! = apply_sip!
};

// Status word shared by the kernels and the host (device memory).
enum : int { DEV_OK = 0, DEV_NONFINITE = 1, DEV_TIMEOUT = 2 };

__device__ __forceinline__ void flag_nonfinite(int* status) {
  if (status) atomicOr(status, DEV_NONFINITE);
}

// Comparisons on bit patterns. GB300 issues a double compare (DSETP), fmax and
// isfinite through the FP64 unit at ~94 cycles per warp instruction per SM
// sub-partition (measured with a micro-probe; a DFMA takes ~64), while the
// same decisions on the IEEE 754 encodings run on the integer pipe at a few
// cycles. For doubles >= +0 (wave speeds, inverse densities, penalties) the
// encodings, read as signed 64-bit integers, order exactly like the numbers,
// so these give the same decisions and the same results as the double forms.
__device__ __forceinline__ bool gt_nonneg(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}
// (a > b) ? a : b for a, b >= +0
__device__ __forceinline__ double max_nonneg(double a, double b) { return gt_nonneg(a, b) ? a : b; }
// x is +-inf or NaN (all exponent bits set)
__device__ __forceinline__ bool nonfinite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) == 0x7ff00000; }
// !(x > 0) || !isfinite(x)
__device__ __forceinline__ bool not_positive_finite(double x) {
  return __double_as_longlong(x) <= 0 || nonfinite_bits(x);
}

// The last levels of a pairwise tree whose 32 (or fewer) remaining values sit
// in the lanes of one warp: lane v adds lane v + w for w = W/2 .. 1, the pairs
// (and so the bits) of the shared-memory tree; lane 0 ends with the sum.
template <int W>
__device__ __forceinline__ double warp_tree_tail(double x) {
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) {
    const double u = __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) < o) x += u;
  }
  return x;
}

// Deterministic sum over the threads of a block (fixed pairwise tree: slot v
// adds slot v + w for w = P2/2 .. 1). P2 is a power of two >= blockDim.x;
// every thread must call it; s_red holds P2 doubles. The levels down to 32
// slots run in shared memory, the last five in warp 0 by shuffles (the same
// pairs). Returns the sum to every thread.
template <int P2>
__device__ __forceinline__ double block_sum(double v, double* s_red) {
  constexpr int W = P2 < 32 ? P2 : 32;
  const int tid = threadIdx.x;
  s_red[tid] = v;
  for (int k = tid + blockDim.x; k < P2; k += blockDim.x) s_red[k] = 0.0;
  __syncthreads();
#pragma unroll
  for (int w = P2 / 2; w >= 32; w >>= 1) {
    if (tid < w) s_red[tid] += s_red[tid + w];
    __syncthreads();
  }
  if (tid < 32) {
    const double x = warp_tree_tail<W>(tid < W ? s_red[tid] : 0.0);
    if (tid == 0) s_red[0] = x;
  }
  __syncthreads();
  const double r = s_red[0];
  __syncthreads();
  return r;
}

// Per-instance inner products of the PCG solve and of its reverse. Every
// block of an instance writes one partial; the instance's sum is the
// canonical warp sum of its partials (warp_sum_partials), formed either by
// the instance's last block inside the producing kernel (cnt set: the block
// fences its partial and counts itself in cnt[inst]; the block that brings
// the count to the instance's number of blocks sums and resets the counter,
// and no block waits for another) or by k2_inst_sum in a separate launch
// (cnt null). Both give the same bits, which do not depend on which block
// finishes last nor on the batch. The fence holds each block's SM slot until
// its partial is visible, which costs more than the extra launch once a
// kernel runs many waves of blocks, so the host fuses only small grids.
//
// What is done with the sum s of instance i (one thread):
//   mode 0: out[i] = s and, with quot set,
//           quot[i] = (qnum ? qnum[i] : s) / ((qden ? qden[i] : s) + eps)
//           (alpha_k = rz_k / (pAp_k + eps), beta_k = rz_{k+1} / (rz_k + eps));
//           eps = 1e-30 in the fixed-count solvers, 0 in cg_solve! (elliptic.jl:292);
//   mode 1 (reverse iteration it, ab = s): RZB[i] = -betab rz_{it+1} / (rz_it + eps)^2
//           + ab / (pAp_it + eps), PAPB[i] = -ab rz_it / (pAp_it + eps)^2,
//           betab = BET[i] (0 when first);
//   mode 2 (betab = s of reverse iteration it): BET[i] = s,
//           RZB1[i] = RZB[i] + s / (rz_it + eps).
// The 1e-30 guards are the reference's (elliptic.jl:338, 343).
struct InstSum {
  int* cnt;          // per-instance completion counters, 0 between launches
  double* out;
  const double *qnum, *qden;
  double* quot;
  int mode, first, it, ni;
  double eps;        // mode 0 quotient guard
  const double *RZ, *PAP;
  double *BET, *RZB, *PAPB, *RZB1;
};

__device__ __forceinline__ void inst_sum_finish(const InstSum& a, int i, double s) {
  if (a.mode == 0) {
    a.out[i] = s;
    if (a.quot) a.quot[i] = (a.qnum ? a.qnum[i] : s) / ((a.qden ? a.qden[i] : s) + a.eps);
    return;
  }
  const double rz0 = a.RZ[(long long)a.it * a.ni + i];
  const double e0 = rz0 + 1e-30;
  if (a.mode == 2) {
    a.BET[i] = s;
    a.RZB1[i] = a.RZB[i] + s / e0;
    return;
  }
  const double rz1 = a.RZ[(long long)(a.it + 1) * a.ni + i];
  const double betab = a.first ? 0.0 : a.BET[i];
  const double den = a.PAP[(long long)a.it * a.ni + i] + 1e-30;
  a.RZB[i] = -betab * rz1 / (e0 * e0) + s / den;
  a.PAPB[i] = -s * rz0 / (den * den);
}

// The canonical sum of count partials: 64 strided lane sums (lane v adds
// partials v, v + 64, ... in order, from 0), then lane l < 32 adds lane
// l + 32's sum to its own, then a fixed shuffle tree. One warp forms it here
// (lane l carries lanes l and l + 32); lane 0 holds the sum. A CTA of 64
// threads forms the same bits with its two warps' lane sums in parallel
// (sum_lanes64), which halves the dependent FP64 adds on its critical path.
__device__ __forceinline__ double warp_sum_partials(const double* p, int count) {
  const int l = threadIdx.x & 31;
  double a0 = 0.0, a1 = 0.0;
#pragma unroll 8
  for (int k = l; k < count; k += 64) {
    a0 += __ldcg(p + k);
    if (k + 32 < count) a1 += __ldcg(p + k + 32);
  }
  double acc = a0 + a1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  return acc;
}

// warp_sum_partials' sum of v[0 .. count) (shared memory) by every thread of
// the CTA (blockDim >= 32): the 64 lane sums in parallel, then warp 0 adds
// them up. Every thread gets the sum (*s_sum: shared).
__device__ __forceinline__ double sum_lanes64(const double* v, int count, double* s_sum) {
  __shared__ double s_acc[64];
  __syncthreads();
  for (int lane = threadIdx.x; lane < 64; lane += blockDim.x) {
    double a = 0.0;
    for (int k = lane; k < count; k += 64) a += v[k];
    s_acc[lane] = a;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double acc = s_acc[threadIdx.x] + s_acc[threadIdx.x + 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *s_sum = acc;
  }
  __syncthreads();
  return *s_sum;
}

// Called by every thread (blockDim >= 32) with the block's partial v, known
// to thread 0, which stores it to partials[slot]. With a.cnt set, the last of
// the instance's `nblocks` blocks then sums partials[first .. first + count)
// and applies inst_sum_finish. Only the partial is fenced: everything else
// the block writes is read by later launches.
__device__ __forceinline__ void inst_sum_last_block(const InstSum& a, int inst, int nblocks, double v, double* partials,
                                                    int slot, int first, int count) {
  __shared__ int s_last;
  if (!a.cnt) {
    if (threadIdx.x == 0) partials[slot] = v;
    return;
  }
  if (threadIdx.x == 0) {
    partials[slot] = v;
    __threadfence();
    s_last = atomicAdd(a.cnt + inst, 1) == nblocks - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x >= 32) return;
  __threadfence();
  const double s = warp_sum_partials(partials + first, count);
  if (threadIdx.x == 0) {
    inst_sum_finish(a, inst, s);
    a.cnt[inst] = 0;
  }
}

// Instance of global node n (binary search over the instances' first nodes).
__device__ __forceinline__ int find_inst(const Inst2D* inst, int ninst, long long n) {
  int lo = 0, hi = ninst - 1;
  while (lo < hi) { const int mid = (lo + hi + 1) / 2; if (inst[mid].off <= n) lo = mid; else hi = mid - 1; }
  return lo;
}

// Quadrature weight w_i w_j Jx Jy and coordinates (mesh.jl:116-122) of the
// instance-local node `local` in the Julia (n_p, n_p, N_ex, N_ey) order.
__device__ __forceinline__ void node_coords2d(const BasisDev& B, const Inst2D& I, long long local, double* c, double* x, double* y) {
  const int nn = B.np * B.np;
  const long long el = local / nn;
  const int nd = (int)(local % nn);
  const int i = nd % B.np, j = nd / B.np;
  const int ex = (int)(el % I.nex), ey = (int)(el / I.nex);
  *c = B.w[i] * B.w[j] * I.jx * I.jy;
  *x = ex * I.dx + I.jx * (1.0 + B.xi[i]);
  *y = ey * I.dy + I.jy * (1.0 + B.xi[j]);
}

// Smallest power of two >= n (n <= 1024), for block_sum's scratch size.
__host__ __device__ constexpr int pow2_at_least(int n) {
  return n <= 1 ? 1 : (n <= 2 ? 2 : (n <= 4 ? 4 : (n <= 8 ? 8 : (n <= 16 ? 16 : (n <= 32 ? 32 : (n <= 64 ? 64 :
         (n <= 128 ? 128 : (n <= 256 ? 256 : (n <= 512 ? 512 : 1024)))))))));
}

}  // namespace igrgpu
