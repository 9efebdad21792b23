// One fixed-count Jacobi-preconditioned CG solve (pcg_fixed!, elliptic.jl:329-347)
// in a single persistent launch.
//
// The two-kernel form (k2_apply<EPI_PCG> + k2_pcg_update per iteration, each
// completing its inner product in its last block) spends much of a small
// instance's iteration on two launches and the latency of two short kernels.
// Here one grid of co-resident CTAs (a cooperative launch; at most one tile per
// CTA) runs the whole solve, with a grid barrier after each inner product:
//   phase A: p_k formed on load, A p_k, per-tile partials of p_k . A p_k
//            | barrier: the last CTA to arrive forms pAp_k and alpha_k |
//   phase B: x_{k+1}, r_{k+1} on the CTA's own tiles, per-tile partials of r . M^-1 r
//            | barrier: the last CTA to arrive forms rz_{k+1} and beta_k |
// The operator runs the same apply_tile code and block tree as k2_apply, the
// update forms each tile's partial in the same 256-slot tree as k2_pcg_update,
// and the scalars come from the same canonical sums of the tile partials, so
// the result is bitwise the two-kernel result.
//
// The barrier counts arrivals in groups of 32 CTAs (one counter per group, on
// its own cache line, then one top counter), so that no single address takes
// an atomic from every CTA, and releases the grid by advancing a generation
// word; its atomics and loads carry GPU-scope release / acquire semantics
// instead of full fences. Waits are bounded: a CTA that waits longer than
// PCG_BARRIER_NS sets DEV_TIMEOUT in the status word and the kernel returns
// (the host reports IGR_ETIMEOUT). With a cooperative launch every CTA is resident, so the limit
// is a guard, not the path.
#pragma once
#include "igr2d_kernels.cuh"
#include "igr2d_pcg_kernels.cuh"

namespace igrgpu {

constexpr int PCG_PERSIST_MAX_INST = 32;            // instances of a plan the persistent form takes
constexpr long long PCG_BARRIER_NS = 1000000000LL;  // grid barrier wait limit (1 s)
constexpr int BAR_GROUP = 32;                       // CTAs per arrival counter
// barrier words: generation at [0], top counter at [32], group counter g at [64 + 32 g] (128-byte lines)
__host__ __device__ constexpr int bar_words(int nblocks) { return 64 + 32 * ((nblocks + BAR_GROUP - 1) / BAR_GROUP); }

struct GridBarrier {
  unsigned* words;  // zero before the launch
  int* status;      // DEV_TIMEOUT on a wait past the limit
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// atomic add with acquire-release semantics at GPU scope; returns the old value
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Thread 0, after a CTA barrier: counts this CTA's arrival (releasing the
// CTA's writes and acquiring those of the CTAs that arrived before it in its
// group); true for the CTA that arrives last overall. Grids of at most
// BAR_GROUP CTAs count on the top counter alone.
__device__ __forceinline__ bool bar_arrive(const GridBarrier& g, unsigned nblocks) {
  const unsigned ngrp = (nblocks + BAR_GROUP - 1) / BAR_GROUP;
  if (ngrp > 1) {
    const unsigned grp = blockIdx.x / BAR_GROUP;
    const unsigned members = min((unsigned)BAR_GROUP, nblocks - grp * BAR_GROUP);
    unsigned* gc = g.words + 64 + 32 * grp;
    if (atom_add_acq_rel_u32(gc, 1u) != members - 1) return false;
    st_relaxed_u32(gc, 0u);  // every member has arrived; none touches it again before the release
  }
  if (atom_add_acq_rel_u32(g.words + 32, 1u) != (ngrp > 1 ? ngrp : nblocks) - 1) return false;
  st_relaxed_u32(g.words + 32, 0u);
  return true;
}

// Grid barrier of the launch's nblocks CTAs; every thread calls it. The CTA
// that arrives last runs last_work() (every thread of it; the partials every
// CTA wrote before arriving are visible to it) and then releases the others by
// advancing the generation. Writes before the barrier are visible to every CTA
// after it. Returns false when a wait timed out (the caller returns).
template <class F>
__device__ __forceinline__ bool grid_barrier(const GridBarrier& g, unsigned nblocks, F&& last_work) {
  __shared__ unsigned s_gen;
  __shared__ int s_last, s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_gen = ld_acquire_u32(g.words);
    s_last = bar_arrive(g, nblocks) ? 1 : 0;
  }
  __syncthreads();
  int ok = 1;
  if (s_last) {
    last_work();
    __syncthreads();
    if (threadIdx.x == 0) atom_add_acq_rel_u32(g.words, 1u);
  } else if (threadIdx.x == 0) {
    const unsigned long long t0 = global_ns();
    while (ld_acquire_u32(g.words) == s_gen) {
      if (global_ns() - t0 > (unsigned long long)PCG_BARRIER_NS) {
        atomicOr(g.status, DEV_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
  }
  if (threadIdx.x == 0) {
    if (ok && (*(volatile int*)g.status & DEV_TIMEOUT)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

struct PcgPersistArgs {
  ApplyArgs2D op;                  // tiles, instances, basis, coefficients, b, cinvM; op.partials: per tile
  int ntiles, ninst, n_iter;
  const double* x0;                // warm start (read only)
  double *xout, *r, *p[2], *ap;    // solution and the CG vectors
  double* upart;                   // per-tile partials of r . M^-1 r
  double* scal;                    // per instance: rz_0..rz_n, pAp_0..pAp_{n-1}, alpha, beta (as pcg_solve)
  double* beta_cta;                // per CTA and instance: beta_{k-1} for the operator loads
  double eps;
  GridBarrier bar;
};

// Warp 0 (of the last CTA): the canonical sum of each instance's tile
// partials, handed to f(i, sum) on lane 0.
template <class F>
__device__ __forceinline__ void inst_tile_sums(const Inst2D* inst, int ninst, const double* partials, F&& f) {
  if (threadIdx.x >= 32) return;
  for (int i = 0; i < ninst; ++i) {
    const Inst2D I = inst[i];
    const double s = warp_sum_partials(partials + I.tile0, I.ntiles);
    if (threadIdx.x == 0) f(i, s);
  }
}

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT, 8) k2_pcg_persist(PcgPersistArgs a) {
  using TL = Tiling2D<NP>;
  constexpr int P2 = pow2_at_least(TL::NT);
  constexpr int UV = PCG_THREADS;        // slots of a tile's update tree
  constexpr int cnt = TL::TE * NP * NP;  // nodes of a tile
  static_assert(cnt <= UV, "one tree slot per node");
  __shared__ ApplySmem<NP> sm;
  __shared__ double s_red[UV > P2 ? UV : P2];
  const unsigned G = gridDim.x;
  const int ni = a.ninst, n = a.n_iter;
  double* RZ = a.scal;
  double* PAP = a.scal + (long long)(n + 1) * ni;
  double* AL = a.scal + (long long)(2 * n + 1) * ni;
  double* BT = a.scal + (long long)(3 * n + 1) * ni;
  double* beta = a.beta_cta + (long long)blockIdx.x * ni;
  const double eps = a.eps;

  // ---- r_0 = b - A x_0, p_0 = M^-1 r_0, partials of r_0 . p_0
  {
    ApplyArgs2D op = a.op;
    op.x = a.x0; op.r_out = a.r; op.p_out = a.p[0];
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const Tile2D tl = op.tiles[t];
      const Inst2D I = op.inst[tl.inst];
      const double tot = block_sum<P2>(apply_tile<NP, EPI_PCG0>(op, tl, I, sm), s_red);
      if (threadIdx.x == 0) op.partials[t] = tot;
    }
  }
  if (!grid_barrier(a.bar, G, [&] {
        inst_tile_sums(a.op.inst, ni, a.op.partials, [&](int i, double s) { RZ[i] = s; });
      }))
    return;

  for (int k = 0; k < n; ++k) {
    // ---- phase A: A p_k (p_k = M^-1 r_k + beta_{k-1} p_{k-1} formed on load for k > 0)
    {
      ApplyArgs2D op = a.op;
      if (k == 0) {
        op.x = a.p[0];
      } else {
        if (threadIdx.x < ni) beta[threadIdx.x] = __ldcg(BT + (long long)(k - 1) * ni + threadIdx.x);
        __syncthreads();
        op.pcg_r = a.r; op.pcg_p = a.p[(k - 1) & 1]; op.pcg_beta = beta;
        op.p_out = a.p[k & 1];
      }
      op.ap_out = a.ap;
      for (int t = blockIdx.x; t < a.ntiles; t += G) {
        const Tile2D tl = op.tiles[t];
        const Inst2D I = op.inst[tl.inst];
        const double tot = block_sum<P2>(apply_tile<NP, EPI_PCG>(op, tl, I, sm), s_red);
        if (threadIdx.x == 0) op.partials[t] = tot;
      }
    }
    if (!grid_barrier(a.bar, G, [&] {
          inst_tile_sums(a.op.inst, ni, a.op.partials, [&](int i, double s) {
            PAP[(long long)k * ni + i] = s;
            AL[(long long)k * ni + i] = __ldcg(RZ + (long long)k * ni + i) / (s + eps);  // alpha_k
          });
        }))
      return;
    // ---- phase B on the CTA's own tiles (whose p_k and A p_k it wrote in phase A):
    // x_{k+1} = x_k + alpha_k p_k, r_{k+1} = r_k - alpha_k A p_k, tile partials of r . M^-1 r
    {
      const double* xin = k == 0 ? a.x0 : a.xout;
      const double* pk = a.p[k & 1];
      for (int t = blockIdx.x; t < a.ntiles; t += G) {
        const Tile2D tl = a.op.tiles[t];
        const Inst2D I = a.op.inst[tl.inst];
        const double al = __ldcg(AL + (long long)k * ni + tl.inst);
        for (int v = threadIdx.x; v < UV; v += blockDim.x) {
          double part = 0.0;
          long long nd;
          if (v < cnt && tile_node<NP>(tl, I, v, &nd)) {
            const double p = pk[nd], apv = a.ap[nd], x = xin[nd], r = a.r[nd], im = a.op.cinvM[nd];
            a.xout[nd] = fma(al, p, x);
            const double rn = fma(-al, apv, r);
            a.r[nd] = rn;
            part = fma(rn, rn * im, 0.0);
          }
          s_red[v] = part;
        }
        __syncthreads();
        tile_tree<UV>(s_red, threadIdx.x, blockDim.x);
        if (threadIdx.x == 0) a.upart[t] = s_red[0];
        __syncthreads();
      }
    }
    if (!grid_barrier(a.bar, G, [&] {
          inst_tile_sums(a.op.inst, ni, a.upart, [&](int i, double rzn) {
            RZ[(long long)(k + 1) * ni + i] = rzn;
            BT[(long long)k * ni + i] = rzn / (__ldcg(RZ + (long long)k * ni + i) + eps);  // beta_k
          });
        }))
      return;
  }
}

}  // namespace igrgpu
