// One fixed-count Jacobi-preconditioned CG solve (pcg_fixed!, elliptic.jl:329-347)
// in a single persistent launch.
//
// The two-kernel form (k2_apply<EPI_PCG> + k2_pcg_update per iteration, each
// completing its inner product in its last block) spends much of a small
// instance's iteration on two launches and the latency of two short kernels.
// Here one grid of co-resident CTAs (a cooperative launch, one tile per CTA)
// runs the whole solve. Instances are independent, so there is no grid-wide
// barrier, only a hand-off of each inner product among the instance's CTAs:
//   phase A: p_k formed on load, A p_k; the tile's partial of p_k . A p_k
//            | pAp_k, alpha_k = rz_k / (pAp_k + eps) |
//   phase B: x_{k+1}, r_{k+1} on the CTA's tile; its partial of r . M^-1 r
//            | rz_{k+1}, beta_k = rz_{k+1} / (rz_k + eps) |
// The operator runs the same apply_tile code and block tree as k2_apply, the
// update forms each tile's partial in the same 256-slot tree as k2_pcg_update,
// and the partials are summed in warp_sum_partials' order (sum_lanes64), so
// the result is bitwise the two-kernel result.
//
// Every reduction e (0: r_0 . p_0; 2k + 1: p_k . A p_k; 2k + 2:
// r_{k+1} . M^-1 r_{k+1}) has its own partial slot per tile, so no slot is
// reused within a launch. The hand-off has two forms, by instance size:
//   counted (instances of at most PCG_COUNTED_TILES tiles): a CTA stores its
//     partial and adds 1 to its instance's arrival counter with release
//     semantics; each CTA waits (acquire loads of the one counter word) until
//     the count reaches (e + 1) x tiles, then reads all of the instance's
//     partials and forms the sum itself;
//   published (larger instances, whose partials all CTAs reading at once
//     would crowd a few L2 lines): the partial slots and the scalars' slots
//     hold PCG_SENTINEL (a signalling-NaN bit pattern, which no arithmetic
//     produces) from a fill before the launch; a CTA stores its partial with
//     release semantics; the instance's first tile (its writer CTA) polls the
//     instance's slots (relaxed loads, many in flight at once) until none
//     holds the sentinel, acquires, sums and publishes the scalar with release
//     semantics to PCG_BCAST copies on separate lines, and every other CTA
//     polls the copy of its own tile number modulo PCG_BCAST.
// Waits are bounded: a CTA that waits longer than PCG_WAIT_NS sets DEV_TIMEOUT
// in the status word and the kernel returns (the host reports IGR_ETIMEOUT).
// With a cooperative launch every CTA is resident, so the limit is a guard,
// not the path.
#pragma once
#include "igr2d_kernels.cuh"
#include "igr2d_pcg_kernels.cuh"

namespace igrgpu {

constexpr int PCG_PERSIST_MAX_INST = 32;             // instances of a plan the persistent form takes
constexpr long long PCG_WAIT_NS = 1000000000LL;      // limit of one wait (1 s)
constexpr unsigned long long PCG_SENTINEL = 0x7FF4DEAD7FF4DEADull;  // "not yet written" (signalling NaN)
constexpr int PCG_COUNTED_TILES = 256;               // instances up to this many tiles: counted hand-off
constexpr int PCG_BCAST = 32;                        // copies of a published scalar
constexpr int PCG_CNT_STRIDE = 32;                   // words between arrival counters (one 128-byte line each)

// Partial slots each writer thread polls, and so the tiles an instance may
// have (slots per thread x threads per CTA, about 1280).
template <int NP>
__host__ __device__ constexpr int persist_slots_per_thread() {
  return (1280 + Tiling2D<NP>::NT - 1) / Tiling2D<NP>::NT < 32 ? (1280 + Tiling2D<NP>::NT - 1) / Tiling2D<NP>::NT : 32;
}
template <int NP>
__host__ __device__ constexpr int persist_max_inst_tiles() { return persist_slots_per_thread<NP>() * Tiling2D<NP>::NT; }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_f64(double* p, double v) {
  asm volatile("st.release.gpu.global.b64 [%0], %1;" :: "l"(p), "l"(__double_as_longlong(v)) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

struct PcgPersistArgs {
  ApplyArgs2D op;                  // tiles, instances, basis, coefficients, b, cinvM
  int ntiles, ninst, n_iter;
  int counted;                     // counted hand-off (else published)
  const double* x0;                // warm start (read only)
  double *xout, *r, *p[2], *ap;    // solution and the CG vectors
  double* slots;                   // partials: reduction e, tile t at slots[e * ntiles + t]
  double* scal;                    // per instance: rz_0..rz_n, pAp_0..pAp_{n-1}, alpha, beta (as pcg_solve)
  double* bcast;                   // published: copy j of reduction e's scalar of instance i at
  long long bcast_stride;          //   bcast[j * bcast_stride + e * ninst + i]
  unsigned* cnt;                   // counted: arrivals of instance i at cnt[i * PCG_CNT_STRIDE]
  double eps;
  int* status;
  int drop_tile;                   // test hook: this tile's CTA leaves before its first p.Ap hand-off (-1: none)
  // at the launch: counted, cnt zero; published, slots and bcast PCG_SENTINEL
};

// Counted hand-off, every thread; thread 0 has stored the CTA's partial.
// Counts the CTA's arrival, waits for the instance's target count, stages the
// partials and returns their sum. *s_ok = 0 on timeout.
__device__ __forceinline__ double counted_sum(unsigned* cnt, unsigned target, const double* part, int count,
                                              double* stage, int* status, double* s_sum, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    red_release_add_u32(cnt, 1u);
    int ok = 1;
    const unsigned long long t0 = global_ns();
    while ((int)(ld_acquire_u32(cnt) - target) < 0) {
      if (global_ns() - t0 > (unsigned long long)PCG_WAIT_NS) {
        atomicOr(status, DEV_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(20);
    }
    *s_ok = ok;
  }
  __syncthreads();
#pragma unroll 4
  for (int j = threadIdx.x; j < count; j += blockDim.x) stage[j] = __ldcg(part + j);
  return sum_lanes64(stage, count, s_sum);
}

// Published hand-off, writer CTA, every thread: waits until none of the
// instance's partial slots (slots[0 .. count)) holds the sentinel, stages
// them, acquires and returns their sum. Thread j polls slots j, j + NT, ...
// with up to 16 of its pending loads in flight at once. *s_ok = 0 on timeout.
template <int NP>
__device__ __forceinline__ double gathered_sum(const double* slots, int count, double* stage, int* status,
                                               double* s_sum, int* s_ok) {
  constexpr int SPT = persist_slots_per_thread<NP>();
  constexpr int NT = Tiling2D<NP>::NT;
  constexpr int CH = 16;  // loads in flight per thread (registers)
  const int tid = threadIdx.x;
  __syncthreads();
  if (tid == 0) *s_ok = 1;
  __syncthreads();
  unsigned pend = 0;
#pragma unroll
  for (int m = 0; m < SPT; ++m)
    if (tid + m * NT < count) pend |= 1u << m;
  const unsigned long long t0 = global_ns();
  while (pend) {
#pragma unroll
    for (int c0 = 0; c0 < SPT; c0 += CH) {
      unsigned long long v[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int m = c0 + j;
        v[j] = m < SPT && ((pend >> m) & 1u) ? ld_relaxed_u64(slots + tid + m * NT) : PCG_SENTINEL;
      }
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int m = c0 + j;
        if (m < SPT && ((pend >> m) & 1u) && v[j] != PCG_SENTINEL) {
          stage[tid + m * NT] = __longlong_as_double((long long)v[j]);
          pend &= ~(1u << m);
        }
      }
    }
    if (!pend) break;
    if (global_ns() - t0 > (unsigned long long)PCG_WAIT_NS) {
      atomicOr(status, DEV_TIMEOUT);
      *s_ok = 0;
      break;
    }
    __nanosleep(20);
  }
  fence_acq_rel_gpu();
  return sum_lanes64(stage, count, s_sum);
}

// Published hand-off, every thread of a CTA other than the writer: waits
// until *slot no longer holds the sentinel and returns it (acquired).
// *s_ok = 0 on timeout.
__device__ __forceinline__ double wait_published(const double* slot, int* status, double* s_val, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned long long v;
    const unsigned long long t0 = global_ns();
    while ((v = ld_relaxed_u64(slot)) == PCG_SENTINEL) {
      if (global_ns() - t0 > (unsigned long long)PCG_WAIT_NS) {
        atomicOr(status, DEV_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(20);
    }
    fence_acq_rel_gpu();
    *s_val = __longlong_as_double((long long)v);
    *s_ok = ok;
  }
  __syncthreads();
  return *s_val;
}

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT, 8) k2_pcg_persist(PcgPersistArgs a) {
  using TL = Tiling2D<NP>;
  constexpr int P2 = pow2_at_least(TL::NT);
  constexpr int UV = PCG_THREADS;        // slots of a tile's update tree
  constexpr int cnt = TL::TE * NP * NP;  // nodes of a tile
  static_assert(cnt <= UV, "one tree slot per node");
  static_assert(TL::NT >= PCG_BCAST, "one thread per published copy");
  __shared__ ApplySmem<NP> sm;
  __shared__ double s_red[UV > P2 ? UV : P2];
  __shared__ double s_val, s_beta[PCG_PERSIST_MAX_INST], s_stage[persist_max_inst_tiles<NP>()];
  __shared__ int s_ok;
  const int t = blockIdx.x;  // the CTA's tile (the grid is the plan's tiles)
  const int ni = a.ninst, n = a.n_iter;
  const Tile2D tl = a.op.tiles[t];
  const Inst2D I = a.op.inst[tl.inst];
  const bool writer = t == I.tile0;  // the instance's first tile records (and publishes) its scalars
  const long long is = tl.inst;
  double* RZ = a.scal;
  double* PAP = a.scal + (long long)(n + 1) * ni;
  double* AL = a.scal + (long long)(2 * n + 1) * ni;
  double* BT = a.scal + (long long)(3 * n + 1) * ni;
  const double eps = a.eps;

  // Reduction e of the instance, after the CTA's partial tot (known to thread
  // 0) is formed: stores it and sets *scalar = scal_of(sum) in every thread;
  // CTAs that form the sum also get it in *sum. False on timeout.
  auto reduce = [&](int e, double tot, auto&& scal_of, double* sum, double* scalar) -> bool {
    if (e == 1 && t == a.drop_tile) return false;  // a CTA that stops early: the others' waits run out
    double* part = a.slots + (long long)e * a.ntiles;
    if (a.counted) {
      if (threadIdx.x == 0) part[t] = tot;
      *sum = counted_sum(a.cnt + is * PCG_CNT_STRIDE, (unsigned)(e + 1) * (unsigned)I.ntiles, part + I.tile0, I.ntiles,
                         s_stage, a.status, &s_val, &s_ok);
      if (!s_ok) return false;
      *scalar = scal_of(*sum);
      return true;
    }
    if (threadIdx.x == 0) st_release_f64(part + t, tot);
    double* pub = a.bcast + (long long)e * ni + is;
    if (writer) {
      *sum = gathered_sum<NP>(part + I.tile0, I.ntiles, s_stage, a.status, &s_val, &s_ok);
      if (!s_ok) return false;
      *scalar = scal_of(*sum);
      if (threadIdx.x < PCG_BCAST) st_release_f64(pub + threadIdx.x * a.bcast_stride, *scalar);
      return true;
    }
    *scalar = wait_published(pub + (t % PCG_BCAST) * a.bcast_stride, a.status, &s_val, &s_ok);
    return s_ok != 0;
  };

  // ---- r_0 = b - A x_0, p_0 = M^-1 r_0, partial of r_0 . p_0
  double rz = 0.0, sum = 0.0, scalar = 0.0;  // rz_k: CTAs that form the sums
  {
    ApplyArgs2D op = a.op;
    op.x = a.x0; op.r_out = a.r; op.p_out = a.p[0];
    const double tot = block_sum<P2>(apply_tile<NP, EPI_PCG0>(op, tl, I, sm), s_red);
    if (!reduce(0, tot, [](double s) { return s; }, &sum, &scalar)) return;
    rz = sum;
    if (writer && threadIdx.x == 0) RZ[is] = rz;
  }

  for (int k = 0; k < n; ++k) {
    // ---- phase A: A p_k (p_k = M^-1 r_k + beta_{k-1} p_{k-1} formed on load for k > 0)
    {
      ApplyArgs2D op = a.op;
      if (k == 0) {
        op.x = a.p[0];
      } else {
        op.pcg_r = a.r; op.pcg_p = a.p[(k - 1) & 1]; op.pcg_beta = s_beta;
        op.p_out = a.p[k & 1];
      }
      op.ap_out = a.ap;
      const double tot = block_sum<P2>(apply_tile<NP, EPI_PCG>(op, tl, I, sm), s_red);
      if (!reduce(2 * k + 1, tot, [&](double pap) { return rz / (pap + eps); }, &sum, &scalar)) return;
    }
    const double al = scalar;  // alpha_k
    if (writer && threadIdx.x == 0) {
      PAP[(long long)k * ni + is] = sum;
      AL[(long long)k * ni + is] = al;
    }
    // ---- phase B on the CTA's tile (whose p_k and A p_k it wrote in phase A):
    // x_{k+1} = x_k + alpha_k p_k, r_{k+1} = r_k - alpha_k A p_k, tile partial of r . M^-1 r
    {
      const double* xin = k == 0 ? a.x0 : a.xout;
      const double* pk = a.p[k & 1];
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
      if (!reduce(2 * k + 2, s_red[0], [&](double rzn) { return rzn / (rz + eps); }, &sum, &scalar)) return;
    }
    const double bt = scalar;  // beta_k
    rz = sum;
    if (writer && threadIdx.x == 0) {
      RZ[(long long)(k + 1) * ni + is] = sum;
      BT[(long long)k * ni + is] = bt;
    }
    if (threadIdx.x == 0) s_beta[is] = bt;
    __syncthreads();  // s_beta before the next operator's loads
  }
}

// Fills [p, p + n) with PCG_SENTINEL.
static __global__ void k2_pcg_persist_fill(double* p, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = __longlong_as_double((long long)PCG_SENTINEL);
}

}  // namespace igrgpu
