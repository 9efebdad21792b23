// 1D IGR-Euler kernels (IGR_adjoints_1d): one CTA per instance, persistent
// over the whole trajectory.
//
// A 1D instance is small (N_e <= a few thousand elements, 4 nodes each at
// P3), so instead of one launch per operator application (whose launch
// latency would dominate) each CTA advances its own instance through every
// RK stage, solver iteration and step, with barriers between phases
// and deterministic block reductions for the solver inner products. A batch
// of instances with different N_e, gamma, alpha, dt and step counts is one
// launch; instances are independent, so no grid-wide synchronisation exists.
//
// Thread mapping: one thread per element (strided over the CTA), the
// element's NP nodes in registers; face partners are read from the
// neighbouring elements' nodes (L1/L2 resident: an instance's fields are a
// few tens of KB). Node order is the reference's Julia (n_p, N_e) layout.
#pragma once
#include <cooperative_groups.h>

#include "igr2d_kernels.cuh"  // line contractions dot_row / dot_end / dot_col

namespace igrgpu {

constexpr int T1 = 256;  // threads per 1D CTA (power of two: block_sum scratch size)
constexpr int E1_FIELDS = 2;  // per-element work at the start of an instance's scratch

// Per-CTA view of one instance. An instance is advanced by `cs` CTAs (a
// thread-block cluster when cs > 1, so that one small instance can use up to
// 16 SMs); CTA rank r owns elements [e0, e1). Phases end with sync() (a CTA
// or cluster barrier, release/acquire). Inner products are reduced from
// per-element partials in one fixed order that does not depend on cs, so a
// result is bitwise the same whatever the cluster size.
template <int NP>
struct View1 {
  Inst1D I;
  int N;          // nodes
  double* scr;    // this instance's scratch (fields of N doubles)
  double* ew;     // per-element work: 2 ne reduction slots, ne d/dgamma, ne d/dalpha accumulators
  int e0, e1, cs;
  mutable int flip;
  __device__ double* f(int k) const { return scr + (long long)k * N; }
  __device__ int m0() const { return e0 * NP; }
  __device__ int m1() const { return e1 * NP; }
  __device__ double* slot() const { return ew + (flip & 1) * I.ne; }
  __device__ double* gbe() const { return ew + 2 * I.ne; }
  __device__ double* abe() const { return ew + 3 * I.ne; }
  __device__ void sync() const {
    if (cs > 1) cooperative_groups::this_cluster().sync();
    else __syncthreads();
  }
  // Sum of per-element values pe[0..ne) written before the call (by any CTA
  // of the instance); every CTA returns the same value.
  __device__ double esum(const double* pe, double* s_red) const {
    sync();
    double acc = 0.0;
    for (int e = threadIdx.x; e < I.ne; e += T1) acc += pe[e];
    return block_sum<T1>(acc, s_red);
  }
  // esum of the current slot, then switch slots (ping-pong: between two uses
  // of one slot there is always another reduction's barrier).
  __device__ double reduce(double* s_red) const {
    const double t = esum(slot(), s_red);
    flip ^= 1;
    return t;
  }
};

// Set up the view of CTA blockIdx.x: instance order[blockIdx.x / cs].
template <int NP>
__device__ __forceinline__ View1<NP> make_view1(const Inst1D* inst, const int* order, double* scr_base, int cs, int* idx) {
  View1<NP> v;
  const int rank = blockIdx.x % cs;
  *idx = order[blockIdx.x / cs];
  v.I = inst[*idx];
  v.N = NP * v.I.ne;
  v.ew = scr_base + v.I.soff;
  v.scr = v.ew + (long long)E1_FIELDS * v.N;
  v.cs = cs;
  v.e0 = (int)((long long)v.I.ne * rank / cs);
  v.e1 = (int)((long long)v.I.ne * (rank + 1) / cs);
  v.flip = 0;
  return v;
}

__device__ __forceinline__ int wrap_left(int e, int ne) { return e == 0 ? ne - 1 : e - 1; }
__device__ __forceinline__ int wrap_right(int e, int ne) { return e == ne - 1 ? 0 : e + 1; }

// ---------------------------------------------------------------------------
// Physics at one node (IGR_adjoints_1d/euler.jl:46-111)
//   P = (gamma-1)(E - mu^2/(2 rho)),  P_bar = P + Sigma
//   f = (mu^2/rho + P_bar, mu, (E + P_bar) mu/rho),  |u| + sqrt(gamma P / rho)
// ---------------------------------------------------------------------------
struct Node1 { double f[3], P, u; };
__device__ __forceinline__ Node1 node1(double g, double mu, double E, double S, double ir) {
  Node1 o;
  o.u = mu * ir;
  o.P = (g - 1.0) * (E - 0.5 * mu * o.u);
  const double pb = o.P + S;
  o.f[0] = fma(mu, o.u, pb); o.f[1] = mu; o.f[2] = (E + pb) * o.u;
  return o;
}
__device__ __forceinline__ double ws1(double g, const Node1& o, double ir) { return fabs(o.u) + sqrt(g * o.P * ir); }

// ---------------------------------------------------------------------------
// Stage setup (IGR_adjoints_1d/elliptic.jl:126-154, 206-253): IGR source
// b = w_i J 2 alpha (d_x u)^2, diag(A), and the operator coefficients
//   cm = w_i J / rho, ck = alpha w_i / (J rho), cpR[e] = alpha eta max(1/rho_L, 1/rho_R) / dx
// (cpR: the penalty of element e's right face). All threads call it.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_setup(const View1<NP>& v, const BasisDev& B, const double* mu, const double* ir, double* b, double* cm,
                         double* ck, double* cpR, double* cinvM, double* cM) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double eta = (double)(NP * NP);
  const double al = I.alpha;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double r[NP], u[NP], kk[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { r[i] = ir[base + i]; u[i] = mu[base + i] * r[i]; }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const double du = I.iJ * dot_row<NP>(B, i, u);
      b[base + i] = (B.w[i] * I.J) * (2.0 * al * (du * du));
      cm[base + i] = (B.w[i] * I.J) * r[i];
      kk[i] = (al * B.w[i] * I.iJ) * r[i];
      ck[base + i] = kk[i];
    }
    const double irLL = ir[eL * NP + L], irR0 = ir[eR * NP];
    const double cpr = al * eta * I.idx * max_nonneg(irR0, r[L]);
    const double cpl = al * eta * I.idx * max_nonneg(r[0], irLL);
    cpR[e] = cpr;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      double M = cm[base + k];
#pragma unroll
      for (int i = 0; i < NP; ++i) M = fma(kk[i], B.D[i][k] * B.D[i][k], M);
      if (k == L) M = fma(-kk[L] * B.iwL, B.D[L][L], M) + cpr;
      if (k == 0) M = fma(kk[0] * B.iw0, B.D[0][0], M) + cpl;
      cinvM[base + k] = 1.0 / M;
      if (cM) cM[base + k] = M;
    }
  }
  v.sync();
}

// ---------------------------------------------------------------------------
// SIP operator y = A x (IGR_adjoints_1d/elliptic.jl:32-116) per element, with
// the face terms folded as in the 2D kernels:
//   F = hw (ck_L d_L + ck_R d_R) + cp (x_L - x_R),  hw = -1/(2 w_0)
//   y_L-side += F, y_R-side -= F, symmetry term into the stiffness transpose.
// ldx(n) supplies x at node n; epi(e, x[], y[]) consumes the element's result.
// Does not synchronise (the epilogue decides what it writes). d1_apply picks
// one thread per element (d1_apply_elems) or one lane per node
// (d1_apply_nodes); both give the same bits.
// ---------------------------------------------------------------------------
template <int NP, class LDX, class EPI>
__device__ __forceinline__ void d1_apply_elems(const View1<NP>& v, const BasisDev& B, LDX ldx, const double* cm,
                                               const double* ck, const double* cpR, EPI epi) {
  constexpr int L = NP - 1;
  const int ne = v.I.ne;
  const double hw = B.hw;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, ne), eR = wrap_right(e, ne);
    const int base = e * NP;
    double x[NP], g[NP], xl[NP], xr[NP], kc[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { x[i] = ldx(base + i); kc[i] = ck[base + i]; }
#pragma unroll
    for (int i = 0; i < NP; ++i) { xl[i] = ldx(eL * NP + i); xr[i] = ldx(eR * NP + i); }
#pragma unroll
    for (int i = 0; i < NP; ++i) g[i] = dot_row<NP>(B, i, x);
    const double gl = dot_end<NP>(B, true, xl), gr = dot_end<NP>(B, false, xr);
    const double ckl = ck[eL * NP + L], ckr = ck[eR * NP];
    const double jl = xl[L] - x[0];
    const double Fl = fma(cpR[eL], jl, hw * fma(ckl, gl, kc[0] * g[0]));
    const double jr = x[L] - xr[0];
    const double Fr = fma(cpR[e], jr, hw * fma(kc[L], g[L], ckr * gr));
    double sx[NP];
#pragma unroll
    for (int i = 1; i < L; ++i) sx[i] = kc[i] * g[i];
    sx[0] = kc[0] * fma(hw, jl, g[0]);
    sx[L] = kc[L] * fma(hw, jr, g[L]);
    double y[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k)
      y[k] = dot_col<NP>(B, k, sx, fma(cm[base + k], x[k], (k == 0) ? -Fl : ((k == L) ? Fr : 0.0)));
    epi(e, x, y);
  }
}

// Lanes per element in d1_apply_nodes: NP rounded up to a power of two.
template <int NP>
__host__ __device__ constexpr int group1() { return NP <= 2 ? 2 : (NP <= 4 ? 4 : 8); }

// d1_apply with one lane per node, for CTAs holding at most T1 / (2 group1)
// elements (a small instance spread over a cluster). GB300's FP64 unit
// issues one warp instruction per ~64 cycles per SM sub-partition whatever
// the number of active lanes (measured with a DFMA micro-probe: 64.1 cycles
// per warp instruction for 1 to 32 active lanes), so one thread per element
// left 3/4 of the lanes of every FP64 instruction idle there. A group of
// group1<NP>() lanes takes one element and lane i its node i: every lane
// forms the derivative at its node, the lanes of nodes 0 and L the left and
// right face terms (interior lanes run the same instructions on the right
// face and discard them), each lane its stiffness-transpose input; the group
// exchanges those by shuffles, lane i forms y_i, and the group's first lane
// runs the element epilogue. Every output is the expression of
// d1_apply_elems evaluated in the same order, so the results are bitwise
// equal; operands are chosen by register selects so that the warp runs one
// instruction stream.
// NODE_EPI: epi(m, x_m, y_m) is a per-node epilogue that every node lane runs
// for its own node; otherwise the group's first lane runs the element
// epilogue epi(e, x[], y[]). The coefficients are read through accessors
// cmf(m), ckf(m) (node m) and cpf(e) (element e).
template <int NP, bool NODE_EPI, class LDX, class CMF, class CKF, class CPF, class EPI>
__device__ __forceinline__ void d1_apply_nodes(const View1<NP>& v, const BasisDev& B, LDX ldx, CMF cmf, CKF ckf,
                                               CPF cpf_, EPI epi) {
  constexpr int L = NP - 1, G = group1<NP>();
  const int ne = v.I.ne;
  const double hw = B.hw;
  const int li = threadIdx.x % G;
  const int ii = li < NP ? li : L;  // lanes past the element's nodes shadow node L (results unused)
  const bool interior = ii > 0 && ii < L;
  const bool left = ii == 0;        // the face this lane evaluates: left of node 0, else right of node L
  const bool face = !interior;
  double Dr[NP], Dc[NP];            // D[ii][k] and D[k][ii]
#pragma unroll
  for (int k = 0; k < NP; ++k) { Dr[k] = B.D[0][k]; Dc[k] = B.D[k][0]; }
#pragma unroll
  for (int r = 1; r < NP; ++r)
    if (ii == r) {
#pragma unroll
      for (int k = 0; k < NP; ++k) { Dr[k] = B.D[r][k]; Dc[k] = B.D[k][r]; }
    }
  for (int eb = v.e0; eb < v.e1; eb += T1 / G) {
    if (eb + (int)(threadIdx.x & ~31u) / G >= v.e1) continue;  // a warp without elements (warp-uniform)
    const int e = eb + threadIdx.x / G;
    const bool live = e < v.e1;
    const int ec = live ? e : v.e0;  // groups past the range shadow a live element; they store nothing
    const int base = ec * NP;
    double x[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) x[k] = ldx(base + k);
    double xo = x[0];
#pragma unroll
    for (int r = 1; r < NP; ++r) xo = (ii == r) ? x[r] : xo;
    // derivative at the lane's node: dot_row<NP>(B, ii, x)
    double g = Dr[0] * x[0];
#pragma unroll
    for (int k = 1; k < NP; ++k) {
      const double t = fma(Dr[k], x[k], g);
      g = (interior && k == ii) ? g : t;
    }
    // the lane's face (d1_apply_elems: Fl for node 0, Fr for node L)
    const int eL = wrap_left(ec, ne), eR = wrap_right(ec, ne);
    const int pe = left ? eL : eR;
    double xp[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) xp[k] = ldx(pe * NP + k);
    const double gp = dot_end<NP>(B, left, xp);
    const double kco = ckf(base + ii);
    const double ckp = ckf(left ? eL * NP + L : eR * NP);
    const double cpf = cpf_(left ? eL : ec);
    const double jmp = (left ? xp[L] : x[L]) - (left ? x[0] : xp[0]);
    const double inner = fma(left ? ckp : kco, left ? gp : g, (left ? kco : ckp) * (left ? g : gp));
    const double F = fma(cpf, jmp, hw * inner);
    const double sxi = kco * (face ? fma(hw, jmp, g) : g);
    double sx[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) sx[k] = __shfl_sync(0xffffffffu, sxi, k, G);
    // y at the lane's node: dot_col<NP>(B, ii, sx, fma(cm, x_ii, -Fl | Fr | 0))
    double y = fma(cmf(base + ii), xo, left ? -F : (ii == L ? F : 0.0));
#pragma unroll
    for (int r = 0; r < NP; ++r) {
      const double t = fma(Dc[r], sx[r], y);
      y = (interior && r == ii) ? y : t;
    }
    if constexpr (NODE_EPI) {
      if (live && li < NP) epi(base + li, xo, y);
    } else {
      double yv[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) yv[k] = __shfl_sync(0xffffffffu, y, k, G);
      if (live && li == 0) epi(e, x, yv);
    }
  }
}

template <int NP, class LDX, class EPI>
__device__ __forceinline__ void d1_apply(const View1<NP>& v, const BasisDev& B, LDX ldx, const double* cm, const double* ck,
                                         const double* cpR, EPI epi) {
  // node form for CTAs filling at most half their threads with nodes: there the
  // element form leaves lanes idle; a CTA of a batch with more elements is
  // already bound by FP64 throughput, where both forms issue the same number
  // of warp instructions and the element form needs no shuffles
  if ((v.e1 - v.e0) * group1<NP>() <= T1 / 2)
    d1_apply_nodes<NP, false>(v, B, ldx, [&](int m) { return cm[m]; }, [&](int m) { return ck[m]; },
                              [&](int e) { return cpR[e]; }, epi);
  else d1_apply_elems<NP>(v, B, ldx, cm, ck, cpR, epi);
}

// d1_apply with a per-node epilogue nepi(m, x_m, y_m) (no per-element
// coupling): in the node form each node lane runs it for its node.
template <int NP, class LDX, class NEPI>
__device__ __forceinline__ void d1_apply_pointwise(const View1<NP>& v, const BasisDev& B, LDX ldx, const double* cm,
                                                   const double* ck, const double* cpR, NEPI nepi) {
  if ((v.e1 - v.e0) * group1<NP>() <= T1 / 2) {
    d1_apply_nodes<NP, true>(v, B, ldx, [&](int m) { return cm[m]; }, [&](int m) { return ck[m]; },
                             [&](int e) { return cpR[e]; }, nepi);
  } else {
    d1_apply_elems<NP>(v, B, ldx, cm, ck, cpR, [&](int e, const double* xx, const double* y) {
#pragma unroll
      for (int i = 0; i < NP; ++i) nepi(e * NP + i, xx[i], y[i]);
    });
  }
}

// ---------------------------------------------------------------------------
// Solver tape of one stage (adjoint only). Jacobi / Chebyshev: x_k, r_k for
// k < n. PCG: x_0, r_0..r_n, p_k, A p_k (k < n) and the scalars rz_0..rz_n,
// pAp_0..pAp_{n-1}.
// ---------------------------------------------------------------------------
struct SolveTape1 {
  double* base = nullptr;  // null: untaped
  int N = 0, n = 0, pcg = 0;
  __device__ double* x(int k) const { return base + (long long)k * N; }                  // Jac/Cheb x_k, PCG x_0
  __device__ double* r(int k) const { return base + (long long)((pcg ? 1 : n) + k) * N; }
  __device__ double* p(int k) const { return base + (long long)(n + 2 + k) * N; }
  __device__ double* ap(int k) const { return base + (long long)(2 * n + 2 + k) * N; }
  __device__ double* scal() const { return base + (long long)(3 * n + 2) * N; }          // rz[0..n], pAp[0..n-1]
};
__host__ __device__ inline int solve_tape_fields1(int solver, int n, int N) {
  if (solver == 0) return 3 * n + 2 + (2 * n + 1 + N - 1) / N;
  return 2 * n;
}

// Chebyshev recurrence coefficients for iteration it = 1..n (elliptic.jl:383-391)
__device__ __forceinline__ void cheb_coef(const BasisDev& B, int it, double& rc, double* ca, double* cc) {
  if (it == 1) { *ca = 0.0; *cc = 1.0 / B.cheb_theta; rc = 1.0 / B.cheb_sigma; return; }
  const double rn = 1.0 / (2.0 * B.cheb_sigma - rc);
  *ca = rn * rc; *cc = 2.0 * rn / B.cheb_delta;
  rc = rn;
}

// The solvers' scalar recurrences are evaluated by one thread of the CTA and
// read by all from shared memory: an FP64 divide is a software sequence of
// ~20 FP64 instructions on GB300, and 256 threads repeating it every iteration
// cost as much FP64 issue as the element work of a small instance. All
// threads of the CTA call these; every CTA of a cluster computes the same bits.
__device__ __forceinline__ double cta_div(double x, double y) {
  __shared__ double s_q;
  if (threadIdx.x == 0) s_q = x / y;
  __syncthreads();
  const double r = s_q;
  __syncthreads();
  return r;
}
// cheb_coef on thread 0 (rc is carried by thread 0 only), coefficients to all.
__device__ __forceinline__ void cta_cheb(const BasisDev& B, int it, double& rc, double* ca, double* cc) {
  __shared__ double s_c[2];
  if (threadIdx.x == 0) {
    cheb_coef(B, it, rc, ca, cc);
    s_c[0] = *ca; s_c[1] = *cc;
  }
  __syncthreads();
  *ca = s_c[0]; *cc = s_c[1];
  __syncthreads();
}

// Jacobi / Chebyshev for an instance whose CTAs hold at most T1 / (2 group1)
// elements each (a small instance, usually spread over a cluster), in node
// form with the iterate, its coefficients, b and 1/M in shared memory. The
// two halo elements are read from the neighbouring CTAs' shared memory (the
// cluster's distributed shared memory), so after each cluster barrier an
// iteration waits for a DSMEM load instead of an L2 round trip, and touches
// global memory only for the tape and the result. The arithmetic is
// d1_solve's, so the results are bitwise equal. The choice depends only on
// the instance (N_e, CTAs per instance), so all CTAs of a cluster agree.
template <int NP>
__device__ __forceinline__ bool d1_local_ok(const View1<NP>& v) {
  const int per = (v.I.ne + v.cs - 1) / v.cs;
  return v.I.ne >= v.cs && per * group1<NP>() <= T1 / 2;
}

template <int NP>
__device__ void d1_solve_local(const View1<NP>& v, const BasisDev& B, int solver, int n, const double* b, const double* x0,
                               double* xout, const double* cm, const double* ck, const double* cpR, const double* cinvM,
                               const SolveTape1& tp) {
  constexpr int L = NP - 1, MAXE = T1 / 2 / group1<NP>(), MAXN = MAXE * NP;
  __shared__ double s_x[2][MAXN], s_d[MAXN], s_cm[MAXN], s_ck[MAXN], s_b[MAXN], s_im[MAXN], s_cp[MAXE], s_h[3];
  const int ne = v.I.ne, cs = v.cs, m0 = v.m0(), nl = (v.e1 - v.e0) * NP;
  const bool taped = tp.base != nullptr;
  for (int j = threadIdx.x; j < nl; j += blockDim.x) {
    const int m = m0 + j;
    s_x[0][j] = x0[m]; s_cm[j] = cm[m]; s_ck[j] = ck[m]; s_b[j] = b[m]; s_im[j] = cinvM[m];
  }
  for (int j = threadIdx.x; j < v.e1 - v.e0; j += blockDim.x) s_cp[j] = cpR[v.e0 + j];
  const int eLh = wrap_left(v.e0, ne), eRh = v.e1 == ne ? 0 : v.e1;  // the halo elements
  if (threadIdx.x == 0) { s_h[0] = ck[eLh * NP + L]; s_h[1] = ck[eRh * NP]; s_h[2] = cpR[eLh]; }
  // neighbouring ranks (eLh is the last element of rank rank_l, eRh the first of rank rank_r)
  const int rank = blockIdx.x % cs, rank_l = (rank + cs - 1) % cs, rank_r = (rank + 1) % cs;
  const int nl_left = (int)((long long)ne * (rank_l + 1) / cs - (long long)ne * rank_l / cs) * NP;
  v.sync();
  auto cmf = [&](int m) { return s_cm[m - m0]; };
  auto ckf = [&](int m) {
    const int j = m - m0;
    return (j >= 0 && j < nl) ? s_ck[j] : (m == eLh * NP + L ? s_h[0] : s_h[1]);
  };
  auto cpf = [&](int e) { return (e >= v.e0 && e < v.e1) ? s_cp[e - v.e0] : s_h[2]; };
  double rc = 0.0;
  for (int k = 0; k < n; ++k) {
    double ca = 0.0, cc = 0.0;
    if (solver == 2) cta_cheb(B, k + 1, rc, &ca, &cc);
    double* xs = s_x[k & 1];
    double* xd = s_x[(k + 1) & 1];
    const double* xl = xs;
    const double* xr = xs;
    if (cs > 1) {
      cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
      xl = cl.map_shared_rank(xs, rank_l);
      xr = cl.map_shared_rank(xs, rank_r);
    }
    auto ldx = [&](int m) -> double {
      const int j = m - m0;
      if (j >= 0 && j < nl) return xs[j];
      return (m / NP == eLh) ? xl[nl_left - NP + m % NP] : xr[m % NP];
    };
    d1_apply_nodes<NP, true>(v, B, ldx, cmf, ckf, cpf, [&](int m, double xm, double ym) {
      const int j = m - m0;
      const double rr = s_b[j] - ym;
      if (taped) { tp.x(k)[m] = xm; tp.r(k)[m] = rr; }
      double xn;
      if (solver == 2) {
        const double z = rr * s_im[j];
        const double dn = k == 0 ? cc * z : fma(ca, s_d[j], cc * z);
        s_d[j] = dn;
        xn = xm + dn;
      } else {
        xn = fma((2.0 / 3.0) * rr, s_im[j], xm);
      }
      xd[j] = xn;
      if (k == n - 1) xout[m] = xn;
    });
    v.sync();
  }
}

// Fixed-count solve A x = b on the instance (pcg_fixed! / jacobi_fixed! /
// chebyshev_fixed!, elliptic.jl:307-430): x0 warm start, result in xout
// (!= x0); w0..w3: scratch fields. All threads call it; ends synchronised.
template <int NP>
__device__ void d1_solve(const View1<NP>& v, const BasisDev& B, int solver, int n, const double* b, const double* x0,
                         double* xout, const double* cm, const double* ck, const double* cpR, const double* cinvM,
                         double* w0, double* w1, double* w2, double* w3, const SolveTape1& tp, double* s_red) {
  const int N = v.N;
  const bool taped = tp.base != nullptr;
  if (solver == 0) {
    // ---- PCG: w0 = r, w1 = p, w2 = A p
    double* r = w0; double* p = w1; double* ap = w2;
    double* red = v.slot();
    d1_apply<NP>(v, B, [&](int m) { return x0[m]; }, cm, ck, cpR, [&](int e, const double* xx, const double* y) {
      double pe = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = e * NP + i;
        const double rr = b[m] - y[i], z = rr * cinvM[m];
        r[m] = rr; p[m] = z;
        pe = fma(rr, z, pe);
        if (taped) { tp.x(0)[m] = xx[i]; tp.r(0)[m] = rr; }
      }
      red[e] = pe;
    });
    double rz = v.reduce(s_red);
    if (taped && threadIdx.x == 0) tp.scal()[0] = rz;  // every CTA of the instance writes the same value
    for (int k = 0; k < n; ++k) {
      red = v.slot();
      d1_apply<NP>(v, B, [&](int m) { return p[m]; }, cm, ck, cpR, [&](int e, const double* xx, const double* y) {
        double pe = 0.0;
#pragma unroll
        for (int i = 0; i < NP; ++i) {
          const int m = e * NP + i;
          ap[m] = y[i];
          pe = fma(xx[i], y[i], pe);
          if (taped) { tp.p(k)[m] = xx[i]; tp.ap(k)[m] = y[i]; }
        }
        red[e] = pe;
      });
      const double pAp = v.reduce(s_red);
      if (taped && threadIdx.x == 0) tp.scal()[n + 1 + k] = pAp;
      const double a = cta_div(rz, pAp + 1e-30);
      const double* xin = k == 0 ? x0 : xout;
      red = v.slot();
      for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
        double pe = 0.0;
#pragma unroll
        for (int i = 0; i < NP; ++i) {
          const int m = e * NP + i;
          xout[m] = fma(a, p[m], xin[m]);
          const double rr = fma(-a, ap[m], r[m]);
          r[m] = rr;
          pe = fma(rr, rr * cinvM[m], pe);
          if (taped) tp.r(k + 1)[m] = rr;
        }
        red[e] = pe;
      }
      const double rzn = v.reduce(s_red);
      if (taped && threadIdx.x == 0) tp.scal()[k + 1] = rzn;
      const double beta = cta_div(rzn, rz + 1e-30);
      for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) p[m] = fma(beta, p[m], r[m] * cinvM[m]);
      rz = rzn;
      v.sync();
    }
    return;
  }
  // ---- Jacobi / Chebyshev: one apply per iteration, x ping-pong in w0/w1, d in w2
  if (d1_local_ok(v)) {
    d1_solve_local<NP>(v, B, solver, n, b, x0, xout, cm, ck, cpR, cinvM, tp);
    return;
  }
  double rc = 0.0;
  const double* x = x0;
  for (int k = 0; k < n; ++k) {
    double* xo = (k == n - 1) ? xout : ((k % 2 == 0) ? w0 : w1);
    double ca = 0.0, cc = 0.0;
    if (solver == 2) cta_cheb(B, k + 1, rc, &ca, &cc);
    double* d = w2;
    d1_apply_pointwise<NP>(v, B, [&](int m) { return x[m]; }, cm, ck, cpR, [&](int m, double xm, double ym) {
      const double rr = b[m] - ym;
      if (taped) { tp.x(k)[m] = xm; tp.r(k)[m] = rr; }
      if (solver == 2) {
        const double z = rr * cinvM[m];
        const double dn = k == 0 ? cc * z : fma(ca, d[m], cc * z);
        d[m] = dn;
        xo[m] = xm + dn;
      } else {
        xo[m] = fma((2.0 / 3.0) * rr, cinvM[m], xm);
      }
    });
    v.sync();
    x = xo;
  }
}

// ---------------------------------------------------------------------------
// Hyperbolic DG RHS (IGR_adjoints_1d/hyperbolic.jl:134-194) fused with the
// SSP-RK3 stage combination q_out = c0 q^n + c1 q_s + c2 dt k(q_s, Sigma),
// plus 1/rho of q_out. Optional raw RHS output (kout). All threads call it.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_hyp_rk(const View1<NP>& v, const BasisDev& B, const double* const q[3], const double* ir,
                          const double* S, const double* const qn[3], double c0, double c1, double c2, double dt,
                          double* const qo[3], double* iro, double* const kout[3], int* status) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double g = I.gamma, iJ = I.iJ, c2dt = c2 * dt;
  bool bad = false;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double qq[3][NP], f[3][NP], k[3][NP];
    Node1 n0, nL;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      qq[0][i] = q[0][m]; qq[1][i] = q[1][m]; qq[2][i] = q[2][m];
      const Node1 o = node1(g, qq[0][i], qq[2][i], S[m], ir[m]);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c][i] = o.f[c];
      if (i == 0) n0 = o;
      if (i == L) nL = o;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) k[c][i] = -iJ * dot_row<NP>(B, i, f[c]);
    // right face (own node L | node 0 of eR)
    {
      const int m = eR * NP;
      const double pq[3] = {q[0][m], q[1][m], q[2][m]};
      const double pir = ir[m];
      const Node1 o = node1(g, pq[0], pq[2], S[m], pir);
      const double wl = ws1(g, nL, ir[base + L]), wr = ws1(g, o, pir);
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(lam, qq[c][L] - pq[c], f[c][L] + o.f[c]);
        k[c][L] = fma(-iJ * B.iwL, fs - f[c][L], k[c][L]);
      }
    }
    // left face (node L of eL | own node 0)
    {
      const int m = eL * NP + L;
      const double pq[3] = {q[0][m], q[1][m], q[2][m]};
      const double pir = ir[m];
      const Node1 o = node1(g, pq[0], pq[2], S[m], pir);
      const double wl = ws1(g, o, pir), wr = ws1(g, n0, ir[base]);
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(lam, pq[c] - qq[c][0], o.f[c] + f[c][0]);
        k[c][0] = fma(iJ * B.iw0, fs - f[c][0], k[c][0]);
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      double out[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (kout) kout[c][m] = k[c][i];
        double val = fma(c2dt, k[c][i], c1 * qq[c][i]);
        if (c0 != 0.0) val = fma(c0, qn[c][m], val);
        out[c] = val;
      }
      if (qo) {
#pragma unroll
        for (int c = 0; c < 3; ++c) qo[c][m] = out[c];
        iro[m] = 1.0 / out[1];
      }
      bad |= not_positive_finite(out[1]) || nonfinite_bits(out[0]) || nonfinite_bits(out[2]);
    }
  }
  if (bad) flag_nonfinite(status);
  v.sync();
}

template <int NP>
__device__ void d1_recip(const View1<NP>& v, const double* x, double* y) {
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) y[m] = 1.0 / x[m];
  v.sync();
}
template <int NP>
__device__ void d1_copy(const View1<NP>& v, const double* x, double* y) {
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) y[m] = x[m];
  v.sync();
}
template <int NP>
__device__ void d1_zero(const View1<NP>& v, double* y) {
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) y[m] = 0.0;
  v.sync();
}

// SSP-RK3 stage coefficients (IGR_adjoints_1d/forward.jl:61-79):
// q_out = c0 q^n + c1 q_s + c2 dt k(q_s)
__device__ __forceinline__ void rk1_coef(int s, double* c0, double* c1, double* c2) {
  *c0 = s == 0 ? 0.0 : (s == 1 ? 0.75 : 1.0 / 3.0);
  *c1 = s == 0 ? 1.0 : (s == 1 ? 0.25 : 2.0 / 3.0);
  *c2 = *c1;
}

// Scratch fields of one untaped step (per instance, N doubles each)
enum : int {
  F1_Q1 = 0, F1_Q2 = 3, F1_IR1 = 6, F1_IR2 = 7, F1_B = 8, F1_CM = 9, F1_CK = 10, F1_CINVM = 11, F1_CPR = 12,
  F1_W0 = 13, F1_W1 = 14, F1_W2 = 15, F1_W3 = 16, F1_STEP_FIELDS = 17
};

// Tape of one RK stage (adjoint): stage input, Sigma in/out, setup outputs
// and the solver tape.
struct StageTape1 {
  double *q[3], *ir, *sin, *sout, *b, *cm, *ck, *cpR, *cinvM, *cM;
  SolveTape1 st;
};
constexpr int STAGE1_FIELDS = 12;

// Lay a stage tape over `fields` consecutive fields starting at base.
template <int NP>
__device__ StageTape1 stage_tape1(const View1<NP>& v, double* base, int solver, int n) {
  StageTape1 t;
  auto f = [&](int k) { return base + (long long)k * v.N; };
  t.q[0] = f(0); t.q[1] = f(1); t.q[2] = f(2);
  t.ir = f(3); t.sin = f(4); t.sout = f(5); t.b = f(6); t.cm = f(7); t.ck = f(8); t.cpR = f(9); t.cinvM = f(10); t.cM = f(11);
  t.st.base = f(STAGE1_FIELDS); t.st.N = v.N; t.st.n = n; t.st.pcg = solver == 0 ? 1 : 0;
  return t;
}

// One SSP-RK3 step of IGR_adjoints_1d/forward.jl:61-79 (compute_igr_euler_rhs!
// per stage: Sigma solve with the warm-start chain, then the DG RHS).
// q (3 fields) and ir = 1/rho are advanced in place; Sx is the current Sigma
// (warm start in, solution out), Sy a spare buffer (the two may be swapped).
// wk: F1_STEP_FIELDS work fields. tp: 3 stage tapes or null.
template <int NP>
__device__ void d1_step(const View1<NP>& v, const BasisDev& B, int solver, int n_iter, double* const q[3], double* ir,
                        double*& Sx, double*& Sy, double* wk, StageTape1* tp, int* status, double* s_red) {
  const Inst1D& I = v.I;
  const bool apos = I.alpha > 0;
  auto W = [&](int k) { return wk + (long long)k * v.N; };
  double* q1[3] = {W(F1_Q1), W(F1_Q1 + 1), W(F1_Q1 + 2)};
  double* q2[3] = {W(F1_Q2), W(F1_Q2 + 1), W(F1_Q2 + 2)};
  double* irs[3] = {ir, W(F1_IR1), W(F1_IR2)};
  const SolveTape1 none;
  for (int s = 0; s < 3; ++s) {
    double* const* qs = s == 0 ? q : (s == 1 ? q1 : q2);
    StageTape1* t = tp ? &tp[s] : nullptr;
    if (t) {
      for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
        t->q[0][m] = qs[0][m]; t->q[1][m] = qs[1][m]; t->q[2][m] = qs[2][m];
        t->ir[m] = irs[s][m]; t->sin[m] = Sx[m];
      }
      v.sync();
    }
    if (apos) {
      double* b = t ? t->b : W(F1_B);
      double* cm = t ? t->cm : W(F1_CM);
      double* ck = t ? t->ck : W(F1_CK);
      double* cpR = t ? t->cpR : W(F1_CPR);
      double* ci = t ? t->cinvM : W(F1_CINVM);
      d1_setup(v, B, qs[0], irs[s], b, cm, ck, cpR, ci, t ? t->cM : nullptr);
      d1_solve(v, B, solver, n_iter, b, Sx, Sy, cm, ck, cpR, ci, W(F1_W0), W(F1_W1), W(F1_W2), W(F1_W3),
               t ? t->st : none, s_red);
      double* tmp = Sx; Sx = Sy; Sy = tmp;
    }
    if (t) {
      for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) t->sout[m] = Sx[m];
      v.sync();
    }
    const double* qsc[3] = {qs[0], qs[1], qs[2]};
    const double* qnc[3] = {q[0], q[1], q[2]};
    double* const* qo = s == 0 ? q1 : (s == 1 ? q2 : q);
    double c0, c1, c2;
    rk1_coef(s, &c0, &c1, &c2);
    d1_hyp_rk(v, B, qsc, irs[s], Sx, qnc, c0, c1, c2, I.dt, qo, s < 2 ? irs[s + 1] : irs[0], nullptr, status);
  }
}

// Forward kernel scratch: the step work fields, 1/rho and the spare Sigma.
enum : int { F1_IR0 = F1_STEP_FIELDS, F1_SA = F1_STEP_FIELDS + 1, F1_FIELDS = F1_STEP_FIELDS + 2 };

// Batch layout: instance i's state is the block q + 3 off_i = (mu, rho, E),
// N_i doubles each, and its Sigma is sig + off_i.
struct Fwd1DArgs {
  const Inst1D* inst; const int* order; BasisDev B;
  double* q;          // batch state, in place
  double* sig;        // batch Sigma out
  double* scr;        // scratch arena
  int solver, n_iter, final_solve;
  int cs;             // CTAs per instance (cluster size)
  int* status;
};

// run_forward! (IGR_adjoints_1d/forward.jl:50-87) for one instance per CTA:
// n_steps SSP-RK3 steps of size dt with the Sigma warm-start chain, then the
// final solve at T when final_solve and alpha > 0.
template <int NP>
__global__ void __launch_bounds__(T1, 2) k1_forward(Fwd1DArgs a) {
  __shared__ double s_red[T1];
  int inst;
  const View1<NP> v = make_view1<NP>(a.inst, a.order, a.scr, a.cs, &inst);
  const BasisDev& B = a.B;
  const Inst1D& I = v.I;
  double* q[3] = {a.q + 3 * I.off, a.q + 3 * I.off + v.N, a.q + 3 * I.off + 2 * v.N};
  double* ir = v.f(F1_IR0);
  double* sig = a.sig + I.off;
  double* Sx = sig;
  double* Sy = v.f(F1_SA);
  d1_zero(v, Sx);
  d1_recip(v, q[1], ir);
  for (int step = 0; step < I.n_steps; ++step) d1_step(v, B, a.solver, a.n_iter, q, ir, Sx, Sy, v.scr, nullptr, a.status, s_red);
  if (I.alpha > 0 && a.final_solve) {
    const SolveTape1 none;
    d1_setup(v, B, q[0], ir, v.f(F1_B), v.f(F1_CM), v.f(F1_CK), v.f(F1_CPR), v.f(F1_CINVM), nullptr);
    d1_solve(v, B, a.solver, a.n_iter, v.f(F1_B), Sx, Sy, v.f(F1_CM), v.f(F1_CK), v.f(F1_CPR), v.f(F1_CINVM), v.f(F1_W0),
             v.f(F1_W1), v.f(F1_W2), v.f(F1_W3), none, s_red);
    double* t = Sx; Sx = Sy; Sy = t;
  }
  if (Sx != sig) d1_copy(v, Sx, sig);
}

}  // namespace igrgpu
