// 2D IGR-Euler forward kernels (sm_103a, FP64 CUDA cores).
//
// Thread mapping: a CTA owns a TX x TY tile of elements of one instance and
// runs one thread per element *line*: in the xi-phase thread t of element e
// owns row j = t (nodes (0..NP-1, t)), in the eta-phase column i = t. The
// 1D contractions with the LGL differentiation matrix then run in registers,
// loop-unrolled per line, which lets the compiler skip the structurally zero
// interior diagonal entries of D for every lane alike (no divergence), and
// face work lands on the threads that own the face nodes.
//
// GB300 has ~1.2 TFLOP/s of FP64 against 6.6 TB/s of HBM (about 5.6 B per
// FP64 flop), so these kernels trade memory for FP64 instructions: per-stage
// operator coefficients are precomputed once and re-read in every solver
// iteration, reciprocals replace divisions, and the SIP face terms are folded
// into the stiffness transpose (see apply_sip below).
#pragma once
#include "igr_device.cuh"

namespace igrgpu {

template <int NP>
struct Tiling2D {
  static constexpr int TX = NP <= 4 ? 4 : 2;  // element tile (keeps static smem < 48 KB)
  static constexpr int TY = 4;
  static constexpr int TE = TX * TY;       // elements per tile
  static constexpr int NN = NP * NP;       // nodes per element
  static constexpr int NT = TE * NP;       // threads per CTA (one per line)
  static constexpr int L = NP - 1;
};

// Per-thread view of its element and of the periodic neighbours.
struct ElemView {
  int e, t, ext, eyt, ex, ey;
  bool valid;
  long long base;  // first node of the element
};

template <int NP>
__device__ __forceinline__ ElemView elem_view(const Tile2D& tl, const Inst2D& I) {
  ElemView v;
  v.e = threadIdx.x / NP;
  v.t = threadIdx.x % NP;
  v.ext = v.e % Tiling2D<NP>::TX;
  v.eyt = v.e / Tiling2D<NP>::TX;
  v.ex = tl.ex0 + v.ext;
  v.ey = tl.ey0 + v.eyt;
  v.valid = (v.ex < I.nex) && (v.ey < I.ney);
  v.base = I.off + (long long)NP * NP * ((long long)v.ex + (long long)I.nex * v.ey);
  return v;
}

// Neighbour element (dx, dy in {-1,0,1}) with periodic wrap; returns its base
// node and its index inside the tile (or -1 when it is not in this tile).
template <int NP>
__device__ __forceinline__ long long neighbour(const Tile2D& tl, const Inst2D& I, int ex, int ey, int ddx, int ddy,
                                               int* in_tile) {
  constexpr int TX = Tiling2D<NP>::TX, TY = Tiling2D<NP>::TY;
  int nx = ex + ddx, ny = ey + ddy;
  nx = nx < 0 ? I.nex - 1 : (nx >= I.nex ? 0 : nx);
  ny = ny < 0 ? I.ney - 1 : (ny >= I.ney ? 0 : ny);
  const int lx = nx - tl.ex0, ly = ny - tl.ey0;
  *in_tile = (lx >= 0 && lx < TX && ly >= 0 && ly < TY) ? (lx + TX * ly) : -1;
  return I.off + (long long)NP * NP * ((long long)nx + (long long)I.nex * ny);
}

// The diagonal of the LGL differentiation matrix vanishes at interior nodes
// (exactly 0.0 in double for P3 as built by basis.jl:38-49; |D_ii| < 1e-15 for
// P4), so those products are skipped. Callers unroll the loops, making i and k
// compile-time constants and the skip free of branches.
__device__ __forceinline__ constexpr bool d_zero(int np, int i, int k) { return i == k && i > 0 && i < np - 1; }

// sum_k D[i][k] v[k] (reference derivative of a line at node i)
template <int NP>
__device__ __forceinline__ double dot_row(const BasisDev& B, int i, const double* v) {
  double s = 0.0;
  bool first = true;
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    if (d_zero(NP, i, k)) continue;
    s = first ? B.D[i][k] * v[k] : fma(B.D[i][k], v[k], s);
    first = false;
  }
  return s;
}

// acc + sum_i D[i][k] v[i] (transpose contraction, node k)
template <int NP>
__device__ __forceinline__ double dot_col(const BasisDev& B, int k, const double* v, double acc) {
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    if (d_zero(NP, i, k)) continue;
    acc = fma(B.D[i][k], v[i], acc);
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Stage setup: IGR source b (elliptic.jl:159-197), diag(A) (elliptic.jl:205-264)
// and the per-node operator coefficients reused by every solver iteration:
//   cm  = w_i w_j Jx Jy / rho                     (mass)
//   ckx = alpha w_i w_j (Jy/Jx) / rho             (x stiffness)
//   cky = alpha w_i w_j (Jx/Jy) / rho             (y stiffness)
//   cpx = alpha (w_j Jy) eta max(1/rho_L,1/rho_R)/dx   at x-face nodes (penalty)
//   cpy = alpha (w_i Jx) eta max(1/rho_L,1/rho_R)/dy   at y-face nodes
//   cinvM = 1 / diag(A)
// ---------------------------------------------------------------------------
struct SetupArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *mx, *my, *invr;
  double *b, *cm, *ckx, *cky, *cinvM, *cpx, *cpy;
  double *cM;  // diag(A) itself (optional; the reverse needs it for d/d alpha)
  int always;  // compute the coefficients even when alpha <= 0 (operator application on its own)
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_setup(SetupArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_ux[TE][NN], s_uy[TE][NN], s_ir[TE][NN], s_uxx[TE][NN], s_uyx[TE][NN], s_mx[TE][NN];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double invJx = I.ijx, invJy = I.ijy;
  if (I.alpha <= 0.0 && !a.always) return;  // no elliptic solve for this instance (forward.jl:24-28)

  // ---- row phase (row t): velocities, x-derivatives, x part of the stiffness diagonal
  double ux[NP], uy[NP], ir[NP];
  if (v.valid) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = v.base + t * NP + i;
      ir[i] = a.invr[n];
      ux[i] = a.mx[n] * ir[i];
      uy[i] = a.my[n] * ir[i];
      s_ux[e][t * NP + i] = ux[i]; s_uy[e][t * NP + i] = uy[i]; s_ir[e][t * NP + i] = ir[i];
    }
    const double cxs = I.alpha * B.w[t] * I.jy * invJx;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      s_uxx[e][t * NP + i] = dot_row<NP>(B, i, ux) * invJx;
      s_uyx[e][t * NP + i] = dot_row<NP>(B, i, uy) * invJx;
      double m = B.W2[0][i] * ir[0];
#pragma unroll
      for (int k = 1; k < NP; ++k) m = fma(B.W2[k][i], ir[k], m);
      s_mx[e][t * NP + i] = cxs * m;
    }
  }
  __syncthreads();
  if (!v.valid) return;

  // ---- column phase (column t): y-derivatives, source, diagonal, coefficients
  double cux[NP], cuy[NP], cir[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) { cux[l] = s_ux[e][l * NP + t]; cuy[l] = s_uy[e][l * NP + t]; cir[l] = s_ir[e][l * NP + t]; }
  const double cys = I.alpha * B.w[t] * I.jx * invJy;
  const double eta = (double)(NP * NP);
  // partner 1/rho across the x-faces of column t (t == 0 or t == L) and the y-faces (l == 0, l == L)
  double irx[NP];  // partner for the x-face at node (t, l)
  if (t == 0 || t == L) {
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, t == 0 ? -1 : 1, 0, &it);
    const int pi = t == 0 ? L : 0;
#pragma unroll
    for (int l = 0; l < NP; ++l) irx[l] = it >= 0 ? s_ir[it][l * NP + pi] : a.invr[pb + l * NP + pi];
  }
  double iry[2];
  {
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, -1, &it);  // bottom partner: node (t, L)
    iry[0] = it >= 0 ? s_ir[it][L * NP + t] : a.invr[pb + L * NP + t];
    const long long pt = neighbour<NP>(tl, I, v.ex, v.ey, 0, 1, &it);   // top partner: node (t, 0)
    iry[1] = it >= 0 ? s_ir[it][t] : a.invr[pt + t];
  }
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    double uxy = dot_row<NP>(B, l, cux) * invJy;
    double uyy = dot_row<NP>(B, l, cuy) * invJy;
    const double uxx = s_uxx[e][l * NP + t], uyx = s_uyx[e][l * NP + t];
    const double s = uxx + uyy;
    double R = fma(s, s, uxx * uxx);
    R = fma(2.0 * uxy, uyx, R);
    R = fma(uyy, uyy, R);
    const double ww = B.w[t] * B.w[l];
    a.b[n] = ww * I.jx * I.jy * (I.alpha * R);
    double my_ = B.W2[0][l] * cir[0];
#pragma unroll
    for (int k = 1; k < NP; ++k) my_ = fma(B.W2[k][l], cir[k], my_);
    const double mass = ww * I.jx * I.jy * cir[l];
    double M = mass + s_mx[e][l * NP + t] + cys * my_;
    double px = 0.0, py = 0.0;
    if (t == 0 || t == L) {
      const double wf = B.w[l] * I.jy;
      const double sig = eta * fmax(t == L ? cir[l] : irx[l], t == L ? irx[l] : cir[l]) * I.idx;
      px = I.alpha * sig * wf;
      // x-face self terms: right side of its left face (t == 0) / left side of its right face (t == L)
      M += (t == L ? -I.alpha * invJx * B.D[L][L] : I.alpha * invJx * B.D[0][0]) * cir[l] * wf + px;
    }
    if (l == 0 || l == L) {
      const double wf = B.w[t] * I.jx;
      const double ip = iry[l == 0 ? 0 : 1];
      const double sig = eta * fmax(l == L ? cir[l] : ip, l == L ? ip : cir[l]) * I.idy;
      py = I.alpha * sig * wf;
      M += (l == L ? -I.alpha * invJy * B.D[L][L] : I.alpha * invJy * B.D[0][0]) * cir[l] * wf + py;
    }
    a.cm[n] = mass;
    a.ckx[n] = I.alpha * ww * I.jy * invJx * cir[l];
    a.cky[n] = I.alpha * ww * I.jx * invJy * cir[l];
    a.cpx[n] = px;
    a.cpy[n] = py;
    a.cinvM[n] = 1.0 / M;
    if (a.cM) a.cM[n] = M;
  }
}

// ---------------------------------------------------------------------------
// SIP operator application y = A x (elliptic.jl:30-145) with a solver
// epilogue. The face terms of a face-node pair (L, R) are
//   F = hw*(kx_L d_L + kx_R d_R) + p (x_L - x_R),  hw = -1/(2 w_0)
//   y_L += F, y_R -= F                    (consistency + penalty)
//   sx_L += hw kx_L jump, sx_R += hw kx_R jump   (symmetry term, folded into
//                                                  the stiffness transpose)
// where d is the reference derivative of x at the face node on each side.
// Each side computes F itself (owner computes), so no atomics are needed.
// ---------------------------------------------------------------------------
enum { EPI_CHEB = 0, EPI_JACOBI = 1, EPI_RESID = 2 };

struct ApplyArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double* x;                       // x_k (read with halo)
  const double *cm, *ckx, *cky, *cpx, *cpy, *b, *cinvM;
  const double* d_in;                    // Chebyshev d_k (null on the first iteration)
  double *d_out, *x_out;                 // d_{k+1}, x_{k+1}
  double *tape_x, *tape_r;               // optional tape of x_k and r_k = b - A x_k
  double *y_out;                         // EPI_RESID: raw y = A x
  double ca, cc, omega;                  // d_{k+1} = ca d_k + cc M^-1 r_k ; Jacobi omega
};

template <int NP, int EPI>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_apply(ApplyArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_x[TE][NN], s_yx[TE][NN], s_gxf[TE][NP][2], s_gyf[TE][NP][2];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double hw = B.hw;

  // ---- xi-phase part 1: row t, derivatives
  double xr[NP], gx[NP];
  double xc[NP], gy[NP];
  if (v.valid) {
#pragma unroll
    for (int i = 0; i < NP; ++i) { xr[i] = a.x[v.base + t * NP + i]; s_x[e][t * NP + i] = xr[i]; }
#pragma unroll
    for (int i = 0; i < NP; ++i) gx[i] = dot_row<NP>(B, i, xr);
    s_gxf[e][t][0] = gx[0]; s_gxf[e][t][1] = gx[L];
    if (a.tape_x) {
#pragma unroll
      for (int i = 0; i < NP; ++i) a.tape_x[v.base + t * NP + i] = xr[i];
    }
  }
  __syncthreads();
  if (v.valid) {
#pragma unroll
    for (int l = 0; l < NP; ++l) xc[l] = s_x[e][l * NP + t];
#pragma unroll
    for (int l = 0; l < NP; ++l) gy[l] = dot_row<NP>(B, l, xc);
    s_gyf[e][t][0] = gy[0]; s_gyf[e][t][1] = gy[L];

    // ---- xi-phase part 2: x-faces of row t and the x-stiffness transpose
    double kxr[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) kxr[i] = a.ckx[v.base + t * NP + i];
    // partner values across the left (s = 0) and right (s = 1) faces
    double px_[2], pd_[2], pk_[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;  // partner face node index along x
      pk_[s] = a.ckx[pb + t * NP + pi];
      if (it >= 0) {
        px_[s] = s_x[it][t * NP + pi];
        pd_[s] = s_gxf[it][t][s == 0 ? 1 : 0];
      } else {
        double pr[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) pr[k] = a.x[pb + t * NP + k];
        px_[s] = pr[pi];
        pd_[s] = dot_row<NP>(B, pi, pr);
      }
    }
    // left face: own node (0,t) is the R side; right face: own node (L,t) is the L side
    const double jl = px_[0] - xr[0];
    const double Fl = fma(a.cpx[v.base + t * NP], jl, hw * fma(pk_[0], pd_[0], kxr[0] * gx[0]));
    const double jr = xr[L] - px_[1];
    const double Fr = fma(a.cpx[v.base + t * NP + L], jr, hw * fma(kxr[L], gx[L], pk_[1] * pd_[1]));
    double sx[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) sx[i] = kxr[i] * gx[i];
    sx[0] = kxr[0] * fma(hw, jl, gx[0]);
    sx[L] = kxr[L] * fma(hw, jr, gx[L]);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const double acc = (k == 0) ? -Fl : ((k == L) ? Fr : 0.0);
      s_yx[e][t * NP + k] = dot_col<NP>(B, k, sx, acc);
    }
  }
  __syncthreads();
  if (!v.valid) return;

  // ---- eta-phase: y-faces of column t, y-stiffness transpose, mass, epilogue
  double kyc[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) kyc[l] = a.cky[v.base + l * NP + t];
  double qx_[2], qd_[2], qk_[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, s == 0 ? -1 : 1, &it);
    const int pl = s == 0 ? L : 0;
    qk_[s] = a.cky[pb + pl * NP + t];
    if (it >= 0) {
      qx_[s] = s_x[it][pl * NP + t];
      qd_[s] = s_gyf[it][t][s == 0 ? 1 : 0];
    } else {
      double pc[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) pc[k] = a.x[pb + k * NP + t];
      qx_[s] = pc[pl];
      qd_[s] = dot_row<NP>(B, pl, pc);
    }
  }
  const double jb = qx_[0] - xc[0];
  const double Fb = fma(a.cpy[v.base + t], jb, hw * fma(qk_[0], qd_[0], kyc[0] * gy[0]));
  const double jt = xc[L] - qx_[1];
  const double Ft = fma(a.cpy[v.base + L * NP + t], jt, hw * fma(kyc[L], gy[L], qk_[1] * qd_[1]));
  double sy[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) sy[l] = kyc[l] * gy[l];
  sy[0] = kyc[0] * fma(hw, jb, gy[0]);
  sy[L] = kyc[L] * fma(hw, jt, gy[L]);
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    double y = fma(a.cm[n], xc[l], s_yx[e][l * NP + t] + ((l == 0) ? -Fb : ((l == L) ? Ft : 0.0)));
    y = dot_col<NP>(B, l, sy, y);
    if (EPI == EPI_RESID) { a.y_out[n] = y; continue; }
    const double r = a.b[n] - y;
    if (a.tape_r) a.tape_r[n] = r;
    if (EPI == EPI_CHEB) {
      const double z = r * a.cinvM[n];
      const double d = a.d_in ? fma(a.ca, a.d_in[n], a.cc * z) : a.cc * z;
      a.d_out[n] = d;
      a.x_out[n] = xc[l] + d;
    } else {  // EPI_JACOBI: x + omega (b - A x) / M   (elliptic.jl:358)
      a.x_out[n] = fma(a.omega * r, a.cinvM[n], xc[l]);
    }
  }
}

// ---------------------------------------------------------------------------
// Hyperbolic DG RHS (hyperbolic.jl:27-119) fused with the SSP-RK3 stage
// combination (forward.jl:53-68):  q_out = c0*q^n + c1*q_s + c2*dt*k(q_s, Sigma).
// Also writes 1/rho of q_out for the next stage's setup and flags non-finite
// values or rho <= 0 in the status word.
// ---------------------------------------------------------------------------
struct HypArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *invr, *S;   // stage input
  const double *qn[4];             // step-start state (stages 2 and 3)
  double c0, c1, c2;
  double *qo[4], *invro;           // stage output (may alias qn: pointwise)
  double *k_out[4];                // optional: raw RHS k (compute_hyperbolic_rhs!)
  int* status;
};

template <int NP>
struct FaceState { double q[4], f[4], ws; };

// Physical flux in direction dir at one node (euler.jl:156-186) and |u_n| + c.
__device__ __forceinline__ void node_flux(int dir, double g, double mx, double my, double r, double E, double S, double ir,
                                          double f[4], double* ws) {
  const double ux = mx * ir, uy = my * ir;
  const double kin = fma(mx, mx, my * my) * (0.5 * ir);
  const double P = (g - 1.0) * (E - kin);
  const double pb = P + S;
  const double un = dir == 0 ? ux : uy;
  if (dir == 0) { f[0] = fma(mx, ux, pb); f[1] = my * ux; f[2] = mx; }
  else { f[0] = mx * uy; f[1] = fma(my, uy, pb); f[2] = my; }
  f[3] = (E + pb) * un;
  if (ws) *ws = fabs(un) + sqrt(g * P * ir);
}

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_hyp_rk(HypArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_fy[4][TE][NN];    // y fluxes
  __shared__ double s_k[4][TE][NN];     // x part of the RHS
  __shared__ FaceState<NP> s_xf[TE][NP][2];  // x-face node data (left, right) per row
  __shared__ FaceState<NP> s_yf[TE][NP][2];  // y-face node data (bottom, top) per column
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double g = I.gamma;
  const double invJx = I.ijx, invJy = I.ijy;

  double q[4][NP], fx[4][NP];
  if (v.valid) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = v.base + t * NP + i;
      const double mx = a.q[0][n], my = a.q[1][n], r = a.q[2][n], E = a.q[3][n], S = a.S[n], ir = a.invr[n];
      q[0][i] = mx; q[1][i] = my; q[2][i] = r; q[3][i] = E;
      double f[4], fyv[4], ws;
      node_flux(0, g, mx, my, r, E, S, ir, f, (i == 0 || i == L) ? &ws : nullptr);
#pragma unroll
      for (int c = 0; c < 4; ++c) fx[c][i] = f[c];
      node_flux(1, g, mx, my, r, E, S, ir, fyv, nullptr);
#pragma unroll
      for (int c = 0; c < 4; ++c) s_fy[c][e][t * NP + i] = fyv[c];
      if (i == 0 || i == L) {
        FaceState<NP>& fs = s_xf[e][t][i == 0 ? 0 : 1];
#pragma unroll
        for (int c = 0; c < 4; ++c) { fs.q[c] = q[c][i]; fs.f[c] = f[c]; }
        fs.ws = ws;
      }
    }
  }
  __syncthreads();
  if (v.valid) {
    // y-face node data of column t (bottom l = 0, top l = L)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int l = s == 0 ? 0 : L;
      const long long n = v.base + l * NP + t;
      double f[4], ws;
      node_flux(1, g, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], f, &ws);
      FaceState<NP>& fs = s_yf[e][t][s];
      fs.q[0] = a.q[0][n]; fs.q[1] = a.q[1][n]; fs.q[2] = a.q[2][n]; fs.q[3] = a.q[3][n];
#pragma unroll
      for (int c = 0; c < 4; ++c) fs.f[c] = f[c];
      fs.ws = ws;
    }
    // ---- x volume term of row t
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) s_k[c][e][t * NP + i] = -invJx * dot_row<NP>(B, i, fx[c]);
  }
  __syncthreads();
  if (v.valid) {
    // ---- x faces of row t (LLF, euler.jl:222-236), owner computes its side
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;
      FaceState<NP> pf;
      if (it >= 0) {
        pf = s_xf[it][t][s == 0 ? 1 : 0];
      } else {
        const long long n = pb + t * NP + pi;
        pf.q[0] = a.q[0][n]; pf.q[1] = a.q[1][n]; pf.q[2] = a.q[2][n]; pf.q[3] = a.q[3][n];
        node_flux(0, g, pf.q[0], pf.q[1], pf.q[2], pf.q[3], a.S[n], a.invr[n], pf.f, &pf.ws);
      }
      const FaceState<NP>& of = s_xf[e][t][s];
      const FaceState<NP>& Ls = s == 0 ? pf : of;
      const FaceState<NP>& Rs = s == 0 ? of : pf;
      const double lam = (Rs.ws > Ls.ws) ? Rs.ws : Ls.ws;
      const int io = s == 0 ? 0 : L;
      const double cf = s == 0 ? invJx * B.iw0 : -invJx * B.iwL;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double fs = 0.5 * fma(lam, Ls.q[c] - Rs.q[c], Ls.f[c] + Rs.f[c]);
        s_k[c][e][t * NP + io] = fma(cf, fs - of.f[c], s_k[c][e][t * NP + io]);
      }
    }
  }
  __syncthreads();
  if (!v.valid) return;
  // ---- column t: y volume term, y faces, RK combination
  double kc[4][NP];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    double fyc[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) fyc[l] = s_fy[c][e][l * NP + t];
#pragma unroll
    for (int l = 0; l < NP; ++l) kc[c][l] = fma(-invJy, dot_row<NP>(B, l, fyc), s_k[c][e][l * NP + t]);
  }
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, s == 0 ? -1 : 1, &it);
    const int pl = s == 0 ? L : 0;
    FaceState<NP> pf;
    if (it >= 0) {
      pf = s_yf[it][t][s == 0 ? 1 : 0];
    } else {
      const long long n = pb + pl * NP + t;
      pf.q[0] = a.q[0][n]; pf.q[1] = a.q[1][n]; pf.q[2] = a.q[2][n]; pf.q[3] = a.q[3][n];
      node_flux(1, g, pf.q[0], pf.q[1], pf.q[2], pf.q[3], a.S[n], a.invr[n], pf.f, &pf.ws);
    }
    const FaceState<NP>& of = s_yf[e][t][s];
    const FaceState<NP>& Ls = s == 0 ? pf : of;
    const FaceState<NP>& Rs = s == 0 ? of : pf;
    const double lam = (Rs.ws > Ls.ws) ? Rs.ws : Ls.ws;
    const int lo = s == 0 ? 0 : L;
    const double cf = s == 0 ? invJy * B.iw0 : -invJy * B.iwL;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double fs = 0.5 * fma(lam, Ls.q[c] - Rs.q[c], Ls.f[c] + Rs.f[c]);
      kc[c][lo] = fma(cf, fs - of.f[c], kc[c][lo]);
    }
  }
  const double c2dt = a.c2 * I.dt;
  bool bad = false;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    double qo[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (a.k_out[c]) a.k_out[c][n] = kc[c][l];
      const double qs = a.q[c][n];
      double val = fma(c2dt, kc[c][l], a.c1 * qs);
      if (a.c0 != 0.0) val = fma(a.c0, a.qn[c][n], val);
      qo[c] = val;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) if (a.qo[c]) a.qo[c][n] = qo[c];
    if (a.invro) a.invro[n] = 1.0 / qo[2];
    bad |= !(qo[2] > 0.0) || !isfinite(qo[0]) || !isfinite(qo[1]) || !isfinite(qo[3]) || !isfinite(qo[2]);
  }
  if (bad) flag_nonfinite(a.status);
}

}  // namespace igrgpu
