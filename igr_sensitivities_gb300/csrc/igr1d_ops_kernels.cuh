// Operator-level calls of the 1D package (IGR_adjoints_1d): one evaluation of
// one operator per instance of a batch, one CTA (or thread-block cluster) per
// instance, built from the device functions the persistent solvers use
// (d1_setup, d1_apply, d1_solve, d1_hyp_rk), so the results are those of the
// corresponding steps inside the RK loop.
#pragma once
#include "igr1d_kernels.cuh"

namespace igrgpu {

// Scratch fields of one instance (N doubles each), after the per-element work.
enum : int {
  O1_IR = 0, O1_B = 1, O1_CM = 2, O1_CK = 3, O1_CPR = 4, O1_CINVM = 5, O1_W0 = 6, O1_W1 = 7, O1_W2 = 8, O1_W3 = 9,
  O1_SY = 10, O1_FIELDS = 11
};

// Batch layout as the forward kernel's: instance i's state is q + 3 off_i =
// (mu, rho, E), N_i doubles each; single fields (x, rho, b, Sigma, y) start at
// off_i. Which pointers an operation reads or writes:
//   APPLY_SIP: x, rho -> out (y)
//   IGR_RHS:   q -> out (b), diag (diag(A), optional)
//   SOLVE:     q, sig (in/out)
//   HYP_RHS:   q, sig -> out (3 fields at 3 off_i)
//   EULER_RHS: q, sig (in/out) -> out (3 fields at 3 off_i)
//   CG:        rho, b, x (in/out: initial guess -> solution) -> iters[i]
struct Ops1DArgs {
  const Inst1D* inst; const int* order; BasisDev B;
  const double *q, *rho, *b;
  double *x, *sig, *out, *diag;
  int* iters;
  double* scr;
  int op, solver, n_iter;
  double tol;
  int maxiter, fixed;
  int cs;
  int* status;
};

// Conjugate gradients on A x = b with M = I (cg_fixed! with its 1e-30 guards;
// cg_solve! without them and with the exit `sqrt(rs_old) < tol` checked before
// each iteration). x: initial guess in, solution out; r, p, ap: scratch.
// Returns the count the reference returns. Every CTA of the instance forms the
// same inner products, so every thread takes the same exit.
template <int NP>
__device__ int d1_cg(const View1<NP>& v, const BasisDev& B, const double* b, double* x, const double* cm,
                     const double* ck, const double* cpR, double* r, double* p, double* ap, double tol, int maxiter,
                     bool fixed, double* s_red) {
  const double eps = fixed ? 1e-30 : 0.0;
  double* red = v.slot();
  d1_apply<NP>(v, B, [&](int m) { return x[m]; }, cm, ck, cpR, [&](int e, const double*, const double* y) {
    double pe = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = e * NP + i;
      const double rr = b[m] - y[i];
      r[m] = rr; p[m] = rr;
      pe = fma(rr, rr, pe);
    }
    red[e] = pe;
  });
  double rs = v.reduce(s_red);
  for (int it = 1; it <= maxiter; ++it) {
    if (!fixed && sqrt(rs) < tol) return it;
    red = v.slot();
    d1_apply<NP>(v, B, [&](int m) { return p[m]; }, cm, ck, cpR, [&](int e, const double* xx, const double* y) {
      double pe = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        ap[e * NP + i] = y[i];
        pe = fma(xx[i], y[i], pe);
      }
      red[e] = pe;
    });
    const double pAp = v.reduce(s_red);
    const double a = cta_div(rs, pAp + eps);
    red = v.slot();
    for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
      double pe = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = e * NP + i;
        x[m] = fma(a, p[m], x[m]);
        const double rr = fma(-a, ap[m], r[m]);
        r[m] = rr;
        pe = fma(rr, rr, pe);
      }
      red[e] = pe;
    }
    const double rsn = v.reduce(s_red);
    const double beta = cta_div(rsn, rs + eps);
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) p[m] = fma(beta, p[m], r[m]);
    rs = rsn;
    v.sync();
  }
  return maxiter;
}

template <int NP>
__global__ void __launch_bounds__(T1, 2) k1_ops(Ops1DArgs a) {
  __shared__ double s_red[T1];
  int inst;
  const View1<NP> v = make_view1<NP>(a.inst, a.order, a.scr, a.cs, &inst);
  const BasisDev& B = a.B;
  const Inst1D& I = v.I;
  const double* q[3] = {a.q ? a.q + 3 * I.off : nullptr, a.q ? a.q + 3 * I.off + v.N : nullptr,
                        a.q ? a.q + 3 * I.off + 2 * v.N : nullptr};
  double* ir = v.f(O1_IR);
  const SolveTape1 none;
  switch (a.op) {
    case OP1_APPLY_SIP: {
      const double* rho = a.rho + I.off;
      const double* x = a.x + I.off;
      double* y = a.out + I.off;
      d1_recip(v, rho, ir);
      d1_setup(v, B, rho, ir, v.f(O1_B), v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR), v.f(O1_CINVM), nullptr);
      d1_apply<NP>(v, B, [&](int m) { return x[m]; }, v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR),
                   [&](int e, const double*, const double* yy) {
#pragma unroll
                     for (int i = 0; i < NP; ++i) y[e * NP + i] = yy[i];
                   });
      break;
    }
    case OP1_IGR_RHS: {
      d1_recip(v, q[1], ir);
      d1_setup(v, B, q[0], ir, a.out + I.off, v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR), v.f(O1_CINVM),
               a.diag ? a.diag + I.off : nullptr);
      break;
    }
    case OP1_SOLVE:
    case OP1_EULER_RHS: {
      double* sig = a.sig + I.off;
      d1_recip(v, q[1], ir);
      if (a.op == OP1_SOLVE || I.alpha > 0) {
        d1_setup(v, B, q[0], ir, v.f(O1_B), v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR), v.f(O1_CINVM), nullptr);
        d1_copy(v, sig, v.f(O1_SY));  // warm start (the solve writes its result to another field)
        d1_solve(v, B, a.solver, a.n_iter, v.f(O1_B), v.f(O1_SY), sig, v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR),
                 v.f(O1_CINVM), v.f(O1_W0), v.f(O1_W1), v.f(O1_W2), v.f(O1_W3), none, s_red);
      } else {
        d1_zero(v, sig);  // forward.jl:27-29
      }
      if (a.op == OP1_SOLVE) break;
      double* ko[3] = {a.out + 3 * I.off, a.out + 3 * I.off + v.N, a.out + 3 * I.off + 2 * v.N};
      d1_hyp_rk(v, B, q, ir, sig, q, 0.0, 1.0, 0.0, 0.0, nullptr, nullptr, ko, nullptr);
      break;
    }
    case OP1_HYP_RHS: {
      d1_recip(v, q[1], ir);
      double* ko[3] = {a.out + 3 * I.off, a.out + 3 * I.off + v.N, a.out + 3 * I.off + 2 * v.N};
      d1_hyp_rk(v, B, q, ir, a.sig + I.off, q, 0.0, 1.0, 0.0, 0.0, nullptr, nullptr, ko, nullptr);
      break;
    }
    case OP1_CG: {
      const double* rho = a.rho + I.off;
      d1_recip(v, rho, ir);
      d1_setup(v, B, rho, ir, v.f(O1_B), v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR), v.f(O1_CINVM), nullptr);
      const int it = d1_cg<NP>(v, B, a.b + I.off, a.x + I.off, v.f(O1_CM), v.f(O1_CK), v.f(O1_CPR), v.f(O1_W0),
                               v.f(O1_W1), v.f(O1_W2), a.tol, a.maxiter, a.fixed != 0, s_red);
      if (threadIdx.x == 0 && blockIdx.x % a.cs == 0) a.iters[inst] = it;
      break;
    }
    default: break;
  }
}

}  // namespace igrgpu
