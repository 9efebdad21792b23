// 1D host engine: batch plans and drivers of the per-instance persistent
// kernels (igr1d_kernels.cuh).
#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

#include "igr1d_launch.h"
#include "igr1d_ops_kernels.cuh"
#include "igr1d_rev_kernels.cuh"
#include "igr1d_pde_kernels.cuh"
#include "igr1d_sens_kernels.cuh"
#include "igr_engine.h"

namespace igrgpu {

#define NP1_DISPATCH(np, CALL)                        \
  switch (np) {                                       \
    case 2: { constexpr int NPV = 2; CALL; } break;   \
    case 3: { constexpr int NPV = 3; CALL; } break;   \
    case 4: { constexpr int NPV = 4; CALL; } break;   \
    case 5: { constexpr int NPV = 5; CALL; } break;   \
    default: throw Error(1, "unsupported polynomial degree"); \
  }

Plan1D make_plan1d(Ctx& c, const BasisDev& B, const std::vector<Inst1DDesc>& insts,
                   const std::function<long long(const Inst1DDesc&, int)>& scratch_fields, const std::string& tag) {
  Plan1D P;
  P.B = B;
  P.np = B.np;
  long long off = 0, soff = 0;
  std::vector<double> cost;
  for (const Inst1DDesc& d : insts) {
    if (d.ne < 1) throw Error(1, "mesh must have at least one element");
    if (!(d.L > 0)) throw Error(1, "domain length must be positive");
    if (d.n_steps < 0) throw Error(1, "n_steps must be >= 0");
    Inst1D I;
    std::memset(&I, 0, sizeof(I));
    I.off = off;
    I.soff = soff;
    I.ne = d.ne;
    I.n_steps = d.n_steps;
    I.L = d.L;
    I.dx = d.L / d.ne;        // mesh.jl:22-23
    I.J = I.dx / 2.0;
    I.iJ = 1.0 / I.J;
    I.idx = 1.0 / I.dx;
    I.gamma = d.gamma; I.alpha = d.alpha; I.dt = d.dt;
    I.t_end = d.t_end;
    I.h = d.h;
    P.inst.push_back(I);
    const long long n = (long long)P.np * d.ne;
    P.inst_nodes.push_back(n);
    off += n;
    soff += scratch_fields(d, (int)n) * n;
    cost.push_back((double)n * std::max(d.n_steps, 1));
  }
  P.NG = off;
  P.scratch = soff;
  // largest work first, so the long CTAs start early and short ones fill in
  P.order.resize(insts.size());
  std::iota(P.order.begin(), P.order.end(), 0);
  std::stable_sort(P.order.begin(), P.order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  P.d_inst = static_cast<Inst1D*>(c.ws.get(tag + ":inst1", sizeof(Inst1D) * P.inst.size()));
  P.d_order = static_cast<int*>(c.ws.get(tag + ":order1", sizeof(int) * P.order.size()));
  cuda_check(cudaMemcpyAsync(P.d_inst, P.inst.data(), sizeof(Inst1D) * P.inst.size(), cudaMemcpyHostToDevice, c.stream),
             "upload inst1");
  cuda_check(cudaMemcpyAsync(P.d_order, P.order.data(), sizeof(int) * P.order.size(), cudaMemcpyHostToDevice, c.stream),
             "upload order1");
  c.cur_nodes = off;
  return P;
}

long long forward1d_scratch_fields(const Inst1DDesc&, int) { return E1_FIELDS + F1_FIELDS; }

// CTAs per instance. Results do not depend on it (fixed-order reductions), so
// it is chosen for speed. One CTA advances an instance at one element per
// thread; its SM's FP64 rate bounds it (a 256-element Jacobi iteration: ~6 us).
// Small batches of instances with at least T1 elements therefore spread each
// over a cluster of up to 16 SMs (at least 16 elements per CTA); below T1
// elements the cluster barrier costs more than it saves (measured on GB300:
// N_e = 64 and 128 run 10-20% faster on one CTA), and batches that fill the
// GPU use one CTA per instance. A context setting overrides the choice, and
// autotuning replaces it with a measurement (cluster_size).
static int cluster_heuristic(Ctx& c, const Plan1D& P) {
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device), "attr");
  const long long ni = (long long)P.inst.size();
  int min_ne = 1 << 30;
  for (auto& I : P.inst) min_ne = std::min(min_ne, I.ne);
  int cs = 1;
  while (cs < 16 && min_ne >= T1 && ni * cs * 2 * 2 <= sms && min_ne / (cs * 2) >= 16) cs *= 2;
  return cs;
}

// Launch with the chosen cluster size, falling back to smaller clusters when
// the device refuses one (results are identical for every size).
template <class Args, class F>
static void launch_1d(Ctx& c, Args& a, int n_inst, F launch, const char* what) {
  for (;;) {
    cudaError_t e;
    {
      LaunchScope ls(c, KID_1D);
      e = launch(a, n_inst);
    }
    if (e == cudaSuccess) { c.last_cluster1d = a.cs; return; }
    if (a.cs <= 1) cuda_check(e, what);
    (void)cudaGetLastError();  // clear the refused launch
    a.cs /= 2;
  }
}

// CTAs per instance for this launch: the context setting, else (with
// autotuning on and the state q at hand) the fastest candidate measured for
// this batch shape, else cluster_heuristic. The measurement advances a copy
// of q by up to 3 steps of the forward kernel for every candidate (powers of
// two up to 16 that keep at least 16 elements per CTA), after one untimed
// run, timed with CUDA events; results do not depend on the choice.
static int cluster_size(Ctx& c, const Plan1D& P, const Solve2DOpts& o, const double* q) {
  if (c.cluster1d > 0) return c.cluster1d;
  const int h = cluster_heuristic(c, P);
  if (!c.tune.on || !q || P.inst.empty()) return h;
  int ne_min = 1 << 30, ne_max = 0;
  long long ne_sum = 0;
  for (auto& I : P.inst) {
    ne_min = std::min(ne_min, I.ne); ne_max = std::max(ne_max, I.ne); ne_sum += I.ne;
    if (!(I.dt > 0)) return h;
  }
  char key[160];
  std::snprintf(key, sizeof(key), "1d.cluster np=%d inst=%d ne_min=%d ne_max=%d ne_sum=%lld solver=%d iters=%d", P.np,
                (int)P.inst.size(), ne_min, ne_max, ne_sum, o.solver, o.n_iter);
  int v = 0;
  if (c.tune.get(key, &v)) return v;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cuda_check(cudaStreamIsCapturing(c.stream, &cap), "stream capture status");
  if (cap != cudaStreamCaptureStatusNone) return h;

  std::vector<Inst1DDesc> d(P.inst.size());
  for (size_t i = 0; i < P.inst.size(); ++i) {
    const Inst1D& I = P.inst[i];
    d[i].ne = I.ne; d[i].L = I.L; d[i].gamma = I.gamma; d[i].alpha = I.alpha; d[i].dt = I.dt;
    d[i].n_steps = std::min(std::max(I.n_steps, 1), 3);
  }
  const long long nodes_saved = c.cur_nodes, launches_saved = c.launches;
  const int last_saved = c.last_cluster1d;
  Plan1D Q;
  double *qq = nullptr, *sg = nullptr, *scr = nullptr;
  int* status = nullptr;
  try {  // no room for the probe's copies: keep the heuristic's choice, untuned
    Q = make_plan1d(c, P.B, d, forward1d_scratch_fields, "tune1");
    qq = c.ws.dbl("tune1:q", (size_t)3 * Q.NG);
    sg = c.ws.dbl("tune1:sig", (size_t)Q.NG);
    scr = c.ws.dbl("tune1:scr", (size_t)std::max<long long>(Q.scratch, 1));
    status = static_cast<int*>(c.ws.get("tune1:status", sizeof(int)));
  } catch (const Error&) {
    (void)cudaGetLastError();
    c.cur_nodes = nodes_saved;
    c.ws.release("tune1:q"); c.ws.release("tune1:sig"); c.ws.release("tune1:scr");
    return h;
  }
  c.cur_nodes = nodes_saved;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cuda_check(cudaEventCreate(&e0), "tune event");
  cuda_check(cudaEventCreate(&e1), "tune event");
  int best = h;
  float best_ms = 0.f;
  try {
    std::vector<int> cand{h};
    for (int cs = 1; cs <= 16; cs *= 2)
      if (cs != h && ne_min / cs >= 16) cand.push_back(cs);
    for (size_t k = 0; k <= cand.size(); ++k) {  // k = 0: untimed run with the heuristic's choice
      const int cs = cand[k == 0 ? 0 : k - 1];
      cuda_check(cudaMemcpyAsync(qq, q, sizeof(double) * 3 * Q.NG, cudaMemcpyDeviceToDevice, c.stream), "tune copy");
      cuda_check(cudaMemsetAsync(sg, 0, sizeof(double) * Q.NG, c.stream), "tune sigma");
      Fwd1DArgs a;
      std::memset(&a, 0, sizeof(a));
      a.inst = Q.d_inst; a.order = Q.d_order; a.B = Q.B;
      a.q = qq; a.sig = sg; a.scr = scr;
      a.solver = o.solver; a.n_iter = o.n_iter; a.final_solve = 0;
      a.status = status;
      a.cs = cs;
      cuda_check(cudaEventRecord(e0, c.stream), "tune event record");
      NP1_DISPATCH(Q.np, launch_1d(c, a, (int)Q.inst.size(),
                                   [&](const Fwd1DArgs& x, int n) { return launch_k1_forward<NPV>(x, n, c.stream); },
                                   "k1_forward launch (autotune)"));
      cuda_check(cudaEventRecord(e1, c.stream), "tune event record");
      cuda_check(cudaEventSynchronize(e1), "tune event sync");
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "tune event time");
      if (k > 0 && a.cs == cs && (k == 1 || ms < best_ms)) { best = cs; best_ms = ms; }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c.ws.release("tune1:q"); c.ws.release("tune1:sig"); c.ws.release("tune1:scr");  // frees after the stream drains
  c.launches = launches_saved;
  c.last_cluster1d = last_saved;
  c.tune.put(key, best);
  return best;
}

void forward1d(Ctx& c, const Plan1D& P, double* q, double* sig, const Solve2DOpts& o, bool final_solve) {
  double* scr = c.ws.dbl("f1:scr", (size_t)std::max<long long>(P.scratch, 1));
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  Fwd1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q = q; a.sig = sig; a.scr = scr;
  a.solver = o.solver; a.n_iter = o.n_iter; a.final_solve = final_solve ? 1 : 0;
  a.status = c.d_status;
  a.cs = cluster_size(c, P, o, q);
  NP1_DISPATCH(P.np, launch_1d(c, a, (int)P.inst.size(),
                               [&](const Fwd1DArgs& x, int n) { return launch_k1_forward<NPV>(x, n, c.stream); },
                               "k1_forward launch"));
  int st = 0;
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
}

int adjoint1d_segment(const std::vector<Inst1DDesc>& insts, int np, const Solve2DOpts& o, size_t budget) {
  int nmax = 0;
  for (auto& d : insts) nmax = std::max(nmax, d.n_steps);
  if (nmax <= 1) return 1;
  auto bytes = [&](int seg) {
    long long t = 0;
    for (auto& d : insts) {
      const int N = np * d.ne;
      t += (E1_FIELDS + adjoint1d_fields(o.solver, o.n_iter, N, d.n_steps, seg)) * N;
    }
    return (size_t)t * sizeof(double);
  };
  // every step's state kept (one forward re-run) when it fits in half the
  // budget, else sqrt(n)-long segments (two re-runs, O(sqrt n) snapshots)
  if (bytes(nmax) <= budget / 2) return nmax;
  const int s = (int)std::ceil(std::sqrt((double)nmax));
  if (bytes(s) > budget) throw Error(5, "device memory too small for the 1D adjoint of this batch");
  return s;
}

void adjoint1d(Ctx& c, const Plan1D& P, const double* q0, double* dq0, const Solve2DOpts& o, int objective,
               const double* prm, int seg, double* J, double* dgamma, double* dalpha) {
  const int ni = (int)P.inst.size();
  double* scr = c.ws.dbl("a1:scr", (size_t)std::max<long long>(P.scratch, 1));
  double* outs = c.ws.dbl("a1:out", (size_t)3 * ni);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  Adj1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q0 = q0; a.dq0 = dq0;
  a.J = outs; a.dgamma = outs + ni; a.dalpha = outs + 2 * ni;
  a.scr = scr;
  a.solver = o.solver; a.n_iter = o.n_iter; a.objective = objective; a.seg = seg;
  for (int k = 0; k < 4; ++k) a.prm[k] = prm ? prm[k] : 0.0;
  a.status = c.d_status;
  c.plan_seg = seg;
  c.plan_groups = 1;
  c.plan_group_size = ni;
  a.cs = cluster_size(c, P, o, q0);
  NP1_DISPATCH(P.np, launch_1d(c, a, ni,
                               [&](const Adj1DArgs& x, int n) { return launch_k1_adjoint<NPV>(x, n, c.stream); },
                               "k1_adjoint launch"));
  std::vector<double> h(3 * ni);
  int st = 0;
  cuda_check(cudaMemcpyAsync(h.data(), outs, sizeof(double) * 3 * ni, cudaMemcpyDeviceToHost, c.stream), "readback");
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
  for (int i = 0; i < ni; ++i) {
    J[i] = h[i];
    if (dgamma) dgamma[i] = h[ni + i];
    if (dalpha) dalpha[i] = h[2 * ni + i];
  }
}

long long adjoint1d_scratch_fields(const Inst1DDesc& d, int N, const Solve2DOpts& o, int seg) {
  return E1_FIELDS + adjoint1d_fields(o.solver, o.n_iter, N, d.n_steps, seg);
}

long long tangent1d_scratch_fields(const Inst1DDesc&, int) { return E1_FIELDS + T1_FIELDS; }

void tangent1d(Ctx& c, const Plan1D& P, double* q, double* s, double* sig, double* vs, const Solve2DOpts& o, int form,
               double s_gamma) {
  if (form != 1 && form != 2) throw Error(1, "Unknown elliptic_rhs (use :form1 or :form2)");
  double* scr = c.ws.dbl("t1:scr", (size_t)std::max<long long>(P.scratch, 1));
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  Tan1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q = q; a.s = s; a.sig = sig; a.vs = vs; a.scr = scr;
  a.solver = o.solver; a.n_iter = o.n_iter; a.form = form; a.s_gamma = s_gamma;
  a.status = c.d_status;
  a.cs = cluster_size(c, P, o, q);
  NP1_DISPATCH(P.np, launch_1d(c, a, (int)P.inst.size(),
                               [&](const Tan1DArgs& x, int n) { return launch_k1_tangent<NPV>(x, n, c.stream); },
                               "k1_tangent launch"));
  int st = 0;
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
}

long long pde1d_scratch_fields(const Inst1DDesc& d, int, int mode, int seg) {
  return E1_FIELDS + P1_SNAP + (mode == 0 ? pde1_snap_fields(d.n_steps, seg) : 0);
}

// Snapshot segment of the 1D continuous adjoint: every snapshot resident when
// the batch's scratch fits the budget, else sqrt(n)-step segments.
int pde1d_segment(const std::vector<Inst1DDesc>& insts, int np, size_t budget) {
  int nmax = 0;
  for (auto& d : insts) nmax = std::max(nmax, d.n_steps);
  if (nmax <= 1) return std::max(nmax, 1);
  auto bytes = [&](int seg) {
    long long t = 0;
    for (auto& d : insts) t += pde1d_scratch_fields(d, np * d.ne, 0, seg) * (long long)np * d.ne;
    return (size_t)t * sizeof(double);
  };
  if (bytes(nmax) <= budget) return nmax;
  const int s = (int)std::ceil(std::sqrt((double)nmax));
  if (bytes(s) > budget) throw Error(5, "device memory too small for the 1D continuous adjoint of this batch");
  return s;
}

void pde_adjoint1d(Ctx& c, const Plan1D& P, int mode, const double* q0, const double* ain, double* a0, double* pi,
                   double* snaps, const long long* snap_off_dev, const Solve2DOpts& o, int objective, const double* prm,
                   int seg) {
  double* scr = c.ws.dbl("p1:scr", (size_t)std::max<long long>(P.scratch, 1));
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  Pde1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q0 = q0; a.ain = ain; a.a0 = a0; a.pi = pi; a.snaps = snaps; a.snap_off = snap_off_dev;
  a.scr = scr;
  a.mode = mode; a.solver = o.solver; a.n_iter = o.n_iter; a.objective = objective; a.seg = std::max(seg, 1);
  for (int k = 0; k < 4; ++k) a.prm[k] = prm ? prm[k] : 0.0;
  a.status = c.d_status;
  c.plan_seg = seg;
  c.plan_groups = 1;
  c.plan_group_size = (int)P.inst.size();
  a.cs = cluster_size(c, P, o, mode <= 1 ? q0 : nullptr);
  NP1_DISPATCH(P.np, launch_1d(c, a, (int)P.inst.size(),
                               [&](const Pde1DArgs& x, int n) { return launch_k1_pde_adjoint<NPV>(x, n, c.stream); },
                               "k1_pde_adjoint launch"));
  int st = 0;
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
}

long long ops1d_scratch_fields(const Inst1DDesc&, int) { return E1_FIELDS + O1_FIELDS; }

int ops1d(Ctx& c, const Plan1D& P, int op, const Solve2DOpts& o, const double* q, const double* rho, const double* b,
          double* x, double* sig, double* out, double* diag, double tol, int maxiter, bool fixed) {
  const int ni = (int)P.inst.size();
  double* scr = c.ws.dbl("o1:scr", (size_t)std::max<long long>(P.scratch, 1));
  int* iters = static_cast<int*>(c.ws.get("o1:iters", sizeof(int) * ni));
  Ops1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q = q; a.rho = rho; a.b = b; a.x = x; a.sig = sig; a.out = out; a.diag = diag; a.iters = iters;
  a.scr = scr;
  a.op = op; a.solver = o.solver; a.n_iter = o.n_iter;
  a.tol = tol; a.maxiter = maxiter; a.fixed = fixed ? 1 : 0;
  a.status = c.d_status;
  a.cs = cluster_size(c, P, o, nullptr);
  NP1_DISPATCH(P.np, launch_1d(c, a, ni, [&](const Ops1DArgs& v, int n) { return launch_k1_ops<NPV>(v, n, c.stream); },
                               "k1_ops launch"));
  int it = 0;
  if (op == OP1_CG) cuda_check(cudaMemcpyAsync(&it, iters, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "iterations");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  return it;
}

}  // namespace igrgpu
