// 1D host engine: batch plans and drivers of the per-instance persistent
// kernels (igr1d_kernels.cuh).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "igr1d_kernels.cuh"
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

Plan1D make_plan1d(Ctx& c, const BasisDev& B, const std::vector<Inst1DDesc>& insts, int scratch_fields,
                   const std::string& tag) {
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
    P.inst.push_back(I);
    const long long n = (long long)P.np * d.ne;
    P.inst_nodes.push_back(n);
    off += n;
    soff += (long long)scratch_fields * n;
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

int forward1d_scratch_fields() { return F1_FIELDS; }

void forward1d(Ctx& c, const Plan1D& P, double* q, double* sig, const Solve2DOpts& o, bool final_solve) {
  double* scr = c.ws.dbl("f1:scr", (size_t)std::max<long long>(P.scratch, 1));
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  Fwd1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.order = P.d_order; a.B = P.B;
  a.q = q; a.sig = sig; a.scr = scr;
  a.solver = o.solver; a.n_iter = o.n_iter; a.final_solve = final_solve ? 1 : 0;
  a.status = c.d_status;
  {
    LaunchScope ls(c, KID_1D);
    NP1_DISPATCH(P.np, (k1_forward<NPV><<<(int)P.inst.size(), T1, 0, c.stream>>>(a)));
  }
  cuda_check(cudaGetLastError(), "k1_forward launch");
  int st = 0;
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
}

}  // namespace igrgpu
