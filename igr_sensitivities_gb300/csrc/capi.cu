// extern "C" boundary (include/igr_gb300.h): argument checks, host<->device
// transfers and status codes around the engine.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/igr_gb300.h"
#include "igr_engine.h"

using namespace igrgpu;

struct igr_ctx {
  Ctx c;
};

namespace {

template <class F>
int guarded(igr_ctx* ctx, F&& f) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.err.clear();
  ctx->c.launches = 0;
  try {
    cuda_check(cudaSetDevice(ctx->c.device), "cudaSetDevice");
    f();
    return IGR_OK;
  } catch (const Error& e) {
    ctx->c.err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    ctx->c.err = "host allocation failed";
    return IGR_ENOMEM;
  } catch (const std::exception& e) {
    ctx->c.err = e.what();
    return IGR_ECUDA;
  }
}

void check_disc(const igr_disc2d* d) {
  if (!d || !d->xi || !d->w || !d->D) throw Error(IGR_EINVAL, "null discretisation");
  if (d->p < 1 || d->p > 4) throw Error(IGR_EINVAL, "polynomial degree p must be in 1..4");
  if (d->n_ex < 1 || d->n_ey < 1 || !(d->lx > 0) || !(d->ly > 0)) throw Error(IGR_EINVAL, "bad mesh");
}

void check_solver(int solver, int n_iter) {
  if (solver < 0 || solver > 2) throw Error(IGR_EINVAL, "Unknown solver (use :pcg, :jacobi, or :chebyshev)");
  if (n_iter < 1) throw Error(IGR_EINVAL, "n_iter must be >= 1");
}

long long nodes2d(const igr_disc2d* d) { return (long long)(d->p + 1) * (d->p + 1) * d->n_ex * d->n_ey; }

void h2d(Ctx& c, double* dst, const double* src, long long n) {
  if (!src) throw Error(IGR_EINVAL, "null array");
  cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, c.stream), "H2D");
}
void d2h(Ctx& c, double* dst, const double* src, long long n) {
  if (!dst) throw Error(IGR_EINVAL, "null array");
  cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream), "D2H");
}
void sync(Ctx& c) { cuda_check(cudaStreamSynchronize(c.stream), "stream sync"); }

// Batched arrays cross the boundary instance-major, [inst][var][N]; on the
// device every variable is one field over all instances, [var][inst * N].
// The reordering is one contiguous copy of the whole block (through a device
// staging buffer when the caller's array is in host memory) and a transpose
// kernel: pitched host copies are avoided, since the driver may touch a whole
// pitch past the last row of the caller's array.
__global__ void k_interleave(const double* __restrict__ src, double* __restrict__ dst, int nv, long long N, int n_inst,
                             int to_fields) {
  const long long tot = (long long)nv * N * n_inst;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < tot; k += (long long)gridDim.x * blockDim.x) {
    const long long m = k % N, bv = k / N;      // k indexes the instance-major block: (b, v, m)
    const int v = (int)(bv % nv), b = (int)(bv / nv);
    const long long f = ((long long)v * n_inst + b) * N + m;
    if (to_fields) dst[f] = src[k];
    else dst[k] = src[f];
  }
}

void interleave(Ctx& c, const double* src, double* dst, int nv, long long N, int n_inst, int to_fields) {
  const long long tot = (long long)nv * N * n_inst;
  LaunchScope ls(c, KID_OTHER);
  k_interleave<<<(int)std::min<long long>((tot + 255) / 256, 152LL * 16), 256, 0, c.stream>>>(src, dst, nv, N, n_inst, to_fields);
}

// instance-major block `src` (host, or device when src_dev) -> device fields at `fields`
void gather_block(Ctx& c, double* fields, const double* src, int nv, long long N, int n_inst, bool src_dev) {
  if (!src) throw Error(IGR_EINVAL, "null array");
  const double* s = src;
  if (!src_dev) {
    const long long tot = (long long)nv * N * n_inst;
    double* st = c.ws.dbl("capi:stage", (size_t)tot);
    cuda_check(cudaMemcpyAsync(st, src, tot * sizeof(double), cudaMemcpyHostToDevice, c.stream), "H2D block");
    s = st;
  }
  interleave(c, s, fields, nv, N, n_inst, 1);
}

// device fields -> instance-major block `dst` (host, or device when dst_dev)
void scatter_block(Ctx& c, double* dst, const double* fields, int nv, long long N, int n_inst, bool dst_dev) {
  if (!dst) throw Error(IGR_EINVAL, "null array");
  if (dst_dev) { interleave(c, fields, dst, nv, N, n_inst, 0); return; }
  const long long tot = (long long)nv * N * n_inst;
  double* st = c.ws.dbl("capi:stage", (size_t)tot);
  interleave(c, fields, st, nv, N, n_inst, 0);
  cuda_check(cudaMemcpyAsync(dst, st, tot * sizeof(double), cudaMemcpyDeviceToHost, c.stream), "D2H block");
}

Plan2D plan_single(Ctx& c, const igr_disc2d* d, double gamma, double alpha, double dt, const char* tag) {
  check_disc(d);
  BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
  Inst2DDesc I{d->n_ex, d->n_ey, d->lx, d->ly, gamma, alpha, dt};
  return make_plan2d(c, B, {I}, tag);
}

}  // namespace

extern "C" {

int igr_ctx_create(int device, igr_ctx** out) {
  if (!out) return IGR_EINVAL;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return IGR_ECUDA;
  std::unique_ptr<igr_ctx> ctx(new igr_ctx());
  ctx->c.device = device;
  if (cudaSetDevice(device) != cudaSuccess) return IGR_ECUDA;
  if (cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess) return IGR_ECUDA;
  if (cudaMalloc(&ctx->c.d_status, sizeof(int)) != cudaSuccess) return IGR_ECUDA;
  if (cudaMemset(ctx->c.d_status, 0, sizeof(int)) != cudaSuccess) return IGR_ECUDA;
  *out = ctx.release();
  return IGR_OK;
}

int igr_ctx_destroy(igr_ctx* ctx) {
  if (!ctx) return IGR_OK;
  cudaSetDevice(ctx->c.device);
  if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
  ctx->c.ws.release_all();
  if (ctx->c.d_status) cudaFree(ctx->c.d_status);
  if (ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
  delete ctx;
  return IGR_OK;
}

const char* igr_last_error(const igr_ctx* ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int igr_set_tape_budget(igr_ctx* ctx, size_t bytes) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.tape_budget = bytes;
  return IGR_OK;
}

int igr_set_cluster_size_1d(igr_ctx* ctx, int cs) {
  if (!ctx || cs < 0 || cs > 16 || (cs & (cs - 1)) != 0) return IGR_EINVAL;
  ctx->c.cluster1d = cs;
  return IGR_OK;
}

int igr_set_graphs(igr_ctx* ctx, int on) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.use_graphs = on != 0;
  return IGR_OK;
}

int igr_set_pcg_persistent(igr_ctx* ctx, int on) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.pcg_persistent = on != 0;
  return IGR_OK;
}

int igr_test_pcg_drop_tile(igr_ctx* ctx, int tile) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.pcg_drop_tile = tile;
  return IGR_OK;
}

int igr_set_autotune(igr_ctx* ctx, int on, const char* cache_path) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.err.clear();
  ctx->c.tune.on = on != 0;
  ctx->c.tune.path = cache_path ? cache_path : "";
  ctx->c.tune.load();  // a missing file is an empty cache
  try {
    ctx->c.tune.save();  // the path must be writable: fail here, not inside a solve
  } catch (const Error& e) {
    ctx->c.err = e.what();
    ctx->c.tune.path.clear();
    return e.code;
  }
  return IGR_OK;
}

int igr_autotune_count(const igr_ctx* ctx, int* n) {
  if (!ctx || !n) return IGR_EINVAL;
  *n = (int)ctx->c.tune.table.size();
  return IGR_OK;
}

int igr_last_cluster_size_1d(const igr_ctx* ctx, int* out) {
  if (!ctx || !out) return IGR_EINVAL;
  *out = ctx->c.last_cluster1d;
  return IGR_OK;
}

int igr_last_launch_count(const igr_ctx* ctx, long long* out) {
  if (!ctx || !out) return IGR_EINVAL;
  *out = ctx->c.launches;
  return IGR_OK;
}

int igr_profile_enable(igr_ctx* ctx, int on) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.prof.harvest();
  ctx->c.prof.on = on != 0;
  return IGR_OK;
}

int igr_profile_reset(igr_ctx* ctx) {
  if (!ctx) return IGR_EINVAL;
  ctx->c.prof.reset();
  return IGR_OK;
}

int igr_profile_read(igr_ctx* ctx, int kernel_family, double* total_ms, long long* launches) {
  if (!ctx || !total_ms || !launches || kernel_family < 0 || kernel_family >= KID_COUNT) return IGR_EINVAL;
  ctx->c.prof.harvest();
  *total_ms = ctx->c.prof.ms[kernel_family];
  *launches = ctx->c.prof.count[kernel_family];
  return IGR_OK;
}

int igr_profile_nodes(igr_ctx* ctx, int kernel_family, double* nodes) {
  if (!ctx || !nodes || kernel_family < 0 || kernel_family >= KID_COUNT) return IGR_EINVAL;
  ctx->c.prof.harvest();
  *nodes = ctx->c.prof.nodes[kernel_family];
  return IGR_OK;
}

int igr_last_adjoint_plan(const igr_ctx* ctx, int* groups, int* group_size, int* segment_steps, int* segments) {
  if (!ctx || !groups || !group_size || !segment_steps || !segments) return IGR_EINVAL;
  *groups = ctx->c.plan_groups;
  *group_size = ctx->c.plan_group_size;
  *segment_steps = ctx->c.plan_seg;
  *segments = ctx->c.plan_nseg;
  return IGR_OK;
}

int igr_last_checkpoint_schedule(const igr_ctx* ctx, int* tape_steps, int* snapshots, long long* step_evaluations) {
  if (!ctx || !tape_steps || !snapshots || !step_evaluations) return IGR_EINVAL;
  *tape_steps = ctx->c.plan_seg;
  *snapshots = ctx->c.plan_snapshots;
  *step_evaluations = ctx->c.plan_step_evals;
  return IGR_OK;
}

int igr_probe_fp64_peak(igr_ctx* ctx, double* tflops) {
  return guarded(ctx, [&] {
    if (!tflops) throw Error(IGR_EINVAL, "null output");
    *tflops = probe_fp64_tflops(ctx->c);
  });
}

int igr_probe_fp64_tensor_peak(igr_ctx* ctx, double* tflops) {
  return guarded(ctx, [&] {
    if (!tflops) throw Error(IGR_EINVAL, "null output");
    *tflops = probe_dmma_tflops(ctx->c);
  });
}

int igr2d_run_forward(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                      int n_iter, int solver, double* mux, double* muy, double* rho, double* E, double* sigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
    // forward.jl:48-49
    const int n_steps = (int)std::ceil(t_end / dt);
    const double dtr = t_end / n_steps;
    Plan2D P = plan_single(c, d, gamma, alpha, dtr, "fwd");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:q", 5 * N);
    double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* S = buf + 4 * N;
    const double* in[4] = {mux, muy, rho, E};
    for (int v = 0; v < 4; ++v) h2d(c, q[v], in[v], N);
    cuda_check(cudaMemsetAsync(S, 0, N * sizeof(double), c.stream), "zero Sigma");  // forward.jl:42
    Solve2DOpts o{n_iter, solver};
    forward2d(c, P, q, S, n_steps, o);
    if (alpha > 0) {  // forward.jl:71-73
      const double* qc[4] = {q[0], q[1], q[2], q[3]};
      solve_elliptic2d(c, P, qc, S, o);
    }
    double* out[4] = {mux, muy, rho, E};
    for (int v = 0; v < 4; ++v) d2h(c, out[v], q[v], N);
    d2h(c, sigma, S, N);
    sync(c);
  });
}

int igr2d_run_sensitivity(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                          int n_iter, int solver, double s_gamma, double* mux, double* muy, double* rho, double* E,
                          double* sigma, double* zetax, double* zetay, double* srho, double* eta, double* varsigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
    // sensitivity.jl:361-362 (same re-rounding as run_forward!)
    const int n_steps = (int)std::ceil(t_end / dt);
    const double dtr = t_end / n_steps;
    Plan2D P = plan_single(c, d, gamma, alpha, dtr, "sen");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:qs", 10 * N);
    double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* sv[4] = {buf + 4 * N, buf + 5 * N, buf + 6 * N, buf + 7 * N};
    double* S = buf + 8 * N;
    double* V = buf + 9 * N;
    double* qh[4] = {mux, muy, rho, E};
    double* sh[4] = {zetax, zetay, srho, eta};
    for (int v = 0; v < 4; ++v) { h2d(c, q[v], qh[v], N); h2d(c, sv[v], sh[v], N); }
    Solve2DOpts o{n_iter, solver};
    sensitivity2d(c, P, q, S, sv, V, n_steps, o, s_gamma);
    for (int v = 0; v < 4; ++v) { d2h(c, qh[v], q[v], N); d2h(c, sh[v], sv[v], N); }
    d2h(c, sigma, S, N);
    d2h(c, varsigma, V, N);
    sync(c);
  });
}

int igr2d_adjoint_batch_meshes(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                               const int* n_ex, const int* n_ey, const double* lx, const double* ly,
                               const double* gammas, const double* alphas, const double* dts, int n_steps, int n_iter,
                               int solver, int objective, const double* obj_params, const double* q0, double* J,
                               double* dq0, double* dgamma, double* dalpha) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    if (!xi || !w || !D || p < 1 || p > 4) throw Error(IGR_EINVAL, "bad basis");
    if (n_inst < 1 || !n_ex || !n_ey || !lx || !ly || !gammas || !alphas || !dts || !q0 || !J || !dq0 || n_steps < 0)
      throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(p, xi, w, D);
    const int np = p + 1;
    std::vector<long long> Ni(n_inst), off(n_inst + 1, 0);
    for (int i = 0; i < n_inst; ++i) {
      if (n_ex[i] < 1 || n_ey[i] < 1 || !(lx[i] > 0) || !(ly[i] > 0)) throw Error(IGR_EINVAL, "bad mesh");
      Ni[i] = (long long)np * np * n_ex[i] * n_ey[i];
      off[i + 1] = off[i] + 4 * Ni[i];
    }
    // groups: consecutive instances while their full tapes fit (an instance that
    // does not fit alone runs by itself with segment checkpointing)
    size_t budget = (size_t)-1;
    if (c.tape_budget == 0) {
      size_t fr = 0, tot = 0;
      cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
      const size_t avail = fr + c.ws.bytes();
      const size_t reserve = (size_t)4 << 30;
      budget = avail > reserve ? (size_t)((avail - reserve) * 0.92) : 0;
    }
    const Solve2DOpts o{n_iter, solver};
    std::vector<int> gstart{0};
    size_t used = 0;
    for (int i = 0; i < n_inst; ++i) {
      const size_t F = (size_t)stage_fields2d(o, alphas[i] > 0, Ni[i], 1);
      const size_t bytes = ((size_t)3 * F * std::max(n_steps, 1) + 6 + 110) * Ni[i] * sizeof(double);
      if (i > gstart.back() && used + bytes > budget) { gstart.push_back(i); used = 0; }
      used += bytes;
    }
    gstart.push_back(n_inst);
    c.plan_groups = (int)gstart.size() - 1;
    c.plan_group_size = 0;
    for (size_t gi = 0; gi + 1 < gstart.size(); ++gi) {
      const int g0 = gstart[gi], g1 = gstart[gi + 1];
      c.plan_group_size = std::max(c.plan_group_size, g1 - g0);
      std::vector<Inst2DDesc> insts;
      for (int b = g0; b < g1; ++b) insts.push_back(Inst2DDesc{n_ex[b], n_ey[b], lx[b], ly[b], gammas[b], alphas[b], dts[b]});
      Plan2D P = make_plan2d(c, B, insts, "adjm");
      const long long NG = P.NG;
      double* buf = c.ws.dbl("capi:bqm", 8 * (size_t)NG);
      double* q[4];
      double* dq[4];
      for (int v = 0; v < 4; ++v) { q[v] = buf + v * NG; dq[v] = buf + (4 + v) * NG; }
      for (int b = g0; b < g1; ++b)  // [var][N_b] of instance b -> its slice of each field
        for (int v = 0; v < 4; ++v) h2d(c, q[v] + P.inst[b - g0].off, q0 + off[b] + v * Ni[b], Ni[b]);
      const double* qc[4] = {q[0], q[1], q[2], q[3]};
      adjoint2d(c, P, qc, n_steps, o, objective, obj_params, J + g0, dq, dgamma ? dgamma + g0 : nullptr,
                dalpha ? dalpha + g0 : nullptr);
      for (int b = g0; b < g1; ++b)
        for (int v = 0; v < 4; ++v) d2h(c, dq0 + off[b] + v * Ni[b], dq[v] + P.inst[b - g0].off, Ni[b]);
      sync(c);
    }
  });
}

int igr2d_sensitivity_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                            const double* dts, int n_steps, int n_iter, int solver, double s_gamma, double* q,
                            double* s, double* sigma, double* varsigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc(d);
    check_solver(solver, n_iter);
    if (n_inst < 1 || !gammas || !alphas || !dts || !q || !s || !sigma || !varsigma || n_steps < 0)
      throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    const long long N = nodes2d(d);
    std::vector<Inst2DDesc> insts;
    for (int b = 0; b < n_inst; ++b) insts.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], alphas[b], dts[b]});
    Plan2D P = make_plan2d(c, B, insts, "senb");
    const long long NG = P.NG;
    double* buf = c.ws.dbl("capi:senb", 10 * (size_t)NG);
    double* qd[4];
    double* sd[4];
    for (int v = 0; v < 4; ++v) { qd[v] = buf + v * NG; sd[v] = buf + (4 + v) * NG; }
    double* S = buf + 8 * NG;
    double* V = buf + 9 * NG;
    gather_block(c, qd[0], q, 4, N, n_inst, false);
    gather_block(c, sd[0], s, 4, N, n_inst, false);
    Solve2DOpts o{n_iter, solver};
    sensitivity2d(c, P, qd, S, sd, V, n_steps, o, s_gamma);
    scatter_block(c, q, qd[0], 4, N, n_inst, false);
    sync(c);  // the staging buffer is reused by the next scatter
    scatter_block(c, s, sd[0], 4, N, n_inst, false);
    d2h(c, sigma, S, NG);
    d2h(c, varsigma, V, NG);
    sync(c);
  });
}

int igr2d_objective(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_steps, double dt,
                    int n_iter, int solver, int objective, const double* obj_params, double* mux, double* muy,
                    double* rho, double* E, double* J) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    Plan2D P = plan_single(c, d, gamma, alpha, dt, "obj");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:q", 5 * N);
    double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* io[4] = {mux, muy, rho, E};
    for (int v = 0; v < 4; ++v) h2d(c, q[v], io[v], N);
    Solve2DOpts o{n_iter, solver};
    objective2d(c, P, q, n_steps, o, objective, obj_params, J);
    for (int v = 0; v < 4; ++v) d2h(c, io[v], q[v], N);
    sync(c);
  });
}

// Instances per group of a batched 2D adjoint on one mesh of N nodes: as many
// as fit with a full tape (no recompute); a single instance that does not fit
// runs with a revolve checkpoint schedule. Without a budget: the free device
// memory less a reserve, with ~110 working fields per instance beside the tape;
// with one (igr_set_tape_budget): the full tapes and checkpoints of the group
// within the budget.
static int adjoint_group_size(Ctx& c, long long N, int n_inst, int n_steps, int n_iter, int solver, bool apos) {
  const size_t F = (size_t)stage_fields2d(Solve2DOpts{n_iter, solver}, apos, N, 1);
  const size_t tape_inst = ((size_t)3 * F * std::max(n_steps, 1) + 6) * N * sizeof(double);
  size_t fit = 0;
  if (c.tape_budget == 0) {
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    const size_t avail = fr + c.ws.bytes();  // workspace buffers are reused or regrown
    const size_t reserve = (size_t)4 << 30;
    const size_t per_inst = tape_inst + (size_t)110 * N * sizeof(double);
    fit = avail > reserve ? (size_t)((avail - reserve) * 0.92) / per_inst : 0;
  } else {
    fit = c.tape_budget / tape_inst;
  }
  return (int)std::max<size_t>(1, std::min<size_t>((size_t)n_inst, fit));
}

int igr2d_adjoint_plan(igr_ctx* ctx, const igr_disc2d* d, int n_inst, int n_steps, int n_iter, int solver, double alpha,
                       int* group_size, int* tape_steps, int* snapshots, long long* step_evaluations) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc(d);
    check_solver(solver, n_iter);
    if (n_inst < 1 || n_steps < 0 || !group_size || !tape_steps || !snapshots || !step_evaluations)
      throw Error(IGR_EINVAL, "bad arguments");
    const long long N = nodes2d(d);
    const int G = adjoint_group_size(c, N, n_inst, n_steps, n_iter, solver, alpha > 0);
    const long long NG = N * G;
    const int F = stage_fields2d(Solve2DOpts{n_iter, solver}, alpha > 0, NG, G);
    const RevolvePlan rp = adjoint_checkpoints2d(c, NG, F, n_steps);
    if (rp.w < 1) throw Error(IGR_ENOMEM, "device memory too small for one taped step and one checkpoint");
    *group_size = G;
    *tape_steps = rp.w;
    *snapshots = rp.slots;
    *step_evaluations = rp.evals;
  });
}

static void adjoint_batch_impl(Ctx& c, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                               const double* dts, int n_steps, int n_iter, int solver, int objective,
                               const double* obj_params, const double* q0, bool q0_dev, double* J, double* dq0,
                               bool dq0_dev, double* dgamma, double* dalpha) {
  check_disc(d);
  check_solver(solver, n_iter);
  if (n_inst < 1 || !gammas || !alphas || !dts || !J) throw Error(IGR_EINVAL, "bad batch arguments");
  BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
  const long long N = nodes2d(d);
  int G = adjoint_group_size(c, N, n_inst, n_steps, n_iter, solver, alphas[0] > 0);
  // balanced groups: sizes differ by at most one (workspace sized for the largest)
  const int ngroups = (n_inst + G - 1) / G;
  std::vector<int> gstart(ngroups + 1, 0);
  for (int g = 0; g < ngroups; ++g) gstart[g + 1] = gstart[g] + n_inst / ngroups + (g < n_inst % ngroups ? 1 : 0);
  G = gstart[1];
  c.plan_groups = ngroups;
  c.plan_group_size = G;
  for (int gi = 0; gi < ngroups; ++gi) {
    const int g0 = gstart[gi], gn = gstart[gi + 1] - gstart[gi];
    std::vector<Inst2DDesc> insts;
    for (int b = g0; b < g0 + gn; ++b) insts.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], alphas[b], dts[b]});
    Plan2D P = make_plan2d(c, B, insts, "adj");
    const long long NG = P.NG;
    double* buf = c.ws.dbl("capi:bq", 8 * (size_t)N * G);
    double* q[4];
    double* dq[4];
    for (int v = 0; v < 4; ++v) { q[v] = buf + v * NG; dq[v] = buf + (4 + v) * NG; }
    gather_block(c, q[0], q0 + (size_t)g0 * 4 * N, 4, N, gn, q0_dev);
    Solve2DOpts o{n_iter, solver};
    const double* qc[4] = {q[0], q[1], q[2], q[3]};
    adjoint2d(c, P, qc, n_steps, o, objective, obj_params, J + g0, dq, dgamma ? dgamma + g0 : nullptr,
              dalpha ? dalpha + g0 : nullptr);
    scatter_block(c, dq0 + (size_t)g0 * 4 * N, dq[0], 4, N, gn, dq0_dev);
    if (!dq0_dev) sync(c);  // the host copy has left the staging buffer before the next group reuses it
  }
  sync(c);
}

int igr2d_adjoint_ic(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_steps, double dt,
                     int n_iter, int solver, int objective, const double* obj_params, const double* mux0,
                     const double* muy0, const double* rho0, const double* E0, double* J, double* dmux0,
                     double* dmuy0, double* drho0, double* dE0, double* dgamma, double* dalpha) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc(d);
    const long long N = nodes2d(d);
    std::vector<double> q0(4 * N), dq0(4 * N);
    const double* in[4] = {mux0, muy0, rho0, E0};
    for (int v = 0; v < 4; ++v) {
      if (!in[v]) throw Error(IGR_EINVAL, "null array");
      std::memcpy(q0.data() + v * N, in[v], N * sizeof(double));
    }
    adjoint_batch_impl(c, d, 1, &gamma, &alpha, &dt, n_steps, n_iter, solver, objective, obj_params, q0.data(), false, J,
                       dq0.data(), false, dgamma, dalpha);
    double* out[4] = {dmux0, dmuy0, drho0, dE0};
    for (int v = 0; v < 4; ++v) {
      if (!out[v]) throw Error(IGR_EINVAL, "null array");
      std::memcpy(out[v], dq0.data() + v * N, N * sizeof(double));
    }
  });
}

int igr2d_adjoint_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                        const double* dts, int n_steps, int n_iter, int solver, int objective,
                        const double* obj_params, const double* q0, double* J, double* dq0, double* dgamma,
                        double* dalpha) {
  return guarded(ctx, [&] {
    if (!q0 || !dq0) throw Error(IGR_EINVAL, "null array");
    adjoint_batch_impl(ctx->c, d, n_inst, gammas, alphas, dts, n_steps, n_iter, solver, objective, obj_params, q0, false, J, dq0,
                       false, dgamma, dalpha);
  });
}

int igr2d_adjoint_batch_dev(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas,
                            const double* alphas, const double* dts, int n_steps, int n_iter, int solver,
                            int objective, const double* obj_params, const double* q0_dev, double* J,
                            double* dq0_dev, double* dgamma, double* dalpha) {
  return guarded(ctx, [&] {
    if (!q0_dev || !dq0_dev) throw Error(IGR_EINVAL, "null array");
    adjoint_batch_impl(ctx->c, d, n_inst, gammas, alphas, dts, n_steps, n_iter, solver, objective, obj_params, q0_dev, true, J,
                       dq0_dev, true, dgamma, dalpha);
  });
}

namespace {
// Device memory the continuous adjoint may use for snapshots: the budget set
// on the context, else free memory (plus what the snapshot buffers already
// hold) less a reserve.
size_t snapshot_budget(Ctx& c) {
  if (c.tape_budget) return c.tape_budget;
  size_t fr = 0, tot = 0;
  cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
  const size_t avail = fr + c.ws.held("capi:snaps");
  const size_t reserve = (size_t)2 << 30;
  return avail > reserve ? avail - reserve : 0;
}

int store_steps(double dt, double t_end) {
  if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
  return (int)std::ceil(t_end / dt);  // forward.jl:131-132
}
}  // namespace

int igr2d_run_forward_store(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                            int n_iter, int solver, const double* mux0, const double* muy0, const double* rho0,
                            const double* E0, double* snapshots, long long snapshots_len, int* n_steps) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    const int n = store_steps(dt, t_end);
    Plan2D P = plan_single(c, d, gamma, alpha, t_end / n, "fst");
    const long long N = P.NG;
    if (!snapshots || !n_steps || snapshots_len != (long long)(n + 1) * 5 * N)
      throw Error(IGR_EINVAL, "snapshots must hold (ceil(T/dt) + 1) * 5 * N doubles");
    const Solve2DOpts o{n_iter, solver};
    const double* in[4] = {mux0, muy0, rho0, E0};
    const size_t bytes = (size_t)(n + 1) * 5 * N * sizeof(double);
    if (bytes <= snapshot_budget(c)) {
      double* S = c.ws.dbl("capi:snaps", (size_t)(n + 1) * 5 * N);
      for (int v = 0; v < 4; ++v) h2d(c, S + v * N, in[v], N);
      const double* q0[4] = {S, S + N, S + 2 * N, S + 3 * N};
      forward_store_init2d(c, P, o, q0, S);
      forward_store_range2d(c, P, o, [&](int k) { return S + (long long)k * 5 * N; }, 0, n);
      d2h(c, snapshots, S, (long long)(n + 1) * 5 * N);
    } else {  // two device slots, each snapshot copied out after its step
      double* S = c.ws.dbl("capi:snaps", (size_t)2 * 5 * N);
      for (int v = 0; v < 4; ++v) h2d(c, S + v * N, in[v], N);
      const double* q0[4] = {S, S + N, S + 2 * N, S + 3 * N};
      forward_store_init2d(c, P, o, q0, S);
      auto ring = [&](int k) { return S + (long long)(k % 2) * 5 * N; };
      d2h(c, snapshots, S, 5 * N);
      for (int k = 0; k < n; ++k) {
        forward_store_range2d(c, P, o, ring, k, k + 1);
        d2h(c, snapshots + (long long)(k + 1) * 5 * N, ring(k + 1), 5 * N);
      }
    }
    sync(c);
    *n_steps = n;
  });
}

int igr2d_run_adjoint_conservative(igr_ctx* ctx, const igr_disc2d* d, const double* snapshots, long long snapshots_len,
                                   int n_steps, double dt, double t_end, double gamma, double alpha, int n_iter,
                                   int objective, int solver, const double* obj_params, double* amux, double* amuy,
                                   double* arho, double* aE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    if (objective < 0 || objective > IGR_OBJ_WINDOW_RHO2) throw Error(IGR_EINVAL, "Unknown objective");
    if (n_steps < 0) throw Error(IGR_EINVAL, "n_steps must be >= 0");
    if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
    Plan2D P = plan_single(c, d, gamma, alpha, std::min(dt, t_end), "pdea");  // adjoint_pde.jl:587
    const long long N = P.NG;
    if (!snapshots || snapshots_len < (long long)(n_steps + 1) * 5 * N)
      throw Error(IGR_EINVAL, "snapshots must hold (n_steps + 1) * 5 * N doubles");
    const Solve2DOpts o{n_iter, solver};
    double* out = c.ws.dbl("capi:aout", 4 * (size_t)N);
    double* ao[4] = {out, out + N, out + 2 * N, out + 3 * N};
    const size_t bytes = (size_t)(n_steps + 1) * 5 * N * sizeof(double);
    if (bytes <= snapshot_budget(c)) {
      double* S = c.ws.dbl("capi:snaps", (size_t)(n_steps + 1) * 5 * N);
      h2d(c, S, snapshots, (long long)(n_steps + 1) * 5 * N);
      pde_adjoint2d(c, P, n_steps, o, objective, obj_params, [&](int k) { return S + (long long)k * 5 * N; }, ao);
    } else {  // upload each snapshot just before its step (two device slots, stream-ordered)
      double* S = c.ws.dbl("capi:snaps", (size_t)2 * 5 * N);
      auto ring = [&](int k) {
        double* dst = S + (long long)(k % 2) * 5 * N;
        h2d(c, dst, snapshots + (long long)k * 5 * N, 5 * N);
        return dst;
      };
      pde_adjoint2d(c, P, n_steps, o, objective, obj_params, ring, ao);
    }
    double* outs[4] = {amux, amuy, arho, aE};
    for (int v = 0; v < 4; ++v) d2h(c, outs[v], ao[v], N);
    sync(c);
  });
}

int igr2d_adjoint_conservative_ic(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt,
                                  double t_end, int n_iter, int solver, int objective, const double* obj_params,
                                  const double* mux0, const double* muy0, const double* rho0, const double* E0,
                                  double* amux, double* amuy, double* arho, double* aE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    if (objective < 0 || objective > IGR_OBJ_WINDOW_RHO2) throw Error(IGR_EINVAL, "Unknown objective");
    const int n = store_steps(dt, t_end);
    Plan2D Pf = plan_single(c, d, gamma, alpha, t_end / n, "pdef");
    Plan2D Pa = plan_single(c, d, gamma, alpha, std::min(dt, t_end), "pdea");
    const long long N = Pf.NG;
    double* buf = c.ws.dbl("capi:pdeq", 8 * (size_t)N);
    double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* ao[4] = {buf + 4 * N, buf + 5 * N, buf + 6 * N, buf + 7 * N};
    const double* in[4] = {mux0, muy0, rho0, E0};
    for (int v = 0; v < 4; ++v) h2d(c, q[v], in[v], N);
    const double* qc[4] = {q[0], q[1], q[2], q[3]};
    const Solve2DOpts o{n_iter, solver};
    pde_adjoint_ic2d(c, Pf, Pa, qc, n, o, objective, obj_params, ao);
    double* outs[4] = {amux, amuy, arho, aE};
    for (int v = 0; v < 4; ++v) d2h(c, outs[v], ao[v], N);
    sync(c);
  });
}

int igr2d_adjoint_conservative_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas,
                                     const double* alphas, const double* dts, double t_end, int n_iter, int solver,
                                     int objective, const double* obj_params, const double* q0, double* a0) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc(d);
    check_solver(solver, n_iter);
    if (objective < 0 || objective > IGR_OBJ_WINDOW_RHO2) throw Error(IGR_EINVAL, "Unknown objective");
    if (n_inst < 1 || !gammas || !alphas || !dts || !q0 || !a0) throw Error(IGR_EINVAL, "bad batch arguments");
    const int n = store_steps(dts[0], t_end);
    for (int b = 1; b < n_inst; ++b)
      if (store_steps(dts[b], t_end) != n) throw Error(IGR_EINVAL, "ceil(T/dt) must be the same for every instance");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    std::vector<Inst2DDesc> fi, ai;
    for (int b = 0; b < n_inst; ++b) {
      fi.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], alphas[b], t_end / n});
      ai.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], alphas[b], std::min(dts[b], t_end)});
    }
    Plan2D Pf = make_plan2d(c, B, fi, "pdef");
    Plan2D Pa = make_plan2d(c, B, ai, "pdea");
    const long long N = nodes2d(d), NG = Pf.NG;
    double* buf = c.ws.dbl("capi:pdeq", 8 * (size_t)NG);
    double* q[4];
    double* ao[4];
    for (int v = 0; v < 4; ++v) { q[v] = buf + v * NG; ao[v] = buf + (4 + v) * NG; }
    gather_block(c, q[0], q0, 4, N, n_inst, false);
    const double* qc[4] = {q[0], q[1], q[2], q[3]};
    const Solve2DOpts o{n_iter, solver};
    pde_adjoint_ic2d(c, Pf, Pa, qc, n, o, objective, obj_params, ao);
    scatter_block(c, a0, ao[0], 4, N, n_inst, false);
    sync(c);
  });
}

int igr2d_adjoint_rhs_conservative(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_iter,
                                   int solver, const double* mux, const double* muy, const double* rho,
                                   const double* E, const double* sigma, double* pi, const double* amux,
                                   const double* amuy, const double* arho, const double* aE, double* damux,
                                   double* damuy, double* darho, double* daE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    Plan2D P = plan_single(c, d, gamma, alpha, 0.0, "pder");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:pder", 14 * (size_t)N);
    const double* qin[5] = {mux, muy, rho, E, sigma};
    for (int v = 0; v < 5; ++v) h2d(c, buf + v * N, qin[v], N);
    double* Pi = buf + 5 * N;
    if (alpha > 0) h2d(c, Pi, pi, N);
    const double* ain[4] = {amux, amuy, arho, aE};
    double* a[4];
    double* da[4];
    for (int v = 0; v < 4; ++v) { a[v] = buf + (6 + v) * N; da[v] = buf + (10 + v) * N; h2d(c, a[v], ain[v], N); }
    const double* ac[4] = {a[0], a[1], a[2], a[3]};
    const Solve2DOpts o{n_iter, solver};
    pde_adjoint_rhs2d(c, P, o, buf, Pi, ac, da);
    double* outs[4] = {damux, damuy, darho, daE};
    for (int v = 0; v < 4; ++v) d2h(c, outs[v], da[v], N);
    if (alpha > 0) d2h(c, pi, Pi, N);
    sync(c);
  });
}

int igr2d_apply_sip(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* x, const double* rho, double* y) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    Plan2D P = plan_single(c, d, 1.4, alpha, 0.0, "sip");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:sip", 3 * N);
    h2d(c, buf, x, N);
    h2d(c, buf + N, rho, N);
    apply_sip2d(c, P, buf, buf + N, buf + 2 * N);
    d2h(c, y, buf + 2 * N, N);
    sync(c);
  });
}

int igr2d_hyperbolic_rhs(igr_ctx* ctx, const igr_disc2d* d, double gamma, const double* mux, const double* muy,
                         const double* rho, const double* E, const double* sigma, double* dmux, double* dmuy,
                         double* drho, double* dE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    Plan2D P = plan_single(c, d, gamma, 0.0, 0.0, "rhs");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:rhs", 9 * N);
    const double* in[5] = {mux, muy, rho, E, sigma};
    for (int v = 0; v < 5; ++v) h2d(c, buf + v * N, in[v], N);
    const double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* k[4] = {buf + 5 * N, buf + 6 * N, buf + 7 * N, buf + 8 * N};
    hyperbolic_rhs2d(c, P, q, buf + 4 * N, k);
    double* out[4] = {dmux, dmuy, drho, dE};
    for (int v = 0; v < 4; ++v) d2h(c, out[v], k[v], N);
    sync(c);
  });
}

int igr2d_solve_elliptic(igr_ctx* ctx, const igr_disc2d* d, double alpha, int n_iter, int solver,
                         const double* mux, const double* muy, const double* rho, const double* E, double* sigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    Plan2D P = plan_single(c, d, 1.4, alpha, 0.0, "sol");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:sol", 5 * N);
    const double* in[4] = {mux, muy, rho, E};
    for (int v = 0; v < 4; ++v) h2d(c, buf + v * N, in[v], N);
    h2d(c, buf + 4 * N, sigma, N);
    const double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    Solve2DOpts o{n_iter, solver};
    solve_elliptic2d(c, P, q, buf + 4 * N, o, true);  // elliptic.jl:413-427 solves for any alpha
    d2h(c, sigma, buf + 4 * N, N);
    sync(c);
  });
}

int igr2d_igr_euler_rhs(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_iter, int solver,
                        const double* mux, const double* muy, const double* rho, const double* E, double* sigma,
                        double* dmux, double* dmuy, double* drho, double* dE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_solver(solver, n_iter);
    Plan2D P = plan_single(c, d, gamma, alpha, 0.0, "eul");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:eul", 9 * N);
    const double* in[4] = {mux, muy, rho, E};
    for (int v = 0; v < 4; ++v) h2d(c, buf + v * N, in[v], N);
    double* S = buf + 4 * N;
    if (alpha > 0) h2d(c, S, sigma, N);  // warm start; alpha <= 0 sets Sigma = 0 (forward.jl:26-27)
    const double* q[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* k[4] = {buf + 5 * N, buf + 6 * N, buf + 7 * N, buf + 8 * N};
    Solve2DOpts o{n_iter, solver};
    igr_euler_rhs2d(c, P, q, S, k, o);
    double* out[4] = {dmux, dmuy, drho, dE};
    for (int v = 0; v < 4; ++v) d2h(c, out[v], k[v], N);
    d2h(c, sigma, S, N);
    sync(c);
  });
}

int igr2d_igr_rhs(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* mux, const double* muy,
                  const double* rho, const double* E, double* b) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    (void)E;  // the reference's argument list; R(q) does not depend on E
    Plan2D P = plan_single(c, d, 1.4, alpha, 0.0, "igrb");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:igrb", 4 * N);
    const double* in[3] = {mux, muy, rho};
    for (int v = 0; v < 3; ++v) h2d(c, buf + v * N, in[v], N);
    const double* q[4] = {buf, buf + N, buf + 2 * N, nullptr};
    igr_rhs_diag2d(c, P, q, buf + 3 * N, nullptr);
    d2h(c, b, buf + 3 * N, N);
    sync(c);
  });
}

int igr2d_sip_diagonal(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, double* M) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    Plan2D P = plan_single(c, d, 1.4, alpha, 0.0, "sipd");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:sipd", 2 * N);
    h2d(c, buf, rho, N);
    const double* q[4] = {nullptr, nullptr, buf, nullptr};
    igr_rhs_diag2d(c, P, q, nullptr, buf + N);
    d2h(c, M, buf + N, N);
    sync(c);
  });
}

namespace {
int cg2d_call(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, const double* b, double* x,
              double tol, int maxiter, bool fixed, int* iters) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (maxiter < 0) throw Error(IGR_EINVAL, fixed ? "n_iter must be >= 0" : "maxiter must be >= 0");
    Plan2D P = plan_single(c, d, 1.4, alpha, 0.0, "cg");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:cg", 3 * N);
    h2d(c, buf, rho, N);
    h2d(c, buf + N, b, N);
    h2d(c, buf + 2 * N, x, N);
    const int it = cg2d(c, P, buf, buf + N, buf + 2 * N, tol, maxiter, fixed);
    d2h(c, x, buf + 2 * N, N);
    sync(c);
    if (iters) *iters = it;
  });
}
}  // namespace

int igr2d_cg_solve(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, const double* b, double* x,
                   double tol, int maxiter, int* iters) {
  return cg2d_call(ctx, d, alpha, rho, b, x, tol, maxiter, false, iters);
}

int igr2d_cg_fixed(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, const double* b, double* x,
                   int n_iter) {
  return cg2d_call(ctx, d, alpha, rho, b, x, 0.0, n_iter, true, nullptr);
}

}  // extern "C"

namespace {

void check_disc1(int p, const double* xi, const double* w, const double* D) {
  if (!xi || !w || !D) throw Error(IGR_EINVAL, "null basis arrays");
  if (p < 1 || p > 4) throw Error(IGR_EINVAL, "polynomial degree p must be in 1..4");
}

}  // namespace

extern "C" {

int igr1d_run_forward(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                      int n_iter, int solver, double* mu, double* rho, double* E, double* sigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    check_solver(solver, n_iter);
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
    const int n_steps = (int)std::ceil(t_end / dt);  // IGR_adjoints_1d/forward.jl:58-59
    const double dtr = t_end / n_steps;
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Plan1D P = make_plan1d(c, B, {Inst1DDesc{d->n_e, d->L, gamma, alpha, dtr, n_steps}}, forward1d_scratch_fields, "f1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:q", 4 * N);
    double* in[3] = {mu, rho, E};
    for (int v = 0; v < 3; ++v) h2d(c, buf + v * N, in[v], N);
    Solve2DOpts o{n_iter, solver};
    forward1d(c, P, buf, buf + 3 * N, o, true);
    for (int v = 0; v < 3; ++v) d2h(c, in[v], buf + v * N, N);
    d2h(c, sigma, buf + 3 * N, N);
    sync(c);
  });
}

namespace {
// One 1D operator evaluation on one instance through k1_ops. in: host fields
// copied to the device slots the operation reads (q = (mu, rho, E), x, rho,
// b, sigma); outputs copied back as the operation writes them.
struct Op1Io {
  const double *mu = nullptr, *rho = nullptr, *E = nullptr, *x = nullptr, *b = nullptr;
  double* sigma = nullptr;  // in/out when set
  const double* sigma_in = nullptr;  // read only
  double* out[3] = {nullptr, nullptr, nullptr};
  double* diag = nullptr;
  double* x_out = nullptr;
};
int op1d_call(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, int op, int n_iter, int solver,
              const Op1Io& io, double tol, int maxiter, bool fixed, int* iters, bool args_ok) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!args_ok) throw Error(IGR_EINVAL, "null array");
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    if (op == OP1_SOLVE || op == OP1_EULER_RHS) check_solver(solver, n_iter);
    if (op == OP1_CG && maxiter < 0) throw Error(IGR_EINVAL, fixed ? "n_iter must be >= 0" : "maxiter must be >= 0");
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Plan1D P = make_plan1d(c, B, {Inst1DDesc{d->n_e, d->L, gamma, alpha, 0.0, 0}}, ops1d_scratch_fields, "o1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:ops", 12 * N);
    double* q = buf;             // mu, rho, E
    double* xs = buf + 3 * N;    // x
    double* rs = buf + 4 * N;    // rho (operator)
    double* bs = buf + 5 * N;    // b
    double* ss = buf + 6 * N;    // Sigma
    double* os = buf + 7 * N;    // outputs (3 fields)
    double* ds = buf + 10 * N;   // diag(A)
    if (io.mu) h2d(c, q, io.mu, N);
    if (io.rho) { h2d(c, q + N, io.rho, N); h2d(c, rs, io.rho, N); }
    if (io.E) h2d(c, q + 2 * N, io.E, N);
    if (io.x) h2d(c, xs, io.x, N);
    if (io.b) h2d(c, bs, io.b, N);
    if (io.sigma) h2d(c, ss, io.sigma, N);
    if (io.sigma_in) h2d(c, ss, io.sigma_in, N);
    Solve2DOpts o{n_iter, solver};
    const int it = ops1d(c, P, op, o, q, rs, bs, xs, ss, os, io.diag ? ds : nullptr, tol, maxiter, fixed);
    for (int v = 0; v < 3; ++v)
      if (io.out[v]) d2h(c, io.out[v], os + v * N, N);
    if (io.diag) d2h(c, io.diag, ds, N);
    if (io.sigma) d2h(c, io.sigma, ss, N);
    if (io.x_out) d2h(c, io.x_out, xs, N);
    sync(c);
    if (iters) *iters = it;
  });
}
}  // namespace

int igr1d_apply_sip(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* x, const double* rho, double* y) {
  Op1Io io;
  io.x = x; io.rho = rho; io.out[0] = y;
  return op1d_call(ctx, d, 1.4, alpha, OP1_APPLY_SIP, 1, 0, io, 0.0, 0, false, nullptr, x && rho && y);
}

int igr1d_igr_rhs(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* mu, const double* rho, const double* E,
                  double* b) {
  (void)E;  // the reference's argument list; the source does not depend on E
  Op1Io io;
  io.mu = mu; io.rho = rho; io.out[0] = b;
  return op1d_call(ctx, d, 1.4, alpha, OP1_IGR_RHS, 1, 0, io, 0.0, 0, false, nullptr, mu && rho && b);
}

int igr1d_sip_diagonal(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, double* M) {
  Op1Io io;
  io.mu = rho; io.rho = rho; io.diag = M;  // the source formed on the way is discarded
  return op1d_call(ctx, d, 1.4, alpha, OP1_IGR_RHS, 1, 0, io, 0.0, 0, false, nullptr, rho && M);
}

int igr1d_solve_elliptic(igr_ctx* ctx, const igr_disc1d* d, double alpha, int n_iter, int solver, const double* mu,
                         const double* rho, const double* E, double* sigma) {
  Op1Io io;
  io.mu = mu; io.rho = rho; io.E = E; io.sigma = sigma;
  return op1d_call(ctx, d, 1.4, alpha, OP1_SOLVE, n_iter, solver, io, 0.0, 0, false, nullptr, mu && rho && E && sigma);
}

int igr1d_hyperbolic_rhs(igr_ctx* ctx, const igr_disc1d* d, double gamma, const double* mu, const double* rho,
                         const double* E, const double* sigma, double* dmu, double* drho, double* dE) {
  Op1Io io;
  io.mu = mu; io.rho = rho; io.E = E;
  io.out[0] = dmu; io.out[1] = drho; io.out[2] = dE;
  io.sigma_in = sigma;
  return op1d_call(ctx, d, gamma, 0.0, OP1_HYP_RHS, 1, 0, io, 0.0, 0, false, nullptr,
                   mu && rho && E && sigma && dmu && drho && dE);
}

int igr1d_igr_euler_rhs(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, int n_iter, int solver,
                        const double* mu, const double* rho, const double* E, double* sigma, double* dmu, double* drho,
                        double* dE) {
  Op1Io io;
  io.mu = mu; io.rho = rho; io.E = E; io.sigma = sigma;
  io.out[0] = dmu; io.out[1] = drho; io.out[2] = dE;
  return op1d_call(ctx, d, gamma, alpha, OP1_EULER_RHS, n_iter, solver, io, 0.0, 0, false, nullptr,
                   mu && rho && E && sigma && dmu && drho && dE);
}

int igr1d_cg_solve(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, const double* b, double* x,
                   double tol, int maxiter, int* iters) {
  Op1Io io;
  io.rho = rho; io.b = b; io.x = x; io.x_out = x;
  return op1d_call(ctx, d, 1.4, alpha, OP1_CG, 1, 0, io, tol, maxiter, false, iters, rho && b && x);
}

int igr1d_cg_fixed(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, const double* b, double* x,
                   int n_iter) {
  Op1Io io;
  io.rho = rho; io.b = b; io.x = x; io.x_out = x;
  return op1d_call(ctx, d, 1.4, alpha, OP1_CG, 1, 0, io, 0.0, n_iter, true, nullptr, rho && b && x);
}

int igr1d_forward_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                        const int* n_e, const double* L, const double* gammas, const double* alphas,
                        const double* dts, const int* n_steps, int n_iter, int solver, int final_solve, double* q,
                        double* sigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc1(p, xi, w, D);
    check_solver(solver, n_iter);
    if (n_inst < 1 || !n_e || !L || !gammas || !alphas || !dts || !n_steps || !q || !sigma)
      throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(p, xi, w, D);
    std::vector<Inst1DDesc> insts;
    for (int i = 0; i < n_inst; ++i) insts.push_back(Inst1DDesc{n_e[i], L[i], gammas[i], alphas[i], dts[i], n_steps[i]});
    Plan1D P = make_plan1d(c, B, insts, forward1d_scratch_fields, "f1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:qb", 4 * N);
    h2d(c, buf, q, 3 * N);
    Solve2DOpts o{n_iter, solver};
    forward1d(c, P, buf, buf + 3 * N, o, final_solve != 0);
    d2h(c, q, buf, 3 * N);
    d2h(c, sigma, buf + 3 * N, N);
    sync(c);
  });
}

int igr1d_adjoint_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                        const int* n_e, const double* L, const double* gammas, const double* alphas,
                        const double* dts, const int* n_steps, int n_iter, int solver, int objective,
                        const double* obj_params, const double* q0, double* J, double* dq0, double* dgamma,
                        double* dalpha) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc1(p, xi, w, D);
    check_solver(solver, n_iter);
    if (n_inst < 1 || !n_e || !L || !gammas || !alphas || !dts || !n_steps || !q0 || !J || !dq0)
      throw Error(IGR_EINVAL, "bad batch arguments");
    if (objective != 0 && objective != 1 && objective != 2 && objective != 4 && objective != 6)
      throw Error(IGR_EINVAL, "Unknown objective");
    if (objective == 6 && !obj_params) throw Error(IGR_EINVAL, "interval objective needs obj_params = {a, b}");
    BasisDev B = make_basis_dev(p, xi, w, D);
    std::vector<Inst1DDesc> insts;
    for (int i = 0; i < n_inst; ++i) insts.push_back(Inst1DDesc{n_e[i], L[i], gammas[i], alphas[i], dts[i], n_steps[i]});
    Solve2DOpts o{n_iter, solver};
    size_t budget = c.tape_budget;
    if (budget == 0) {
      size_t fr = 0, tot = 0;
      cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
      const size_t avail = fr + c.ws.held("a1:scr");
      budget = avail > ((size_t)2 << 30) ? avail - ((size_t)2 << 30) : 0;
    }
    const int seg = adjoint1d_segment(insts, p + 1, o, budget);
    Plan1D P = make_plan1d(c, B, insts,
                           [&](const Inst1DDesc& d, int N) { return adjoint1d_scratch_fields(d, N, o, seg); }, "a1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:adj", 6 * N);
    h2d(c, buf, q0, 3 * N);
    adjoint1d(c, P, buf, buf + 3 * N, o, objective, obj_params, seg, J, dgamma, dalpha);
    d2h(c, dq0, buf + 3 * N, 3 * N);
    sync(c);
  });
}

int igr1d_run_sensitivity(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                          int n_iter, int solver, int elliptic_rhs, double s_gamma, double* mu, double* rho, double* E,
                          double* sigma, double* smu, double* srho, double* sE, double* ssigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    check_solver(solver, n_iter);
    if (elliptic_rhs != 1 && elliptic_rhs != 2) throw Error(IGR_EINVAL, "Unknown elliptic_rhs (use :form1 or :form2)");
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    if (!(dt > 0) || !(t_end >= 0)) throw Error(IGR_EINVAL, "dt must be positive and T non-negative");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Inst1DDesc desc{d->n_e, d->L, gamma, alpha, dt, 0};
    desc.t_end = t_end;
    Plan1D P = make_plan1d(c, B, {desc}, tangent1d_scratch_fields, "t1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:tan", 8 * N);
    double* qh[3] = {mu, rho, E};
    double* sh[3] = {smu, srho, sE};
    for (int v = 0; v < 3; ++v) { h2d(c, buf + v * N, qh[v], N); h2d(c, buf + (3 + v) * N, sh[v], N); }
    Solve2DOpts o{n_iter, solver};
    tangent1d(c, P, buf, buf + 3 * N, buf + 6 * N, buf + 7 * N, o, elliptic_rhs, s_gamma);
    for (int v = 0; v < 3; ++v) { d2h(c, qh[v], buf + v * N, N); d2h(c, sh[v], buf + (3 + v) * N, N); }
    d2h(c, sigma, buf + 6 * N, N);
    d2h(c, ssigma, buf + 7 * N, N);
    sync(c);
  });
}

int igr1d_sensitivity_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                            const int* n_e, const double* L, const double* gammas, const double* alphas,
                            const double* dts, const double* t_ends, int n_iter, int solver, int elliptic_rhs,
                            const double* s_gammas, double* q, double* s, double* sigma, double* ssigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc1(p, xi, w, D);
    check_solver(solver, n_iter);
    if (n_inst < 1 || !n_e || !L || !gammas || !alphas || !dts || !t_ends || !q || !s || !sigma || !ssigma)
      throw Error(IGR_EINVAL, "bad batch arguments");
    if (s_gammas) {
      for (int i = 1; i < n_inst; ++i)
        if (s_gammas[i] != s_gammas[0]) throw Error(IGR_EINVAL, "s_gamma must be the same for every instance of a batch");
    }
    BasisDev B = make_basis_dev(p, xi, w, D);
    std::vector<Inst1DDesc> insts;
    for (int i = 0; i < n_inst; ++i) {
      Inst1DDesc dsc{n_e[i], L[i], gammas[i], alphas[i], dts[i], 0};
      dsc.t_end = t_ends[i];
      insts.push_back(dsc);
    }
    Plan1D P = make_plan1d(c, B, insts, tangent1d_scratch_fields, "t1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:tanb", 8 * N);
    h2d(c, buf, q, 3 * N);
    h2d(c, buf + 3 * N, s, 3 * N);
    Solve2DOpts o{n_iter, solver};
    tangent1d(c, P, buf, buf + 3 * N, buf + 6 * N, buf + 7 * N, o, elliptic_rhs, s_gammas ? s_gammas[0] : 0.0);
    d2h(c, q, buf, 3 * N);
    d2h(c, s, buf + 3 * N, 3 * N);
    d2h(c, sigma, buf + 6 * N, N);
    d2h(c, ssigma, buf + 7 * N, N);
    sync(c);
  });
}

// ---- 1D continuous adjoint ------------------------------------------------------------------
namespace {
size_t budget1(Ctx& c, const char* name) {
  if (c.tape_budget) return c.tape_budget;
  size_t fr = 0, tot = 0;
  cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
  const size_t avail = fr + c.ws.held(name);
  return avail > ((size_t)2 << 30) ? avail - ((size_t)2 << 30) : 0;
}
void check_obj1(int objective, const double* obj_params) {
  if (objective != 0 && objective != 1 && objective != 2 && objective != 4 && objective != 6)
    throw Error(IGR_EINVAL, "Unknown objective (use :l2_density, :l2_pressure, or :kinetic_energy)");
  if (objective == 6 && !obj_params) throw Error(IGR_EINVAL, "interval objective needs obj_params = {a, b}");
}
Inst1DDesc pde1_desc(int ne, double L, double gamma, double alpha, double dt, double t_end) {
  if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
  const int n = (int)std::ceil(t_end / dt);  // IGR_adjoints_1d/forward.jl:158-159
  Inst1DDesc d{ne, L, gamma, alpha, t_end / n, n};
  d.h = std::min(dt, t_end);                  // IGR_adjoints_1d/adjoint_pde.jl:531
  return d;
}
}  // namespace

int igr1d_run_forward_store(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                            int n_iter, int solver, const double* mu0, const double* rho0, const double* E0,
                            double* snapshots, long long snapshots_len, int* n_steps) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    check_solver(solver, n_iter);
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    const Inst1DDesc dsc = pde1_desc(d->n_e, d->L, gamma, alpha, dt, t_end);
    const long long N = (long long)(d->p + 1) * d->n_e, n = dsc.n_steps;
    if (!snapshots || !n_steps || snapshots_len != (n + 1) * 4 * N)
      throw Error(IGR_EINVAL, "snapshots must hold (ceil(T/dt) + 1) * 4 * N doubles");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Plan1D P = make_plan1d(c, B, {dsc}, [&](const Inst1DDesc& x, int NN) { return pde1d_scratch_fields(x, NN, 1, 1); }, "p1");
    double* q = c.ws.dbl("capi1:pq", 3 * N);
    const double* in[3] = {mu0, rho0, E0};
    for (int v = 0; v < 3; ++v) h2d(c, q + v * N, in[v], N);
    double* S = c.ws.dbl("capi1:psnap", (size_t)(n + 1) * 4 * N);
    long long* off = static_cast<long long*>(c.ws.get("capi1:psoff", sizeof(long long)));
    cuda_check(cudaMemsetAsync(off, 0, sizeof(long long), c.stream), "offset");
    Solve2DOpts o{n_iter, solver};
    pde_adjoint1d(c, P, 1, q, nullptr, nullptr, nullptr, S, off, o, 0, nullptr, 1);
    d2h(c, snapshots, S, (n + 1) * 4 * N);
    sync(c);
    *n_steps = (int)n;
  });
}

int igr1d_run_adjoint_conservative(igr_ctx* ctx, const igr_disc1d* d, const double* snapshots, long long snapshots_len,
                                   int n_steps, double dt, double t_end, double gamma, double alpha, int n_iter,
                                   int objective, int solver, const double* obj_params, double* amu, double* arho,
                                   double* aE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    check_solver(solver, n_iter);
    check_obj1(objective, obj_params);
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    if (n_steps < 0) throw Error(IGR_EINVAL, "n_steps must be >= 0");
    if (!(dt > 0) || !(t_end > 0)) throw Error(IGR_EINVAL, "dt and T must be positive");
    const long long N = (long long)(d->p + 1) * d->n_e;
    if (!snapshots || snapshots_len < (long long)(n_steps + 1) * 4 * N)
      throw Error(IGR_EINVAL, "snapshots must hold (n_steps + 1) * 4 * N doubles");
    Inst1DDesc dsc{d->n_e, d->L, gamma, alpha, t_end / std::max(n_steps, 1), n_steps};
    dsc.h = std::min(dt, t_end);  // adjoint_pde.jl:531
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Plan1D P = make_plan1d(c, B, {dsc}, [&](const Inst1DDesc& x, int NN) { return pde1d_scratch_fields(x, NN, 2, 1); }, "p1");
    double* S = c.ws.dbl("capi1:psnap", (size_t)(n_steps + 1) * 4 * N);
    h2d(c, S, snapshots, (long long)(n_steps + 1) * 4 * N);
    double* out = c.ws.dbl("capi1:pout", 3 * N);
    long long* off = static_cast<long long*>(c.ws.get("capi1:psoff", sizeof(long long)));
    cuda_check(cudaMemsetAsync(off, 0, sizeof(long long), c.stream), "offset");
    Solve2DOpts o{n_iter, solver};
    pde_adjoint1d(c, P, 2, nullptr, nullptr, out, nullptr, S, off, o, objective, obj_params, 1);
    double* outs[3] = {amu, arho, aE};
    for (int v = 0; v < 3; ++v) d2h(c, outs[v], out + v * N, N);
    sync(c);
  });
}

int igr1d_adjoint_rhs_conservative(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, int n_iter, int solver,
                                   const double* mu, const double* rho, const double* E, const double* sigma, double* pi,
                                   const double* amu, const double* arho, const double* aE, double* damu, double* darho,
                                   double* daE) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!d) throw Error(IGR_EINVAL, "null discretisation");
    check_disc1(d->p, d->xi, d->w, d->D);
    check_solver(solver, n_iter);
    if (d->n_e < 1 || !(d->L > 0)) throw Error(IGR_EINVAL, "bad mesh");
    Inst1DDesc dsc{d->n_e, d->L, gamma, alpha, 0.0, 0};
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    Plan1D P = make_plan1d(c, B, {dsc}, [&](const Inst1DDesc& x, int NN) { return pde1d_scratch_fields(x, NN, 3, 1); }, "p1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:prhs", 11 * N);
    const double* qin[4] = {mu, rho, E, sigma};
    for (int v = 0; v < 4; ++v) h2d(c, buf + v * N, qin[v], N);
    const double* ain[3] = {amu, arho, aE};
    for (int v = 0; v < 3; ++v) h2d(c, buf + (4 + v) * N, ain[v], N);
    double* Pi = buf + 7 * N;
    if (alpha > 0) h2d(c, Pi, pi, N);
    double* k = buf + 8 * N;
    Solve2DOpts o{n_iter, solver};
    pde_adjoint1d(c, P, 3, buf, buf + 4 * N, k, Pi, nullptr, nullptr, o, 0, nullptr, 1);
    double* outs[3] = {damu, darho, daE};
    for (int v = 0; v < 3; ++v) d2h(c, outs[v], k + v * N, N);
    if (alpha > 0) d2h(c, pi, Pi, N);
    sync(c);
  });
}

int igr1d_adjoint_conservative_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                                     const int* n_e, const double* L, const double* gammas, const double* alphas,
                                     const double* dts, const double* t_ends, int n_iter, int solver, int objective,
                                     const double* obj_params, const double* q0, double* a0) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc1(p, xi, w, D);
    check_solver(solver, n_iter);
    check_obj1(objective, obj_params);
    if (n_inst < 1 || !n_e || !L || !gammas || !alphas || !dts || !t_ends || !q0 || !a0)
      throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(p, xi, w, D);
    std::vector<Inst1DDesc> insts;
    for (int i = 0; i < n_inst; ++i) {
      if (n_e[i] < 1 || !(L[i] > 0)) throw Error(IGR_EINVAL, "bad mesh");
      insts.push_back(pde1_desc(n_e[i], L[i], gammas[i], alphas[i], dts[i], t_ends[i]));
    }
    Solve2DOpts o{n_iter, solver};
    const int seg = pde1d_segment(insts, p + 1, budget1(c, "p1:scr"));
    Plan1D P = make_plan1d(c, B, insts, [&](const Inst1DDesc& x, int NN) { return pde1d_scratch_fields(x, NN, 0, seg); },
                           "p1");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi1:pbatch", 6 * N);
    h2d(c, buf, q0, 3 * N);
    pde_adjoint1d(c, P, 0, buf, nullptr, buf + 3 * N, nullptr, nullptr, nullptr, o, objective, obj_params, seg);
    d2h(c, a0, buf + 3 * N, 3 * N);
    sync(c);
  });
}

// ---- initial conditions -------------------------------------------------------------------
namespace {
Plan2D ic_plan(Ctx& c, const igr_disc2d* d, int ic_type, int n_inst, const double* gammas, const double* amps,
               const double* params) {
  check_disc(d);
  if (ic_type < 0 || ic_type > 5) throw Error(IGR_EINVAL, "Unknown IC type");
  if (n_inst < 1 || !gammas || !amps) throw Error(IGR_EINVAL, "bad batch arguments");
  if (ic_type == 5 && !params) throw Error(IGR_EINVAL, "the multi-blast IC needs params");
  BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
  std::vector<Inst2DDesc> insts;
  for (int b = 0; b < n_inst; ++b) insts.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], 0.0, 0.0});
  return make_plan2d(c, B, insts, "ic");
}
}  // namespace

int igr2d_build_ic(igr_ctx* ctx, const igr_disc2d* d, int ic_type, int n_inst, const double* gammas, const double* amps,
                   const double* params, double* q) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!q) throw Error(IGR_EINVAL, "null output");
    Plan2D P = ic_plan(c, d, ic_type, n_inst, gammas, amps, params);
    const long long N = nodes2d(d), NG = P.NG;
    double* buf = c.ws.dbl("capi:ic", 4 * (size_t)NG);
    double* f[4] = {buf, buf + NG, buf + 2 * NG, buf + 3 * NG};
    build_ic2d(c, P, ic_type, amps, params, f);
    scatter_block(c, q, f[0], 4, N, n_inst, false);
    sync(c);
  });
}

int igr2d_build_ic_dev(igr_ctx* ctx, const igr_disc2d* d, int ic_type, int n_inst, const double* gammas,
                       const double* amps, const double* params, double* q_dev) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!q_dev) throw Error(IGR_EINVAL, "null output");
    Plan2D P = ic_plan(c, d, ic_type, n_inst, gammas, amps, params);
    const long long N = nodes2d(d), NG = P.NG;
    double* buf = c.ws.dbl("capi:ic", 4 * (size_t)NG);
    double* f[4] = {buf, buf + NG, buf + 2 * NG, buf + 3 * NG};
    build_ic2d(c, P, ic_type, amps, params, f);
    scatter_block(c, q_dev, f[0], 4, N, n_inst, true);
    sync(c);
  });
}

int igr2d_l2_error(igr_ctx* ctx, const igr_disc2d* d, const double* u, const double* u_ref, double* err) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    if (!err) throw Error(IGR_EINVAL, "null output");
    Plan2D P = plan_single(c, d, 1.4, 0.0, 0.0, "l2e");
    const long long N = P.NG;
    double* buf = c.ws.dbl("capi:l2e", 2 * (size_t)N);
    h2d(c, buf, u, N);
    h2d(c, buf + N, u_ref, N);
    *err = l2_error2d(c, P, buf, buf + N);
  });
}

int igr1d_build_ic(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst, const int* n_e,
                   const double* L, int ic_type, const double* gammas, const double* amps, double* q) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc1(p, xi, w, D);
    if (ic_type < 0 || ic_type > 4) throw Error(IGR_EINVAL, "Unknown IC type");
    if (n_inst < 1 || !n_e || !L || !gammas || !amps || !q) throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(p, xi, w, D);
    std::vector<Inst1DDesc> insts;
    for (int i = 0; i < n_inst; ++i) {
      if (n_e[i] < 1 || !(L[i] > 0)) throw Error(IGR_EINVAL, "bad mesh");
      insts.push_back(Inst1DDesc{n_e[i], L[i], gammas[i], 0.0, 0.0, 0});
    }
    Plan1D P = make_plan1d(c, B, insts, [](const Inst1DDesc&, int) { return 0LL; }, "ic1");
    double* buf = c.ws.dbl("capi1:ic", 3 * (size_t)P.NG);
    build_ic1d(c, P, ic_type, amps, buf);
    d2h(c, q, buf, 3 * P.NG);
    sync(c);
  });
}

int igr2d_forward_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                        const double* dts, int n_steps, int n_iter, int solver, int final_solve, double* q,
                        double* sigma) {
  return guarded(ctx, [&] {
    Ctx& c = ctx->c;
    check_disc(d);
    check_solver(solver, n_iter);
    if (n_inst < 1 || !gammas || !alphas || !dts || !q || !sigma || n_steps < 0) throw Error(IGR_EINVAL, "bad batch arguments");
    BasisDev B = make_basis_dev(d->p, d->xi, d->w, d->D);
    std::vector<Inst2DDesc> insts;
    for (int b = 0; b < n_inst; ++b) insts.push_back(Inst2DDesc{d->n_ex, d->n_ey, d->lx, d->ly, gammas[b], alphas[b], dts[b]});
    Plan2D P = make_plan2d(c, B, insts, "fwdb");
    const long long N = nodes2d(d), NG = P.NG;
    double* buf = c.ws.dbl("capi:fwdb", 5 * (size_t)NG);
    double* qd[4] = {buf, buf + NG, buf + 2 * NG, buf + 3 * NG};
    double* S = buf + 4 * NG;
    gather_block(c, qd[0], q, 4, N, n_inst, false);
    cuda_check(cudaMemsetAsync(S, 0, NG * sizeof(double), c.stream), "zero Sigma");  // forward.jl:42
    Solve2DOpts o{n_iter, solver};
    forward2d(c, P, qd, S, n_steps, o);
    if (final_solve) {  // forward.jl:71-73
      const double* qc[4] = {qd[0], qd[1], qd[2], qd[3]};
      solve_elliptic2d(c, P, qc, S, o);
    }
    scatter_block(c, q, qd[0], 4, N, n_inst, false);
    d2h(c, sigma, S, NG);
    sync(c);
  });
}

}  // extern "C"
