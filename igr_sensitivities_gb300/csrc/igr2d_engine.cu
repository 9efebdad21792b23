// 2D host engine: plans, forward / adjoint drivers and the small pointwise and
// reduction kernels that do not depend on the polynomial degree.
#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>

#include "igr2d_kernels.cuh"
#include "igr2d_launch.h"
#include "igr2d_pcg_kernels.cuh"
#include "igr2d_pcg_persist.cuh"
#include "igr2d_pde_kernels.cuh"
#include "igr2d_rev_kernels.cuh"
#include "igr2d_sens_kernels.cuh"
#include "igr_engine.h"

namespace igrgpu {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(4, std::string(what) + ": " + cudaGetErrorString(e));
}

Workspace::~Workspace() { release_all(); }
void* Workspace::get(const std::string& name, size_t bytes) {
  if (bytes == 0) bytes = 8;
  Buf& b = bufs_[name];
  if (b.n < bytes) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    cuda_check(cudaMalloc(&b.p, bytes), ("cudaMalloc " + name).c_str());
    b.n = bytes;
  }
  return b.p;
}
void Workspace::release(const std::string& name) {
  auto it = bufs_.find(name);
  if (it == bufs_.end()) return;
  if (it->second.p) cudaFree(it->second.p);
  bufs_.erase(it);
}
void Workspace::release_all() {
  for (auto& kv : bufs_) if (kv.second.p) cudaFree(kv.second.p);
  bufs_.clear();
}
size_t Workspace::held(const std::string& name) const {
  auto it = bufs_.find(name);
  return it == bufs_.end() ? 0 : it->second.n;
}
size_t Workspace::bytes() const {
  size_t s = 0;
  for (auto& kv : bufs_) s += kv.second.n;
  return s;
}

cudaEvent_t Profiler::get() {
  if (next < pool.size()) return pool[next++];
  cudaEvent_t e;
  cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  pool.push_back(e);
  ++next;
  return e;
}
void Profiler::begin(cudaStream_t s, int kid, long long n) {
  Rec r{kid, n, get(), get()};
  cudaEventRecord(r.a, s);
  recs.push_back(r);
}
void Profiler::end(cudaStream_t s) { cudaEventRecord(recs.back().b, s); }
void Profiler::harvest() {
  for (auto& r : recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    ms[r.kid] += t;
    count[r.kid] += 1;
    nodes[r.kid] += (double)r.nodes;
  }
  recs.clear();
  next = 0;
}
void Profiler::reset() {
  harvest();
  for (int k = 0; k < KID_COUNT; ++k) { ms[k] = 0; count[k] = 0; nodes[k] = 0; }
}
Profiler::~Profiler() {
  for (auto e : pool) cudaEventDestroy(e);
}

BasisDev make_basis_dev(int p, const double* xi, const double* w, const double* D) {
  if (p < 1 || p > MAXNP - 1) throw Error(1, "polynomial degree p must be in 1..4");
  BasisDev B;
  std::memset(&B, 0, sizeof(B));
  B.np = p + 1;
  for (int i = 0; i < B.np; ++i) { B.w[i] = w[i]; B.xi[i] = xi[i]; }
  for (int i = 0; i < B.np; ++i)
    for (int k = 0; k < B.np; ++k) B.D[i][k] = D[i + (size_t)k * B.np];
  for (int i = 0; i < B.np; ++i)
    for (int k = 0; k < B.np; ++k) B.W2[i][k] = B.w[i] * (B.D[i][k] * B.D[i][k]);
  // chebyshev_fixed!, elliptic.jl:373-378
  const double table[4] = {1.5, 2.0, 2.1, 2.2};
  const double lmax = table[std::min(p, 4) - 1], lmin = 1.0;
  B.cheb_theta = (lmax + lmin) / 2;
  B.cheb_delta = (lmax - lmin) / 2;
  B.cheb_sigma = B.cheb_theta / std::max(B.cheb_delta, 1e-10);
  B.hw = -0.5 / B.w[0];
  B.iw0 = 1.0 / B.w[0];
  B.iwL = 1.0 / B.w[B.np - 1];
  return B;
}

// Chebyshev recurrence coefficients of iteration it = 1..n:
// d_it = a_it d_{it-1} + c_it M^-1 r_{it-1} (elliptic.jl:383-391).
static void cheb_coeffs(const BasisDev& B, int n, std::vector<double>& a, std::vector<double>& cc) {
  a.assign(n + 1, 0.0);
  cc.assign(n + 1, 0.0);
  double rc = 1 / B.cheb_sigma;
  for (int it = 1; it <= n; ++it) {
    if (it == 1) { a[it] = 0.0; cc[it] = 1.0 / B.cheb_theta; }
    else { const double rn = 1 / (2 * B.cheb_sigma - rc); a[it] = rn * rc; cc[it] = 2 * rn / B.cheb_delta; rc = rn; }
  }
}

static void tile_shape(int np, int* tx, int* ty) {
  switch (np) {
    case 2: tile_shape2d<2>(tx, ty); break;
    case 3: tile_shape2d<3>(tx, ty); break;
    case 4: tile_shape2d<4>(tx, ty); break;
    case 5: tile_shape2d<5>(tx, ty); break;
    default: throw Error(1, "unsupported polynomial degree");
  }
}

Plan2D make_plan2d(Ctx& c, const BasisDev& B, const std::vector<Inst2DDesc>& insts, const std::string& tag) {
  Plan2D P;
  P.B = B;
  P.np = B.np;
  int tx, ty;
  tile_shape(P.np, &tx, &ty);
  long long off = 0;
  for (size_t i = 0; i < insts.size(); ++i) {
    const Inst2DDesc& d = insts[i];
    if (d.nex < 1 || d.ney < 1) throw Error(1, "mesh must have at least one element per direction");
    Inst2D I;
    I.off = off;
    I.nex = d.nex; I.ney = d.ney;
    I.lx = d.lx; I.ly = d.ly;
    I.dx = d.lx / d.nex; I.dy = d.ly / d.ney;
    I.jx = I.dx / 2.0; I.jy = I.dy / 2.0;
    I.gamma = d.gamma; I.alpha = d.alpha; I.dt = d.dt;
    I.ijx = 1.0 / I.jx; I.ijy = 1.0 / I.jy; I.idx = 1.0 / I.dx; I.idy = 1.0 / I.dy;
    I.ialpha = d.alpha > 0 ? 1.0 / d.alpha : 0.0;
    I.tile0 = (int)P.tiles.size();
    for (int ey0 = 0; ey0 < d.ney; ey0 += ty)
      for (int ex0 = 0; ex0 < d.nex; ex0 += tx) P.tiles.push_back(Tile2D{(int)i, ex0, ey0, 0});
    I.ntiles = (int)P.tiles.size() - I.tile0;
    for (int g = 0; g < I.ntiles; g += TILE_GROUP)
      P.groups.push_back(TileGroup{(int)i, I.tile0 + g, std::min(TILE_GROUP, I.ntiles - g), 0});
    P.inst.push_back(I);
    const long long n = (long long)P.np * P.np * d.nex * d.ney;
    P.inst_nodes.push_back(n);
    off += n;
  }
  P.NG = off;
  c.cur_nodes = off;
  P.d_inst = static_cast<Inst2D*>(c.ws.get(tag + ":inst", sizeof(Inst2D) * P.inst.size()));
  P.d_tiles = static_cast<Tile2D*>(c.ws.get(tag + ":tiles", sizeof(Tile2D) * P.tiles.size()));
  cuda_check(cudaMemcpyAsync(P.d_inst, P.inst.data(), sizeof(Inst2D) * P.inst.size(), cudaMemcpyHostToDevice, c.stream), "upload inst");
  cuda_check(cudaMemcpyAsync(P.d_tiles, P.tiles.data(), sizeof(Tile2D) * P.tiles.size(), cudaMemcpyHostToDevice, c.stream), "upload tiles");
  P.d_groups = static_cast<TileGroup*>(c.ws.get(tag + ":groups", sizeof(TileGroup) * P.groups.size()));
  cuda_check(cudaMemcpyAsync(P.d_groups, P.groups.data(), sizeof(TileGroup) * P.groups.size(), cudaMemcpyHostToDevice,
                             c.stream), "upload tile groups");
  return P;
}

// ------------------------------------------------------------------------------------------
// Pointwise and reduction kernels (degree independent)
// ------------------------------------------------------------------------------------------
__global__ void k_recip(const double* __restrict__ x, double* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) y[i] = 1.0 / x[i];
}

// Per-node objective integrands (IGR_adjoints_2d/enzyme_adjoint.jl:72-229 and the nodal
// window extension). j1 = integrand, j2 = mass integrand (kinetic energy only).
struct ObjArgs2D {
  const Inst2D* inst; int ninst; BasisDev B;
  const double *q[4];
  int obj; double prm[4];
  double *j1, *j2;
  const double *s1, *s2;       // per-instance sums (gradient kernel)
  double *qb[4], *gb;          // gradient outputs: d/dq and per-node d/dgamma
  long long NG;
};


__global__ void k2_obj_nodes(ObjArgs2D a) {
  const double pi = 3.14159265358979323846;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.NG; n += (long long)gridDim.x * blockDim.x) {
    const Inst2D I = a.inst[find_inst(a.inst, a.ninst, n)];
    double c, x, y;
    node_coords2d(a.B, I, n - I.off, &c, &x, &y);
    const double mx = a.q[0][n], my = a.q[1][n], r = a.q[2][n], E = a.q[3][n];
    double v1 = 0.0, v2 = 0.0;
    switch (a.obj) {
      case OBJ_L2_DENSITY: v1 = c * (r * r); break;
      case OBJ_L2_PRESSURE: { const double P = (I.gamma - 1.0) * (E - (mx * mx + my * my) / (2.0 * r)); v1 = c * (P * P); break; }
      case OBJ_KINETIC_ENERGY: v1 = c * (mx * mx + my * my) / (2.0 * r); v2 = c * r; break;
      case OBJ_WINDOWED_KE: {
        const double wx = exp(-((x - 0.55) * (x - 0.55) + (y - 0.50) * (y - 0.50)) / (0.15 * 0.15));
        v1 = c * wx * (mx * mx + my * my) / (2.0 * r); break;
      }
      case OBJ_WEIGHTED_MOMENTUM: {
        const double Lx = I.lx, Ly = I.ly;
        v1 = c * mx * (sin(2 * pi * x / Lx) * sin(2 * pi * y / Ly)); break;
      }
      case OBJ_WINDOW_RHO2: {
        const bool in = x >= a.prm[0] && x <= a.prm[0] + a.prm[2] && y >= a.prm[1] && y <= a.prm[1] + a.prm[2];
        v1 = in ? c * (r * r) : 0.0; break;
      }
      default: break;
    }
    a.j1[n] = v1;
    if (a.j2) a.j2[n] = v2;
  }
}

__global__ void k2_obj_grad(ObjArgs2D a) {
  const double pi = 3.14159265358979323846;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.NG; n += (long long)gridDim.x * blockDim.x) {
    const int ii = find_inst(a.inst, a.ninst, n);
    const Inst2D I = a.inst[ii];
    double c, x, y;
    node_coords2d(a.B, I, n - I.off, &c, &x, &y);
    const double mx = a.q[0][n], my = a.q[1][n], r = a.q[2][n], E = a.q[3][n];
    double g0 = 0, g1 = 0, g2 = 0, g3 = 0, gg = 0;
    switch (a.obj) {
      case OBJ_L2_DENSITY: g2 = 2.0 * c * r; break;
      case OBJ_L2_PRESSURE: {
        const double K = (mx * mx + my * my) / (2.0 * r), P = (I.gamma - 1.0) * (E - K);
        const double Pb = 2.0 * c * P, Kb = -Pb * (I.gamma - 1.0);
        gg = Pb * (E - K); g3 = Pb * (I.gamma - 1.0); g0 = Kb * mx / r; g1 = Kb * my / r; g2 = -Kb * K / r; break;
      }
      case OBJ_KINETIC_ENERGY: {
        const double KE = a.s1[ii], Ms = a.s2[ii];
        const double KEb = 1.0 / Ms, Mb = -KE / (Ms * Ms);
        g0 = KEb * c * mx / r; g1 = KEb * c * my / r; g2 = -KEb * c * (mx * mx + my * my) / (2.0 * r * r) + Mb * c; break;
      }
      case OBJ_WINDOWED_KE: {
        const double wx = exp(-((x - 0.55) * (x - 0.55) + (y - 0.50) * (y - 0.50)) / (0.15 * 0.15));
        g0 = c * wx * mx / r; g1 = c * wx * my / r; g2 = -c * wx * (mx * mx + my * my) / (2.0 * r * r); break;
      }
      case OBJ_WEIGHTED_MOMENTUM: {
        const double Lx = I.lx, Ly = I.ly;
        g0 = c * (sin(2 * pi * x / Lx) * sin(2 * pi * y / Ly)); break;
      }
      case OBJ_WINDOW_RHO2: {
        const bool in = x >= a.prm[0] && x <= a.prm[0] + a.prm[2] && y >= a.prm[1] && y <= a.prm[1] + a.prm[2];
        g2 = in ? 2.0 * c * r : 0.0; break;
      }
      default: break;
    }
    a.qb[0][n] = g0; a.qb[1][n] = g1; a.qb[2][n] = g2; a.qb[3][n] = g3;
    if (a.gb) a.gb[n] = gg;   // per-node d/dgamma of the objective (l2_pressure)
  }
}

// Deterministic per-instance sum: one block per instance, fixed order.
__global__ void k_inst_sum(const double* __restrict__ f, const long long* __restrict__ off, const long long* __restrict__ cnt,
                           double* __restrict__ out) {
  __shared__ double s[256];
  const long long o = off[blockIdx.x], n = cnt[blockIdx.x];
  double acc = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += f[o + i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

__global__ void k_fill(double* p, double v, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) p[i] = v;
}

// ------------------------------------------------------------------------------------------
// Launch helpers
// ------------------------------------------------------------------------------------------
static int grid_for(long long n) { return (int)std::min<long long>((n + 255) / 256, 152LL * 16); }

#define NP_DISPATCH(np, CALL)                         \
  switch (np) {                                       \
    case 2: { constexpr int NPV = 2; CALL; } break;   \
    case 3: { constexpr int NPV = 3; CALL; } break;   \
    case 4: { constexpr int NPV = 4; CALL; } break;   \
    case 5: { constexpr int NPV = 5; CALL; } break;   \
    default: throw Error(1, "unsupported polynomial degree"); \
  }

void launch_recip(const double* x, double* y, long long n, cudaStream_t s) {
  k_recip<<<(int)std::min<long long>((n + 255) / 256, 152LL * 16), 256, 0, s>>>(x, y, n);
}

static void recip(Ctx& c, const double* x, double* y, long long n) {
  LaunchScope ls(c, KID_OTHER);
  k_recip<<<grid_for(n), 256, 0, c.stream>>>(x, y, n);
}

// Per-stage storage: tape slot or scratch.
struct StageBuf {
  double* q[4] = {nullptr, nullptr, nullptr, nullptr};
  double* invr = nullptr;
  double* Sout = nullptr;
  double *b = nullptr, *cm = nullptr, *ckx = nullptr, *cky = nullptr, *cinvM = nullptr, *cpx = nullptr, *cpy = nullptr, *cM = nullptr;
  double *wsx = nullptr, *wsy = nullptr;  // LLF wave speeds at face nodes
  // taped solver iterates (empty when untaped). Jacobi / Chebyshev: xk = x_k,
  // rk = r_k (k < n). PCG: x0t = x_0, rk = r_0..r_n, pk = p_k, apk = A p_k,
  // scal = per-instance rz_0..rz_n, pAp_0..pAp_{n-1}, alpha_0..alpha_{n-1},
  // beta_0..beta_{n-1} (pcg_scal_count).
  std::vector<double*> xk, rk;
  std::vector<double*> gxk, gyk;  // taped reference derivatives of the iterates (optional)
  std::vector<double*> pk, apk;
  double* x0t = nullptr;
  double* scal = nullptr;
};

constexpr int STAGE_FIXED_FIELDS = 16;  // q(4) invr Sout b cm ckx cky cinvM cpx cpy cM wsx wsy
// Taping the reference derivatives of the Jacobi / Chebyshev iterates saves
// two line contractions per reverse apply but adds two fields per iteration to
// the tape; on the 32 x 128^2 P3 Chebyshev-5 adjoint the smaller tape (more
// instances per group) measured faster (3.77 vs 3.59 gradients/s), so the
// reverse recomputes them.
constexpr bool TAPE_ITERATE_DERIVATIVES = false;

// Per-instance scalars of one PCG solve: rz (n + 1), pAp, alpha, beta (n each).
static long long pcg_scal_count(int n_iter, int ni) { return (long long)(4 * n_iter + 1) * ni; }

static int pcg_scal_fields(const Solve2DOpts& o, long long NG, int ni) {
  const long long need = pcg_scal_count(o.n_iter, ni);
  return (int)((need + NG - 1) / NG);
}

int stage_fields2d(const Solve2DOpts& o, bool alpha_pos, long long NG, int ni) {
  if (!alpha_pos) return STAGE_FIXED_FIELDS;
  if (o.solver == SOLVER_PCG) return STAGE_FIXED_FIELDS + 1 + (o.n_iter + 1) + 2 * o.n_iter + pcg_scal_fields(o, NG, ni);
  return STAGE_FIXED_FIELDS + (TAPE_ITERATE_DERIVATIVES ? 4 : 2) * o.n_iter;
}

static StageBuf stage_from(double* base, long long NG, const Solve2DOpts& o, bool alpha_pos, bool taped, int ni) {
  StageBuf s;
  int f = 0;
  auto nxt = [&]() { return base + (long long)(f++) * NG; };
  for (int v = 0; v < 4; ++v) s.q[v] = nxt();
  s.invr = nxt(); s.Sout = nxt(); s.b = nxt(); s.cm = nxt(); s.ckx = nxt(); s.cky = nxt();
  s.cinvM = nxt(); s.cpx = nxt(); s.cpy = nxt(); s.cM = nxt();
  s.wsx = nxt(); s.wsy = nxt();
  if (taped && alpha_pos) {
    if (o.solver == SOLVER_PCG) {
      s.x0t = nxt();
      for (int k = 0; k <= o.n_iter; ++k) s.rk.push_back(nxt());
      for (int k = 0; k < o.n_iter; ++k) s.pk.push_back(nxt());
      for (int k = 0; k < o.n_iter; ++k) s.apk.push_back(nxt());
      s.scal = base + (long long)f * NG;
      f += pcg_scal_fields(o, NG, ni);
    } else {
      for (int k = 0; k < o.n_iter; ++k) s.xk.push_back(nxt());
      for (int k = 0; k < o.n_iter; ++k) s.rk.push_back(nxt());
      if (TAPE_ITERATE_DERIVATIVES) {
        for (int k = 0; k < o.n_iter; ++k) s.gxk.push_back(nxt());
        for (int k = 0; k < o.n_iter; ++k) s.gyk.push_back(nxt());
      }
    }
  }
  return s;
}

static bool any_alpha_pos(const Plan2D& P) {
  for (auto& I : P.inst) if (I.alpha > 0) return true;
  return false;
}
static bool all_alpha_pos(const Plan2D& P) {
  for (auto& I : P.inst) if (!(I.alpha > 0)) return false;
  return true;
}

// The PCG inner products are completed inside their producing kernels
// (InstSum with counters) for grids of at most this many tiles, and by a
// separate k2_inst_sum launch above it: the fused form saves a launch per
// product but holds every block until its partial is fenced, which costs
// more once a kernel runs many waves (16 x 256^2 P3: 1.56 fused vs 1.63
// separate tangent + adjoint + FD sets/hour; one 128^2 PCG-60 forward solve:
// 3.72 vs 3.88 s). Both forms give the same bits.
constexpr int FUSED_SUM_MAX_TILES = 4096;

// Per-instance completion counters of the fused inner products, zeroed
// before each solve (the kernels leave them at 0).
static int* inst_counters(Ctx& c, const Plan2D& P) {
  int* cnt = static_cast<int*>(c.ws.get("pcg:cnt", sizeof(int) * P.inst.size()));
  cuda_check(cudaMemsetAsync(cnt, 0, sizeof(int) * P.inst.size(), c.stream), "zero instance counters");
  return cnt;
}

// Whether a solve on this plan completes its inner products inside the
// kernels. Without autotuning: grids of at most FUSED_SUM_MAX_TILES tiles.
// With it, the first solve of a new shape runs fused and the second
// separate, each timed with CUDA events (both give the same bits), and the
// faster is remembered. No trial runs while the stream is being captured.
struct SumChoice {
  bool fused = false, trial = false;
  std::string key;
};
static SumChoice sum_choice(Ctx& c, const Plan2D& P, bool allow_trial) {
  SumChoice ch;
  ch.fused = P.ntiles() <= FUSED_SUM_MAX_TILES;
  if (!c.tune.on) return ch;
  char key[96];
  std::snprintf(key, sizeof(key), "2d.pcg_sums np=%d tiles=%d inst=%d", P.np, P.ntiles(), (int)P.inst.size());
  int v = 0;
  if (c.tune.get(key, &v)) {
    ch.fused = v != 0;
    return ch;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cuda_check(cudaStreamIsCapturing(c.stream, &cap), "stream capture status");
  if (!allow_trial || cap != cudaStreamCaptureStatusNone) return ch;
  ch.trial = true;
  ch.key = key;
  ch.fused = c.tune.trial_ms.count(ch.key) == 0;
  return ch;
}

// Times one trial solve (CUDA events on the engine's stream).
struct TrialTimer {
  Ctx& c;
  cudaEvent_t a = nullptr, b = nullptr;
  explicit TrialTimer(Ctx& cc, bool on) : c(cc) {
    if (!on) return;
    cuda_check(cudaEventCreate(&a), "trial event");
    cuda_check(cudaEventCreate(&b), "trial event");
    cuda_check(cudaEventRecord(a, c.stream), "trial event record");
  }
  ~TrialTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  double stop() {
    float ms = 0.f;
    cuda_check(cudaEventRecord(b, c.stream), "trial event record");
    cuda_check(cudaEventSynchronize(b), "trial event sync");
    cuda_check(cudaEventElapsedTime(&ms, a, b), "trial event time");
    return ms;
  }
};

static void sum_trial_done(Ctx& c, const SumChoice& ch, double ms) {
  if (ch.fused) {
    c.tune.trial_ms[ch.key] = ms;
    return;
  }
  const double fused_ms = c.tune.trial_ms[ch.key];
  c.tune.trial_ms.erase(ch.key);
  c.tune.put(ch.key, fused_ms <= ms ? 1 : 0);
}

// InstSum in mode 0: out[inst] = sum, and with quot
// quot = (qnum or the sum) / ((qden or the sum) + eps), eps = 1e-30 (the
// fixed-count solvers' guard) unless given.
static InstSum inst_sum0(int* cnt, double* out, const double* qnum = nullptr, const double* qden = nullptr,
                         double* quot = nullptr, double eps = 1e-30) {
  InstSum s;
  std::memset(&s, 0, sizeof(s));
  s.cnt = cnt; s.out = out; s.qnum = qnum; s.qden = qden; s.quot = quot; s.mode = 0; s.eps = eps;
  return s;
}

// Completes an InstSum in a separate launch when its kernel did not (cnt null).
static void inst_sum_after(Ctx& c, const Plan2D& P, const double* partials, bool grouped, const InstSum& s) {
  if (s.cnt) return;
  LaunchScope ls(c, KID_OTHER);
  k2_inst_sum<<<(int)P.inst.size(), 64, 0, c.stream>>>(P.d_inst, partials, grouped ? 1 : 0, s);
}

// Fixed-count Jacobi-preconditioned CG (pcg_fixed!, elliptic.jl:329-347) on
// the stage's operator: x_0 = warm start, result in st.Sout. Per iteration
// one operator kernel (A p_k and p_k . A p_k, with p_k formed on load; its
// last block per instance forms pAp_k and alpha_k) and one pointwise kernel
// (x, r and r . M^-1 r; its last block forms rz_{k+1} and beta_k). With a
// tape slot, r_k, p_k, A p_k and the scalars are written straight into it.
// CTAs of the persistent PCG kernel that the device holds at once.
static int pcg_persist_capacity(Ctx& c, int np) {
  int per_sm = 0, sms = 0;
  NP_DISPATCH(np, per_sm = pcg_persist_blocks_per_sm<NPV>());
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device), "attr");
  return per_sm * sms;
}

// The untaped solve runs as one persistent launch (k2_pcg_persist, bitwise the
// two-kernel result) when the plan's tiles fit one wave of resident CTAs (one
// tile per CTA) and it has at most PCG_PERSIST_MAX_INST instances: there the
// two-kernel form pays two launches and two short kernels' latency per
// iteration. Larger plans keep the two-kernel form, whose waves of tiles
// hide those costs.
static bool pcg_persistent(Ctx& c, const Plan2D& P, bool taped, int n_iter) {
  if (taped || !c.pcg_persistent || (int)P.inst.size() > PCG_PERSIST_MAX_INST) return false;
  // one partial slot per tile and reduction: keep that under 64 MB (about 3,000 iterations at 1,216 tiles),
  // which also keeps the arrival counts ((2 n_iter + 1) x tiles) far below 2^31
  if ((2LL * n_iter + 1) * P.ntiles() * (long long)sizeof(double) > (64LL << 20)) return false;
  int max_tiles = 0;
  NP_DISPATCH(P.np, max_tiles = persist_max_inst_tiles<NPV>());
  for (const auto& I : P.inst)
    if (I.ntiles > max_tiles) return false;
  const int cap = pcg_persist_capacity(c, P.np);
  return cap >= 1 && P.ntiles() <= cap;
}

// Returns false, having launched nothing that matters (the slot fill only),
// when the device refuses the cooperative launch (too many CTAs to be
// resident at once, e.g. beside another process's work); the caller then
// runs the two-kernel form.
static bool pcg_solve_persistent(Ctx& c, const Plan2D& P, const Solve2DOpts& o, StageBuf& st, const double* b,
                                 const double* x0, double* xout, double* xa, double* xb, double* dbuf) {
  const int nb = P.ntiles(), n = o.n_iter, ni = (int)P.inst.size();
  PcgPersistArgs a;
  std::memset(&a, 0, sizeof(a));
  a.op.tiles = P.d_tiles; a.op.inst = P.d_inst; a.op.B = P.B;
  a.op.cm = st.cm; a.op.ckx = st.ckx; a.op.cky = st.cky; a.op.cpx = st.cpx; a.op.cpy = st.cpy; a.op.b = b;
  a.op.cinvM = st.cinvM;
  // partial slots of the 2n + 1 reductions, the scalar record and (published hand-off) the scalars' copies
  int max_inst_tiles = 0;
  for (const auto& I : P.inst) max_inst_tiles = std::max(max_inst_tiles, I.ntiles);
  a.counted = max_inst_tiles <= PCG_COUNTED_TILES ? 1 : 0;
  const long long npart = (2LL * n + 1) * nb, nscal = pcg_scal_count(n, ni);
  const long long stride = ((2LL * n + 1) * ni + 15) / 16 * 16;  // copies on separate 128-byte lines
  const long long nbc = a.counted ? 0 : PCG_BCAST * stride;
  double* slots = c.ws.dbl("pcgp:slots", (size_t)(npart + nbc + nscal));
  a.slots = slots;
  a.bcast = slots + npart;
  a.bcast_stride = stride;
  a.scal = slots + npart + nbc;
  a.cnt = static_cast<unsigned*>(c.ws.get("pcgp:cnt", sizeof(unsigned) * PCG_CNT_STRIDE * ni));
  a.ntiles = nb; a.ninst = ni; a.n_iter = n;
  a.x0 = x0; a.xout = xout; a.r = xa; a.p[0] = xb; a.p[1] = dbuf; a.ap = c.ws.dbl("pcg:ap", P.NG);
  a.eps = 1e-30;
  a.status = c.d_status;
  a.drop_tile = c.pcg_drop_tile;
  c.pcg_drop_tile = -1;  // one launch
  if (a.counted) {
    cuda_check(cudaMemsetAsync(a.cnt, 0, sizeof(unsigned) * PCG_CNT_STRIDE * ni, c.stream), "arrival counters");
  } else {
    LaunchScope ls(c, KID_OTHER);
    k2_pcg_persist_fill<<<grid_for(npart + nbc), 256, 0, c.stream>>>(slots, npart + nbc);
  }
  cuda_check(cudaGetLastError(), "persistent PCG slot fill");
  cudaError_t e = cudaSuccess;
  {
    LaunchScope ls(c, KID_APPLY);
    NP_DISPATCH(P.np, e = launch_k2_pcg_persist<NPV>(a, nb, c.stream));
  }
  if (e == cudaErrorCooperativeLaunchTooLarge) {
    (void)cudaGetLastError();  // clear it: nothing was launched
    --c.launches;
    return false;
  }
  cuda_check(e, "persistent PCG launch");
  return true;
}

static void pcg_solve(Ctx& c, const Plan2D& P, const Solve2DOpts& o, StageBuf& st, const double* b, const double* x0,
                      double* xout, bool taped, double* xa, double* xb, double* dbuf) {
  if (pcg_persistent(c, P, taped, o.n_iter) && pcg_solve_persistent(c, P, o, st, b, x0, xout, xa, xb, dbuf)) return;
  const int nb = P.ntiles(), n = o.n_iter, ni = (int)P.inst.size();
  const long long NG = P.NG;
  double* part = c.ws.dbl("red:part", nb);
  const SumChoice ch = sum_choice(c, P, true);
  int* cnt = ch.fused ? inst_counters(c, P) : nullptr;
  TrialTimer timer(c, ch.trial);
  double* scal = taped ? st.scal : c.ws.dbl("pcg:scal", (size_t)pcg_scal_count(n, ni));
  double* apbuf = taped ? nullptr : c.ws.dbl("pcg:ap", NG);
  auto RZ = [&](int k) { return scal + (long long)k * ni; };
  auto PAP = [&](int k) { return scal + (long long)(n + 1 + k) * ni; };
  auto AL = [&](int k) { return scal + (long long)(2 * n + 1 + k) * ni; };
  auto BT = [&](int k) { return scal + (long long)(3 * n + 1 + k) * ni; };
  auto R = [&](int k) { return taped ? st.rk[k] : xa; };
  auto PK = [&](int k) { return taped ? st.pk[k] : ((k % 2 == 0) ? xb : dbuf); };
  auto AP = [&](int k) { return taped ? st.apk[k] : apbuf; };
  ApplyArgs2D base;
  std::memset(&base, 0, sizeof(base));
  base.tiles = P.d_tiles; base.inst = P.d_inst; base.B = P.B;
  base.cm = st.cm; base.ckx = st.ckx; base.cky = st.cky; base.cpx = st.cpx; base.cpy = st.cpy; base.b = b; base.cinvM = st.cinvM;
  base.partials = part;
  {  // r_0 = b - A x_0, p_0 = M^-1 r_0, rz_0
    ApplyArgs2D a = base;
    a.x = x0;
    a.tape_x = taped ? st.x0t : nullptr;
    a.r_out = R(0); a.p_out = PK(0);
    a.isum = inst_sum0(cnt, RZ(0));
    {
      LaunchScope ls(c, KID_APPLY);
      NP_DISPATCH(P.np, launch_k2_apply<NPV>(EPI_PCG0, a, nb, c.stream));
    }
    inst_sum_after(c, P, part, false, a.isum);
  }
  for (int k = 0; k < n; ++k) {
    {
      ApplyArgs2D a = base;
      if (k == 0) {
        a.x = PK(0);
      } else {
        a.pcg_r = R(k); a.pcg_p = PK(k - 1); a.pcg_beta = BT(k - 1);
        a.p_out = PK(k);
      }
      a.ap_out = AP(k);
      a.isum = inst_sum0(cnt, PAP(k), RZ(k), nullptr, AL(k));  // alpha_k = rz_k / (pAp_k + eps)
      {
        LaunchScope ls(c, KID_APPLY);
        NP_DISPATCH(P.np, launch_k2_apply<NPV>(EPI_PCG, a, nb, c.stream));
      }
      inst_sum_after(c, P, part, false, a.isum);
    }
    PcgUpdateArgs u;
    u.tiles = P.d_tiles; u.groups = P.d_groups; u.inst = P.d_inst;
    u.x_in = k == 0 ? x0 : xout; u.x_out = xout;
    u.p = PK(k); u.ap = AP(k); u.r_in = R(k); u.r_out = R(k + 1); u.cinvM = st.cinvM;
    u.al = AL(k);
    u.partials = part;
    u.isum = inst_sum0(cnt, RZ(k + 1), nullptr, RZ(k), BT(k));  // beta_k = rz_{k+1} / (rz_k + eps)
    {
      LaunchScope ls(c, KID_OTHER);
      NP_DISPATCH(P.np, launch_k2_pcg_update<NPV>(u, P.ngroups(), c.stream));
    }
    inst_sum_after(c, P, part, false, u.isum);
  }
  if (ch.trial) sum_trial_done(c, ch, timer.stop());
}

// Operator coefficients, IGR source b and diag(A) of one stage (the setup
// part of solve_elliptic!, elliptic.jl:413-416).
// always: also for instances with alpha <= 0 (the stand-alone solve_elliptic!
// has no alpha test; the RK stages skip the solve there, forward.jl:24-28).
static void stage_setup(Ctx& c, const Plan2D& P, StageBuf& st, bool always = false) {
  SetupArgs2D sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.tiles = P.d_tiles; sa.inst = P.d_inst; sa.B = P.B;
  sa.mx = st.q[0]; sa.my = st.q[1]; sa.invr = st.invr;
  sa.b = st.b; sa.cm = st.cm; sa.ckx = st.ckx; sa.cky = st.cky; sa.cinvM = st.cinvM; sa.cpx = st.cpx; sa.cpy = st.cpy; sa.cM = st.cM;
  sa.always = always ? 1 : 0;
  LaunchScope ls(c, KID_SETUP);
  NP_DISPATCH(P.np, launch_k2_setup<NPV>(sa, P.ntiles(), c.stream));
}

// Fixed-count solve A x = b on the stage's operator (set up by stage_setup):
// x0 = warm start (read only), result in xout (!= x0). taped: record the
// iterates into the stage's tape slots. xa/xb/dbuf: scratch.
static void stage_solve_b(Ctx& c, const Plan2D& P, const Solve2DOpts& o, StageBuf& st, const double* b, const double* x0,
                          double* xout, bool taped, double* xa, double* xb, double* dbuf) {
  if (o.solver == SOLVER_PCG) {
    pcg_solve(c, P, o, st, b, x0, xout, taped, xa, xb, dbuf);
    return;
  }
  const int nb = P.ntiles();
  const int epi = o.solver == SOLVER_CHEBYSHEV ? EPI_CHEB : EPI_JACOBI;
  std::vector<double> ca, cc;
  cheb_coeffs(P.B, o.n_iter, ca, cc);
  const double* x = x0;
  for (int k = 0; k < o.n_iter; ++k) {
    ApplyArgs2D a;
    std::memset(&a, 0, sizeof(a));
    a.tiles = P.d_tiles; a.inst = P.d_inst; a.B = P.B;
    a.x = x;
    a.cm = st.cm; a.ckx = st.ckx; a.cky = st.cky; a.cpx = st.cpx; a.cpy = st.cpy; a.b = b; a.cinvM = st.cinvM;
    a.d_in = k == 0 ? nullptr : dbuf;
    a.d_out = dbuf;
    double* xo = (k == o.n_iter - 1) ? xout : ((k % 2 == 0) ? xa : xb);
    a.x_out = xo;
    if (taped) {
      a.tape_x = st.xk.empty() ? nullptr : st.xk[k];
      a.tape_r = st.rk.empty() ? nullptr : st.rk[k];
      a.tape_gx = st.gxk.empty() ? nullptr : st.gxk[k];
      a.tape_gy = st.gyk.empty() ? nullptr : st.gyk[k];
    }
    a.ca = ca[k + 1]; a.cc = cc[k + 1];
    a.omega = 2.0 / 3.0;
    { LaunchScope ls(c, KID_APPLY); NP_DISPATCH(P.np, launch_k2_apply<NPV>(epi, a, nb, c.stream)); }
    x = xo;
  }
}

// Setup + fixed-count solve of one stage: x0 = warm start, result in st.Sout
// (taped when the stage buffer carries tape slots).
static void stage_solve(Ctx& c, const Plan2D& P, const Solve2DOpts& o, StageBuf& st, const double* x0, double* xa,
                        double* xb, double* dbuf) {
  stage_setup(c, P, st);
  const bool taped = st.x0t != nullptr || !st.xk.empty();
  stage_solve_b(c, P, o, st, st.b, x0, st.Sout, taped, xa, xb, dbuf);
}

// One SSP-RK3 step: stage inputs st[0..2] (st[0].q holds q^n), warm start
// Sin, output state into (qout, invrout) (may alias st[0].q: pointwise).
// SSP-RK3 stage coefficients (forward.jl:53-68): q_out = c0 q^n + c1 q_s + c2 dt k(q_s)
static const double RK_C0[3] = {0.0, 3.0 / 4, 1.0 / 3}, RK_C1[3] = {1.0, 1.0 / 4, 2.0 / 3}, RK_C2[3] = {1.0, 1.0 / 4, 2.0 / 3};

// Hyperbolic RHS + RK combination of stage s (inputs st[s], step start st[0]).
static void hyp_stage(Ctx& c, const Plan2D& P, StageBuf st[3], int s, double* const qout[4], double* invrout) {
  HypArgs2D h;
  std::memset(&h, 0, sizeof(h));
  h.tiles = P.d_tiles; h.inst = P.d_inst; h.B = P.B;
  for (int v = 0; v < 4; ++v) { h.q[v] = st[s].q[v]; h.qn[v] = st[0].q[v]; }
  h.invr = st[s].invr;
  h.S = st[s].Sout;
  h.c0 = RK_C0[s]; h.c1 = RK_C1[s]; h.c2 = RK_C2[s];
  for (int v = 0; v < 4; ++v) h.qo[v] = s < 2 ? st[s + 1].q[v] : qout[v];
  h.invro = s < 2 ? st[s + 1].invr : invrout;
  h.ws_x = st[s].wsx; h.ws_y = st[s].wsy;
  h.status = c.d_status;
  LaunchScope ls(c, KID_HYP);
  NP_DISPATCH(P.np, launch_k2_hyp_rk<NPV>(h, P.ntiles(), c.stream));
}

// setup0 = false: st[0] already holds the operator coefficients and IGR
// source of its state (the caller just solved on it).
static void step_forward(Ctx& c, const Plan2D& P, const Solve2DOpts& o, StageBuf st[3], const double* Sin, double* const qout[4],
                         double* invrout, double* xa, double* xb, double* dbuf, bool setup0 = true) {
  const bool apos = any_alpha_pos(P);
  const double* sprev = Sin;
  for (int s = 0; s < 3; ++s) {
    if (apos && s == 0 && !setup0) stage_solve_b(c, P, o, st[0], st[0].b, sprev, st[0].Sout, false, xa, xb, dbuf);
    else if (apos) stage_solve(c, P, o, st[s], sprev, xa, xb, dbuf);
    hyp_stage(c, P, st, s, qout, invrout);
    sprev = st[s].Sout;
  }
}

static void check_status(Ctx& c) {
  int st = 0;
  cuda_check(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.stream), "status readback");
  cuda_check(cudaStreamSynchronize(c.stream), "stream sync");
  if (st & DEV_TIMEOUT) throw Error(6, "a hand-off wait of the persistent PCG solve gave up (a CTA stopped early)");
  if (st & DEV_NONFINITE) throw Error(3, "non-finite value or non-positive density in the state");
}

static void check_alpha_uniform(const Plan2D& P) {
  if (any_alpha_pos(P) && !all_alpha_pos(P)) throw Error(1, "a batch must have alpha > 0 for all instances or for none");
}

// A piece of stream work replayed as a CUDA graph: captured on its first
// run, launched as one graph afterwards. The work must use the same buffers
// and launch arguments every time and allocate nothing (run it once eagerly
// first so that the workspace holds every buffer it names).
struct StreamGraph {
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;  // kernel launches per replay
  StreamGraph() = default;
  StreamGraph(const StreamGraph&) = delete;
  StreamGraph& operator=(const StreamGraph&) = delete;
  ~StreamGraph() { if (exec) cudaGraphExecDestroy(exec); }
  template <class F>
  void run(Ctx& c, F&& work) {
    if (!exec) {
      cuda_check(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal), "begin graph capture");
      const long long l0 = c.launches;
      cudaGraph_t g = nullptr;
      try {
        work();
      } catch (...) {
        cudaStreamEndCapture(c.stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      launches = c.launches - l0;
      c.launches = l0;
      cuda_check(cudaStreamEndCapture(c.stream, &g), "end graph capture");
      const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      cuda_check(e, "graph instantiate");
    }
    cuda_check(cudaGraphLaunch(exec, c.stream), "graph launch");
    c.launches += launches;
  }
};

void forward2d(Ctx& c, const Plan2D& P, double* const q[4], double* Sig, int n_steps, const Solve2DOpts& o) {
  check_alpha_uniform(P);
  const long long NG = P.NG;
  const bool apos = any_alpha_pos(P);
  double* scratch = c.ws.dbl("fwd:stages", (size_t)NG * 3 * STAGE_FIXED_FIELDS);
  StageBuf st[3];
  for (int s = 0; s < 3; ++s) st[s] = stage_from(scratch + (long long)s * STAGE_FIXED_FIELDS * NG, NG, o, apos, false, (int)P.inst.size());
  double* xa = c.ws.dbl("fwd:xa", NG);
  double* xb = c.ws.dbl("fwd:xb", NG);
  double* db = c.ws.dbl("fwd:d", NG);
  for (int v = 0; v < 4; ++v) st[0].q[v] = q[v];
  recip(c, q[2], st[0].invr, NG);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  if (!apos) cuda_check(cudaMemsetAsync(Sig, 0, NG * sizeof(double), c.stream), "zero Sigma");
  // Sigma ping-pong: the stage-3 output of step s is the warm start of step
  // s+1, copied back to Sig, so every step runs the same launches on the same
  // buffers. From the second step on the step is replayed as a CUDA graph
  // (one graph launch instead of 3 (2 n_iter + 3) kernel launches for PCG):
  // the single-instance solves are bound by launch gaps, not by the kernels.
  for (int k = 0; k < 3; ++k) st[k].Sout = !apos ? Sig : ((k % 2 == 0) ? c.ws.dbl("fwd:sA", NG) : c.ws.dbl("fwd:sB", NG));
  auto step = [&]() {
    step_forward(c, P, o, st, Sig, q, st[0].invr, xa, xb, db);
    if (apos) cuda_check(cudaMemcpyAsync(Sig, st[2].Sout, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "Sigma copy");
  };
  StreamGraph graph;
  const bool use_graph = c.use_graphs && !c.prof.on;
  for (int s = 0; s < n_steps; ++s) {
    if (use_graph && s > 0) graph.run(c, step);
    else step();
  }
  check_status(c);
}

// ------------------------------------------------------------------------------------------
// Tangent (run_sensitivity, sensitivity.jl:353-413)
// ------------------------------------------------------------------------------------------
static void sens_rhs(Ctx& c, const Plan2D& P, const StageBuf& st, double* const s[4], double* b) {
  SensRhsArgs2D a;
  std::memset(&a, 0, sizeof(a));
  a.tiles = P.d_tiles; a.inst = P.d_inst; a.B = P.B;
  for (int v = 0; v < 3; ++v) { a.q[v] = st.q[v]; a.s[v] = s[v]; }
  a.invr = st.invr; a.S = st.Sout;
  a.b_out = b;
  LaunchScope ls(c, KID_TAN);
  NP_DISPATCH(P.np, launch_k2_sens_rhs<NPV>(a, P.ntiles(), c.stream));
}

void sensitivity2d(Ctx& c, const Plan2D& P, double* const q[4], double* Sig, double* const s[4], double* vs, int n_steps,
                   const Solve2DOpts& o, double s_gamma) {
  check_alpha_uniform(P);
  const long long NG = P.NG;
  const bool apos = any_alpha_pos(P);
  const int ni = (int)P.inst.size();
  double* scratch = c.ws.dbl("sen:stages", (size_t)NG * 3 * STAGE_FIXED_FIELDS);
  StageBuf st[3];
  for (int k = 0; k < 3; ++k) st[k] = stage_from(scratch + (long long)k * STAGE_FIXED_FIELDS * NG, NG, o, apos, false, ni);
  double* tsb = c.ws.dbl("sen:tan", (size_t)NG * 8);
  double* ts[3][4];
  for (int v = 0; v < 4; ++v) { ts[0][v] = s[v]; ts[1][v] = tsb + v * NG; ts[2][v] = tsb + (4 + v) * NG; }
  double* bs = c.ws.dbl("sen:bs", NG);
  double* xa = c.ws.dbl("sen:xa", NG);
  double* xb = c.ws.dbl("sen:xb", NG);
  double* db = c.ws.dbl("sen:d", NG);
  double* sigAlt = c.ws.dbl("sen:sig", NG);
  double* vsAlt = c.ws.dbl("sen:vs", NG);
  for (int v = 0; v < 4; ++v) st[0].q[v] = q[v];
  recip(c, q[2], st[0].invr, NG);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  cuda_check(cudaMemsetAsync(Sig, 0, NG * sizeof(double), c.stream), "zero Sigma");      // sensitivity.jl:364
  cuda_check(cudaMemsetAsync(vs, 0, NG * sizeof(double), c.stream), "zero varsigma");
  // Sigma and varsigma chains: warm start in *_cur, solution into the other buffer
  double* sig_cur = Sig; double* sig_nxt = sigAlt;
  double* vs_cur = vs; double* vs_nxt = vsAlt;
  auto step_body = [&]() {
    for (int k = 0; k < 3; ++k) {
      if (apos) {
        st[k].Sout = sig_nxt;
        stage_solve(c, P, o, st[k], sig_cur, xa, xb, db);
        std::swap(sig_cur, sig_nxt);
        sens_rhs(c, P, st[k], ts[k], bs);
        stage_solve_b(c, P, o, st[k], bs, vs_cur, vs_nxt, false, xa, xb, db);
        std::swap(vs_cur, vs_nxt);
      } else {
        st[k].Sout = sig_cur;  // zero
      }
      hyp_stage(c, P, st, k, q, st[0].invr);
      SensHypArgs2D h;
      std::memset(&h, 0, sizeof(h));
      h.tiles = P.d_tiles; h.inst = P.d_inst; h.B = P.B;
      for (int v = 0; v < 4; ++v) { h.q[v] = st[k].q[v]; h.s[v] = ts[k][v]; h.sn[v] = ts[0][v]; h.so[v] = k < 2 ? ts[k + 1][v] : s[v]; }
      h.invr = st[k].invr; h.S = st[k].Sout; h.vs = vs_cur;
      h.ws_x = st[k].wsx; h.ws_y = st[k].wsy;
      h.c0 = RK_C0[k]; h.c1 = RK_C1[k]; h.c2 = RK_C2[k]; h.s_gamma = s_gamma;
      h.status = c.d_status;
      LaunchScope ls(c, KID_TAN);
      NP_DISPATCH(P.np, launch_k2_sens_hyp_rk<NPV>(h, P.ntiles(), c.stream));
    }
  };
  // The host-side effect of one step on the Sigma / varsigma chains.
  auto step_pointers = [&]() {
    for (int k = 0; k < 3; ++k) {
      if (apos) {
        st[k].Sout = sig_nxt;
        std::swap(sig_cur, sig_nxt);
        std::swap(vs_cur, vs_nxt);
      } else {
        st[k].Sout = sig_cur;
      }
    }
  };
  // Three swaps per step: the buffers repeat every second step, so steps of
  // one parity replay one CUDA graph (captured at steps 2 and 3, after the
  // first steps have allocated every buffer).
  StreamGraph graphs[2];
  const bool use_graph = c.use_graphs && !c.prof.on;
  for (int step = 0; step < n_steps; ++step) {
    StreamGraph& g = graphs[step % 2];
    if (!use_graph || step < 2) {
      step_body();
    } else {
      const bool replay = g.exec != nullptr;
      g.run(c, step_body);  // runs step_body only while capturing
      if (replay) step_pointers();
    }
  }
  if (apos) {  // sensitivity.jl:404-409: Sigma and varsigma at the final state
    recip(c, q[2], st[0].invr, NG);
    st[0].Sout = sig_nxt;
    stage_solve(c, P, o, st[0], sig_cur, xa, xb, db);
    std::swap(sig_cur, sig_nxt);
    sens_rhs(c, P, st[0], s, bs);
    stage_solve_b(c, P, o, st[0], bs, vs_cur, vs_nxt, false, xa, xb, db);
    std::swap(vs_cur, vs_nxt);
  }
  if (sig_cur != Sig) cuda_check(cudaMemcpyAsync(Sig, sig_cur, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "Sigma");
  if (vs_cur != vs) cuda_check(cudaMemcpyAsync(vs, vs_cur, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "varsigma");
  check_status(c);
}

void solve_elliptic2d(Ctx& c, const Plan2D& P, const double* const q[4], double* Sig, const Solve2DOpts& o, bool always) {
  const long long NG = P.NG;
  if (!always && !any_alpha_pos(P)) return;
  if (!always) check_alpha_uniform(P);
  double* scratch = c.ws.dbl("sol:stage", (size_t)NG * STAGE_FIXED_FIELDS);
  StageBuf st = stage_from(scratch, NG, o, true, false, (int)P.inst.size());
  for (int v = 0; v < 4; ++v) st.q[v] = const_cast<double*>(q[v]);
  recip(c, q[2], st.invr, NG);
  double* x0 = c.ws.dbl("sol:x0", NG);
  cuda_check(cudaMemcpyAsync(x0, Sig, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "x0 copy");
  st.Sout = Sig;
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  stage_setup(c, P, st, always);
  stage_solve_b(c, P, o, st, st.b, x0, st.Sout, false, c.ws.dbl("sol:xa", NG), c.ws.dbl("sol:xb", NG),
                c.ws.dbl("sol:d", NG));
  check_status(c);
}

void hyperbolic_rhs2d(Ctx& c, const Plan2D& P, const double* const q[4], const double* Sig, double* const k[4]) {
  const long long NG = P.NG;
  double* ir = c.ws.dbl("rhs:invr", NG);
  recip(c, q[2], ir, NG);
  HypArgs2D h;
  std::memset(&h, 0, sizeof(h));
  h.tiles = P.d_tiles; h.inst = P.d_inst; h.B = P.B;
  for (int v = 0; v < 4; ++v) { h.q[v] = q[v]; h.qn[v] = q[v]; h.k_out[v] = k[v]; h.qo[v] = nullptr; }
  h.invr = ir; h.S = Sig;
  h.c0 = 0.0; h.c1 = 1.0; h.c2 = 0.0;
  h.status = nullptr;
  { LaunchScope ls(c, KID_HYP); NP_DISPATCH(P.np, launch_k2_hyp_rk<NPV>(h, P.ntiles(), c.stream)); }
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
}

// Operator coefficients of A(rho, alpha) into the stage buffer st (for any
// alpha), its IGR source from (mx, my, rho) when mx is given (else st.b is not
// written) and diag(A) into st.cM when set.
static void operator_setup(Ctx& c, const Plan2D& P, StageBuf& st, const double* rho, const double* mx, const double* my) {
  recip(c, rho, st.invr, P.NG);
  SetupArgs2D sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.tiles = P.d_tiles; sa.inst = P.d_inst; sa.B = P.B;
  sa.mx = mx; sa.my = my; sa.invr = st.invr;
  sa.b = mx ? st.b : nullptr;
  sa.cm = st.cm; sa.ckx = st.ckx; sa.cky = st.cky; sa.cinvM = st.cinvM; sa.cpx = st.cpx; sa.cpy = st.cpy; sa.cM = st.cM;
  sa.always = 1;
  LaunchScope ls(c, KID_SETUP);
  NP_DISPATCH(P.np, launch_k2_setup<NPV>(sa, P.ntiles(), c.stream));
}

void apply_sip2d(Ctx& c, const Plan2D& P, const double* x, const double* rho, double* y) {
  const long long NG = P.NG;
  double* scratch = c.ws.dbl("sip:stage", (size_t)NG * STAGE_FIXED_FIELDS);
  Solve2DOpts o;
  StageBuf st = stage_from(scratch, NG, o, true, false, (int)P.inst.size());
  st.cM = nullptr;
  operator_setup(c, P, st, rho, nullptr, nullptr);
  ApplyArgs2D a;
  std::memset(&a, 0, sizeof(a));
  a.tiles = P.d_tiles; a.inst = P.d_inst; a.B = P.B;
  a.x = x; a.cm = st.cm; a.ckx = st.ckx; a.cky = st.cky; a.cpx = st.cpx; a.cpy = st.cpy; a.b = st.b; a.cinvM = st.cinvM;
  a.y_out = y;
  { LaunchScope ls(c, KID_APPLY); NP_DISPATCH(P.np, launch_k2_apply<NPV>(EPI_RESID, a, P.ntiles(), c.stream)); }
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
}

void igr_rhs_diag2d(Ctx& c, const Plan2D& P, const double* const q[4], double* b, double* M) {
  const long long NG = P.NG;
  Solve2DOpts o;
  StageBuf st = stage_from(c.ws.dbl("sip:stage", (size_t)NG * STAGE_FIXED_FIELDS), NG, o, true, false, (int)P.inst.size());
  if (b) st.b = b;
  st.cM = M;
  operator_setup(c, P, st, q[2], b ? q[0] : nullptr, q[1]);
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
}

void igr_euler_rhs2d(Ctx& c, const Plan2D& P, const double* const q[4], double* Sig, double* const k[4],
                     const Solve2DOpts& o) {
  check_alpha_uniform(P);
  if (any_alpha_pos(P)) solve_elliptic2d(c, P, q, Sig, o);
  else cuda_check(cudaMemsetAsync(Sig, 0, P.NG * sizeof(double), c.stream), "zero Sigma");  // forward.jl:26-27
  hyperbolic_rhs2d(c, P, q, Sig, k);
}

// Conjugate gradients on A(rho, alpha) x = b with M = I: the PCG kernels
// (k2_apply<EPI_PCG0 / EPI_PCG>, k2_pcg_update) with a field of ones as
// M^-1, so p_0 = r_0, rz = r . r and p_{k+1} = r_{k+1} + beta_k p_k
// (cg_fixed!, elliptic.jl:304-320, with its 1e-30 guards). Without `fixed`
// (cg_solve!, :278-297) the guards are 0 and the loop stops before iteration
// `it` (1-based) at the first it with sqrt(rz_{it-1}) < tol, returning it and
// x_{it-1}; else it returns maxiter and x_maxiter. The test reads rz back
// after every CG_CHUNK - 1 iterations, whose iterates x_k sit in a ring of
// CG_CHUNK fields, so the stop costs no extra work beyond the chunk.
constexpr int CG_CHUNK = 32;
int cg2d(Ctx& c, const Plan2D& P, const double* rho, const double* b, double* x, double tol, int maxiter, bool fixed) {
  if (P.inst.size() != 1) throw Error(1, "the CG solve takes one instance");
  if (maxiter < 0) throw Error(1, "maxiter must be >= 0");
  const long long NG = P.NG;
  const int nb = P.ntiles(), n = maxiter;
  Solve2DOpts o;
  StageBuf st = stage_from(c.ws.dbl("cg:stage", (size_t)NG * STAGE_FIXED_FIELDS), NG, o, true, false, 1);
  st.cM = nullptr;
  operator_setup(c, P, st, rho, nullptr, nullptr);
  double* ones = c.ws.dbl("cg:ones", NG);
  { LaunchScope ls(c, KID_OTHER); k_fill<<<grid_for(NG), 256, 0, c.stream>>>(ones, 1.0, NG); }
  double* r = c.ws.dbl("cg:r", NG);
  double* pv[2] = {c.ws.dbl("cg:pA", NG), c.ws.dbl("cg:pB", NG)};
  double* ap = c.ws.dbl("cg:ap", NG);
  const int K = fixed ? 1 : CG_CHUNK;
  double* ring = fixed ? x : c.ws.dbl("cg:xring", (size_t)NG * K);
  double* part = c.ws.dbl("red:part", nb);
  double* scal = c.ws.dbl("cg:scal", (size_t)pcg_scal_count(n, 1));
  auto RZ = [&](int k) { return scal + k; };
  auto PAP = [&](int k) { return scal + (n + 1) + k; };
  auto AL = [&](int k) { return scal + (2 * n + 1) + k; };
  auto BT = [&](int k) { return scal + (3 * n + 1) + k; };
  auto XK = [&](int k) { return (fixed || k == 0) ? x : ring + (long long)((k - 1) % K) * NG; };  // x_k
  const double eps = fixed ? 1e-30 : 0.0;
  int* cnt = sum_choice(c, P, false).fused ? inst_counters(c, P) : nullptr;
  ApplyArgs2D base;
  std::memset(&base, 0, sizeof(base));
  base.tiles = P.d_tiles; base.inst = P.d_inst; base.B = P.B;
  base.cm = st.cm; base.ckx = st.ckx; base.cky = st.cky; base.cpx = st.cpx; base.cpy = st.cpy; base.b = b; base.cinvM = ones;
  base.partials = part;
  {  // r_0 = b - A x_0, p_0 = r_0, rz_0 = r_0 . r_0
    ApplyArgs2D a = base;
    a.x = x; a.r_out = r; a.p_out = pv[0];
    a.isum = inst_sum0(cnt, RZ(0));
    { LaunchScope ls(c, KID_APPLY); NP_DISPATCH(P.np, launch_k2_apply<NPV>(EPI_PCG0, a, nb, c.stream)); }
    inst_sum_after(c, P, part, false, a.isum);
  }
  auto iteration = [&](int k) {
    ApplyArgs2D a = base;
    if (k == 0) {
      a.x = pv[0];
    } else {
      a.pcg_r = r; a.pcg_p = pv[(k - 1) % 2]; a.pcg_beta = BT(k - 1);
      a.p_out = pv[k % 2];
    }
    a.ap_out = ap;
    a.isum = inst_sum0(cnt, PAP(k), RZ(k), nullptr, AL(k), eps);
    { LaunchScope ls(c, KID_APPLY); NP_DISPATCH(P.np, launch_k2_apply<NPV>(EPI_PCG, a, nb, c.stream)); }
    inst_sum_after(c, P, part, false, a.isum);
    PcgUpdateArgs u;
    u.tiles = P.d_tiles; u.groups = P.d_groups; u.inst = P.d_inst;
    u.x_in = XK(k); u.x_out = XK(k + 1);
    u.p = pv[k % 2]; u.ap = ap; u.r_in = r; u.r_out = r; u.cinvM = ones;
    u.al = AL(k);
    u.partials = part;
    u.isum = inst_sum0(cnt, RZ(k + 1), nullptr, RZ(k), BT(k), eps);
    { LaunchScope ls(c, KID_OTHER); NP_DISPATCH(P.np, launch_k2_pcg_update<NPV>(u, P.ngroups(), c.stream)); }
    inst_sum_after(c, P, part, false, u.isum);
  };
  int iters = n;
  if (fixed) {
    for (int k = 0; k < n; ++k) iteration(k);
  } else {
    std::vector<double> rz(K);
    int k0 = 0, stop = -1;
    while (stop < 0 && k0 < n) {
      const int k1 = std::min(n, k0 + K - 1);  // iterations k0 .. k1-1 keep x_k0 .. x_k1 in the ring
      for (int k = k0; k < k1; ++k) iteration(k);
      cuda_check(cudaMemcpyAsync(rz.data(), RZ(k0), sizeof(double) * (k1 - k0), cudaMemcpyDeviceToHost, c.stream),
                 "rz readback");
      cuda_check(cudaStreamSynchronize(c.stream), "sync");
      for (int k = k0; k < k1 && stop < 0; ++k)
        if (std::sqrt(rz[k - k0]) < tol) stop = k;
      k0 = k1;
    }
    const int kx = stop >= 0 ? stop : n;
    iters = stop >= 0 ? stop + 1 : n;
    if (kx > 0) cuda_check(cudaMemcpyAsync(x, XK(kx), NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "x copy");
  }
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
  return iters;
}

// ------------------------------------------------------------------------------------------
// Objective and adjoint
// ------------------------------------------------------------------------------------------
static void inst_sums(Ctx& c, const Plan2D& P, const double* f, double* out_dev) {
  const int ni = (int)P.inst.size();
  std::vector<long long> off(ni), cnt(ni);
  for (int i = 0; i < ni; ++i) { off[i] = P.inst[i].off; cnt[i] = P.inst_nodes[i]; }
  long long* d = static_cast<long long*>(c.ws.get("sum:meta", sizeof(long long) * 2 * ni));
  cuda_check(cudaMemcpyAsync(d, off.data(), sizeof(long long) * ni, cudaMemcpyHostToDevice, c.stream), "meta");
  cuda_check(cudaMemcpyAsync(d + ni, cnt.data(), sizeof(long long) * ni, cudaMemcpyHostToDevice, c.stream), "meta");
  LaunchScope ls(c, KID_OTHER);
  k_inst_sum<<<ni, 256, 0, c.stream>>>(f, d, d + ni, out_dev);
}

static ObjArgs2D obj_args(const Plan2D& P, const double* const q[4], int objective, const double* prm) {
  ObjArgs2D a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.ninst = (int)P.inst.size(); a.B = P.B;
  for (int v = 0; v < 4; ++v) a.q[v] = q[v];
  a.obj = objective;
  for (int k = 0; k < 4; ++k) a.prm[k] = prm ? prm[k] : 0.0;
  a.NG = P.NG;
  return a;
}

// J per instance (device array out, ninst) from the final state q.
static void objective_value(Ctx& c, const Plan2D& P, const double* const q[4], int objective, const double* prm, double* J_host,
                            double* s1_dev, double* s2_dev) {
  const long long NG = P.NG;
  const int ni = (int)P.inst.size();
  ObjArgs2D a = obj_args(P, q, objective, prm);
  a.j1 = c.ws.dbl("obj:j1", NG);
  a.j2 = c.ws.dbl("obj:j2", NG);
  { LaunchScope ls(c, KID_OTHER); k2_obj_nodes<<<grid_for(NG), 256, 0, c.stream>>>(a); }
  inst_sums(c, P, a.j1, s1_dev);
  inst_sums(c, P, a.j2, s2_dev);
  std::vector<double> s1(ni), s2(ni);
  cuda_check(cudaMemcpyAsync(s1.data(), s1_dev, sizeof(double) * ni, cudaMemcpyDeviceToHost, c.stream), "J readback");
  cuda_check(cudaMemcpyAsync(s2.data(), s2_dev, sizeof(double) * ni, cudaMemcpyDeviceToHost, c.stream), "J readback");
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
  for (int i = 0; i < ni; ++i) J_host[i] = objective == OBJ_KINETIC_ENERGY ? s1[i] / s2[i] : s1[i];
}

static void check_objective(int objective) {
  if (objective < 0 || objective > OBJ_WINDOW_RHO2) throw Error(1, "Unknown objective");
}
static void check_solver(const Solve2DOpts& o) {
  if (o.solver < 0 || o.solver > 2) throw Error(1, "Unknown solver (use :pcg, :jacobi, or :chebyshev)");
  if (o.n_iter < 1) throw Error(1, "n_iter must be >= 1");
}

void objective2d(Ctx& c, const Plan2D& P, double* const q[4], int n_steps, const Solve2DOpts& o, int objective,
                 const double* prm, double* J) {
  check_objective(objective);
  check_solver(o);
  double* Sig = c.ws.dbl("obj:Sig", P.NG);
  cuda_check(cudaMemsetAsync(Sig, 0, P.NG * sizeof(double), c.stream), "zero Sigma");
  forward2d(c, P, q, Sig, n_steps, o);
  const double* qc[4] = {q[0], q[1], q[2], q[3]};
  objective_value(c, P, qc, objective, prm, J, c.ws.dbl("obj:s1", P.inst.size()), c.ws.dbl("obj:s2", P.inst.size()));
}

// Binomial checkpointing (revolve) over super-steps. cost(n, s) = the fewest
// forward super-step evaluations that reverse n super-steps when the first
// one's state sits in a slot and s more slots are free: the last super-step is
// taped and reversed first, and
//   cost(1, s) = 1,   cost(n, 0) = n (n + 1) / 2   (every super-step re-run from the first state),
//   cost(n, s) = min over 0 < m < n of  m + cost(n - m, s - 1) + cost(m, s)
// (advance m super-steps, store the state, reverse the right part with one
// slot fewer, then the left part with the slot back). Tabulated once for up to
// REVOLVE_MAX super-steps, with the minimising m of each entry.
constexpr int REVOLVE_MAX = 512;
struct RevolveTable {
  std::vector<long long> cost;  // [n][s], s < n
  std::vector<int> split;
  long long at(int n, int s) const { return cost[(size_t)n * (REVOLVE_MAX + 1) + std::min(s, n - 1)]; }
};
static const RevolveTable& revolve_table() {
  static const RevolveTable t = [] {
    RevolveTable r;
    const size_t W = REVOLVE_MAX + 1;
    r.cost.assign(W * W, 0);
    r.split.assign(W * W, 1);
    for (int n = 1; n <= REVOLVE_MAX; ++n)
      for (int s = 0; s < n; ++s) {
        long long best;
        int bm = 1;
        if (n == 1) best = 1;
        else if (s == 0) best = (long long)n * (n + 1) / 2;
        else {
          best = -1;
          for (int m = 1; m < n; ++m) {
            const long long v = m + r.cost[(size_t)(n - m) * W + std::min(s - 1, n - m - 1)] + r.cost[(size_t)m * W + std::min(s, m - 1)];
            if (best < 0 || v < best) { best = v; bm = m; }
          }
        }
        r.cost[(size_t)n * W + s] = best;
        r.split[(size_t)n * W + s] = bm;
      }
    return r;
  }();
  return t;
}
// Where the schedule stores its next checkpoint within a range of n super-steps
// with `free` slots (1 <= result < n).
static int revolve_split(int n, int free) {
  return revolve_table().split[(size_t)n * (REVOLVE_MAX + 1) + std::min(free, n - 1)];
}

// Tape window w (RK steps per super-step) and checkpoint slots for n steps
// within `budget` bytes (w taped steps + the first state + `slots` states),
// minimising the forward step evaluations; w = 0 when nothing fits.
static RevolvePlan plan_revolve(int n, size_t step_bytes, size_t ckpt_bytes, size_t budget) {
  const RevolveTable& t = revolve_table();
  RevolvePlan best;
  for (int w = n; w >= 1; --w) {
    const int ns = (n + w - 1) / w;
    if (ns > REVOLVE_MAX) break;
    if ((size_t)w * step_bytes + ckpt_bytes > budget) continue;
    const long long avail = (long long)((budget - (size_t)w * step_bytes) / ckpt_bytes) - 1;
    const int slots = (int)std::min<long long>(avail, ns - 1);
    const long long evals = t.at(ns, slots) * w;
    if (best.w == 0 || evals < best.evals) { best.w = w; best.slots = slots; best.evals = evals; }
  }
  return best;
}

RevolvePlan adjoint_checkpoints2d(Ctx& c, long long NG, int F, int n_steps) {
  const size_t step_bytes = (size_t)3 * F * NG * sizeof(double);
  const size_t ckpt_bytes = (size_t)6 * NG * sizeof(double);
  size_t budget = c.tape_budget;
  if (budget == 0) {
    // free memory plus what the tape and checkpoint buffers already hold (they are reused)
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    const size_t avail = fr + c.ws.held("adj:tape") + c.ws.held("adj:ckpt");
    const size_t reserve = (size_t)1 << 30;
    budget = avail > reserve ? avail - reserve : 0;
  }
  return plan_revolve(std::max(n_steps, 1), step_bytes, ckpt_bytes, budget);
}

void adjoint2d(Ctx& c, const Plan2D& P, const double* const q0[4], int n_steps, const Solve2DOpts& o, int objective,
               const double* prm, double* J, double* const dq0[4], double* dgamma, double* dalpha) {
  check_objective(objective);
  check_solver(o);
  check_alpha_uniform(P);
  if (n_steps < 0) throw Error(1, "n_steps must be >= 0");
  const long long NG = P.NG;
  const int ni = (int)P.inst.size();
  const bool apos = any_alpha_pos(P);
  const int F = stage_fields2d(o, apos, NG, ni);
  // scratch for untaped steps and final state
  double* scr = c.ws.dbl("adj:scr", (size_t)NG * 3 * STAGE_FIXED_FIELDS);
  StageBuf ust[3];
  for (int s = 0; s < 3; ++s) ust[s] = stage_from(scr + (long long)s * STAGE_FIXED_FIELDS * NG, NG, o, apos, false, ni);
  double* xa = c.ws.dbl("adj:xa", NG);
  double* xb = c.ws.dbl("adj:xb", NG);
  double* dbuf = c.ws.dbl("adj:d", NG);
  double* qend = c.ws.dbl("adj:qend", 5 * NG);
  double* qendp[4] = {qend, qend + NG, qend + 2 * NG, qend + 3 * NG};
  double* sigA = c.ws.dbl("adj:sigA", NG);
  double* sigB = c.ws.dbl("adj:sigB", NG);
  double* sig0 = c.ws.dbl("adj:sig0", NG);
  double* rb = c.ws.dbl("adj:rev", (size_t)NG * 24);
  double* gnode = c.ws.dbl("adj:gnode", NG);
  double* anode = c.ws.dbl("adj:anode", NG);
  c.ws.dbl("obj:j1", NG);
  c.ws.dbl("obj:j2", NG);
  // ---- memory plan: a binomial (revolve) checkpoint schedule over super-steps
  // of w RK steps. The tape holds one super-step (w taped steps); checkpoint
  // slots hold (q, 1/rho, Sigma) at super-step boundaries, slot 0 the initial
  // state. Among the tape windows that fit the budget with their slots, the one
  // with the fewest forward step evaluations is taken (the full tape, w = n,
  // when it fits: no recomputation).
  const int nsteps_eff = std::max(n_steps, 1);
  const RevolvePlan rp = adjoint_checkpoints2d(c, NG, F, nsteps_eff);
  if (rp.w < 1) throw Error(5, "device memory too small for one taped step and one checkpoint of this batch");
  const int w = rp.w, n_super = (nsteps_eff + w - 1) / w;
  c.plan_seg = w;
  c.plan_nseg = n_super;
  c.plan_snapshots = rp.slots;
  c.plan_step_evals = 0;
  double* ckpt = c.ws.dbl("adj:ckpt", (size_t)(rp.slots + 1) * 6 * NG);
  double* tape = c.ws.dbl("adj:tape", (size_t)w * 3 * F * NG);
  auto slot = [&](int local_step, int stage) {
    return stage_from(tape + ((long long)local_step * 3 + stage) * F * NG, NG, o, apos, true, ni);
  };

  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  cuda_check(cudaMemsetAsync(sig0, 0, NG * sizeof(double), c.stream), "zero Sigma");
  // untaped state: ust[0].q / invr hold q^s
  for (int v = 0; v < 4; ++v)
    cuda_check(cudaMemcpyAsync(ust[0].q[v], q0[v], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "q0 copy");
  recip(c, ust[0].q[2], ust[0].invr, NG);
  if (!apos) {
    for (int s = 0; s < 3; ++s) cuda_check(cudaMemsetAsync(ust[s].Sout, 0, NG * sizeof(double), c.stream), "zero Sout");
  }
  const double* sig_cur = sig0;

  // Runs steps [s0, s1) taped into slots 0.. (state enters in slot 0 of s0),
  // the final step's output goes to qend (or the next step's slot).
  auto taped_range = [&](int s0, int s1, const double* sig_in) {
    const double* sg = sig_in;
    for (int s = s0; s < s1; ++s) {
      StageBuf st[3] = {slot(s - s0, 0), slot(s - s0, 1), slot(s - s0, 2)};
      if (!apos) for (int k = 0; k < 3; ++k) cuda_check(cudaMemsetAsync(st[k].Sout, 0, NG * sizeof(double), c.stream), "zero Sout");
      double* qo[4];
      double* iro;
      if (s + 1 < s1) { StageBuf nx = slot(s + 1 - s0, 0); for (int v = 0; v < 4; ++v) qo[v] = nx.q[v]; iro = nx.invr; }
      else { for (int v = 0; v < 4; ++v) qo[v] = qendp[v]; iro = qend + 4 * NG; }
      step_forward(c, P, o, st, sg, qo, iro, xa, xb, dbuf);
      sg = st[2].Sout;
      ++c.plan_step_evals;
    }
    return sg;
  };
  auto copy_nd = [&](double* dst, const double* src, const char* what) {
    cuda_check(cudaMemcpyAsync(dst, src, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), what);
  };
  // checkpoint slot k <-> the untaped state (q, 1/rho and the carried Sigma)
  auto save_slot = [&](int k) {
    double* ck = ckpt + (long long)k * 6 * NG;
    for (int v = 0; v < 4; ++v) copy_nd(ck + v * NG, ust[0].q[v], "ckpt");
    copy_nd(ck + 4 * NG, ust[0].invr, "ckpt");
    copy_nd(ck + 5 * NG, sig_cur, "ckpt");
  };
  auto restore_slot = [&](int k) {
    const double* ck = ckpt + (long long)k * 6 * NG;
    for (int v = 0; v < 4; ++v) copy_nd(ust[0].q[v], ck + v * NG, "restore");
    copy_nd(ust[0].invr, ck + 4 * NG, "restore");
    copy_nd(sig0, ck + 5 * NG, "restore");
    sig_cur = sig0;
  };
  auto super_begin = [&](int k) { return k * w; };
  auto super_end = [&](int k) { return std::min(n_steps, (k + 1) * w); };
  // untaped steps of super-steps [k0, k1) from the untaped state
  auto advance = [&](int k0, int k1) {
    for (int s = super_begin(k0); s < super_begin(k1); ++s) {
      if (apos) for (int kk = 0; kk < 3; ++kk) ust[kk].Sout = (kk % 2 == 0) ? sigA : sigB;
      step_forward(c, P, o, ust, sig_cur, ust[0].q, ust[0].invr, xa, xb, dbuf);
      if (apos) {  // carried Sigma lives in sig0 (its zero start is only read by step 0)
        copy_nd(sig0, ust[2].Sout, "Sigma carry");
        sig_cur = sig0;
      }
      ++c.plan_step_evals;
    }
  };
  // tape super-step k from the untaped state (its output state goes to qend)
  auto tape_super = [&](int k) {
    const int s0 = super_begin(k), s1 = super_end(k);
    if (s1 <= s0) {  // no steps at all: the final state is the initial one
      for (int v = 0; v < 4; ++v) copy_nd(qendp[v], ust[0].q[v], "q end");
      return;
    }
    StageBuf first = slot(0, 0);
    for (int v = 0; v < 4; ++v) copy_nd(first.q[v], ust[0].q[v], "seg in");
    copy_nd(first.invr, ust[0].invr, "seg in");
    taped_range(s0, s1, sig_cur);
  };
  save_slot(0);

  // ---- objective and its gradient at the final state (once the last super-step has run)
  const double* qf[4] = {qendp[0], qendp[1], qendp[2], qendp[3]};
  double* s1d = c.ws.dbl("adj:s1", ni);
  double* s2d = c.ws.dbl("adj:s2", ni);
  // reverse buffers
  double* QB[4]; double* QN[4]; double* Q2b[4]; double* Q1b[4];
  for (int v = 0; v < 4; ++v) { QB[v] = rb + v * NG; QN[v] = rb + (4 + v) * NG; Q2b[v] = rb + (8 + v) * NG; Q1b[v] = rb + (12 + v) * NG; }
  double* Sb = rb + 16 * NG;
  double* U[2] = {rb + 17 * NG, rb + 18 * NG};
  double* db = rb + 19 * NG;
  double* bb = rb + 20 * NG;
  double* Mb = rb + 21 * NG;
  double* Zm = rb + 22 * NG;
  double* Zs = rb + 23 * NG;
  auto objective_and_seed = [&]() {
    objective_value(c, P, qf, objective, prm, J, s1d, s2d);
    ObjArgs2D a = obj_args(P, qf, objective, prm);
    a.s1 = s1d; a.s2 = s2d;
    for (int v = 0; v < 4; ++v) a.qb[v] = QB[v];
    a.gb = gnode;   // initialises the per-node gamma accumulator
    LaunchScope ls(c, KID_OTHER);
    k2_obj_grad<<<grid_for(NG), 256, 0, c.stream>>>(a);
  };
  cuda_check(cudaMemsetAsync(Sb, 0, NG * sizeof(double), c.stream), "zero Sb");
  cuda_check(cudaMemsetAsync(anode, 0, NG * sizeof(double), c.stream), "zero anode");
  std::vector<double> ca, cc;
  cheb_coeffs(P.B, o.n_iter, ca, cc);
  const int srev = !apos ? SREV_NONE : (o.solver == SOLVER_CHEBYSHEV ? SREV_CHEB : (o.solver == SOLVER_JACOBI ? SREV_JACOBI : SREV_PCG));
  double* part = srev == SREV_PCG ? c.ws.dbl("red:part", P.ntiles()) : nullptr;
  double* pscal = c.ws.dbl("adj:pcgscal", (size_t)4 * ni);  // BET, RZB, PAPB, RZB1 per instance
  const int nb = P.ntiles();
  const double c0s[3] = {0.0, 3.0 / 4, 1.0 / 3}, c1s[3] = {1.0, 1.0 / 4, 2.0 / 3}, c2s[3] = {1.0, 1.0 / 4, 2.0 / 3};

  // Reverse of one stage's PCG solve (the tape of pcg_solve), given Sb = the
  // adjoint of its result: leaves the adjoint of the warm start in Sb and
  // bb, iMb (Mb), Zm, Zs for the setup reverse.
  auto pcg_reverse = [&](StageBuf& sb) {
    const int n = o.n_iter;
    double* PB = U[0];
    double* RB = U[1];
    double* BET = pscal; double* RZB = pscal + ni; double* PAPB = pscal + 2 * ni; double* RZB1 = pscal + 3 * ni;
    const double* RZ = sb.scal;
    const double* PAP = sb.scal + (long long)(n + 1) * ni;
    const double* AL = sb.scal + (long long)(2 * n + 1) * ni;
    const double* BT = sb.scal + (long long)(3 * n + 1) * ni;
    int* cnt = sum_choice(c, P, false).fused ? inst_counters(c, P) : nullptr;
    for (int it = n - 1; it >= 0; --it) {
      PcgRevArgs g;
      g.tiles = P.d_tiles; g.groups = P.d_groups; g.inst = P.d_inst;
      g.first = it == n - 1 ? 1 : 0;
      g.pb = PB; g.rb = RB; g.iMb = Mb;
      g.r1 = sb.rk[it + 1]; g.cinvM = sb.cinvM; g.ap = sb.apk[it]; g.p = sb.pk[it]; g.xb = Sb;
      g.beta = BT + (long long)it * ni; g.rzb1 = RZB1;
      g.partials = part;
      std::memset(&g.isum, 0, sizeof(g.isum));  // ab, then RZB and PAPB
      g.isum.cnt = cnt; g.isum.mode = 1; g.isum.first = g.first; g.isum.it = it; g.isum.ni = ni;
      g.isum.RZ = RZ; g.isum.PAP = PAP; g.isum.BET = BET; g.isum.RZB = RZB; g.isum.PAPB = PAPB;
      { LaunchScope ls(c, KID_OTHER); NP_DISPATCH(P.np, launch_k2_pcg_rev_update<NPV>(g, P.ngroups(), c.stream)); }
      inst_sum_after(c, P, part, true, g.isum);
      ApplyRevArgs2D r;
      std::memset(&r, 0, sizeof(r));
      r.tiles = P.d_tiles; r.inst = P.d_inst; r.B = P.B;
      r.u = RB; r.xk = sb.pk[it];
      r.cm = sb.cm; r.ckx = sb.ckx; r.cky = sb.cky; r.cpx = sb.cpx; r.cpy = sb.cpy; r.cinvM = sb.cinvM;
      r.invr = sb.invr;
      r.xb = PB; r.bb = bb; r.Zm = Zm; r.Zs = Zs;
      r.first = it == n - 1 ? 1 : 0;
      r.bb_op = 0;
      r.zscale = -1.0;
      r.has_next = it > 0 ? 1 : 0;
      r.al_it = AL + (long long)it * ni; r.papb = PAPB;
      r.xconst = Sb; r.apk = sb.apk[it]; r.p_next = it > 0 ? sb.pk[it - 1] : nullptr;
      r.partials = part;
      if (it > 0) {  // betab of iteration it - 1 and rzb_it = RZB + betab / (rz_{it-1} + eps)
        r.isum.cnt = cnt; r.isum.mode = 2; r.isum.it = it - 1; r.isum.ni = ni;
        r.isum.RZ = RZ; r.isum.BET = BET; r.isum.RZB = RZB; r.isum.RZB1 = RZB1;
      }
      { LaunchScope ls(c, KID_APPLY_REV); NP_DISPATCH(P.np, launch_k2_apply_rev<NPV>(SREV_PCG, r, nb, c.stream)); }
      if (it > 0) inst_sum_after(c, P, part, false, r.isum);
    }
    {
      PcgRevFinalArgs f;
      f.tiles = P.d_tiles; f.inst = P.d_inst;
      f.pb = PB; f.r0 = sb.rk[0]; f.cinvM = sb.cinvM; f.RZB = RZB; f.rb = RB; f.iMb = Mb;
      LaunchScope ls(c, KID_OTHER);
      NP_DISPATCH(P.np, launch_k2_pcg_rev_final<NPV>(f, nb, c.stream));
    }
    // r_0 = b - A x_0
    ApplyRevArgs2D r;
    std::memset(&r, 0, sizeof(r));
    r.tiles = P.d_tiles; r.inst = P.d_inst; r.B = P.B;
    r.u = RB; r.xk = sb.x0t;
    r.cm = sb.cm; r.ckx = sb.ckx; r.cky = sb.cky; r.cpx = sb.cpx; r.cpy = sb.cpy; r.cinvM = sb.cinvM;
    r.invr = sb.invr;
    r.xb = Sb; r.bb = bb; r.Zm = Zm; r.Zs = Zs;
    r.first = 0; r.bb_op = 1;
    r.zscale = -1.0;
    r.has_next = 0;
    LaunchScope ls(c, KID_APPLY_REV);
    NP_DISPATCH(P.np, launch_k2_apply_rev<NPV>(SREV_NONE, r, nb, c.stream));
  };

  auto reverse_step = [&](int local) {
    StageBuf st[3] = {slot(local, 0), slot(local, 1), slot(local, 2)};
    for (int s = 2; s >= 0; --s) {
      HypRevArgs2D h;
      std::memset(&h, 0, sizeof(h));
      h.tiles = P.d_tiles; h.inst = P.d_inst; h.B = P.B;
      for (int v = 0; v < 4; ++v) {
        h.q[v] = st[s].q[v];
        h.A[v] = s == 2 ? QB[v] : (s == 1 ? Q2b[v] : Q1b[v]);
        h.Qn[v] = QN[v];
        h.Qs[v] = s == 2 ? Q2b[v] : (s == 1 ? Q1b[v] : QN[v]);
      }
      h.invr = st[s].invr; h.S = st[s].Sout;
      h.ws_x = st[s].wsx; h.ws_y = st[s].wsy;
      h.c0 = c0s[s]; h.c1 = c1s[s]; h.c2 = c2s[s];
      h.qn_mode = s == 2 ? 1 : (s == 1 ? 2 : 0);
      h.qs_add = s == 0 ? 1 : 0;
      h.Sb = Sb; h.Sb_add = 1;
      h.gnode = gnode;
      h.srev = srev == SREV_PCG ? SREV_NONE : srev;
      h.cinvM = st[s].cinvM;
      h.r_last = (apos && srev != SREV_PCG) ? st[s].rk[o.n_iter - 1] : nullptr;
      h.u_out = U[0]; h.db = db; h.iMb = Mb;
      h.ca = ca[o.n_iter]; h.cc = cc[o.n_iter]; h.omega = 2.0 / 3.0;
      { LaunchScope ls(c, KID_HYP_REV); NP_DISPATCH(P.np, launch_k2_hyp_rev<NPV>(h, nb, c.stream)); }
      if (!apos) continue;
      if (srev == SREV_PCG) {
        pcg_reverse(st[s]);
      } else {
      int cur = 0;
      for (int m = o.n_iter - 1; m >= 0; --m) {
        ApplyRevArgs2D r;
        std::memset(&r, 0, sizeof(r));
        r.tiles = P.d_tiles; r.inst = P.d_inst; r.B = P.B;
        r.u = U[cur]; r.xk = st[s].xk[m];
        r.gxk = st[s].gxk.empty() ? nullptr : st[s].gxk[m];
        r.gyk = st[s].gyk.empty() ? nullptr : st[s].gyk[m];
        r.cm = st[s].cm; r.ckx = st[s].ckx; r.cky = st[s].cky; r.cpx = st[s].cpx; r.cpy = st[s].cpy; r.cinvM = st[s].cinvM;
        r.invr = st[s].invr;
        r.xb = Sb; r.bb = bb; r.Zm = Zm; r.Zs = Zs;
        r.first = (m == o.n_iter - 1) ? 1 : 0;
        r.bb_op = r.first ? 1 : 2;
        r.zscale = -1.0;
        r.has_next = m > 0 ? 1 : 0;
        r.r_prev = m > 0 ? st[s].rk[m - 1] : nullptr;
        r.u_out = U[1 - cur]; r.db = db; r.iMb = Mb;
        r.ca = ca[m > 0 ? m : 1]; r.cc = cc[m > 0 ? m : 1]; r.omega = 2.0 / 3.0;
        { LaunchScope ls(c, KID_APPLY_REV); NP_DISPATCH(P.np, launch_k2_apply_rev<NPV>(srev, r, nb, c.stream)); }
        cur = 1 - cur;
      }
      }
      SetupRevArgs2D sr;
      std::memset(&sr, 0, sizeof(sr));
      sr.tiles = P.d_tiles; sr.inst = P.d_inst; sr.B = P.B;
      sr.mx = st[s].q[0]; sr.my = st[s].q[1]; sr.invr = st[s].invr;
      sr.b = st[s].b; sr.cm = st[s].cm; sr.cM = st[s].cM; sr.cinvM = st[s].cinvM;
      sr.bb = bb; sr.iMb = Mb; sr.Zm = Zm; sr.Zs = Zs;
      double* const* QsP = s == 2 ? Q2b : (s == 1 ? Q1b : QN);
      sr.Qs[0] = QsP[0]; sr.Qs[1] = QsP[1]; sr.Qs[2] = QsP[2];
      sr.anode = anode;
      { LaunchScope ls(c, KID_SETUP_REV); NP_DISPATCH(P.np, launch_k2_setup_rev<NPV>(sr, nb, c.stream)); }
    }
    for (int v = 0; v < 4; ++v) std::swap(QB[v], QN[v]);
  };

  // ---- the schedule: revolve(a, b, k, free) reverses super-steps [a, b) from
  // the state of super-step a held in slot k, with `free` slots above k. The
  // first super-step reversed is the last one, whose taped run also yields the
  // final state for the objective.
  bool seeded = false;
  auto leaf = [&](int a) {
    tape_super(a);
    if (!seeded) { objective_and_seed(); seeded = true; }
    for (int st = super_end(a) - 1; st >= super_begin(a); --st) reverse_step(st - super_begin(a));
  };
  std::function<void(int, int, int, int)> revolve = [&](int a, int b, int k, int free) {
    if (b - a == 1) { restore_slot(k); leaf(a); return; }
    if (free == 0) {  // no slot left: every super-step is re-run from slot k
      for (int j = b - 1; j >= a; --j) { restore_slot(k); advance(a, j); leaf(j); }
      return;
    }
    const int m = a + revolve_split(b - a, free);
    restore_slot(k);
    advance(a, m);
    save_slot(k + 1);
    revolve(m, b, k + 1, free - 1);
    revolve(a, m, k, free);
  };
  revolve(0, n_super, 0, rp.slots);
  for (int v = 0; v < 4; ++v) cuda_check(cudaMemcpyAsync(dq0[v], QB[v], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "dq0");
  // per-instance parameter gradients
  double* gsum = c.ws.dbl("adj:gsum", ni);
  double* asum = c.ws.dbl("adj:asum", ni);
  inst_sums(c, P, gnode, gsum);
  inst_sums(c, P, anode, asum);
  if (dgamma) cuda_check(cudaMemcpyAsync(dgamma, gsum, sizeof(double) * ni, cudaMemcpyDeviceToHost, c.stream), "dgamma");
  if (dalpha) cuda_check(cudaMemcpyAsync(dalpha, asum, sizeof(double) * ni, cudaMemcpyDeviceToHost, c.stream), "dalpha");
  check_status(c);
}

// FP64 throughput probe: independent DFMA chains on every SM (roofline
// denominator of this FP64-bound path). Returns TFLOP/s (2 flops per DFMA).
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5) out[threadIdx.x] = s;  // never true; keeps the chains live
}

// FP64 tensor-core (DMMA) throughput probe: eight independent accumulator
// chains per warp of mma.sync.m8n8k4 f64 (one warp instruction = 8 x 8 x 4
// multiply-adds = 512 flops), the question being whether the 4 x 4 line
// contractions would issue faster on the FP64 tensor path than as DFMAs.
__global__ void k_dmma_probe(double* out, int iters, double a, double b) {
  double c[8][2];
#pragma unroll
  for (int k = 0; k < 8; ++k) { c[k][0] = threadIdx.x * 1e-3 + k; c[k][1] = c[k][0] + 0.5; }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  if (s == 1234.5) out[threadIdx.x] = s;  // never true; keeps the chains live
}

// ------------------------------------------------------------------------------------------
// Continuous adjoint: run_forward_store (forward.jl:111-158) and
// run_adjoint_conservative (adjoint_pde.jl:527-611)
// ------------------------------------------------------------------------------------------

// Terminal condition of run_adjoint_conservative (adjoint_pde.jl:542-584): the
// L2 gradient density of J at t = T (no quadrature weights). s1/s2 hold the
// per-instance kinetic energy and mass sums for the kinetic-energy objective.
__global__ void k2_pde_terminal(ObjArgs2D a) {
  const double pi = 3.14159265358979323846;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.NG; n += (long long)gridDim.x * blockDim.x) {
    const int ii = find_inst(a.inst, a.ninst, n);
    const Inst2D I = a.inst[ii];
    double c, x, y;
    node_coords2d(a.B, I, n - I.off, &c, &x, &y);
    const double mx = a.q[0][n], my = a.q[1][n], r = a.q[2][n], E = a.q[3][n];
    const double ux = mx / r, uy = my / r;
    double g0 = 0, g1 = 0, g2 = 0, g3 = 0;
    switch (a.obj) {
      case OBJ_L2_DENSITY: g2 = 2.0 * r; break;
      case OBJ_L2_PRESSURE: {
        const double gm = I.gamma - 1.0;
        const double P = gm * (E - (mx * mx + my * my) / (2.0 * r));
        g0 = -2.0 * gm * P * ux; g1 = -2.0 * gm * P * uy; g2 = gm * P * (ux * ux + uy * uy); g3 = 2.0 * gm * P;
        break;
      }
      case OBJ_KINETIC_ENERGY: {
        const double KE = a.s1[ii], Ms = a.s2[ii];
        g0 = ux / Ms; g1 = uy / Ms;
        g2 = -(mx * mx + my * my) / (2.0 * (r * r)) / Ms - KE / (Ms * Ms);
        break;
      }
      case OBJ_WINDOWED_KE: {
        const double wx = exp(-((x - 0.55) * (x - 0.55) + (y - 0.50) * (y - 0.50)) / (0.15 * 0.15));
        g0 = wx * ux; g1 = wx * uy; g2 = -wx * (ux * ux + uy * uy) / 2.0;
        break;
      }
      case OBJ_WEIGHTED_MOMENTUM: g0 = sin(2 * pi * x / I.lx) * sin(2 * pi * y / I.ly); break;
      case OBJ_WINDOW_RHO2: {
        const bool in = x >= a.prm[0] && x <= a.prm[0] + a.prm[2] && y >= a.prm[1] && y <= a.prm[1] + a.prm[2];
        g2 = in ? 2.0 * r : 0.0;
        break;
      }
      default: break;
    }
    a.qb[0][n] = g0; a.qb[1][n] = g1; a.qb[2][n] = g2; a.qb[3][n] = g3;
  }
}

void forward_store_init2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const double* const q0[4], double* snap0) {
  const long long NG = P.NG;
  for (int v = 0; v < 4; ++v)
    if (snap0 + v * NG != q0[v])
      cuda_check(cudaMemcpyAsync(snap0 + v * NG, q0[v], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "snapshot 0");
  double* Sig = snap0 + 4 * NG;
  double* zero = c.ws.dbl("fst:zero", NG);
  cuda_check(cudaMemsetAsync(zero, 0, NG * sizeof(double), c.stream), "zero");
  if (!any_alpha_pos(P)) {
    cuda_check(cudaMemsetAsync(Sig, 0, NG * sizeof(double), c.stream), "zero Sigma");
    return;
  }
  StageBuf st = stage_from(c.ws.dbl("fst:stages", (size_t)NG * 3 * STAGE_FIXED_FIELDS), NG, o, true, false, (int)P.inst.size());
  for (int v = 0; v < 4; ++v) st.q[v] = snap0 + v * NG;
  recip(c, st.q[2], st.invr, NG);
  st.Sout = Sig;
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  stage_solve(c, P, o, st, zero, c.ws.dbl("fst:xa", NG), c.ws.dbl("fst:xb", NG), c.ws.dbl("fst:d", NG));
  check_status(c);
}

void forward_store_range2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const SnapSlot& slot, int k0, int k1) {
  check_alpha_uniform(P);
  const long long NG = P.NG;
  const int ni = (int)P.inst.size();
  const bool apos = any_alpha_pos(P);
  double* scratch = c.ws.dbl("fst:stages", (size_t)NG * 3 * STAGE_FIXED_FIELDS);
  StageBuf st[3];
  for (int s = 0; s < 3; ++s) st[s] = stage_from(scratch + (long long)s * STAGE_FIXED_FIELDS * NG, NG, o, apos, false, ni);
  double* xa = c.ws.dbl("fst:xa", NG);
  double* xb = c.ws.dbl("fst:xb", NG);
  double* db = c.ws.dbl("fst:d", NG);
  double* sA = c.ws.dbl("fst:sA", NG);
  double* sB = c.ws.dbl("fst:sB", NG);
  double* zero = c.ws.dbl("fst:zero", NG);
  if (k1 <= k0) return;
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  if (!apos) cuda_check(cudaMemsetAsync(zero, 0, NG * sizeof(double), c.stream), "zero");
  {
    const double* s0 = slot(k0);
    recip(c, s0 + 2 * NG, st[0].invr, NG);
  }
  for (int k = k0; k < k1; ++k) {
    double* cur = slot(k);
    double* nxt = slot(k + 1);
    for (int v = 0; v < 4; ++v) st[0].q[v] = cur + v * NG;
    for (int s = 0; s < 3; ++s) st[s].Sout = !apos ? zero : ((s % 2 == 0) ? sA : sB);
    double* qo[4] = {nxt, nxt + NG, nxt + 2 * NG, nxt + 3 * NG};
    // the last stage writes 1/rho of the new state into st[0].invr (read by the post-step solve);
    // the post-step solve leaves st[0]'s coefficients set up for the next step's first stage
    step_forward(c, P, o, st, cur + 4 * NG, qo, st[0].invr, xa, xb, db, k == k0);
    if (apos) {  // forward.jl:152-154: one more solve on the new state, warm start = stage-3 Sigma
      StageBuf post = st[0];
      for (int v = 0; v < 4; ++v) post.q[v] = qo[v];
      post.Sout = nxt + 4 * NG;
      stage_solve(c, P, o, post, st[2].Sout, xa, xb, db);
    } else {
      cuda_check(cudaMemsetAsync(nxt + 4 * NG, 0, NG * sizeof(double), c.stream), "zero Sigma");
    }
  }
  check_status(c);
}

namespace {
// Device buffers of the continuous adjoint.
struct PdeWork {
  double* a[4]; double* a1[4]; double* a2[4];
  double* Pi[2];
  int cur = 0;
  double* b;
  double* invr; double* src[PDE_SRC]; double* nl[PDE_NL]; double* wsx; double* wsy;
  StageBuf st;
  double *xa, *xb, *db;
};
}  // namespace

static PdeWork pde_work(Ctx& c, const Plan2D& P, const Solve2DOpts& o) {
  const long long NG = P.NG;
  PdeWork w;
  double* f = c.ws.dbl("pde:fields", (size_t)NG * (12 + 2 + 1 + 1 + PDE_SRC + PDE_NL + 2 + 3));
  int k = 0;
  auto nxt = [&]() { return f + (long long)(k++) * NG; };
  for (int v = 0; v < 4; ++v) { w.a[v] = nxt(); w.a1[v] = nxt(); w.a2[v] = nxt(); }
  w.Pi[0] = nxt(); w.Pi[1] = nxt();
  w.b = nxt(); w.invr = nxt();
  for (int v = 0; v < PDE_SRC; ++v) w.src[v] = nxt();
  for (int v = 0; v < PDE_NL; ++v) w.nl[v] = nxt();
  w.wsx = nxt(); w.wsy = nxt();
  w.xa = nxt(); w.xb = nxt(); w.db = nxt();
  w.st = stage_from(c.ws.dbl("pde:stage", (size_t)NG * STAGE_FIXED_FIELDS), NG, o, true, false, (int)P.inst.size());
  return w;
}

// Per-step preparation from one snapshot and, with alpha > 0, the SIP
// operator coefficients of its density (compute_sip_diagonal + the operator
// the Pi solve applies, adjoint_pde.jl:495-502).
static void pde_prep(Ctx& c, const Plan2D& P, PdeWork& w, const double* snap, bool apos) {
  const long long NG = P.NG;
  PdePrepArgs2D p;
  std::memset(&p, 0, sizeof(p));
  p.tiles = P.d_tiles; p.inst = P.d_inst; p.B = P.B;
  for (int v = 0; v < 4; ++v) p.q[v] = snap + v * NG;
  p.S = snap + 4 * NG;
  p.invr = w.invr;
  for (int v = 0; v < PDE_SRC; ++v) p.src[v] = w.src[v];
  for (int v = 0; v < PDE_NL; ++v) p.nl[v] = apos ? w.nl[v] : nullptr;
  p.ws_x = w.wsx; p.ws_y = w.wsy;
  {
    LaunchScope ls(c, KID_PDE_AUX);
    NP_DISPATCH(P.np, launch_k2_pde_prep<NPV>(p, P.ntiles(), c.stream));
  }
  if (apos) {
    for (int v = 0; v < 4; ++v) w.st.q[v] = const_cast<double*>(snap + v * NG);
    w.st.invr = w.invr;
    stage_setup(c, P, w.st);
  }
}

// Pi solve of one stage (adjoint_pde.jl:487-502): b from the stage input,
// warm start = the current Pi; the result becomes the current Pi.
static void pde_pi_solve(Ctx& c, const Plan2D& P, const Solve2DOpts& o, PdeWork& w, const double* snap,
                         const double* const ain[4]) {
  const long long NG = P.NG;
  PdeBArgs2D b;
  std::memset(&b, 0, sizeof(b));
  b.tiles = P.d_tiles; b.inst = P.d_inst; b.B = P.B;
  for (int v = 0; v < 4; ++v) b.a[v] = ain[v];
  b.mx = snap; b.my = snap + NG; b.invr = w.invr;
  b.b = w.b;
  {
    LaunchScope ls(c, KID_PDE_AUX);
    NP_DISPATCH(P.np, launch_k2_pde_b<NPV>(b, P.ntiles(), c.stream));
  }
  stage_solve_b(c, P, o, w.st, w.b, w.Pi[w.cur], w.Pi[1 - w.cur], false, w.xa, w.xb, w.db);
  w.cur = 1 - w.cur;
}

static PdeRkArgs2D pde_rk_args(const Plan2D& P, const PdeWork& w, const double* snap, bool apos) {
  const long long NG = P.NG;
  PdeRkArgs2D r;
  std::memset(&r, 0, sizeof(r));
  r.tiles = P.d_tiles; r.inst = P.d_inst; r.B = P.B;
  for (int v = 0; v < 4; ++v) r.q[v] = snap + v * NG;
  r.S = snap + 4 * NG; r.invr = w.invr; r.ws_x = w.wsx; r.ws_y = w.wsy;
  for (int v = 0; v < PDE_SRC; ++v) r.src[v] = w.src[v];
  for (int v = 0; v < PDE_NL; ++v) r.nl[v] = w.nl[v];
  r.Pi = apos ? w.Pi[w.cur] : nullptr;
  return r;
}

// One backward SSP-RK3 step over one snapshot (adjoint_pde.jl:586-608):
// a -> a1 -> a2 -> a.
static void pde_step(Ctx& c, const Plan2D& P, const Solve2DOpts& o, PdeWork& w, const double* snap, bool apos) {
  pde_prep(c, P, w, snap, apos);
  double* const* ins[3] = {w.a, w.a1, w.a2};
  double* const* outs[3] = {w.a1, w.a2, w.a};
  for (int s = 0; s < 3; ++s) {
    const double* ain[4] = {ins[s][0], ins[s][1], ins[s][2], ins[s][3]};
    if (apos) pde_pi_solve(c, P, o, w, snap, ain);
    PdeRkArgs2D r = pde_rk_args(P, w, snap, apos);
    for (int v = 0; v < 4; ++v) { r.a[v] = ain[v]; r.an[v] = w.a[v]; r.ao[v] = outs[s][v]; }
    r.c0 = RK_C0[s]; r.c1 = RK_C1[s]; r.c2 = RK_C2[s];
    LaunchScope ls(c, KID_PDE);
    NP_DISPATCH(P.np, launch_k2_pde_rk<NPV>(r, P.ntiles(), c.stream));
  }
}

static void pde_terminal(Ctx& c, const Plan2D& P, PdeWork& w, const double* snapT, int objective, const double* prm) {
  const long long NG = P.NG;
  const int ni = (int)P.inst.size();
  const double* qT[4] = {snapT, snapT + NG, snapT + 2 * NG, snapT + 3 * NG};
  ObjArgs2D a = obj_args(P, qT, objective, prm);
  double* s1 = c.ws.dbl("pde:s1", ni);
  double* s2 = c.ws.dbl("pde:s2", ni);
  if (objective == OBJ_KINETIC_ENERGY) {
    a.j1 = c.ws.dbl("obj:j1", NG);
    a.j2 = c.ws.dbl("obj:j2", NG);
    { LaunchScope ls(c, KID_OTHER); k2_obj_nodes<<<grid_for(NG), 256, 0, c.stream>>>(a); }
    inst_sums(c, P, a.j1, s1);
    inst_sums(c, P, a.j2, s2);
  }
  a.s1 = s1; a.s2 = s2;
  for (int v = 0; v < 4; ++v) a.qb[v] = w.a[v];
  LaunchScope ls(c, KID_OTHER);
  k2_pde_terminal<<<grid_for(NG), 256, 0, c.stream>>>(a);
}

// Adjoint steps n = n_hi .. n_lo + 1 over slot(n).
static void pde_steps(Ctx& c, const Plan2D& P, const Solve2DOpts& o, PdeWork& w, const SnapSlot& slot, int n_hi, int n_lo) {
  const bool apos = any_alpha_pos(P);
  for (int n = n_hi; n > n_lo; --n) pde_step(c, P, o, w, slot(n), apos);
}

static void pde_checks(const Plan2D& P, const Solve2DOpts& o, int objective, int n_steps) {
  check_objective(objective);
  check_solver(o);
  check_alpha_uniform(P);
  if (n_steps < 0) throw Error(1, "n_steps must be >= 0");
}

void pde_adjoint2d(Ctx& c, const Plan2D& P, int n_steps, const Solve2DOpts& o, int objective, const double* prm,
                   const SnapSlot& slot, double* const a_out[4]) {
  pde_checks(P, o, objective, n_steps);
  const long long NG = P.NG;
  PdeWork w = pde_work(c, P, o);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  pde_terminal(c, P, w, slot(n_steps), objective, prm);
  cuda_check(cudaMemsetAsync(w.Pi[0], 0, NG * sizeof(double), c.stream), "zero Pi");
  w.cur = 0;
  pde_steps(c, P, o, w, slot, n_steps, 0);
  for (int v = 0; v < 4; ++v)
    cuda_check(cudaMemcpyAsync(a_out[v], w.a[v], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "adjoint out");
  check_status(c);
}

void pde_adjoint_ic2d(Ctx& c, const Plan2D& Pf, const Plan2D& Pa, const double* const q0[4], int n_steps,
                      const Solve2DOpts& o, int objective, const double* prm, double* const a_out[4]) {
  pde_checks(Pa, o, objective, n_steps);
  check_alpha_uniform(Pf);
  const long long NG = Pf.NG;
  const size_t snap = (size_t)5 * NG * sizeof(double);
  size_t budget = c.tape_budget;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    const size_t avail = fr + c.ws.held("pde:snaps") + c.ws.held("pde:ckpt") + c.ws.held("pde:seg");
    const size_t reserve = (size_t)2 << 30;
    budget = avail > reserve ? avail - reserve : 0;
  }
  const int n = n_steps;
  if ((size_t)(n + 1) * snap <= budget) {  // every snapshot resident
    c.plan_seg = std::max(n, 1);
    c.plan_nseg = 1;
    double* S = c.ws.dbl("pde:snaps", (size_t)(n + 1) * 5 * NG);
    auto slot = [&](int k) { return S + (long long)k * 5 * NG; };
    forward_store_init2d(c, Pf, o, q0, slot(0));
    forward_store_range2d(c, Pf, o, slot, 0, n);
    pde_adjoint2d(c, Pa, n, o, objective, prm, slot, a_out);
    return;
  }
  // checkpoints at k = 0, K, 2K, ... and one recomputed segment of K snapshots
  int K = (int)std::ceil(std::sqrt((double)n));
  const size_t need = ((size_t)(n / K + 1) + (size_t)K + 2) * snap;
  if (need > budget) throw Error(5, "device memory too small for the snapshots of the continuous adjoint");
  const int nseg = (n + K - 1) / K;
  c.plan_seg = K;
  c.plan_nseg = nseg;
  double* ck = c.ws.dbl("pde:ckpt", (size_t)(n / K + 1) * 5 * NG);
  double* sg = c.ws.dbl("pde:seg", (size_t)(K + 2) * 5 * NG);
  auto pass1 = [&](int k) {
    return k % K == 0 ? ck + (long long)(k / K) * 5 * NG : sg + (long long)(k % 2) * 5 * NG;
  };
  forward_store_init2d(c, Pf, o, q0, pass1(0));
  forward_store_range2d(c, Pf, o, pass1, 0, n);
  pde_checks(Pa, o, objective, n);
  PdeWork w = pde_work(c, Pa, o);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  pde_terminal(c, Pa, w, pass1(n), objective, prm);
  cuda_check(cudaMemsetAsync(w.Pi[0], 0, NG * sizeof(double), c.stream), "zero Pi");
  w.cur = 0;
  for (int s = nseg - 1; s >= 0; --s) {
    const int k0 = s * K, k1 = std::min(n, k0 + K);
    auto seg = [&](int k) { return k == k0 ? ck + (long long)(k0 / K) * 5 * NG : sg + (long long)(k - k0 - 1) * 5 * NG; };
    forward_store_range2d(c, Pf, o, seg, k0, k1);
    pde_steps(c, Pa, o, w, seg, k1, k0);
  }
  for (int v = 0; v < 4; ++v)
    cuda_check(cudaMemcpyAsync(a_out[v], w.a[v], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "adjoint out");
  check_status(c);
}

void pde_adjoint_rhs2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const double* snap, double* Pi,
                       const double* const a[4], double* const da[4]) {
  check_solver(o);
  check_alpha_uniform(P);
  const long long NG = P.NG;
  const bool apos = any_alpha_pos(P);
  PdeWork w = pde_work(c, P, o);
  cuda_check(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.stream), "status reset");
  pde_prep(c, P, w, snap, apos);
  if (apos) {
    cuda_check(cudaMemcpyAsync(w.Pi[0], Pi, NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "Pi in");
    w.cur = 0;
    pde_pi_solve(c, P, o, w, snap, a);
  }
  PdeRkArgs2D r = pde_rk_args(P, w, snap, apos);
  for (int v = 0; v < 4; ++v) { r.a[v] = a[v]; r.an[v] = a[v]; r.ao[v] = nullptr; r.k_out[v] = da[v]; }
  r.c0 = 0.0; r.c1 = 1.0; r.c2 = 0.0;
  {
    LaunchScope ls(c, KID_PDE);
    NP_DISPATCH(P.np, launch_k2_pde_rk<NPV>(r, P.ntiles(), c.stream));
  }
  if (apos) cuda_check(cudaMemcpyAsync(Pi, w.Pi[w.cur], NG * sizeof(double), cudaMemcpyDeviceToDevice, c.stream), "Pi out");
  check_status(c);
}

double probe_fp64_tflops(Ctx& c) {
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device), "attr");
  double* d = c.ws.dbl("probe", 1024);
  const int grid = sms * 4, tpb = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event");
  cuda_check(cudaEventCreate(&e1), "event");
  k_dfma_probe<<<grid, tpb, 0, c.stream>>>(d, 64, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, c.stream);
    k_dfma_probe<<<grid, tpb, 0, c.stream>>>(d, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1, c.stream);
    cuda_check(cudaEventSynchronize(e1), "probe sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 2.0 * 8.0 * iters * (double)grid * tpb / (best * 1e-3) / 1e12;
}

double probe_dmma_tflops(Ctx& c) {
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device), "attr");
  double* d = c.ws.dbl("probe", 1024);
  const int grid = sms * 4, tpb = 256, iters = 2048;
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event");
  cuda_check(cudaEventCreate(&e1), "event");
  k_dmma_probe<<<grid, tpb, 0, c.stream>>>(d, 32, 1e-3, 1e-3);
  cuda_check(cudaGetLastError(), "dmma probe launch");
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, c.stream);
    k_dmma_probe<<<grid, tpb, 0, c.stream>>>(d, iters, 1e-3, 1e-3);
    cudaEventRecord(e1, c.stream);
    cuda_check(cudaEventSynchronize(e1), "probe sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double warps = (double)grid * tpb / 32.0;
  return 512.0 * 8.0 * iters * warps / (best * 1e-3) / 1e12;
}

}  // namespace igrgpu
