// Host engine shared by the C ABI: context, device workspace, 2D/1D problem
// descriptions and drivers. Not part of the public interface (see
// include/igr_gb300.h for that).
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "igr_device.cuh"

namespace igrgpu {

// Error raised by the engine; converted to an int status at the C boundary.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what);

// Named, grow-only device buffers owned by a context. Reusing the same names
// across calls keeps large tapes allocated between repeated gradient calls.
class Workspace {
 public:
  ~Workspace();
  void* get(const std::string& name, size_t bytes);
  double* dbl(const std::string& name, size_t n) { return static_cast<double*>(get(name, n * sizeof(double))); }
  void release_all();
  void release(const std::string& name);  // frees one buffer (cudaFree: waits for the device)
  size_t bytes() const;
  size_t held(const std::string& name) const;  // current capacity of one named buffer (0 if absent)

 private:
  struct Buf { void* p = nullptr; size_t n = 0; };
  std::map<std::string, Buf> bufs_;
};

// Kernel families timed by the optional per-launch CUDA-event profiler.
enum KernelId { KID_SETUP = 0, KID_APPLY, KID_HYP, KID_HYP_REV, KID_APPLY_REV, KID_SETUP_REV, KID_TAN, KID_1D, KID_OTHER,
                KID_PDE, KID_PDE_AUX, KID_COUNT };

struct Profiler {
  bool on = false;
  struct Rec { int kid; long long nodes; cudaEvent_t a, b; };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> recs;
  size_t next = 0;
  double ms[KID_COUNT] = {0};
  long long count[KID_COUNT] = {0};
  double nodes[KID_COUNT] = {0};
  cudaEvent_t get();
  void begin(cudaStream_t s, int kid, long long nodes);
  void end(cudaStream_t s);
  void harvest();   // synchronises, accumulates ms/count, recycles events
  void reset();
  ~Profiler();
};

// Launch choices that do not change results, measured on this device and
// remembered per problem shape: the 1D CTAs per instance and whether the 2D
// PCG inner products complete inside their kernels. Every candidate gives
// bitwise the same results, so tuning never changes an answer. With a cache
// path the table is read when tuning is switched on and written after every
// new entry (text: one "key<TAB>value" line per entry).
struct Autotune {
  bool on = false;
  std::string path;
  std::map<std::string, int> table;
  std::map<std::string, double> trial_ms;  // 2D sums: time of the fused trial, per key
  void load();
  void save() const;
  bool get(const std::string& key, int* v) const;
  void put(const std::string& key, int v);
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int* d_status = nullptr;      // device status word (DEV_* flags)
  std::string err;
  Workspace ws;
  size_t tape_budget = 0;       // 0: derive from free device memory
  long long launches = 0;       // kernels launched by the last call (host-side count)
  long long cur_nodes = 0;      // nodes of the plan being executed (profiler bookkeeping)
  // memory plan of the last adjoint call: instance groups, instances per group,
  // steps taped per segment and segments per group (1 = no forward recompute)
  int plan_groups = 0, plan_group_size = 0, plan_seg = 0, plan_nseg = 0;
  // 2D discrete adjoint: checkpoint slots of its revolve schedule (beyond the
  // first state) and RK step evaluations of the last group (taped and untaped)
  int plan_snapshots = 0;
  long long plan_step_evals = 0;
  int cluster1d = 0;            // 1D: CTAs per instance (0 = chosen per launch)
  int last_cluster1d = 0;       // 1D: CTAs per instance of the last launch
  bool use_graphs = true;       // replay repeated forward steps as CUDA graphs
  bool pcg_persistent = true;   // 2D untaped PCG solves of one wave of tiles in one persistent launch
  int pcg_drop_tile = -1;       // test hook for the next persistent PCG launch (igr_test_pcg_drop_tile)
  Autotune tune;
  Profiler prof;
};

// Launch bookkeeping: count (and, when profiling, time) one kernel launch.
struct LaunchScope {
  Ctx& c;
  LaunchScope(Ctx& cc, int kid) : c(cc) { if (c.prof.on) c.prof.begin(c.stream, kid, c.cur_nodes); }
  ~LaunchScope() { ++c.launches; if (c.prof.on) c.prof.end(c.stream); }
};

// Basis arrays as the reference stores them: xi, w (n) and D (n x n, Julia
// column-major, D[i + k*n] = D[i,k]).
BasisDev make_basis_dev(int p, const double* xi, const double* w, const double* D_colmajor);

enum Solver { SOLVER_PCG = 0, SOLVER_JACOBI = 1, SOLVER_CHEBYSHEV = 2 };
enum Objective2D { OBJ_L2_DENSITY = 0, OBJ_L2_PRESSURE = 1, OBJ_KINETIC_ENERGY = 2, OBJ_WINDOWED_KE = 3,
                   OBJ_WEIGHTED_MOMENTUM = 4, OBJ_WINDOW_RHO2 = 5, OBJ_INTERVAL_RHO = 6 };

// One 2D instance as described by the caller.
struct Inst2DDesc {
  int nex, ney;
  double lx, ly, gamma, alpha, dt;
};

// Device-side plan of a batch group: instances, tiles, node counts.
struct Plan2D {
  BasisDev B;
  int np = 4;
  std::vector<Inst2D> inst;
  std::vector<Tile2D> tiles;
  std::vector<long long> inst_nodes;
  long long NG = 0;
  Inst2D* d_inst = nullptr;
  Tile2D* d_tiles = nullptr;
  std::vector<TileGroup> groups;   // TILE_GROUP tiles per entry, per instance
  TileGroup* d_groups = nullptr;
  int ntiles() const { return (int)tiles.size(); }
  int ngroups() const { return (int)groups.size(); }
};

Plan2D make_plan2d(Ctx& c, const BasisDev& B, const std::vector<Inst2DDesc>& insts, const std::string& tag);

// Drivers. Field pointers are device pointers to NG doubles each, in the
// instance-major Julia layout.
struct Solve2DOpts { int n_iter = 10; int solver = SOLVER_PCG; };
// FP64 fields (of NG nodes) one taped RK stage holds for this solver setup.
int stage_fields2d(const Solve2DOpts& o, bool alpha_pos, long long NG, int ni);

// In-place forward over n_steps fixed steps (dt per instance), Sigma in/out
// (warm start carried across stages and steps as forward.jl:41-75 does).
void forward2d(Ctx& c, const Plan2D& P, double* const q[4], double* Sig, int n_steps, const Solve2DOpts& o);
// Coupled primal + tangent SSP-RK3 (run_sensitivity, sensitivity.jl:353-413):
// q and the tangent s in place; Sigma and varsigma zeroed at entry and
// returned for the final state. s_gamma adds the direct dP/dgamma source.
void sensitivity2d(Ctx& c, const Plan2D& P, double* const q[4], double* Sig, double* const s[4], double* vs, int n_steps,
                   const Solve2DOpts& o, double s_gamma);
// One elliptic solve (solve_elliptic!, elliptic.jl:413-427) with Sigma as warm
// start. Instances with alpha <= 0 are skipped (Sigma unchanged), as the RK
// stages and the final solve of run_forward! do, unless `always` (the
// stand-alone solve_elliptic!, which has no alpha test).
void solve_elliptic2d(Ctx& c, const Plan2D& P, const double* const q[4], double* Sig, const Solve2DOpts& o,
                      bool always = false);
// compute_igr_rhs! (elliptic.jl:159-197) into b and compute_sip_diagonal
// (elliptic.jl:205-264) into M; either may be null.
void igr_rhs_diag2d(Ctx& c, const Plan2D& P, const double* const q[4], double* b, double* M);
// compute_igr_euler_rhs! (forward.jl:22-31): the Sigma solve (warm start in
// Sig, result out) when alpha > 0, else Sigma = 0; then the DG RHS into k.
void igr_euler_rhs2d(Ctx& c, const Plan2D& P, const double* const q[4], double* Sig, double* const k[4],
                     const Solve2DOpts& o);
// cg_fixed! (fixed, maxiter = n_iter) or cg_solve! (tolerance tol) on
// A(rho, alpha) x = b for one instance, x the initial guess in and the
// solution out (elliptic.jl:278-320 with apply_A! = apply_sip!). Returns the
// iteration count the reference returns.
int cg2d(Ctx& c, const Plan2D& P, const double* rho, const double* b, double* x, double tol, int maxiter, bool fixed);
// One hyperbolic RHS evaluation (compute_hyperbolic_rhs!, hyperbolic.jl:27).
void hyperbolic_rhs2d(Ctx& c, const Plan2D& P, const double* const q[4], const double* Sig, double* const k[4]);
// y = A x (apply_sip!, elliptic.jl:30).
void apply_sip2d(Ctx& c, const Plan2D& P, const double* x, const double* rho, double* y);

// Checkpoint schedule of a 2D adjoint over NG nodes with F taped fields per
// stage: RK steps taped at once (w), checkpoint slots beyond the initial state
// and forward step evaluations (w = 0: not even one taped step fits).
struct RevolvePlan { int w = 0, slots = 0; long long evals = 0; };
RevolvePlan adjoint_checkpoints2d(Ctx& c, long long NG, int F, int n_steps);

// Gradient of the objective after n_steps fixed steps (enzyme_adjoint_ic,
// enzyme_adjoint.jl:270): J[inst], dq0 (4 fields), dgamma[inst], dalpha[inst].
void adjoint2d(Ctx& c, const Plan2D& P, const double* const q0[4], int n_steps, const Solve2DOpts& o, int objective,
               const double* obj_params, double* J, double* const dq0[4], double* dgamma, double* dalpha);

// ---- 1D ---------------------------------------------------------------------
struct Inst1DDesc {
  int ne;
  double L, gamma, alpha, dt;
  int n_steps;
  double t_end = 0.0;  // tangent only: final time of the `while t < T` stepping
  double h = 0.0;      // continuous adjoint only: the backward step min(dt, T)
};
// A batch of 1D instances. State layout on the device: instance i's block of
// 3 N_i doubles (mu, rho, E) starts at 3 * inst[i].off; Sigma at inst[i].off.
struct Plan1D {
  BasisDev B;
  int np = 4;
  std::vector<Inst1D> inst;
  std::vector<long long> inst_nodes;
  std::vector<int> order;      // launch order (largest work first)
  long long NG = 0;            // total nodes
  long long scratch = 0;       // scratch doubles
  Inst1D* d_inst = nullptr;
  int* d_order = nullptr;
};
// scratch_fields(desc, N): scratch fields (of N doubles) the instance needs.
Plan1D make_plan1d(Ctx& c, const BasisDev& B, const std::vector<Inst1DDesc>& insts,
                   const std::function<long long(const Inst1DDesc&, int)>& scratch_fields, const std::string& tag);
long long forward1d_scratch_fields(const Inst1DDesc& d, int N);
// run_forward! (IGR_adjoints_1d/forward.jl:50-87) for every instance: n_steps
// steps of size dt each (the caller re-rounds dt), final solve when asked.
void forward1d(Ctx& c, const Plan1D& P, double* q, double* sig, const Solve2DOpts& o, bool final_solve);
long long tangent1d_scratch_fields(const Inst1DDesc& d, int N);
// run_sensitivity (IGR_adjoints_1d/sensitivity.jl:401-515) for every
// instance: q and the tangent s in place, Sigma and varsigma out; form = 1 or 2
// selects the tangent elliptic source; s_gamma the direct dP/dgamma source.
void tangent1d(Ctx& c, const Plan1D& P, double* q, double* s, double* sig, double* vs, const Solve2DOpts& o, int form,
               double s_gamma);
// Snapshot segment length of the 1D adjoint for this batch within `budget` bytes.
int adjoint1d_segment(const std::vector<Inst1DDesc>& insts, int np, const Solve2DOpts& o, size_t budget);
long long adjoint1d_scratch_fields(const Inst1DDesc& d, int N, const Solve2DOpts& o, int seg);
// Gradient of the objective after each instance's n_steps fixed steps
// (enzyme_adjoint_ic, IGR_adjoints_1d/enzyme_adjoint.jl:267-314, in
// conservative variables): J, dq0 (same layout as q0), dgamma, dalpha.
void adjoint1d(Ctx& c, const Plan1D& P, const double* q0, double* dq0, const Solve2DOpts& o, int objective,
               const double* prm, int seg, double* J, double* dgamma, double* dalpha);

// One operator evaluation per instance of a 1D batch (k1_ops, one CTA or
// cluster per instance): op is one of OP1_APPLY_SIP, OP1_IGR_RHS, OP1_SOLVE,
// OP1_HYP_RHS, OP1_EULER_RHS, OP1_CG (igr1d_ops_kernels.cuh, which lists the
// fields each reads and writes). For OP1_CG returns the first instance's
// iteration count (cg_solve! / cg_fixed!); otherwise 0.
long long ops1d_scratch_fields(const Inst1DDesc& d, int N);
int ops1d(Ctx& c, const Plan1D& P, int op, const Solve2DOpts& o, const double* q, const double* rho, const double* b,
          double* x, double* sig, double* out, double* diag, double tol, int maxiter, bool fixed);

// ---- continuous adjoint (IGR_adjoints_2d/adjoint_pde.jl, forward.jl:111-158) ----
// Snapshot k of the forward store: 5 fields of NG doubles (mux, muy, rho, E,
// Sigma) at a device address given by the caller's slot function.
using SnapSlot = std::function<double*(int)>;
// run_forward_store steps k0+1..k1: snapshot k0 must hold a state and its
// Sigma; every step is followed by one more Sigma solve on the new state,
// which is stored and is the next step's warm start. P carries the
// (re-rounded) forward dt.
void forward_store_range2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const SnapSlot& slot, int k0, int k1);
// Snapshot 0: q0 and the initial Sigma solve from zero (forward.jl:127-130).
void forward_store_init2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const double* const q0[4], double* snap0);
// run_adjoint_conservative (adjoint_pde.jl:527-611) over snapshots 0..n_steps
// given by slot (each called once per adjoint step, n_steps first; a slot may
// upload the snapshot on the way). P carries the adjoint step min(dt, T).
void pde_adjoint2d(Ctx& c, const Plan2D& P, int n_steps, const Solve2DOpts& o, int objective, const double* prm,
                   const SnapSlot& slot, double* const a_out[4]);
// Forward store + adjoint with device-resident snapshots: all of them when they
// fit in the memory budget, else checkpoints every K steps and a recomputed
// segment of K snapshots at a time (c.plan_seg = K, c.plan_nseg = segments).
void pde_adjoint_ic2d(Ctx& c, const Plan2D& Pf, const Plan2D& Pa, const double* const q0[4], int n_steps,
                      const Solve2DOpts& o, int objective, const double* prm, double* const a_out[4]);
// compute_adjoint_rhs_conservative! (adjoint_pde.jl:481-516): da from a at
// the state (q, Sigma); Pi is the warm start and returns the new Pi.
void pde_adjoint_rhs2d(Ctx& c, const Plan2D& P, const Solve2DOpts& o, const double* snap, double* Pi,
                       const double* const a[4], double* const da[4]);

// 1D continuous adjoint (IGR_adjoints_1d/adjoint_pde.jl, forward.jl:137-186),
// one persistent kernel per instance. Instance n_steps = ceil(T/dt), dt the
// re-rounded forward step, h the backward step. mode 0: store + adjoint (q0 ->
// a0, snapshots in scratch: all when seg >= n_steps, else checkpoints every
// seg steps); 1: store only (q0 -> snaps); 2: adjoint only (snaps -> a0);
// 3: one adjoint-operator evaluation (q0 = (mu, rho, E, Sigma) per instance at
// 4 off_i, ain -> a0 = k, pi in/out).
long long pde1d_scratch_fields(const Inst1DDesc& d, int N, int mode, int seg);
int pde1d_segment(const std::vector<Inst1DDesc>& insts, int np, size_t budget);
void pde_adjoint1d(Ctx& c, const Plan1D& P, int mode, const double* q0, const double* ain, double* a0, double* pi,
                   double* snaps, const long long* snap_off_dev, const Solve2DOpts& o, int objective, const double* prm,
                   int seg);

// Initial-condition builders (IGR_adjoints_2d/initial_conditions.jl:15-232;
// 1D :94-204) for every instance of a plan; amps: per-instance amplitude A
// (host); params: the builder's keyword arguments (nullptr = the reference's
// defaults). 2D types: 0 constant, 1 isentropic vortex, 2 Taylor-Green,
// 3 Sedov blast, 4 Oseen pair + blast; 1D: 0 acoustic, 1 entropy wave,
// 2 density, 3 pressure, 4 velocity pulse. q: device fields (2D: 4 of NG;
// 1D: the batch layout).
int ic2d_param_count(int type);
void build_ic2d(Ctx& c, const Plan2D& P, int type, const double* amps, const double* params, double* const q[4]);
void build_ic1d(Ctx& c, const Plan1D& P, int type, const double* amps, double* q);
// l2_error (initial_conditions.jl:74-87) over all nodes of the plan.
double l2_error2d(Ctx& c, const Plan2D& P, const double* u, const double* r);

double probe_fp64_tflops(Ctx& c);
// FP64 tensor-core (mma.sync m8n8k4 f64) throughput in TFLOP/s.
double probe_dmma_tflops(Ctx& c);
// y = 1 / x elementwise on stream s (no bookkeeping).
void launch_recip(const double* x, double* y, long long n, cudaStream_t s);

// Objective value only (the primal of the adjoint call), final state in q.
void objective2d(Ctx& c, const Plan2D& P, double* const q[4], int n_steps, const Solve2DOpts& o, int objective,
                 const double* obj_params, double* J);

}  // namespace igrgpu
