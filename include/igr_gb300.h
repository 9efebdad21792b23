/*
 * igr_gb300.h — C ABI of the GB300 engine for the IGR-regularised Euler
 * forward map and its derivatives (f-t-s/IGR_sensitivities).
 *
 * Every entry point is a drop-in for one function of the reference's Julia
 * module API (IGRAdjoints2D / IGRAdjoints1D); the file:line of the function
 * it replaces is given beside it.
 *
 * Conventions
 *  - Arrays are caller-owned host arrays of double in the reference's Julia
 *    column-major layout: 2D fields are (n_p, n_p, N_ex, N_ey) with the x-node
 *    index fastest; 1D fields are (n_p, N_e). Entry points ending in `_dev`
 *    take device pointers instead.
 *  - The basis is passed as the reference stores it in DGBasis
 *    (IGR_adjoints_2d/basis.jl:7-12): xi and w of length p+1 and D as a
 *    (p+1) x (p+1) column-major matrix, so results use the caller's exact
 *    node and weight values. p must be 1..4.
 *  - Solvers: 0 = :pcg, 1 = :jacobi, 2 = :chebyshev (elliptic.jl:417-425).
 *  - Every function returns an igr_status; on failure igr_last_error(ctx)
 *    holds a message. Unknown solver/objective symbols give IGR_EINVAL with
 *    the reference's error text.
 *  - A context owns a CUDA stream and device buffers; it is not thread-safe.
 *    Use one context per host thread.
 */
#ifndef IGR_GB300_H
#define IGR_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  IGR_OK = 0,
  IGR_EINVAL = 1,      /* bad argument: unknown solver/objective, bad sizes */
  IGR_EUNSUPPORTED = 2,/* valid request this build does not implement */
  IGR_ENONFINITE = 3,  /* NaN/Inf or rho <= 0 appeared in the state */
  IGR_ECUDA = 4,       /* CUDA runtime error */
  IGR_ENOMEM = 5,      /* device memory too small */
  IGR_ETIMEOUT = 6     /* a bounded device-side wait gave up */
} igr_status;

typedef struct igr_ctx igr_ctx;

/* Objectives of enzyme_adjoint_ic (enzyme_objective_fn, IGR_adjoints_2d/enzyme_adjoint.jl:240-254)
 * plus nodal-window extensions. */
typedef enum {
  IGR_OBJ_L2_DENSITY = 0,          /* :l2_density, enzyme_adjoint.jl:48-82 */
  IGR_OBJ_L2_PRESSURE = 1,         /* :l2_pressure, enzyme_adjoint.jl:84-119 */
  IGR_OBJ_KINETIC_ENERGY = 2,      /* :kinetic_energy, enzyme_adjoint.jl:121-156 */
  IGR_OBJ_WINDOWED_KE = 3,         /* :windowed_kinetic_energy, enzyme_adjoint.jl:160-195 */
  IGR_OBJ_WEIGHTED_MOMENTUM = 4,   /* :weighted_momentum, enzyme_adjoint.jl:199-229 */
  IGR_OBJ_WINDOW_RHO2 = 5,         /* sum w_i w_j Jx Jy rho^2 over nodes inside the square
                                      [x0, x0+s] x [y0, y0+s]; obj_params = {x0, y0, s} */
  IGR_OBJ_INTERVAL_RHO = 6         /* 1D: sum w_i J rho over nodes in [a, b]; obj_params = {a, b} */
} igr_objective;

/* Discretisation of one 2D instance: DGBasis + CartesianMesh2D
 * (IGR_adjoints_2d/basis.jl:7-12, mesh.jl:89-125). */
typedef struct {
  int p;
  int n_ex, n_ey;
  double lx, ly;
  const double* xi; /* p+1 */
  const double* w;  /* p+1 */
  const double* D;  /* (p+1)^2, column-major */
} igr_disc2d;

/* Discretisation of one 1D instance: DGBasis + PeriodicMesh1D
 * (IGR_adjoints_1d/basis.jl, mesh.jl:7-33). */
typedef struct {
  int p;
  int n_e;
  double L;
  const double* xi; /* p+1 */
  const double* w;  /* p+1 */
  const double* D;  /* (p+1)^2, column-major */
} igr_disc1d;

/* ---- context -------------------------------------------------------------- */
int igr_ctx_create(int device, igr_ctx** out);
int igr_ctx_destroy(igr_ctx* ctx);
const char* igr_last_error(const igr_ctx* ctx);
/* Device bytes the adjoint may use for its tape; 0 (default) = most of the
 * free memory. A batch runs as groups of instances whose full tapes fit the
 * budget together; an instance whose tape alone exceeds it runs by itself
 * with segment checkpointing. */
int igr_set_tape_budget(igr_ctx* ctx, size_t bytes);
/* 1D: CTAs that advance one instance (a thread-block cluster when > 1):
 * 0 (default) = chosen per launch (small batches spread each instance over up
 * to 16 SMs); 1, 2, 4, 8 or 16 force it. Results do not depend on it.
 * No reference counterpart. */
int igr_set_cluster_size_1d(igr_ctx* ctx, int cs);
/* 2D forward and tangent solves: replay the repeated RK steps as CUDA graphs
 * (1, default) or launch every kernel from the host (0). Results are bitwise
 * the same. No reference counterpart. */
int igr_set_graphs(igr_ctx* ctx, int on);
/* 2D untaped PCG solves (forward, tangent, stand-alone and continuous-adjoint
 * solves) whose tiles fit one wave of resident CTAs: one persistent
 * cooperative launch per solve, whose CTAs hand each inner product on within
 * each instance (1, default), or two kernels per iteration (0). Results are
 * bitwise the same. A hand-off that waits past its time limit (1 s) makes the
 * call return IGR_ETIMEOUT. No reference counterpart. */
int igr_set_pcg_persistent(igr_ctx* ctx, int on);
/* Test hook for the timeout path. The next persistent PCG launch on this
 * context runs with the CTA of tile `tile` (plan order) leaving before its
 * first p.Ap hand-off, as a CTA that stopped early would. The instance's other
 * CTAs give up after 1 s, the call returns IGR_ETIMEOUT and the context stays
 * usable. Nothing faults or hangs. -1 clears it. No reference counterpart. */
int igr_test_pcg_drop_tile(igr_ctx* ctx, int tile);
/* Autotuning of launch choices that leave results bitwise unchanged: the 1D
 * CTAs per instance (when not forced by igr_set_cluster_size_1d) and whether
 * the 2D PCG inner products complete inside their kernels. on = 1 measures
 * the candidates on the first call of each batch shape (CUDA events) and
 * keeps the fastest; cache_path (NULL or "" = memory only) is read now and
 * rewritten after every new entry, so later processes skip the measurement;
 * IGR_EINVAL if it cannot be written (tuning then stays in memory).
 * No reference counterpart. */
int igr_set_autotune(igr_ctx* ctx, int on, const char* cache_path);
/* Entries in the context's autotune table. */
int igr_autotune_count(const igr_ctx* ctx, int* n);
/* CTAs per instance used by the last 1D launch on this context. */
int igr_last_cluster_size_1d(const igr_ctx* ctx, int* out);
/* Kernels launched by the last call on this context. */
int igr_last_launch_count(const igr_ctx* ctx, long long* out);

/* Per-launch CUDA-event timing of the engine's kernel families (no reference
 * counterpart; used by the benchmark for live kernel durations). Families:
 * 0 setup, 1 SIP apply (solver iteration), 2 hyperbolic+RK, 3 hyperbolic
 * reverse, 4 SIP apply reverse, 5 setup reverse, 6 tangent, 7 1D, 8 other,
 * 9 continuous-adjoint operator (k2_pde_rk), 10 continuous-adjoint per-step
 * preparation and Pi source (k2_pde_prep, k2_pde_b). */
int igr_profile_enable(igr_ctx* ctx, int on);
int igr_profile_reset(igr_ctx* ctx);
int igr_profile_read(igr_ctx* ctx, int kernel_family, double* total_ms, long long* launches);
/* Nodes processed by the timed launches of a family (sum over launches). */
int igr_profile_nodes(igr_ctx* ctx, int kernel_family, double* nodes);
/* Memory plan of the last adjoint call: instance groups run one after the
 * other, instances per group, RK steps taped per segment and segments per
 * group (segments > 1 means the forward is recomputed from checkpoints). */
int igr_last_adjoint_plan(const igr_ctx* ctx, int* groups, int* group_size, int* segment_steps, int* segments);
/* Checkpoint schedule of the last 2D discrete adjoint (its last instance
 * group): RK steps taped at once, checkpoint slots beyond the initial state,
 * and the RK step evaluations of the forward sweeps (n_steps when the whole
 * tape fits; more when states are recomputed from checkpoints). The schedule
 * is binomial (revolve) over super-steps of tape_steps steps: with s slots and
 * r re-runs it reverses up to C(s + r, s) super-steps. No reference
 * counterpart (the reference's Enzyme call keeps the whole trajectory). */
int igr_last_checkpoint_schedule(const igr_ctx* ctx, int* tape_steps, int* snapshots, long long* step_evaluations);
/* Measured FP64 FMA throughput of the device in TFLOP/s (the roofline
 * denominator of this FP64-bound path; no reference counterpart). */
int igr_probe_fp64_peak(igr_ctx* ctx, double* tflops);
/* Measured FP64 tensor-core throughput (mma.sync m8n8k4 f64, 512 flops per
 * warp instruction) in TFLOP/s, beside the FMA figure above (no reference
 * counterpart). */
int igr_probe_fp64_tensor_peak(igr_ctx* ctx, double* tflops);

/* ---- 2D ------------------------------------------------------------------- */

/* run_forward! (IGR_adjoints_2d/forward.jl:41-75): in place, Sigma zeroed at
 * entry, n_steps = ceil(T/dt), dt = T/n_steps, final solve at T when alpha > 0. */
int igr2d_run_forward(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                      int n_iter, int solver, double* mux, double* muy, double* rho, double* E, double* sigma);

/* run_sensitivity (IGR_adjoints_2d/sensitivity.jl:353-413): the coupled
 * primal + tangent SSP-RK3 to time T, in place. On entry (mux..E) is the
 * initial state and (zetax, zetay, srho, eta) its tangent direction; on exit
 * both are at T, with sigma = Sigma(T) and varsigma = its tangent. Same dt
 * re-rounding as run_forward!. s_gamma != 0 adds the direct dP/dgamma source
 * s_gamma * rho e to the tangent pressure, as the 1D package does
 * (IGR_adjoints_1d/sensitivity.jl:36-41); the 2D reference has none (pass 0). */
int igr2d_run_sensitivity(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                          int n_iter, int solver, double s_gamma, double* mux, double* muy, double* rho, double* E,
                          double* sigma, double* zetax, double* zetay, double* srho, double* eta, double* varsigma);

/* Batched run_sensitivity over instances sharing one mesh, each with its own
 * gamma, alpha and dt, for n_steps fixed steps (no dt re-rounding; a caller
 * wanting run_sensitivity's semantics passes n_steps = ceil(T/dt) and
 * dt = T/n_steps). q and s are [n_inst][4][N] (mux, muy, rho, E and their
 * tangents), in place; sigma and varsigma are [n_inst][N] out. s_gamma is
 * shared by the batch (the direct dP/dgamma source; 1 with s = 0 gives the
 * state's derivative with respect to gamma at frozen LLF wave speed). */
int igr2d_sensitivity_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                            const double* dts, int n_steps, int n_iter, int solver, double s_gamma, double* q,
                            double* s, double* sigma, double* varsigma);

/* enzyme_adjoint_ic (IGR_adjoints_2d/enzyme_adjoint.jl:270-296): J and
 * dJ/dq0 of the objective after n_steps SSP-RK3 steps of size dt (no dt
 * re-rounding, Sigma warm start from zero). dgamma/dalpha (may be NULL) are
 * dJ/dgamma and dJ/dalpha, which the reference does not compute. */
int igr2d_adjoint_ic(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_steps, double dt,
                     int n_iter, int solver, int objective, const double* obj_params, const double* mux0,
                     const double* muy0, const double* rho0, const double* E0, double* J, double* dmux0,
                     double* dmuy0, double* drho0, double* dE0, double* dgamma, double* dalpha);

/* Batched enzyme_adjoint_ic: n_inst instances on one mesh, each with its own
 * gamma, alpha, dt and initial state. q0 and dq0 are [n_inst][4][N] with the
 * variables ordered (mux, muy, rho, E); J, dgamma, dalpha are [n_inst]. */
int igr2d_adjoint_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                        const double* dts, int n_steps, int n_iter, int solver, int objective,
                        const double* obj_params, const double* q0, double* J, double* dq0, double* dgamma,
                        double* dalpha);
/* Batched enzyme_adjoint_ic over instances with their own meshes (n_ex, n_ey,
 * lx, ly), gamma, alpha and dt, sharing the basis and the step count: one
 * launch per kernel covers the tiles of every instance of a group. q0 / dq0
 * are the concatenation over instances of [4][N_i] blocks,
 * N_i = (p+1)^2 n_ex[i] n_ey[i]. Results equal the single-instance calls. */
int igr2d_adjoint_batch_meshes(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                               const int* n_ex, const int* n_ey, const double* lx, const double* ly,
                               const double* gammas, const double* alphas, const double* dts, int n_steps, int n_iter,
                               int solver, int objective, const double* obj_params, const double* q0, double* J,
                               double* dq0, double* dgamma, double* dalpha);
/* The memory plan igr2d_adjoint_batch would use for n_inst instances of d
 * with this step count and solver, without running it: instances per group,
 * RK steps taped at once, checkpoint slots beyond the initial state and the
 * forward step evaluations of its revolve schedule (per group, an upper bound
 * when tape_steps does not divide n_steps; n_steps means no recomputation).
 * Reads the free device memory or the tape budget. No reference counterpart. */
int igr2d_adjoint_plan(igr_ctx* ctx, const igr_disc2d* d, int n_inst, int n_steps, int n_iter, int solver, double alpha,
                       int* group_size, int* tape_steps, int* snapshots, long long* step_evaluations);
/* Same with q0 and dq0 in device memory (J, dgamma, dalpha stay host arrays). */
int igr2d_adjoint_batch_dev(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas,
                            const double* alphas, const double* dts, int n_steps, int n_iter, int solver,
                            int objective, const double* obj_params, const double* q0_dev, double* J,
                            double* dq0_dev, double* dgamma, double* dalpha);

/* Primal of the objective only (the `result[2]` of enzyme_adjoint_ic). */
int igr2d_objective(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_steps, double dt,
                    int n_iter, int solver, int objective, const double* obj_params, double* mux, double* muy,
                    double* rho, double* E, double* J);

/* apply_sip! (IGR_adjoints_2d/elliptic.jl:30-145): y = A(rho, alpha) x. */
int igr2d_apply_sip(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* x, const double* rho, double* y);

/* compute_hyperbolic_rhs! (IGR_adjoints_2d/hyperbolic.jl:27-119). */
int igr2d_hyperbolic_rhs(igr_ctx* ctx, const igr_disc2d* d, double gamma, const double* mux, const double* muy,
                         const double* rho, const double* E, const double* sigma, double* dmux, double* dmuy,
                         double* drho, double* dE);

/* solve_elliptic! (IGR_adjoints_2d/elliptic.jl:413-427): sigma is the warm
 * start on entry and the solution on exit (for any alpha, as the reference's
 * solve has no alpha test). */
int igr2d_solve_elliptic(igr_ctx* ctx, const igr_disc2d* d, double alpha, int n_iter, int solver,
                         const double* mux, const double* muy, const double* rho, const double* E, double* sigma);

/* compute_igr_euler_rhs! (IGR_adjoints_2d/forward.jl:15-31, both methods):
 * the full IGR Euler operator. When alpha > 0, sigma is the warm start of one
 * solve_elliptic! and holds its result on return; otherwise sigma is set to
 * zero. Then (dmux, dmuy, drho, dE) = compute_hyperbolic_rhs! at
 * (mux, muy, rho, E, sigma). */
int igr2d_igr_euler_rhs(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_iter, int solver,
                        const double* mux, const double* muy, const double* rho, const double* E, double* sigma,
                        double* dmux, double* dmuy, double* drho, double* dE);

/* compute_igr_rhs! (IGR_adjoints_2d/elliptic.jl:159-197): the IGR source b
 * = w_i w_j Jx Jy alpha [(u_x + v_y)^2 + u_x^2 + 2 u_y v_x + v_y^2]. E is part
 * of the reference's argument list and is not read. */
int igr2d_igr_rhs(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* mux, const double* muy,
                  const double* rho, const double* E, double* b);

/* compute_sip_diagonal (IGR_adjoints_2d/elliptic.jl:205-264): M = diag(A). */
int igr2d_sip_diagonal(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, double* M);

/* cg_solve! (IGR_adjoints_2d/elliptic.jl:278-297) with apply_A! = apply_sip!
 * at (rho, alpha), as the reference's manufactured-solution test calls it
 * (tests/run_euler_test.jl:64-65): unpreconditioned CG from the initial guess
 * x (solution on return) that stops before iteration `it` (1-based) at the
 * first it with sqrt(r.r) < tol; *iters = that it, or maxiter. */
int igr2d_cg_solve(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, const double* b, double* x,
                   double tol, int maxiter, int* iters);

/* cg_fixed! (IGR_adjoints_2d/elliptic.jl:304-320) with apply_A! = apply_sip!:
 * n_iter CG iterations with the reference's 1e-30 guards, x in place. */
int igr2d_cg_fixed(igr_ctx* ctx, const igr_disc2d* d, double alpha, const double* rho, const double* b, double* x,
                   int n_iter);

/* y = A(rho, alpha) x like igr2d_apply_sip, for callers that cannot let this
 * library allocate device memory: hosts whose GPU memory belongs to another
 * allocator (a Julia CUDA.jl pool, a framework's caching allocator with a
 * fixed budget) or that cannot afford a synchronising cudaMalloc in their
 * loop. No counterpart in the reference. x_dev, rho_dev and y_dev are device
 * pointers; stream may be NULL (default stream); the call returns after the
 * result is complete. It allocates nothing: its scratch is a fixed device
 * array of about 4.8 MB, so it accepts at most 65,536 nodes
 * ((p+1)^2 n_ex n_ey, any mesh shape) and returns IGR_EINVAL above that. All
 * calls share that array, so calls that overlap on the GPU race. With CUDA's
 * lazy module loading the first call on each device loads the library's
 * kernels there, which reserves the array then: make that first call during
 * set-up. The first call on each device (and the first after the device's
 * context was reset) looks up the array's address. The call synchronises its
 * stream before it returns, so it cannot be recorded into a CUDA graph: on a
 * stream that is capturing it returns IGR_EINVAL without touching the stream. */
int igr2d_apply_sip_noalloc(const igr_disc2d* d, double alpha, const double* x_dev, const double* rho_dev,
                            double* y_dev, void* stream);

/* Batched run_forward! on one mesh: n_inst instances with their own gamma,
 * alpha and dt advance n_steps fixed SSP-RK3 steps together (the caller
 * re-rounds: n_steps = ceil(T/dt), dt = T/n_steps reproduces run_forward!);
 * Sigma starts at zero; final_solve != 0 adds the solve at the final state
 * (forward.jl:71-73). q: (n_inst, 4, N) in place; sigma: (n_inst, N) out.
 * Used for finite-difference stencils of parameter sweeps. No counterpart in
 * the reference. */
int igr2d_forward_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas, const double* alphas,
                        const double* dts, int n_steps, int n_iter, int solver, int final_solve, double* q,
                        double* sigma);

/* ---- 2D continuous adjoint (optimise-then-discretise) ---------------------- */

/* run_forward_store (IGR_adjoints_2d/forward.jl:111-158): the forward with
 * n_steps = ceil(T/dt), dt = T/n_steps, and one more Sigma solve after every
 * step (and at t = 0), whose result is stored and is the next step's warm
 * start. snapshots: (n_steps + 1) x 5 x N doubles, snapshot k (k = 0..n_steps,
 * the state after step k) = (mux, muy, rho, E, Sigma); snapshots_len must
 * equal (ceil(T/dt) + 1) * 5 * N. The step count is returned in *n_steps. */
int igr2d_run_forward_store(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt, double t_end,
                            int n_iter, int solver, const double* mux0, const double* muy0, const double* rho0,
                            const double* E0, double* snapshots, long long snapshots_len, int* n_steps);

/* run_adjoint_conservative (IGR_adjoints_2d/adjoint_pde.jl:527-611): the
 * adjoint PDE integrated backward with SSP-RK3 from the L2 gradient of the
 * objective at T, step n using snapshot n for all three stages, step
 * min(dt, T), one SIP solve for Pi per stage (warm-started, from zero at T).
 * snapshots as igr2d_run_forward_store writes them (snapshots_len >=
 * (n_steps + 1) * 5 * N). Objectives: IGR_OBJ_L2_DENSITY, _L2_PRESSURE,
 * _KINETIC_ENERGY, _WINDOWED_KE, _WEIGHTED_MOMENTUM (adjoint_pde.jl:542-584)
 * and IGR_OBJ_WINDOW_RHO2 (no reference counterpart). Output: the adjoint
 * (a_mux, a_muy, a_rho, a_E) at t = 0. */
int igr2d_run_adjoint_conservative(igr_ctx* ctx, const igr_disc2d* d, const double* snapshots, long long snapshots_len,
                                   int n_steps, double dt, double t_end, double gamma, double alpha, int n_iter,
                                   int objective, int solver, const double* obj_params, double* amux, double* amuy,
                                   double* arho, double* aE);

/* run_forward_store followed by run_adjoint_conservative (the pairing of
 * IGR_adjoints_2d/tests/run_adjoint_test.jl:59-62) with the snapshots kept on
 * the device: all of them when they fit, else checkpoints every K steps and
 * one recomputed K-step segment at a time (igr_last_adjoint_plan reports K
 * and the segment count). dt is the caller's step: the forward re-rounds it,
 * the adjoint steps by min(dt, T), as the two reference calls do. */
int igr2d_adjoint_conservative_ic(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, double dt,
                                  double t_end, int n_iter, int solver, int objective, const double* obj_params,
                                  const double* mux0, const double* muy0, const double* rho0, const double* E0,
                                  double* amux, double* amuy, double* arho, double* aE);

/* Batched igr2d_adjoint_conservative_ic: n_inst instances on one mesh, each
 * with its own gamma, alpha, dt and initial state, one final time T for all;
 * ceil(T/dt[i]) must be the same for every instance. q0 and a0: (n_inst, 4, N)
 * doubles, instance-major. No counterpart in the reference. */
int igr2d_adjoint_conservative_batch(igr_ctx* ctx, const igr_disc2d* d, int n_inst, const double* gammas,
                                     const double* alphas, const double* dts, double t_end, int n_iter, int solver,
                                     int objective, const double* obj_params, const double* q0, double* a0);

/* compute_adjoint_rhs_conservative! (IGR_adjoints_2d/adjoint_pde.jl:481-516):
 * the adjoint operator at the state (q, sigma) applied to a: the local DG
 * part (adjoint flux with LLF, local source) plus, when alpha > 0, the
 * nonlocal source of one Pi solve (pi: warm start in, solution out). */
int igr2d_adjoint_rhs_conservative(igr_ctx* ctx, const igr_disc2d* d, double gamma, double alpha, int n_iter,
                                   int solver, const double* mux, const double* muy, const double* rho,
                                   const double* E, const double* sigma, double* pi, const double* amux,
                                   const double* amuy, const double* arho, const double* aE, double* damux,
                                   double* damuy, double* darho, double* daE);

/* ---- 1D ------------------------------------------------------------------- */

/* run_forward! (IGR_adjoints_1d/forward.jl:50-87): in place, Sigma zeroed at
 * entry, n_steps = ceil(T/dt), dt = T/n_steps, final solve at T when alpha > 0.
 * State ordering (mu, rho, E) as IGR_adjoints_1d/euler.jl:23. */
int igr1d_run_forward(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                      int n_iter, int solver, double* mu, double* rho, double* E, double* sigma);

/* apply_sip! (IGR_adjoints_1d/elliptic.jl:32-116): y = A(rho, alpha) x. */
int igr1d_apply_sip(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* x, const double* rho, double* y);

/* compute_igr_rhs! (IGR_adjoints_1d/elliptic.jl:126-154): b = w_i J 2 alpha
 * (d_x u)^2. E is part of the reference's argument list and is not read. */
int igr1d_igr_rhs(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* mu, const double* rho,
                  const double* E, double* b);

/* compute_sip_diagonal (IGR_adjoints_1d/elliptic.jl:206-253): M = diag(A). */
int igr1d_sip_diagonal(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, double* M);

/* solve_elliptic! (IGR_adjoints_1d/elliptic.jl:446-467): sigma is the warm
 * start on entry and the solution on exit. */
int igr1d_solve_elliptic(igr_ctx* ctx, const igr_disc1d* d, double alpha, int n_iter, int solver, const double* mu,
                         const double* rho, const double* E, double* sigma);

/* compute_hyperbolic_rhs! (IGR_adjoints_1d/hyperbolic.jl:23-83). */
int igr1d_hyperbolic_rhs(igr_ctx* ctx, const igr_disc1d* d, double gamma, const double* mu, const double* rho,
                         const double* E, const double* sigma, double* dmu, double* drho, double* dE);

/* compute_igr_euler_rhs! (IGR_adjoints_1d/forward.jl:17-33, both methods):
 * sigma is the warm start and result of one solve when alpha > 0, else set to
 * zero; then (dmu, drho, dE) = compute_hyperbolic_rhs! at (mu, rho, E, sigma). */
int igr1d_igr_euler_rhs(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, int n_iter, int solver,
                        const double* mu, const double* rho, const double* E, double* sigma, double* dmu, double* drho,
                        double* dE);

/* cg_solve! (IGR_adjoints_1d/elliptic.jl:163-199) with apply_A! = apply_sip!
 * at (rho, alpha) (tests/run_euler_test.jl:160-161); as igr2d_cg_solve. */
int igr1d_cg_solve(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, const double* b, double* x,
                   double tol, int maxiter, int* iters);

/* cg_fixed! (IGR_adjoints_1d/elliptic.jl:265-292) with apply_A! = apply_sip!. */
int igr1d_cg_fixed(igr_ctx* ctx, const igr_disc1d* d, double alpha, const double* rho, const double* b, double* x,
                   int n_iter);

/* Batched 1D forward: n_inst instances sharing the basis (p, xi, w, D), each
 * with its own n_e, L, gamma, alpha, dt and step count, advanced in one
 * launch (one CTA per instance). Fixed steps (no dt re-rounding; callers that
 * want run_forward! semantics pass n_steps = ceil(T/dt) and dt = T/n_steps).
 * q is the concatenation over instances of (mu, rho, E), N_i = (p+1) n_e[i]
 * doubles each, in place; sigma is the concatenation of Sigma (N_i each).
 * final_solve != 0 adds the solve at the final state (forward.jl:83-85). */
int igr1d_forward_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                        const int* n_e, const double* L, const double* gammas, const double* alphas,
                        const double* dts, const int* n_steps, int n_iter, int solver, int final_solve, double* q,
                        double* sigma);

/* run_sensitivity (IGR_adjoints_1d/sensitivity.jl:475-515): the coupled primal
 * + tangent SSP-RK3 to time T with the reference's stepping (`while t < T -
 * 1e-14`, h = min(dt, T - t), no re-rounding), in place: (mu, rho, E) and the
 * tangent (smu, srho, sE) on entry are the initial state and direction; on
 * exit both are at T with sigma = Sigma(T) and ssigma its tangent.
 * elliptic_rhs: 1 = :form1, 2 = :form2 (sensitivity.jl:168-314). s_gamma: the
 * direct dP/dgamma source (sensitivity.jl:36-48). The reference's optional
 * per-step callback has no counterpart. */
int igr1d_run_sensitivity(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                          int n_iter, int solver, int elliptic_rhs, double s_gamma, double* mu, double* rho, double* E,
                          double* sigma, double* smu, double* srho, double* sE, double* ssigma);

/* Batched run_sensitivity: per-instance n_e, L, gamma, alpha, dt, T; one
 * s_gamma for the batch (s_gammas may be NULL = 0; all entries must be equal).
 * q and s: concatenations of (mu, rho, E) / (smu, srho, sE) per instance as in
 * igr1d_forward_batch; sigma, ssigma: N_i each. */
int igr1d_sensitivity_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                            const int* n_e, const double* L, const double* gammas, const double* alphas,
                            const double* dts, const double* t_ends, int n_iter, int solver, int elliptic_rhs,
                            const double* s_gammas, double* q, double* s, double* sigma, double* ssigma);

/* Batched 1D discrete adjoint: for each instance, J and dJ/d(mu0, rho0, E0)
 * (conservative variables) of the objective after n_steps[i] fixed SSP-RK3
 * steps of size dts[i] from q0 (layout as igr1d_forward_batch), plus
 * dJ/dgamma and dJ/dalpha (may be NULL). The gradient enzyme_adjoint_ic
 * returns (IGR_adjoints_1d/enzyme_adjoint.jl:267-314) before its
 * conservative-to-primitive transform, which the host-side mirror applies.
 * Objectives: IGR_OBJ_L2_DENSITY, _L2_PRESSURE, _KINETIC_ENERGY,
 * _WEIGHTED_MOMENTUM (enzyme_adjoint.jl:34-215) and IGR_OBJ_INTERVAL_RHO
 * (obj_params = {a, b}). One CTA per instance; the step history is kept as
 * snapshots (all steps, or sqrt(n)-step segments when memory is short) and
 * every step is re-run with full stage tapes before its reverse. */
int igr1d_adjoint_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                        const int* n_e, const double* L, const double* gammas, const double* alphas,
                        const double* dts, const int* n_steps, int n_iter, int solver, int objective,
                        const double* obj_params, const double* q0, double* J, double* dq0, double* dgamma,
                        double* dalpha);

/* ---- 1D continuous adjoint (optimise-then-discretise) ---------------------- */

/* run_forward_store (IGR_adjoints_1d/forward.jl:137-186): n_steps = ceil(T/dt),
 * dt = T/n_steps, one more Sigma solve after every step (and at t = 0);
 * snapshots: (n_steps + 1) x 4 x N doubles, snapshot k = (mu, rho, E, Sigma)
 * after step k; snapshots_len must equal (ceil(T/dt) + 1) * 4 * N. */
int igr1d_run_forward_store(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, double dt, double t_end,
                            int n_iter, int solver, const double* mu0, const double* rho0, const double* E0,
                            double* snapshots, long long snapshots_len, int* n_steps);

/* run_adjoint_conservative (IGR_adjoints_1d/adjoint_pde.jl:474-551): backward
 * SSP-RK3 of the adjoint PDE over the snapshots (step min(dt, T), one Pi solve
 * per stage). Objectives: IGR_OBJ_L2_DENSITY, _L2_PRESSURE, _KINETIC_ENERGY,
 * _WEIGHTED_MOMENTUM (adjoint_pde.jl:487-525) and IGR_OBJ_INTERVAL_RHO
 * (a_rho = indicator of [a, b], obj_params = {a, b}; no reference
 * counterpart). Output: (a_mu, a_rho, a_E) at t = 0. */
int igr1d_run_adjoint_conservative(igr_ctx* ctx, const igr_disc1d* d, const double* snapshots, long long snapshots_len,
                                   int n_steps, double dt, double t_end, double gamma, double alpha, int n_iter,
                                   int objective, int solver, const double* obj_params, double* amu, double* arho,
                                   double* aE);

/* compute_adjoint_rhs_conservative! (IGR_adjoints_1d/adjoint_pde.jl:410-456):
 * the adjoint operator at (mu, rho, E, sigma) applied to a; pi is the Pi
 * warm start in and the solution out (alpha > 0). */
int igr1d_adjoint_rhs_conservative(igr_ctx* ctx, const igr_disc1d* d, double gamma, double alpha, int n_iter, int solver,
                                   const double* mu, const double* rho, const double* E, const double* sigma, double* pi,
                                   const double* amu, const double* arho, const double* aE, double* damu, double* darho,
                                   double* daE);

/* Store + adjoint for a batch of 1D instances (each with its own n_e, L,
 * gamma, alpha, dt and T) in one launch of per-instance persistent CTAs, the
 * snapshots kept on the device (all, or sqrt(n)-step segments recomputed from
 * checkpoints when memory is short). q0 and a0: concatenations of
 * (mu, rho, E) per instance as in igr1d_forward_batch. No counterpart in the
 * reference. */
int igr1d_adjoint_conservative_batch(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst,
                                     const int* n_e, const double* L, const double* gammas, const double* alphas,
                                     const double* dts, const double* t_ends, int n_iter, int solver, int objective,
                                     const double* obj_params, const double* q0, double* a0);

/* ---- Initial conditions ------------------------------------------------------ */

/* 2D builders (IGR_adjoints_2d/initial_conditions.jl). */
typedef enum {
  IGR_IC2D_CONSTANT = 0,          /* init_constant_state, :15; params (rho0, ux0, uy0, p0) = (1, 1, 1, 1) */
  IGR_IC2D_ISENTROPIC_VORTEX = 1, /* init_isentropic_vortex, :39; params (beta, ux0, uy0) = (5, 1, 1) */
  IGR_IC2D_TAYLOR_GREEN = 2,      /* build_taylor_green_ic!, :105; amplitude A, no params */
  IGR_IC2D_SEDOV_BLAST = 3,       /* build_sedov_blast_ic!, :136; params (p_bg, sigma) = (1, 0.1) */
  IGR_IC2D_OSEEN_PAIR_BLAST = 4,  /* build_oseen_pair_blast_ic!, :175; params (a_core, M_star, blast_xc,
                                     blast_yc, sigma, xc1, yc1, sign1, xc2, yc2, sign2) = (0.05, 0.5, 0.25,
                                     0.5, 0.09, 0.45, 0.6, +1, 0.45, 0.4, -1) */
  IGR_IC2D_MULTI_BLAST = 5        /* rho = 1, u = 0, p = p_bg + sum_k A_k exp(-r_k^2/sigma^2), the several-blast
                                     state of 2d/paper_scripts/generate_otd_refinement_sedov_data.jl:72-86;
                                     params (p_bg, sigma, n <= 4, x_1, y_1, A_1, ..., x_n, y_n, A_n), required;
                                     blast 1's amplitude is the instance's A */
} igr_ic2d;

/* Builds the initial state of n_inst instances on one mesh, each with its own
 * gamma and amplitude A (ignored by the constant state and the vortex), on the
 * GPU: q is (n_inst, 4, N) doubles (mux, muy, rho, E per instance, Julia node
 * order), host memory; params may be NULL (the reference's defaults). */
int igr2d_build_ic(igr_ctx* ctx, const igr_disc2d* d, int ic_type, int n_inst, const double* gammas, const double* amps,
                   const double* params, double* q);
/* The same into device memory (q_dev: n_inst * 4 * N doubles), for batched
 * calls such as igr2d_adjoint_batch_dev that take device inputs. */
int igr2d_build_ic_dev(igr_ctx* ctx, const igr_disc2d* d, int ic_type, int n_inst, const double* gammas,
                       const double* amps, const double* params, double* q_dev);
/* l2_error (IGR_adjoints_2d/initial_conditions.jl:74-87): sqrt(sum w_i w_j Jx Jy (u - u_ref)^2). */
int igr2d_l2_error(igr_ctx* ctx, const igr_disc2d* d, const double* u, const double* u_ref, double* err);

/* 1D builders (IGR_adjoints_1d/initial_conditions.jl:94-204, IC_BUILDERS :218). */
typedef enum {
  IGR_IC1D_ACOUSTIC_PULSE = 0, IGR_IC1D_ENTROPY_WAVE = 1, IGR_IC1D_DENSITY_PULSE = 2, IGR_IC1D_PRESSURE_PULSE = 3,
  IGR_IC1D_VELOCITY_PULSE = 4
} igr_ic1d;
/* n_inst instances with their own n_e, L, gamma and amplitude A; q: the
 * concatenation of (mu, rho, E) per instance as igr1d_forward_batch takes it. */
int igr1d_build_ic(igr_ctx* ctx, int p, const double* xi, const double* w, const double* D, int n_inst, const int* n_e,
                   const double* L, int ic_type, const double* gammas, const double* amps, double* q);

#ifdef __cplusplus
}
#endif

#endif /* IGR_GB300_H */
