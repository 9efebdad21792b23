"""Benchmark: 2D P3 128^2 discrete-adjoint gradients/s, batched vs plain.

Workload (one "step" = one batched gradient call): B = 32 instances of the
2D IGR-Euler discrete adjoint on a 128 x 128 P3 mesh (262,144 nodes x 4
vars each), Chebyshev-Jacobi 5 iterations per stage, 200 SSP-RK3 steps,
objective J = sum over nodes in a seeded square window of w_i w_j Jx Jy rho^2,
gradient w.r.t. the initial state, gamma and alpha. Initial states: seeded
Gaussian pressure pulses (3 pulses, amplitude U[1,10], width 0.03, centres
U[0.2,0.8]; synthetic stand-ins of the reference's pulse family), gamma = 1.4,
alpha = 3 (1/128)^2, dt from CFL 0.1.

`value` times the batched call with inputs and outputs resident in HBM; `e2e`
times the same call through the C ABI with host buffers (H2D of q0, D2H of
dq0 inside the timed region). "plain" runs the same kernels one instance at a
time. The working set (tape) is far larger than L2, so no flush is needed.

Under torchrun (N > 1) every rank runs its own batch (instances shard with no
exchange: weak scaling); rank 0 prints the max-over-ranks timing.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P, NE, N_STEPS, N_ITER, SOLVER, OBJ = 3, 128, 200, 5, "chebyshev", "window_rho2"
GAMMA = 1.4
METRIC = "2D P3 128² adjoint gradients/s: batched vs plain, same GPU, rel err ≤1e-9"

# FP64 flops per node executed by each kernel family, P3, Chebyshev epilogues:
# (2 DFMA + DADD + DMUL) of one ncu capture divided by the launch's nodes
# (profiles/adjoint2d_kernels_128.md). Used for the live roofline.
FLOPS_PER_NODE = {0: 86.0, 1: 47.8, 2: 167.0, 3: 235.5, 4: 78.45, 5: 137.0}
# Algorithmic FP64 bytes per node per launch: one read of every live field and
# one write of every output field (halo re-reads excluded), for the HBM fraction.
BYTES_PER_NODE = {0: 8 * 11, 1: 8 * 13, 2: 8 * 17, 3: 8 * 35, 4: 8 * 23, 5: 8 * 19}
# DRAM bytes per node of one launch of each family, measured with ncu on an
# 8-instance case whose fields exceed L2 (profiles/adjoint2d_kernels_128.md);
# scaled by the launch's node count for `roofline.traffic`.
TRAFFIC_PER_NODE = {0: 61.9, 1: 91.8, 2: 123.7, 3: 208.1, 4: 151.6, 5: 140.8}
# FP64 instructions per node (DFMA + DADD + DMUL thread instructions of the same
# captures): the issue-rate view of the FP64 roof, whose peak is half the DFMA
# probe's flop rate (one DFMA = 2 flops).
INST_PER_NODE = {0: 59.0, 1: 30.0, 2: 107.0, 3: 155.1, 4: 52.1, 5: 90.3}
FAMILY = {0: "k2_setup", 1: "k2_apply", 2: "k2_hyp_rk", 3: "k2_hyp_rev", 4: "k2_apply_rev", 5: "k2_setup_rev"}
# Algorithmic FP64 operations per node: the reference's arithmetic as restated in the oracle, counted with an
# operation-counting scalar (+ - * / sqrt |x| max = 1 each, a multiply-add = 2), and its reverse by the
# operation-by-operation adjoint rule Enzyme applies to the same code (tests/test_opcount.py pins these).
# P3, Chebyshev 5: per launch of each family (the five operator launches of a stage share the solver's cost)
# and per node and RK step of a whole gradient (forward 2892 + reverse 6970.5).
ALG_OPS_PER_NODE = {0: 131.0, 1: (105.0 + 5 * 112.0) / 5, 2: 168.0, 3: 406.5, 4: (247.0 + 5 * 264.0) / 5, 5: 350.0}
ALG_OPS_PER_NODE_STEP = 2892.0 + 6970.5


def instance_seeds(rank, B):
    """Seeds of the B instances rank `rank` runs: ranks shard the instance
    stream with no overlap (weak scaling, no data exchange)."""
    return [rank * B + b for b in range(B)]


def max_over_ranks(t, dist=None, device=None):
    """Slowest rank's elapsed time (the job's time); identity on one rank."""
    if dist is None:
        return t
    import torch
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def gather_by_seed(dist, seeds, *arrays):
    """Every rank's per-instance results in the order of the instance seeds
    (identity on one rank): (seeds, arrays), each array concatenated along its
    first axis over all ranks' instances."""
    if dist is None:
        return list(seeds), [np.asarray(a) for a in arrays]
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (list(seeds), [np.asarray(a) for a in arrays]))
    allseeds = [s for p in parts for s in p[0]]
    order = np.argsort(allseeds, kind="stable")
    cat = [np.concatenate([p[1][k] for p in parts])[order] for k in range(len(arrays))]
    return [allseeds[i] for i in order], cat


def make_batch(igr, W, B, first=0, ne=NE):
    """Instances first .. first + B - 1 of the workload (one seed each) and the
    job's objective window (the same for every instance, whichever rank runs it)."""
    basis = igr.DGBasis(P)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    q0 = np.empty((B, 4, mesh.x.size))
    dts = np.empty(B)
    for b in range(B):
        q = W.seeded_pulses_2d(mesh, GAMMA, W.seed_for(3, first + b), n_pulses=3, width=0.03)
        for v in range(4):
            q0[b, v] = np.asarray(q[v]).reshape(-1, order="F")
        dts[b] = W.cfl_dt_2d(mesh, P, q, GAMMA, 0.1)
    alpha = 3.0 * (1.0 / ne) ** 2
    return basis, mesh, q0, np.full(B, GAMMA), np.full(B, alpha), dts, W.seeded_window(W.seed_for(3, 0))


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "igr_clocks_bench_%d.csv" % os.getpid())

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(B_cpu, n_steps_sample, threads):
    """The CPU oracle (C++ restatement of the reference) on a bounded sample:
    B_cpu instances for n_steps_sample steps, OpenMP over instances. Returns
    (gradients/s scaled to full gradients, seconds, the sample's inputs and the
    oracle's (J, dq0, dgamma, dalpha))."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    from igr_sensitivities_gb300 import workloads as W
    import igr_sensitivities_gb300 as igr
    basis, mesh, q0, gam, alp, dts, prm = make_batch(igr, W, B_cpu)
    G = O.Grid2D(P, NE, NE)
    t0 = time.perf_counter()
    ref = O.adjoint_batch_2d(G, gam, alp, n_steps_sample, float(dts[0]), N_ITER, SOLVER, OBJ, q0, prm,
                             n_threads=threads)
    t = time.perf_counter() - t0
    sample = (basis, mesh, q0, gam, alp, float(dts[0]), prm)
    # per-step cost is uniform: a full 200-step gradient costs 200/n_steps_sample times the sample
    return B_cpu / (t * N_STEPS / n_steps_sample), t, sample, ref


def parity_vs_oracle(igr, ctx, sample, ref, n_steps_sample):
    """The GPU batch on the CPU baseline's sample (same instances, step size and
    steps) against the oracle's result: relative errors of J, the gradient
    w.r.t. q0 (L2 over each instance's four fields; max over instances and over
    the whole batch), dJ/dgamma and dJ/dalpha."""
    basis, mesh, q0, gam, alp, dt, prm = sample
    B = q0.shape[0]
    J, dq, dg, da = igr.adjoint_batch(q0, gam, alp, np.full(B, dt), n_steps_sample, basis, mesh, n_iter=N_ITER,
                                      solver=SOLVER, objective=OBJ, obj_params=prm, ctx=ctx)
    Jr, dqr, dgr, dar = ref
    r = lambda a, b: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))
    per = [float(np.linalg.norm(dq[b] - dqr[b]) / np.linalg.norm(dqr[b])) for b in range(B)]
    # dJ/dgamma and dJ/dalpha on the scale of J: the elasticities (dJ/dgamma) gamma / J and (dJ/dalpha) alpha / J.
    # Over a few steps of this workload both are at the rounding level of J's own sum (the window sees no wave
    # yet), so their relative errors compare rounding noise; the errors on the elasticity scale do not.
    el = lambda d, p: float(np.max(np.abs(d) * p / np.abs(Jr)))
    return {"rel_l2_grad": float(np.linalg.norm(dq - dqr) / np.linalg.norm(dqr)), "rel_l2_grad_max_instance": max(per),
            "rel_J": r(J, Jr), "rel_dgamma": r(dg, dgr), "rel_dalpha": r(da, dar),
            "elasticity_gamma": el(dgr, gam), "err_elasticity_gamma": el(dg - dgr, gam),
            "elasticity_alpha": el(dar, alp), "err_elasticity_alpha": el(da - dar, alp),
            "tolerance": "rel_l2_grad <= 1e-9, rel_J <= 1e-11, elasticity errors <= 1e-9",
            "config": "%d instances of the workload (128x128 P3, Chebyshev 5, window rho^2), %d steps of dt = %.6e, "
                      "GPU batch vs the CPU oracle" % (B, n_steps_sample, dt)}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    B_cpu = threads
    n_sample = 2
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(B_cpu, n_sample, threads)
    for _ in range(args.steps):
        v, t, _, _ = cpu_baseline(B_cpu, n_sample, threads)
        vals.append((v, t))
    value = statistics.median(v for v, _ in vals)
    ms = statistics.median(t for _, t in vals) * 1e3
    sample = "%d instances x %d of %d steps (OpenMP over instances), scaled to full gradients" % (B_cpu, n_sample, N_STEPS)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "gradients/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args.batch),
            "cpu_baseline": {"value": value, "unit": "gradients/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "gradients/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is Julia, absent on this machine; this arm times the C++ CPU oracle (a restatement "
                    "of the reference's algorithm)"}
    print(json.dumps(line))


def config_dict(B):
    return {"workload": "2D IGR-Euler discrete adjoint, P3 128x128 (262,144 nodes x 4 vars per instance), "
                        "Chebyshev-Jacobi 5 iters/stage, 200 SSP-RK3 steps, J = window rho^2",
            "batch": B, "mesh": "128x128", "p": P, "n_steps": N_STEPS, "solver": "chebyshev", "n_iter": N_ITER,
            "objective": OBJ, "gradient_wrt": "q0 (4 fields), gamma, alpha",
            "l2": "inputs and tape far larger than L2 (no flush needed)", "parallelism": "instances per GPU (no exchange)"}


def secondary(args):
    """Other BASELINE configurations, timed the same way (one JSON line each,
    not the headline): forward2d_pcg (2D 128^2 P3, PCG 60, 500 steps),
    forward1d (1D N_e = 256 P3, Jacobi 50, T = 0.1) and batch1d (1024 1D
    instances, N_e in {64..1024}, PCG 102, forward + adjoint; a bounded
    sample of the 2000 steps, scaled)."""
    import torch
    import igr_sensitivities_gb300 as igr
    from igr_sensitivities_gb300 import igr1d, workloads as W
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    ctx = igr.Context(0)
    threads = os.cpu_count() or 1
    flat = lambda a: np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))
    line = {"impl": "gb300", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic (seeded Gaussian pressure pulses)", "vs_baseline": None}
    if args.workload == "forward2d_pcg":
        basis = igr.DGBasis(3)
        mesh = igr.CartesianMesh2D(128, 128, 1.0, 1.0, basis)
        q0 = W.seeded_pulses_2d(mesh, GAMMA, W.seed_for(2, 0), n_pulses=3, width=0.03)
        dt = W.cfl_dt_2d(mesh, 3, q0, GAMMA, 0.1)
        alpha, nst = 3.0 / 128 ** 2, 500
        if args.profile_case:  # 2 steps (ncu captures)
            nst = 2
        T = nst * dt * 0.999
        run = lambda: igr.run_forward(*q0, dt, T, basis, mesh, GAMMA, alpha, n_iter=60, solver="pcg", ctx=ctx)
        if args.profile_case:
            run()
            run()
            print("profile case done")
            return
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        G = O.Grid2D(3, 128, 128)
        ns = 2
        tc0 = time.perf_counter()
        O.run_forward_2d(G, GAMMA, alpha, dt, ns * dt * 0.999, 60, "pcg", [flat(a) for a in q0])
        tc = (time.perf_counter() - tc0) * nst / ns
        line.update(metric="2D P3 128^2 PCG-60 forward solves/s (500 SSP-RK3 steps)", value=1.0 / t,
                    unit="solves/s", ms_per_step=t * 1e3, gpu_launches=ctx.last_launch_count(),
                    config={"workload": "2D IGR-Euler forward, P3 128x128, PCG 60 iters/stage, 500 steps", "mesh": "128x128"},
                    cpu_baseline={"value": 1.0 / tc, "unit": "solves/s", "cores": 1, "kind": "port",
                                  "sample": "%d of %d steps, single thread, scaled" % (ns, nst)})
    elif args.workload == "adjoint2d_64":
        # one 64^2 P3 gradient (Chebyshev 5, 200 steps, window rho^2), the single-instance adjoint configuration
        basis = igr.DGBasis(3)
        mesh = igr.CartesianMesh2D(64, 64, 1.0, 1.0, basis)
        q0 = W.seeded_pulses_2d(mesh, GAMMA, W.seed_for(3, 0), n_pulses=3, width=0.03)
        dt = W.cfl_dt_2d(mesh, 3, q0, GAMMA, 0.1)
        alpha = 3.0 / 64 ** 2
        prm = W.seeded_window(W.seed_for(3, 0))
        run = lambda: igr.enzyme_adjoint_ic(*q0, N_STEPS, dt, basis, mesh, GAMMA, alpha, n_iter=N_ITER, solver=SOLVER,
                                            objective=OBJ, obj_params=prm, with_params=True, ctx=ctx)
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        G = O.Grid2D(3, 64, 64)
        ns = 2
        tc0 = time.perf_counter()
        O.adjoint_2d(G, GAMMA, alpha, ns, dt, N_ITER, SOLVER, OBJ, [flat(a) for a in q0], prm)
        tc = (time.perf_counter() - tc0) * N_STEPS / ns
        line.update(metric="2D P3 64^2 adjoint gradients/s (Chebyshev 5, 200 steps, one instance)", value=1.0 / t,
                    unit="gradients/s", ms_per_step=t * 1e3,
                    config={"workload": "2D IGR-Euler discrete adjoint, P3 64x64, Chebyshev 5, 200 steps, window rho^2"},
                    cpu_baseline={"value": 1.0 / tc, "unit": "gradients/s", "cores": 1, "kind": "port",
                                  "sample": "%d of %d steps, single thread, scaled" % (ns, N_STEPS)})
    elif args.workload == "forward1d":
        basis = igr.DGBasis(3)
        mesh = igr.PeriodicMesh1D(256, 1.0, basis)
        q0 = W.seeded_pulses_1d(mesh, GAMMA, W.seed_for(1, 0), n_pulses=2, width=0.02)
        dt = W.cfl_dt_1d(mesh, 3, q0, GAMMA, 0.1)
        alpha, T = 3.0 * mesh.dx ** 2, 0.1
        run = lambda: igr1d.run_forward(*q0, dt, T, basis, mesh, GAMMA, alpha, n_iter=50, solver="jacobi", ctx=ctx)
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        G = O.Grid1D(3, 256)
        nst = int(np.ceil(T / dt))
        Ts = 0.005
        tc0 = time.perf_counter()
        O.run_forward_1d(G, GAMMA, alpha, dt, Ts, 50, "jacobi", [flat(a) for a in q0])
        tc = (time.perf_counter() - tc0) * T / Ts
        line.update(metric="1D P3 N_e=256 Jacobi-50 forward solves/s (T = 0.1)", value=1.0 / t, unit="solves/s",
                    ms_per_step=t * 1e3, config={"workload": "1D IGR-Euler forward, N_e=256 P3, Jacobi 50, T=0.1",
                                                 "n_steps": nst},
                    cpu_baseline={"value": 1.0 / tc, "unit": "solves/s", "cores": 1, "kind": "port",
                                  "sample": "T = %.3f of %.1f, single thread, scaled" % (Ts, T)})
    elif args.workload == "batch1d":
        basis = igr.DGBasis(3)
        rng = W.SplitMix64(W.seed_for(4, 0xB))
        nes = [64 * 2 ** int(rng.uniform(0, 5)) for _ in range(1024)]
        gs = [rng.uniform(1.2, 1.8) for _ in range(1024)]
        states, dts, als = [], [], []
        for i, ne in enumerate(nes):
            mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
            q0 = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(4, i), n_pulses=2, width=0.02)
            states.append(tuple(flat(a) for a in q0))
            dts.append(W.cfl_dt_1d(mesh, 3, q0, gs[i], 0.1))
            als.append(3.0 * mesh.dx ** 2)
        ns, nfull = args.n_steps if args.n_steps != N_STEPS else 10, 2000
        prm = W.seeded_interval(W.seed_for(4, 0))
        if args.profile_case:  # the first 152 instances for 2 steps, once (ncu captures; ~2 GB on the device)
            k = 152
            igr1d.adjoint_batch(states[:k], basis, nes[:k], 1.0, gs[:k], als[:k], dts[:k], 2, n_iter=102, solver="pcg",
                                objective="interval_rho", obj_params=prm, ctx=ctx)
            print("profile case done")
            return
        run = lambda: igr1d.adjoint_batch(states, basis, nes, 1.0, gs, als, dts, ns, n_iter=102, solver="pcg",
                                          objective="interval_rho", obj_params=prm, ctx=ctx)
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        # CPU: the oracle's 1D adjoint on two instances of each size for 2 steps, single thread
        tc = 0.0
        for ne in (64, 128, 256, 512, 1024):
            G = O.Grid1D(3, ne)
            i = nes.index(ne)
            tc0 = time.perf_counter()
            O.adjoint_1d(G, gs[i], als[i], 2, dts[i], 102, "pcg", "interval_rho", list(states[i]), prm)
            tc += (time.perf_counter() - tc0) * nes.count(ne) * nfull / 2
        line.update(metric="1D batch of 1024 (N_e in {64..1024}, P3, PCG 102) forward+adjoint gradients/s",
                    value=1024 * ns / nfull / t, unit="gradients/s (2000-step equivalents)", ms_per_step=t * 1e3,
                    config={"workload": "1024 1D instances, N_e ~ U{64..1024}, gamma ~ U[1.2,1.8], PCG 102, "
                                        "interval rho objective", "sample_steps": ns, "full_steps": nfull},
                    cpu_baseline={"value": 1024 / tc, "unit": "gradients/s", "cores": 1, "kind": "port",
                                  "sample": "one instance per N_e for 2 steps, scaled by counts and to 2000 steps"})
    elif args.workload == "pde_batch1d":
        # the batch1d instances through the continuous adjoint (store + backward PDE, one persistent CTA per
        # instance, snapshots on the device), a bounded sample of the 2000 steps, scaled
        basis = igr.DGBasis(3)
        rng = W.SplitMix64(W.seed_for(4, 0xB))
        nes = [64 * 2 ** int(rng.uniform(0, 5)) for _ in range(1024)]
        gs = [rng.uniform(1.2, 1.8) for _ in range(1024)]
        states, dts, als = [], [], []
        for i, ne in enumerate(nes):
            mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
            q0 = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(4, i), n_pulses=2, width=0.02)
            states.append(tuple(flat(a) for a in q0))
            dts.append(W.cfl_dt_1d(mesh, 3, q0, gs[i], 0.1))
            als.append(3.0 * mesh.dx ** 2)
        ns, nfull = args.n_steps if args.n_steps != N_STEPS else 10, 2000
        Ts = [ns * dt * 0.999 for dt in dts]  # ceil(T / dt) = ns
        prm = W.seeded_interval(W.seed_for(4, 0))
        k = 152 if args.profile_case else 1024
        run = lambda: igr1d.adjoint_conservative_batch(states[:k], basis, nes[:k], 1.0, gs[:k], als[:k], dts[:k], Ts[:k],
                                                       n_iter=102, solver="pcg", objective="interval_rho",
                                                       obj_params=prm, ctx=ctx)
        if args.profile_case:
            run()
            print("profile case done")
            return
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        tc = 0.0
        for ne in (64, 128, 256, 512, 1024):
            G = O.Grid1D(3, ne)
            i = nes.index(ne)
            tc0 = time.perf_counter()
            sn, n2 = O.run_forward_store_1d(G, gs[i], als[i], dts[i], 2 * dts[i] * 0.999, 102, "pcg", list(states[i]))
            O.run_adjoint_conservative_1d(G, sn, n2, dts[i], 2 * dts[i] * 0.999, gs[i], als[i], 102, "interval_rho", "pcg",
                                          prm)
            tc += (time.perf_counter() - tc0) * nes.count(ne) * nfull / 2
        line.update(metric="1D batch of 1024 (N_e in {64..1024}, P3, PCG 102) continuous-adjoint gradients/s",
                    value=1024 * ns / nfull / t, unit="gradients/s (2000-step equivalents)", ms_per_step=t * 1e3,
                    gpu_launches=ctx.last_launch_count(),
                    config={"workload": "1024 1D instances, N_e ~ U{64..1024}, gamma ~ U[1.2,1.8], PCG 102, interval rho "
                                        "objective, run_forward_store + run_adjoint_conservative",
                            "sample_steps": ns, "full_steps": nfull},
                    cpu_baseline={"value": 1024 / tc, "unit": "gradients/s", "cores": 1, "kind": "port",
                                  "sample": "one instance per N_e for 2 steps, scaled by counts and to 2000 steps"})
    elif args.workload == "batch2d_c5":
        # 2D batched forward sensitivity + adjoint: 16 x 256^2 P3, gamma ~ U[1.3, 1.7], Oseen vortex pair + one
        # Gaussian pressure pulse, PCG 60, 1000 steps; tangent dJ/dgamma vs adjoint dJ/dgamma vs central FD.
        # Timed on a sample of the steps (the per-step cost is uniform) and extrapolated to 1000 steps.
        # profile case (ncu): 8 x 128^2 for 2 steps, every field 16.8 MB (a launch's working set far above L2)
        B = 8 if args.profile_case else 16
        ne5 = 128 if args.profile_case else 256
        S = args.n_steps if args.n_steps != N_STEPS else (2 if args.profile_case else 4)
        full, nit, h = 1000, 60, 1e-6
        basis = igr.DGBasis(3)
        mesh = igr.CartesianMesh2D(ne5, ne5, 1.0, 1.0, basis)
        rng = W.SplitMix64(W.seed_for(5, 0))
        gs = np.array([rng.uniform(1.3, 1.7) for _ in range(B)])
        q0 = np.empty((B, 4, mesh.x.size))
        dts = np.empty(B)
        for b in range(B):
            # build_oseen_pair_blast_ic! with a seeded pair centre, pulse centre, amplitude U[1, 10] and vortex Mach
            # number U[0.25, 0.5] (circulations of order one would make the homentropic core pressure negative)
            xc, yc, bx, by = (rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
            prm = [0.05, rng.uniform(0.25, 0.5), bx, by, 0.05, xc, yc + 0.1, 1.0, xc, yc - 0.1, -1.0]
            q0[b] = igr.build_ic_batch("oseen_pair_blast", basis, mesh, [gs[b]], [rng.uniform(1.0, 10.0)], params=prm,
                                       ctx=ctx)[0]
            dts[b] = W.cfl_dt_2d(mesh, 3, [q0[b, v].reshape(mesh.x.shape, order="F") for v in range(4)], gs[b], 0.1)
        alpha = 3.0 / ne5 ** 2
        prm_w = W.seeded_window(W.seed_for(5, 0))
        c = np.tile(np.outer(basis.w, basis.w).reshape(-1, order="F"), ne5 * ne5) * mesh.Jx * mesh.Jy
        x, y = mesh.x.reshape(-1, order="F"), mesh.y.reshape(-1, order="F")
        chi = ((x >= prm_w[0]) & (x <= prm_w[0] + prm_w[2]) & (y >= prm_w[1]) & (y <= prm_w[1] + prm_w[2])).astype(float)

        def parts():
            t0 = time.perf_counter()
            q, _, s, _ = igr.sensitivity_batch(q0, np.zeros_like(q0), gs, alpha, dts, S, basis, mesh, n_iter=nit,
                                               solver="pcg", s_gamma=1.0, ctx=ctx)
            t1 = time.perf_counter()
            J, _, dg, _ = igr.adjoint_batch(q0, gs, np.full(B, alpha), dts, S, basis, mesh, n_iter=nit, solver="pcg",
                                            objective="window_rho2", obj_params=prm_w, ctx=ctx)
            t2 = time.perf_counter()
            qf, _ = igr.forward_batch(np.concatenate([q0, q0]), np.concatenate([gs + h, gs - h]), alpha,
                                      np.concatenate([dts, dts]), S, basis, mesh, n_iter=nit, solver="pcg",
                                      final_solve=False, ctx=ctx)
            t3 = time.perf_counter()
            tan = np.array([np.sum(c * 2.0 * q[b, 2] * chi * s[b, 2]) for b in range(B)])
            Jf = np.array([np.sum(c * qf[k, 2] ** 2 * chi) for k in range(2 * B)])
            fd = (Jf[:B] - Jf[B:]) / (2 * h)
            return (t1 - t0, t2 - t1, t3 - t2), tan, dg, fd

        if args.profile_case:
            parts()
            print("profile case done")
            return
        for _ in range(args.warmup):
            parts()
        ts = []
        clocks = ClockSampler(0)
        clocks.start()
        for _ in range(args.steps):
            tt, tan, adj, fd = parts()
            ts.append(tt)
        clk = clocks.stop()
        t_tan, t_adj, t_fd = (float(np.median([t[k] for t in ts])) for k in range(3))
        scale = full / S
        # at 1000 steps the adjoint's tape does not fit: the revolve schedule re-runs forward steps from its
        # checkpoints (the FD batch is two forwards of all instances, so half of it is one forward)
        rerun = igr.adjoint_plan(B, full, basis, mesh, alpha, n_iter=nit, solver="pcg", ctx=ctx)
        groups = -(-B // rerun["instances_per_group"])
        extra = (rerun["step_evaluations"] - full) / full * groups * rerun["instances_per_group"] / B
        t_full = (t_tan + t_adj + t_fd) * scale + 0.5 * t_fd * scale * extra
        # CPU: the oracle pipeline for one 64^2 instance and one step, scaled by nodes and steps
        G = O.Grid2D(3, 64, 64)
        m64 = igr.CartesianMesh2D(64, 64, 1.0, 1.0, basis)
        qc = igr.build_ic_batch("oseen_pair_blast", basis, m64, [gs[0]], [5.0], ctx=ctx)[0]
        dtc = W.cfl_dt_2d(m64, 3, [qc[v].reshape(m64.x.shape, order="F") for v in range(4)], gs[0], 0.1)
        tc0 = time.perf_counter()
        O.run_sensitivity_2d(G, gs[0], 3.0 / 64 ** 2, dtc, dtc * 0.999, nit, "pcg", list(qc), [np.zeros(G.N)] * 4,
                             s_gamma=1.0)
        O.adjoint_2d(G, gs[0], 3.0 / 64 ** 2, 1, dtc, nit, "pcg", "window_rho2", list(qc), prm_w)
        for gg in (gs[0] + h, gs[0] - h):
            O.objective_run_2d(G, gg, 3.0 / 64 ** 2, 1, dtc, nit, "pcg", "window_rho2", list(qc), prm_w)
        tcpu = (time.perf_counter() - tc0) * (B * ne5 * ne5 / 64 ** 2) * full * 1.125  # same recompute allowance
        # on the batch's scale: over a short sample some instances' dJ/dgamma is tiny and FD rounding dominates it
        plan = rerun  # the adjoint's memory plan for the whole 1000 steps (revolve schedule of one instance group)
        rel_ta = float(np.max(np.abs(tan - adj)) / np.max(np.abs(adj)))
        rel_af = float(np.max(np.abs(adj - fd)) / np.max(np.abs(fd)))
        line.update(metric="2D batched tangent + adjoint + FD dJ/dgamma sets/hour (16 x 256^2 P3, PCG 60, 1000 steps)",
                    value=3600.0 / t_full, unit="sets/hour", ms_per_step=t_full * 1e3 / full,
                    gpu_launches=ctx.last_launch_count(),
                    config={"workload": "16 x 256x256 P3 Oseen vortex pair + Gaussian pulse (build_oseen_pair_blast_ic!, "
                                        "seeded centres, amplitude U[1,10], vortex Mach U[0.25,0.5]), gamma ~ U[1.3,1.7], "
                                        "PCG 60, window rho^2; batched tangent (s_gamma = 1), batched adjoint (dJ/dgamma), "
                                        "32-instance FD forward batch (h = 1e-6)",
                            "sample_steps": S, "full_steps": full,
                            "sample_seconds": {"tangent": round(t_tan, 3), "adjoint": round(t_adj, 3), "fd": round(t_fd, 3)},
                            "extrapolation": "sample x 1000/S, plus the forward re-runs of the adjoint's checkpoint "
                                             "schedule (adjoint_plan: step_evaluations / 1000 - 1)",
                            "adjoint_plan_1000_steps": plan,
                            "tangent_vs_adjoint_max_rel": rel_ta, "adjoint_vs_fd_max_rel": rel_af},
                    clocks=clk,
                    cpu_baseline={"value": 3600.0 / tcpu, "unit": "sets/hour", "cores": 1, "kind": "port",
                                  "sample": "one 64^2 instance, one step of each part, scaled by nodes and to 1000 steps"})
    elif args.workload == "otd_sedov":
        # the paper's OtD-gap refinement study on three Sedov blasts (p = 4, N_e = 12..30, T = 0.1, PCG 60,
        # kinetic energy): per resolution a continuous adjoint and a two-instance FD forward batch, all on the GPU
        from igr_sensitivities_gb300 import drivers
        cfg = dict(drivers.SEDOV_THREE_BLASTS)
        ic, A = cfg.pop("ic_type"), cfg.pop("A")
        nes = drivers.SEDOV_N_E
        run = lambda: drivers.otd_refinement(ic, A, nes, ctx=ctx, **cfg)
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rows, rates = run()
        t = (time.perf_counter() - t0) / args.steps
        # CPU: the same pipeline on the oracle for 2 steps at N_e = 12, scaled by nodes and step counts
        basis = igr.DGBasis(4)
        G = O.Grid2D(4, 12, 12)
        qs = [O.build_ic_2d(G, ic, GAMMA, a, cfg["params"]) for a in (A, A + cfg["eps"], A - cfg["eps"])]
        dt12 = cfg["CFL"] * G.dx / (9 * W.max_wavespeed_2d(*qs[0], GAMMA))
        ns = 2
        tc0 = time.perf_counter()
        sn, n2 = O.run_forward_store_2d(G, GAMMA, cfg["alpha"], dt12, ns * dt12 * 0.999, 60, "pcg", qs[0])
        O.run_adjoint_conservative_2d(G, sn, n2, dt12, ns * dt12 * 0.999, GAMMA, cfg["alpha"], 60, cfg["objective"], "pcg")
        for q in qs[1:]:
            O.run_forward_2d(G, GAMMA, cfg["alpha"], dt12, ns * dt12 * 0.999, 60, "pcg", q)
        per_step_node = (time.perf_counter() - tc0) / (ns * G.N)
        tc = 0.0
        for ne in nes:
            steps = int(np.ceil(cfg["T"] / (dt12 * 12.0 / ne)))
            tc += per_step_node * steps * 25 * ne * ne
        line.update(metric="OtD refinement sweeps/hour (three Sedov blasts, P4, N_e 12..30, PCG 60, T = 0.1)",
                    value=3600.0 / t, unit="sweeps/hour", ms_per_step=t * 1e3, gpu_launches=ctx.last_launch_count(),
                    config={"workload": "2d/paper_scripts/generate_otd_refinement_sedov_data.jl settings: per N_e one "
                                        "continuous adjoint (store + backward PDE) and a 2-instance central-difference "
                                        "forward batch", "N_e": nes,
                            "gaps": [round(r[1], 6) for r in rows], "rates": [round(r, 3) for r in rates]},
                    cpu_baseline={"value": 3600.0 / tc, "unit": "sweeps/hour", "cores": 1, "kind": "port",
                                  "sample": "the pipeline for 2 steps at N_e = 12, scaled by nodes and step counts"})
    elif args.workload == "pde_adjoint2d":
        # the headline's batch (32 x 128^2 P3, Chebyshev 5, 200 steps, window rho^2) through the continuous
        # adjoint: run_forward_store + run_adjoint_conservative with device-resident snapshots
        B = 8 if args.profile_case else args.batch
        nst = 2 if args.profile_case else args.n_steps
        basis, mesh, q0, gs, als, dts, prm = make_batch(igr, W, B)
        dt = float(dts.min())  # one step for the batch: the most restrictive CFL step
        T = nst * dt
        dtv = np.full(B, dt)
        run = lambda: igr.adjoint_conservative_batch(q0, gs, als, dtv, T, basis, mesh, n_iter=N_ITER, solver=SOLVER,
                                                     objective=OBJ, obj_params=prm, ctx=ctx)
        if args.profile_case:
            run()
            print("profile case done")
            return
        _lib_mod = sys.modules["igr_sensitivities_gb300._lib"]
        lib = _lib_mod.lib()
        import ctypes as C
        for _ in range(args.warmup):
            run()
        lib.igr_profile_reset(ctx.handle)
        lib.igr_profile_enable(ctx.handle, 1)
        run()
        lib.igr_profile_enable(ctx.handle, 0)
        fam = {}
        for k, nm in ((9, "k2_pde_rk"), (10, "k2_pde_prep+k2_pde_b"), (1, "k2_apply"), (0, "k2_setup"), (2, "k2_hyp_rk"),
                      (8, "other")):
            ms, cnt, nodes = C.c_double(0), C.c_longlong(0), C.c_double(0)
            lib.igr_profile_read(ctx.handle, k, C.byref(ms), C.byref(cnt))
            lib.igr_profile_nodes(ctx.handle, k, C.byref(nodes))
            fam[nm] = {"ms": round(ms.value, 2), "launches": cnt.value, "nodes": nodes.value}
        clocks = ClockSampler(0)
        clocks.start()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        t = (time.perf_counter() - t0) / args.steps
        clk = clocks.stop()
        # CPU: the oracle's forward store + continuous adjoint, one instance for 2 steps, single thread
        G = O.Grid2D(3, NE, NE)
        ns = 2
        qi = [np.ascontiguousarray(q0[0, v]) for v in range(4)]
        tc0 = time.perf_counter()
        snaps, n2 = O.run_forward_store_2d(G, GAMMA, als[0], dt, ns * dt, N_ITER, SOLVER, qi)
        O.run_adjoint_conservative_2d(G, snaps, n2, dt, ns * dt, GAMMA, als[0], N_ITER, OBJ, SOLVER, prm)
        tc = (time.perf_counter() - tc0) * nst / ns
        rk = fam["k2_pde_rk"]
        line.update(metric="2D P3 128^2 continuous-adjoint gradients/s (Chebyshev 5, 200 steps, batch %d)" % B,
                    value=B / t, unit="gradients/s", ms_per_step=t * 1e3, gpu_launches=ctx.last_launch_count(),
                    config={"workload": "2D IGR-Euler continuous adjoint (run_forward_store + run_adjoint_conservative), "
                                        "P3 128x128, Chebyshev 5, 200 steps, window rho^2, snapshots resident in HBM",
                            "global_batch": B, "n_steps": nst, "l2": "snapshots and fields >> L2"},
                    e2e={"value": B / t, "unit": "gradients/s", "h2d_bytes_per_step": int(q0.nbytes),
                         "d2h_bytes_per_step": int(q0.nbytes)},
                    kernels=fam,
                    k2_pde_rk_us_per_launch=round(1e3 * rk["ms"] / max(rk["launches"], 1), 1),
                    clocks=clk,
                    cpu_baseline={"value": 1.0 / tc, "unit": "gradients/s", "cores": 1, "kind": "port",
                                  "sample": "1 instance, %d of %d steps, single thread, scaled" % (ns, nst)})
    elif args.workload == "batch_sweep":
        # the headline workload at several batch sizes (B = 1 is the plain path): gradients/s per B
        sizes = [1, 8, 32, 64]
        by_batch = {}
        clk = ClockSampler(0)
        clk.start()
        for B in sizes:
            basis, mesh, q0h, gam, alp, dts, prm = make_batch(igr, W, B)
            q0d = torch.from_numpy(q0h).to(torch.device("cuda", 0))
            run = lambda: igr.adjoint_batch(q0d, gam, alp, dts, N_STEPS, basis, mesh, n_iter=N_ITER, solver=SOLVER,
                                            objective=OBJ, obj_params=prm, ctx=ctx, device_arrays=True)
            run()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            run()
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            pg = ctx.last_adjoint_plan()
            by_batch[B] = {"gradients_per_s": B / t, "s_per_call": t, "tape_plan": pg}
            del q0d
        clk_v = clk.stop()
        line.update(metric=METRIC + " (batch sweep)", value=by_batch[32]["gradients_per_s"], unit="gradients/s",
                    ms_per_step=by_batch[32]["s_per_call"] * 1e3, gpu_launches=ctx.last_launch_count(),
                    config=dict(config_dict(32), batch_sizes=sizes), by_batch=by_batch, clocks=clk_v,
                    batched_over_plain={B: by_batch[B]["gradients_per_s"] / by_batch[1]["gradients_per_s"] for B in sizes})
    else:
        raise SystemExit("unknown workload " + args.workload)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--n-steps", type=int, default=N_STEPS, help="RK steps per gradient (200 = the workload)")
    ap.add_argument("--workload", default="adjoint2d",
                    help="adjoint2d (the headline) | adjoint2d_64 | forward2d_pcg | forward1d | batch1d | pde_adjoint2d | "
                         "pde_batch1d | otd_sedov | batch2d_c5 | batch_sweep")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu captures: batch 2, 4 steps, one call, no timing output")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload != "adjoint2d":
        return secondary(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import igr_sensitivities_gb300 as igr
    from igr_sensitivities_gb300 import _lib, workloads as W
    import ctypes as C

    ctx = igr.Context(local)
    if args.profile_case:
        # one instance group of the metric workload (8 instances: fields of 16.8 MB, the
        # per-kernel working set well above L2) for 2 steps, called twice
        basis, mesh, q0h, gam, alp, dts, prm = make_batch(igr, W, 8)
        q0d = torch.from_numpy(q0h).to(torch.device("cuda", local))
        for _ in range(2):
            igr.adjoint_batch(q0d, gam, alp, dts, 2, basis, mesh, n_iter=N_ITER, solver=SOLVER, objective=OBJ,
                              obj_params=prm, ctx=ctx, device_arrays=True)
        torch.cuda.synchronize()
        print("profile case done")
        return
    n_steps = args.n_steps
    B = args.batch
    basis, mesh, q0h, gam, alp, dts, prm = make_batch(igr, W, B, first=instance_seeds(rank, B)[0])
    dev = torch.device("cuda", local)
    q0d = torch.from_numpy(q0h).to(dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    def run_dev():
        return igr.adjoint_batch(q0d, gam, alp, dts, n_steps, basis, mesh, n_iter=N_ITER, solver=SOLVER, objective=OBJ,
                                 obj_params=prm, ctx=ctx, device_arrays=True)

    for _ in range(args.warmup):
        run_dev()
    lib = _lib.lib()
    clk = ClockSampler(local)
    clk.start()
    barrier()
    t0 = time.perf_counter()
    launches = 0
    for _ in range(args.steps):
        run_dev()
        launches += ctx.last_launch_count()
    barrier()
    t = time.perf_counter() - t0
    clocks = clk.stop()
    # one more step with per-launch CUDA events on the engine's stream: kernel durations and shares
    lib.igr_profile_reset(ctx.handle)
    lib.igr_profile_enable(ctx.handle, 1)
    barrier()
    tp0 = time.perf_counter()
    Jl = run_dev()[0]  # the instances' J, gathered below in seed order (outside the timed region)
    barrier()
    t_prof = time.perf_counter() - tp0
    lib.igr_profile_enable(ctx.handle, 0)
    pg = [C.c_int(0) for _ in range(4)]
    lib.igr_last_adjoint_plan(ctx.handle, *[C.byref(x) for x in pg])
    tape_plan = {"groups": pg[0].value, "instances_per_group": pg[1].value, "steps_per_segment": pg[2].value,
                 "segments": pg[3].value}
    fam = {}
    for k in range(9):
        ms, cnt, nn = C.c_double(0), C.c_longlong(0), C.c_double(0)
        lib.igr_profile_read(ctx.handle, k, C.byref(ms), C.byref(cnt))
        lib.igr_profile_nodes(ctx.handle, k, C.byref(nn))
        fam[k] = (ms.value, cnt.value, nn.value)
    tmax = max_over_ranks(t, dist, dev)
    value = B * world * args.steps / tmax
    seeds_all, (J_all,) = gather_by_seed(dist, instance_seeds(rank, B), Jl)

    # end to end: host buffers through the C ABI (one untimed call first, as for the device-resident timing)
    run_host = lambda: igr.adjoint_batch(q0h, gam, alp, dts, n_steps, basis, mesh, n_iter=N_ITER, solver=SOLVER,
                                         objective=OBJ, obj_params=prm, ctx=ctx)
    run_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        run_host()
    barrier()
    te = (time.perf_counter() - t0) / max(1, args.steps // 2)
    e2e = B * world / te
    e2e_plan = ctx.last_adjoint_plan()

    # plain: the same kernels, one instance per call
    plain = None
    if not args.no_plain:
        nplain = 2
        run1 = lambda b: igr.adjoint_batch(q0d[b:b + 1].contiguous(), gam[b:b + 1], alp[b:b + 1], dts[b:b + 1], n_steps, basis,
                                           mesh, n_iter=N_ITER, solver=SOLVER, objective=OBJ, obj_params=prm, ctx=ctx,
                                           device_arrays=True)
        run1(0)
        barrier()
        t0 = time.perf_counter()
        for b in range(nplain):
            run1(b)
        barrier()
        tp = (time.perf_counter() - t0) / nplain
        plain = {"value": 1.0 / tp, "unit": "gradients/s", "ms_per_gradient": tp * 1e3}

    if rank != 0:
        return
    peak = C.c_double(0)
    lib.igr_probe_fp64_peak(ctx.handle, C.byref(peak))
    tpeak = C.c_double(0)
    lib.igr_probe_fp64_tensor_peak(ctx.handle, C.byref(tpeak))
    share = {FAMILY[k]: fam[k][0] for k in FAMILY}
    tot = sum(v[0] for v in fam.values()) or 1.0
    dom = max(FAMILY, key=lambda k: fam[k][0])
    ms_launch = fam[dom][0] / max(fam[dom][1], 1)
    nodes = fam[dom][2] / max(fam[dom][1], 1)       # nodes per launch (one instance group)
    flops = FLOPS_PER_NODE[dom] * nodes
    achieved = flops / (ms_launch * 1e-3) / 1e12
    hbm = BYTES_PER_NODE[dom] * nodes / (ms_launch * 1e-3) / 1e9
    issue = INST_PER_NODE[dom] * nodes / (ms_launch * 1e-3) / 1e12
    alg_dom = ALG_OPS_PER_NODE[dom] * nodes / (ms_launch * 1e-3) / 1e12
    # whole gradient: forward + reverse operations of every RK step, over the profiled step's device time
    alg_all = ALG_OPS_PER_NODE_STEP * mesh.x.size * B * n_steps / (sum(v[0] for v in fam.values()) * 1e-3) / 1e12
    all_flops = sum(FLOPS_PER_NODE[k] * fam[k][2] for k in FAMILY)
    all_ms = sum(fam[k][0] for k in FAMILY)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        hbm_peak, hbm_src = 6800.0, "fallback"
    traffic = TRAFFIC_PER_NODE[dom] * nodes if dom in TRAFFIC_PER_NODE else None
    roofline = {"bound": "fp64", "kernel": FAMILY[dom], "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                "frac": achieved / peak.value if peak.value else None, "traffic": traffic,
                "traffic_note": "DRAM bytes per launch (ncu, 8-instance case scaled by nodes)",
                "peak_source": "measured live (DFMA-chain probe in libigr_gb300.so)",
                "fp64_tensor_probe_tflops": tpeak.value,
                "ms_per_launch": ms_launch, "flops_per_launch": flops, "nodes_per_launch": nodes,
                "all_kernels_fp64_tflops": all_flops / (all_ms * 1e-3) / 1e12 if all_ms else None,
                "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak, "peak_source": hbm_src},
                "fp64_issue": {"achieved": issue, "peak": peak.value / 2, "unit": "T FP64 instructions/s",
                               "frac": issue / (peak.value / 2) if peak.value else None,
                               "note": "DFMA, DADD and DMUL each take one FP64 issue slot; a third of these kernels' "
                                       "FP64 instructions are DADD/DMUL (1 flop), so the flop fraction is lower"},
                "fp64_algorithmic": {
                    "achieved": alg_dom, "peak": peak.value, "unit": "TFLOP/s", "frac": alg_dom / peak.value if peak.value else None,
                    "whole_gradient_achieved": alg_all, "whole_gradient_frac": alg_all / peak.value if peak.value else None,
                    "ops_per_node_per_launch": ALG_OPS_PER_NODE[dom], "ops_per_node_step": ALG_OPS_PER_NODE_STEP,
                    "note": "the reference's arithmetic (operation-counted restatement, reverse by the adjoint rule) per "
                            "second: above 1 where the kernels need fewer operations than the reference's expressions "
                            "(per-stage coefficients, skipped zero terms, folded face terms)"},
                "time_share": {k: v / tot for k, v in share.items()},
                "profiled_step_ms": t_prof * 1e3, "kernel_ms_in_profiled_step": sum(v[0] for v in fam.values())}
    cfg = config_dict(B)
    cfg["n_steps"] = n_steps
    cfg["tape_plan"] = tape_plan
    cfg["instances_total"] = len(seeds_all)
    cfg["J_sum_over_instances"] = float(np.sum(J_all))
    line = {"metric": METRIC, "value": value, "unit": "gradients/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian pressure pulses)",
            "config": cfg, "plain": plain,
            "batched_over_plain": (value / world / plain["value"]) if plain else None,
            "e2e": {"value": e2e, "unit": "gradients/s", "h2d_bytes_per_step": int(q0h.nbytes),
                    "d2h_bytes_per_step": int(q0h.nbytes + 3 * 8 * B), "tape_plan": e2e_plan},
            "gpu_launches": launches, "roofline": roofline, "clocks": clocks}
    if not args.no_cpu and world == 1:
        threads = os.cpu_count() or 1
        n_sample = 5
        v, tcpu, sample, ref = cpu_baseline(threads, n_sample, threads)
        line["cpu_baseline"] = {"value": v, "unit": "gradients/s", "cores": threads, "kind": "port",
                                "sample": "%d instances x %d of %d steps (OpenMP over instances, %.1f s), scaled to full "
                                          "gradients" % (threads, n_sample, N_STEPS, tcpu)}
        line["parity"] = parity_vs_oracle(igr, ctx, sample, ref, n_sample)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
