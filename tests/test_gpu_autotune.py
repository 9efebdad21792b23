"""Autotuning of result-invariant launch choices (1D CTAs per instance, 2D
fused or separate PCG inner products): tuned runs give bitwise the untuned
results, the choices are remembered per batch shape, and a cache file carries
them to a fresh context."""
import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


def test_1d_tuned_cluster_size_keeps_results_and_is_cached(igr, tmp_path):
    from igr_sensitivities_gb300 import Context, igr1d
    basis = igr.DGBasis(3)
    nes, gs = [256, 64, 512], [1.4, 1.3, 1.6]
    states, dts, als = [], [], []
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        q0 = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(4, 70 + i), width=0.08)
        states.append(tuple(flat(a) for a in q0))
        dts.append(W.cfl_dt_1d(mesh, 3, q0, gs[i], 0.1))
        als.append(3.0 * mesh.dx ** 2)
    nst = [6, 6, 6]
    run = lambda ctx: igr1d.forward_batch(states, basis, nes, 1.0, gs, als, dts, nst, n_iter=9, solver="pcg", ctx=ctx)
    plain = run(Context(0))
    cache = tmp_path / "tune.txt"
    ctx = Context(0)
    ctx.set_autotune(True, str(cache))
    assert ctx.autotune_count() == 0
    tuned = run(ctx)
    assert ctx.autotune_count() == 1
    text = cache.read_text()
    assert "1d.cluster np=4 inst=3 ne_min=64 ne_max=512" in text
    cs = int(text.strip().splitlines()[-1].split("\t")[1])
    assert cs in (1, 2, 4) and ctx.last_cluster_size_1d() == cs  # at least 16 elements per CTA
    again = run(ctx)
    fresh = Context(0)
    fresh.set_autotune(True, str(cache))
    assert fresh.autotune_count() == 1
    cached = run(fresh)
    assert fresh.last_cluster_size_1d() == cs
    for res in (tuned, again, cached):
        for i in range(len(nes)):
            for a, b in zip(plain[i], res[i]):
                assert np.array_equal(a, b)


@pytest.mark.parametrize("solver", ["pcg"])
def test_2d_tuned_pcg_sums_keep_results(igr, oracle, solver, tmp_path):
    """The first two PCG solves of a new shape are the fused and the separate
    trial; the tuned forward equals the untuned one bitwise."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 3), width=0.1)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    alpha = 3.0 * (1 / 8) ** 2
    run = lambda ctx: igr.run_forward(*q0, dt, 5 * dt * 0.999, basis, mesh, g, alpha, n_iter=7, solver=solver, ctx=ctx)
    plain = run(Context(0))
    ctx = Context(0)
    ctx.set_pcg_persistent(False)  # the inner-product form is a choice of the two-kernel PCG iteration
    cache = tmp_path / "tune2d.txt"
    ctx.set_autotune(True, str(cache))
    tuned = run(ctx)
    assert ctx.autotune_count() == 1
    assert "2d.pcg_sums np=4 tiles=4 inst=1\t" in cache.read_text()
    again = run(ctx)
    for res in (tuned, again):
        for a, b in zip(plain, res):
            assert np.array_equal(flat(a), flat(b))
    ctx.set_autotune(False)


def test_unwritable_cache_path_is_rejected_up_front(igr, tmp_path):
    from igr_sensitivities_gb300 import Context
    from igr_sensitivities_gb300._lib import IGRError
    ctx = Context(0)
    with pytest.raises(IGRError) as ei:
        ctx.set_autotune(True, str(tmp_path / "no_such_dir" / "tune.txt"))
    assert "IGR_EINVAL" in str(ei.value) and "autotune cache" in str(ei.value)
    assert ctx.autotune_count() == 0


def test_1d_tuned_adjoint_and_continuous_adjoint_keep_results(igr):
    """The 1D CTA count is also measured inside the discrete and continuous
    adjoint calls (the probe advances a copy of q0); their results do not
    change."""
    from igr_sensitivities_gb300 import Context, igr1d
    basis = igr.DGBasis(3)
    nes, g = [48, 160], 1.4
    states = []
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(4, 80 + i), width=0.08)
        states.append(tuple(flat(a) for a in q0))
    mesh = igr.PeriodicMesh1D(nes[1], 1.0, basis)
    dt = W.cfl_dt_1d(mesh, 3, [a.reshape(4, nes[1], order="F") for a in states[1]], g, 0.1)
    alpha = 3.0 / nes[1] ** 2
    run = lambda ctx: igr1d.adjoint_batch(states, basis, nes, 1.0, g, alpha, dt, 6, n_iter=6, solver="pcg",
                                          objective="l2_pressure", ctx=ctx)
    run_c = lambda ctx: igr1d.adjoint_conservative_batch(states, basis, nes, 1.0, g, alpha, dt, 6 * dt, n_iter=6,
                                                         objective="l2_pressure", ctx=ctx)
    plain, plain_c = run(Context(0)), run_c(Context(0))
    ctx = Context(0)
    ctx.set_autotune(True)
    tuned, tuned_c = run(ctx), run_c(ctx)
    assert ctx.autotune_count() >= 1
    def same(a, b):
        if isinstance(a, (list, tuple)):
            assert len(a) == len(b)
            for x, y in zip(a, b):
                same(x, y)
        else:
            assert np.array_equal(np.asarray(a), np.asarray(b))

    same(plain, tuned)
    same(plain_c, tuned_c)
