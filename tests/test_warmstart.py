"""Learned warm start: the previous-displacement feature, the fit sweeps'
contract, and a gain in Gauss-Seidel sweeps at equal XPBD residual over the
plain solver on held-out trajectories (450-tet cantilever under random body
forces, 30 plain iterations), with the carry start (previous substep's
multipliers) and with fit sweeps."""
import numpy as np
import pytest

from sbs_gb300 import warmstart

pytestmark = pytest.mark.gpu


def test_previous_displacement_feature(capi_mod):
    sc = warmstart.batch_scene([7])
    g = capi_mod.Solver(sc, exec_mode=1)
    dt = sc.frame_dt
    g.detect_contacts()
    g.predict(dt)
    f1 = g.features()
    assert (f1[:, 3:6] == 0).all()          # nothing recorded yet
    xp = g.predicted_all()
    g.solve(dt, 30)
    g.update_velocities(dt)
    x = g.positions()
    g.detect_contacts()
    g.predict(dt)
    f2 = g.features()
    assert np.array_equal(f2[:, 3:6], x - xp)   # the last substep's solve displacement
    assert np.abs(f2[:, 3:6]).max() > 0
    # replacing the state forgets it
    xs, vs = g.get_state(-1)
    g.set_state(-1, xs, vs)
    g.predict(dt)
    assert (g.features()[:, 3:6] == 0).all()
    g.close()


def test_strain_features_match_numpy(capi_mod):
    """Features 6..11: the Green strain (F^T F - I) / 2 of the mean
    deformation gradient of a vertex's incident tets at the predicted
    positions, against numpy in FP64 (the GPU adds the incident gradients in
    eight interleaved partial sums and a fixed tree)."""
    from sbs_gb300 import scenes
    sc = scenes.beam_twist(10, 4, 4, 0.05)
    g = capi_mod.Solver(sc, exec_mode=1)
    g.step(3)
    g.detect_contacts()
    g.predict(sc.frame_dt / sc.substeps)
    f = g.features().astype(np.float64)
    xp = g.predicted_all().astype(np.float64)
    b = sc.bodies[0]
    t = b.tets.astype(np.int64)
    x0 = b.x0
    Dm = np.stack([x0[t[:, 0]] - x0[t[:, 3]], x0[t[:, 1]] - x0[t[:, 3]], x0[t[:, 2]] - x0[t[:, 3]]], axis=2)
    Ds = np.stack([xp[t[:, 0]] - xp[t[:, 3]], xp[t[:, 1]] - xp[t[:, 3]], xp[t[:, 2]] - xp[t[:, 3]]], axis=2)
    F = Ds @ np.linalg.inv(Dm)
    Fsum = np.zeros((len(x0), 3, 3))
    cnt = np.zeros(len(x0))
    for k in range(4):
        np.add.at(Fsum, t[:, k], F)
        np.add.at(cnt, t[:, k], 1)
    Fm = Fsum / cnt[:, None, None]
    E = 0.5 * (np.einsum("vki,vkj->vij", Fm, Fm) - np.eye(3))
    want = np.stack([E[:, 0, 0], E[:, 1, 1], E[:, 2, 2], E[:, 0, 1], E[:, 0, 2], E[:, 1, 2]], axis=1)
    assert np.abs(f[:, 6:12] - want).max() < 2e-5
    assert np.abs(want).max() > 1e-4
    g.close()


def test_fit_sweeps_argument(capi_mod):
    sc = warmstart.batch_scene([7])
    g = capi_mod.Solver(sc, exec_mode=1)
    m = capi_mod.Mlp(device=0, seed=0)
    with pytest.raises(capi_mod.SbsError):
        g.set_warm_start(m, 17)
    g.set_warm_start(m, 0)             # carry start
    g.step(2)
    assert np.isfinite(g.positions()).all()
    m.set_params(np.zeros(m.n_params, np.float32))   # guess = previous displacement
    g.set_warm_start(m, 3)
    g.step(2)                          # frames run through the warm-start path
    assert np.isfinite(g.positions()).all()
    g.set_warm_start(None)
    g.close()


def test_warm_start_saves_sweeps(capi_mod):
    X, Y = warmstart.generate(list(range(1000, 1128)), frames=40, iterations=30)
    m, losses = warmstart.fit(X, Y, steps=3000, batch=32768, lr=1e-3, seed=1, chunk=1000)
    assert losses[-1] < losses[0]
    seeds = list(range(50000, 50012))
    # carry start (previous multipliers): the plain 30-sweep residual in at
    # most 40% of the sweeps on average, fallbacks counted as 30
    res = warmstart.evaluate(m, seeds, frame=20, iterations=30, fit_sweeps=0)
    assert all(r["same_start"] for r in res)
    its = np.array([r["iterations"] for r in res])
    assert (its <= 30).all()
    assert its.mean() <= 12.0, its
    for r in res:
        if not r["fallback"]:
            assert r["r_end"] <= r["r_plain"]
    # the trained network beats its own previous-displacement guess
    m_zero = capi_mod.Mlp(device=0, seed=0)
    m_zero.set_params(np.zeros(m_zero.n_params, np.float32))
    m_zero.set_normalization(X.mean(0), np.maximum(X.std(0), 1e-8), Y.std(0) + 1e-12)
    res0 = warmstart.evaluate(m_zero, seeds, frame=20, iterations=30, fit_sweeps=0)
    assert its.mean() < np.mean([r["iterations"] for r in res0])
    # fit sweeps: never worse than plain (the fallback)
    resf = warmstart.evaluate(m, seeds[:4], frame=20, iterations=30, fit_sweeps=3)
    assert all(r["iterations"] <= 30 for r in resf)


def test_warm_start_with_springs_and_grid_environment(capi_mod):
    """The warm-start path runs distance constraints and grid contacts too."""
    from sbs_gb300 import scenes
    sc = scenes.hanging_block(alpha=1e-6)
    lo = np.array([-1.0, -1.5, -1.0])
    sp = np.array([0.25, 0.25, 0.25])
    nodes = (9, 9, 9)
    y = lo[1] + sp[1] * np.arange(nodes[1])
    vals = np.broadcast_to((y + 0.3)[None, :, None], (nodes[2], nodes[1], nodes[0])).astype(np.float32).copy()
    sc.ground = None
    sc.sdf_grids = [(vals, nodes, lo, sp)]          # a floor at y = -0.3 under the hanging block
    g = capi_mod.Solver(sc, exec_mode=1)
    m = capi_mod.Mlp(device=0, seed=0)
    m.set_params(np.zeros(m.n_params, np.float32))
    g.set_warm_start(m, 2)
    g.step(1)
    assert g.stats().n_contacts > 0                   # the block starts 0.1 m into the floor
    g.step(39)
    x = g.positions()
    assert np.isfinite(x).all()
    offs = np.cumsum([0] + [len(b.x0) for b in sc.bodies])
    assert x[offs[1]:, 1].min() > -0.35               # pushed out of the grid floor
    g.set_warm_start(None)
    g.close()


@pytest.mark.parametrize("fit_sweeps", [0, 2])
def test_warm_start_cluster_matches_graph(capi_mod, oracle_mod, fit_sweeps):
    """Warm-started frames in the cluster-resident mode (one launch per
    substep on the warm-started positions and multipliers) against the same
    frames in the graph mode: the same sweep, so within the FP32 noise floor."""
    from sbs_gb300 import scenes
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    m = capi_mod.Mlp(device=0, seed=3)       # untrained: a small, deterministic correction
    m.set_normalization(np.zeros(16, np.float32), np.ones(16, np.float32), np.full(3, 1e-4, np.float32))
    a = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_CLUSTER)
    b = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_GRAPH)
    a.step(1)
    b.step(1)
    a.set_warm_start(m, fit_sweeps)
    b.set_warm_start(m, fit_sweeps)
    a.step(2, iterations=12)
    b.step(2, iterations=12)
    xa, xb = a.positions(), b.positions()
    assert np.isfinite(xa).all()
    order, off = capi_mod.plan_sweep(sc)
    floor = oracle_mod.noise_floor(sc, 3, order, off, n_seeds=2)
    assert np.abs(xa - xb).max() < 2 * floor + 1e-6 * sc.bbox_diag()
    # the cluster frames ran (one launch per substep plus the global kernels)
    assert a.stats().exec_mode == capi_mod.EXEC_CLUSTER
    a.set_warm_start(None)
    b.set_warm_start(None)
