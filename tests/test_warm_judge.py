"""The plain solver as the judge of warm-started substeps
(sbs_gpu_set_warm_judge), run on the device inside the frame's CUDA graph:
a warm start whose residual is not below the plain start's falls back to the
plain start, and sweeps continue in chunks until the plain solver's residual
target (or the sweep cap) is reached.

A network with huge weights makes every warm start worse than the plain
start; with an unreachable target the substeps then run the full plain sweep
count from the plain start, which must give the plain solver's positions bit
for bit (graph and cluster-resident modes)."""
import numpy as np
import pytest

from sbs_gb300 import scenes, warmstart

pytestmark = pytest.mark.gpu


def _bad_network(capi_mod):
    m = capi_mod.Mlp(device=0, seed=0)
    m.set_params(np.full(m.n_params, 0.5, np.float32))
    return m


@pytest.mark.parametrize("mode,make,frames", [
    ("graph", lambda: warmstart.batch_scene([7]), 3),
    ("cluster", lambda: scenes.beam_twist(16, 4, 4, 0.05), 2),
])
def test_fallback_gives_the_plain_result_bit_for_bit(capi_mod, mode, make, frames):
    sc = make()
    em = capi_mod.EXEC_GRAPH if mode == "graph" else capi_mod.EXEC_CLUSTER
    plain = capi_mod.Solver(sc, exec_mode=em)
    judged = capi_mod.Solver(sc, exec_mode=em)
    m = _bad_network(capi_mod)
    judged.set_warm_start(m, 0)
    judged.set_warm_judge(3, 0, 0, 1e-30)          # target never reached: every substep runs to the cap
    plain.step(frames)
    judged.step(frames)
    assert judged.stats().exec_mode == em
    st = judged.warm_stats()
    n_sub = frames * sc.substeps
    assert st.warm_substeps == n_sub
    assert st.fallbacks == n_sub
    assert st.sweeps == n_sub * sc.iterations      # 30 sweeps in chunks of 3
    assert st.capped == n_sub
    assert st.calibration_substeps == 0
    xp, xj = plain.positions(), judged.positions()
    assert np.isfinite(xj).all()
    assert np.array_equal(xp, xj)
    assert np.array_equal(plain.velocities(), judged.velocities())


def test_calibration_frames_and_targets(capi_mod):
    sc = warmstart.batch_scene([11])
    g = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_GRAPH)
    m = capi_mod.Mlp(device=0, seed=0)
    m.set_params(np.zeros(m.n_params, np.float32))   # guess = the previous substep's displacement
    g.step(2)
    g.set_warm_start(m, 0)
    g.set_warm_judge(2, 0, 3, 0.0)                   # calibrate frames 0, 3, 6, ...
    g.step(7)
    st = g.warm_stats()
    assert st.calibration_substeps == 3
    assert st.warm_substeps == 4
    assert st.last_target > 0.0
    assert st.sweeps <= 4 * sc.iterations and st.sweeps % 2 == 0
    if st.capped == 0:
        assert st.max_residual_ratio <= 1.0
    assert np.isfinite(g.positions()).all()
    # the stats reset with the judge's settings; judge off = the unjudged warm path
    g.set_warm_judge(0, 0, 0, 0.0)
    g.step(1)
    assert g.warm_stats().warm_substeps == 0
    with pytest.raises(capi_mod.SbsError):
        g.set_warm_judge(40, 30, 0, 0.0)             # chunk above the cap


@pytest.fixture(scope="module")
def trained(capi_mod):
    X, Y = warmstart.generate(list(range(1000, 1064)), frames=40, iterations=30)
    m, losses = warmstart.fit(X, Y, steps=3000, batch=32768, lr=1e-3, seed=1, chunk=1000)
    assert losses[-1] < losses[0]
    return m


def test_judged_warm_start_reaches_the_plain_residual_in_fewer_sweeps(capi_mod, trained):
    """Held-out cantilever trajectories: after 10 plain frames a calibration
    frame records the plain residual, then 10 judged frames run; they must
    reach it (or fall back) in fewer sweeps than the plain 30."""
    sweeps, subs, capped = 0, 0, 0
    for seed in (50000, 50001, 50002, 50003):
        sc = warmstart.batch_scene([seed])
        g = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_GRAPH)
        g.step(10)
        g.set_warm_start(trained, 0)
        g.set_warm_judge(2, 0, 0, 0.0)
        g.step(11)                                   # 1 calibration + 10 judged frames
        st = g.warm_stats()
        assert st.calibration_substeps == 1 and st.warm_substeps == 10
        sweeps += st.sweeps
        subs += st.warm_substeps
        capped += st.capped
        g.set_warm_start(None)
        g.close()
    print(f"\njudged cantilever: {sweeps / subs:.1f} sweeps per substep (plain 30), {capped} of {subs} capped")
    assert sweeps / subs < 0.6 * 30


def test_judged_cluster_frames_keep_prescribed_motion(capi_mod):
    """Calibration frames run the frame kernel itself (kinematic targets from
    the frame's start time), judged frames the per-substep kernel: over
    several frames of both the x=max face stays on its analytic rotation."""
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    g = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_CLUSTER)
    m = capi_mod.Mlp(device=0, seed=0)
    m.set_params(np.zeros(m.n_params, np.float32))
    g.step(1)
    g.set_warm_start(m, 0)
    g.set_warm_judge(3, 0, 2, 0.0)            # calibration frames 0, 2, 4
    g.step(6)
    st = g.warm_stats()
    assert st.calibration_substeps == 3 * sc.substeps and st.warm_substeps == 3 * sc.substeps
    b = sc.bodies[0]
    ang = b.kin_omega * 7 * sc.frame_dt
    R = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
    c = np.array(b.kin_center)
    want = (b.x0[b.kin_verts] - c) @ R.T + c
    assert np.abs(g.positions()[b.kin_verts] - want).max() < 1e-6
    assert np.isfinite(g.positions()).all()
