"""GPU kernels (through the C ABI) against the FP64 oracle running the same
Gauss-Seidel sweep order.

Tolerances.  One sweep from an identical state must agree to 2e-5 of the
bounding-box diagonal (FP32 arithmetic: measured 1.6e-6 .. 3.9e-6).  Over
whole frames the sequential loop amplifies rounding differences (a 1e-12 m
perturbation grows to 1e-4 m within a frame of the 450-tet beam, see
test_oracle.py), so multi-frame positions are compared against the oracle's
own noise floor: the spread between the oracle and the oracle restarted from
FP32-rounded initial positions (the larger of two nudge seeds); the GPU must
stay within 2x of it.
"""
import numpy as np
import pytest

from conftest import make_pair
from sbs_gb300 import scenes

pytestmark = pytest.mark.gpu

SWEEP_TOL = 2e-5


def sync_from_oracle(g, o, oracle):
    """Copy the oracle's state, rounded to FP32, into both solvers."""
    x = o.get().astype(np.float32).astype(np.float64)
    v = o.get(oracle.FIELD_V).astype(np.float32).astype(np.float64)
    o.set(oracle.FIELD_X, x)
    o.set(oracle.FIELD_V, v)
    off = 0
    for b, n in enumerate(g.body_sizes):
        g.set_state(b, x[off:off + n], v[off:off + n])
        off += n


def sweeps(g, o, oracle, dt, k):
    o.L.orc_detect_contacts(o.h)
    o.L.orc_predict(o.h, dt)
    o.L.orc_solve(o.h, dt, k)
    g.detect_contacts()
    g.predict(dt)
    g.solve(dt, k)
    return g.get_predicted(0).astype(np.float64), o.get(oracle.FIELD_XI)


def noise_floor(scene, oracle, frames, seed=0):
    from sbs_gb300 import capi
    order, off = capi.plan_sweep(scene)
    return oracle.noise_floor(scene, frames, order, off, seed, n_seeds=2)


@pytest.mark.parametrize("pre", [0, 5])
def test_one_sweep_stvk(capi_mod, oracle_mod, pre):
    sc = scenes.beam_c1()
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.step(pre)
    o.step(pre)
    sync_from_oracle(g, o, oracle_mod)
    xg, xo = sweeps(g, o, oracle_mod, sc.frame_dt, 1)
    assert np.abs(xg - xo).max() / sc.bbox_diag() < SWEEP_TOL
    lg, lo = g.lambdas()[:, 0], o.lambdas()[:, 0]
    assert np.abs(lg - lo).max() <= 1e-2 * np.abs(lo).max()


def test_one_sweep_snh_twist(capi_mod, oracle_mod):
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.step(2)
    o.step(2)
    sync_from_oracle(g, o, oracle_mod)
    xg, xo = sweeps(g, o, oracle_mod, sc.frame_dt / sc.substeps, 1)
    assert np.abs(xg - xo).max() / sc.bbox_diag() < SWEEP_TOL
    lg, lo = g.lambdas(), o.lambdas()
    assert np.abs(lg - lo).max() <= 1e-2 * np.abs(lo).max()


def test_one_sweep_with_contacts(capi_mod, oracle_mod):
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), -0.15)   # plane y = 0.15 cuts the beam
    g, o = make_pair(sc, capi_mod, oracle_mod)
    xg, xo = sweeps(g, o, oracle_mod, sc.frame_dt, 1)
    assert np.abs(xg - xo).max() / sc.bbox_diag() < SWEEP_TOL


def test_contact_set_is_identical(capi_mod, oracle_mod):
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), -0.15)
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.detect_contacts()
    vg, qg = g.contacts()
    vo, qo = o.detect_contacts()
    assert len(vo) > 0
    assert np.array_equal(vg, vo)          # both sorted by (plane, vertex)
    assert np.abs(qg - qo).max() < 1e-6


def test_contact_sets_after_frames(capi_mod, oracle_mod):
    # the beam sags onto a raised ground: compare the frame's contact set on
    # identical (synchronised) states
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), 0.02)
    g, o = make_pair(sc, capi_mod, oracle_mod)
    for _ in range(6):
        g.step(1)
        o.step(1)
        sync_from_oracle(g, o, oracle_mod)
        g.detect_contacts()
        vg, _ = g.contacts()
        vo, _ = o.detect_contacts()
        assert np.array_equal(vg, vo)


@pytest.mark.parametrize("name", ["tetrahedron", "2tets", "3tets", "cube_tet", "tet_bar_5x2x2",
                                  "bar_tet"])
def test_reference_meshes_first_frame(capi_mod, oracle_mod, name):
    from golden.make_golden import golden_scene
    d = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "ref_meshes.npz")
    sc = golden_scene(d[f"{name}_x0"], d[f"{name}_tets"])
    g = capi_mod.Solver(sc)
    g.step(1)
    err = np.abs(g.positions() - d[f"{name}_x1"]).max() / sc.bbox_diag()
    floor = noise_floor(sc, oracle_mod, 1) / sc.bbox_diag()
    assert err < max(2 * floor, SWEEP_TOL)


def test_beam450_frames_within_noise_floor(capi_mod, oracle_mod):
    sc = scenes.beam_c1()
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.step(1)
    o.step(1)
    err = float(np.abs(g.positions() - o.get()).max())
    floor = noise_floor(sc, oracle_mod, 1)
    assert err < 2 * floor + 1e-7


def test_beam98k_first_frame(capi_mod, oracle_mod):
    sc = scenes.beam_twist()
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.step(1)
    o.step(1)
    x = g.positions()
    assert np.all(np.isfinite(x))
    err = float(np.abs(x - o.get()).max())
    order, off = g.tet_order()
    assert err < 2 * oracle_mod.noise_floor(sc, 1, order, off, threads=16, n_seeds=2) + 1e-7
    b = sc.bodies[0]
    assert np.array_equal(x[b.pinned], b.x0[b.pinned].astype(np.float32))


def test_kinematic_face_follows_rotation(capi_mod):
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    g = capi_mod.Solver(sc)
    g.step(10)
    b = sc.bodies[0]
    ang = b.kin_omega * 10 * sc.frame_dt
    R = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
    c = np.array(b.kin_center)
    want = (b.x0[b.kin_verts] - c) @ R.T + c
    assert np.abs(g.positions()[b.kin_verts] - want).max() < 1e-6


def test_masses_and_surface(capi_mod, oracle_mod):
    sc = scenes.beam_twist(8, 3, 3, 0.05)
    g, o = make_pair(sc, capi_mod, oracle_mod)
    m = o.masses()
    w = np.where(m > 0, 1.0 / np.where(m > 0, m, 1), 0.0)
    assert np.allclose(g.inv_masses(), w, rtol=1e-6)
    assert np.array_equal(g.surface(), o.surface())


def test_colouring_is_a_valid_sweep(capi_mod):
    sc = scenes.beam_twist()
    g = capi_mod.Solver(sc)
    order, off = g.tet_order()
    assert np.array_equal(np.sort(order), np.arange(sc.n_tets))
    t = sc.bodies[0].tets
    for c in range(len(off) - 1):
        v = t[order[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)
    # the host planner gives the same colours; the solver may order tets within
    # a colour differently (by owning CTA), which leaves the sweep unchanged
    po, poff = capi_mod.plan_sweep(sc)
    assert np.array_equal(poff, off)
    for c in range(len(off) - 1):
        assert np.array_equal(np.sort(po[off[c]:off[c + 1]]), np.sort(order[off[c]:off[c + 1]]))


@pytest.mark.parametrize("mode", [1, 2])
def test_deterministic(capi_mod, mode):
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    a = capi_mod.Solver(sc, exec_mode=mode)
    b = capi_mod.Solver(sc, exec_mode=mode)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.positions(), b.positions())


def test_graph_and_persistent_agree(capi_mod, oracle_mod):
    sc = scenes.beam_c1()
    a = capi_mod.Solver(sc, exec_mode=1)
    b = capi_mod.Solver(sc, exec_mode=2)
    a.step(1)
    b.step(1)
    floor = noise_floor(sc, oracle_mod, 1)
    assert np.abs(a.positions() - b.positions()).max() < 2 * floor + 1e-7


@pytest.mark.parametrize("make,frames", [(scenes.beam_c1, 1), (lambda: scenes.beam_twist(16, 4, 4, 0.05), 1)])
def test_wavefront_matches_oracle(capi_mod, oracle_mod, make, frames):
    sc = make()
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=capi_mod.EXEC_WAVEFRONT)
    assert g.stats().exec_mode == capi_mod.EXEC_WAVEFRONT
    g.step(frames)
    o.step(frames)
    floor = noise_floor(sc, oracle_mod, frames)
    assert np.abs(g.positions() - o.get()).max() < 2 * floor + 1e-7


def test_wavefront_with_contacts_and_springs(capi_mod, oracle_mod):
    # ground contacts (beam on a raised plane) and distance constraints take
    # the wavefront kernel's grid-barrier paths
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), -0.05)
    a = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_WAVEFRONT)
    b = capi_mod.Solver(sc, exec_mode=1)
    a.step(3)
    b.step(3)
    floor = noise_floor(sc, oracle_mod, 3)
    assert a.stats().n_contacts > 0
    assert np.abs(a.positions() - b.positions()).max() < 2 * floor + 1e-7
    hb = scenes.hanging_block()
    a = capi_mod.Solver(hb, exec_mode=capi_mod.EXEC_WAVEFRONT)
    b = capi_mod.Solver(hb, exec_mode=1)
    a.step(5)
    b.step(5)
    assert np.abs(a.positions() - b.positions()).max() < 1e-3


def test_wavefront_deterministic(capi_mod):
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    a = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_WAVEFRONT)
    b = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_WAVEFRONT)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.positions(), b.positions())


def test_residual_matches_oracle(capi_mod, oracle_mod):
    for sc in (scenes.beam_c1(), scenes.beam_twist(16, 4, 4, 0.05)):
        g, o = make_pair(sc, capi_mod, oracle_mod)
        g.step(2)
        o.step(2)
        sync_from_oracle(g, o, oracle_mod)
        dt = sc.frame_dt / sc.substeps
        sweeps(g, o, oracle_mod, dt, 1)
        r, e = g.residual(dt)
        ro = np.zeros(3)
        o.L.orc_residual(o.h, dt, ro)
        assert r == pytest.approx(ro[0], rel=1e-3)
        assert e == pytest.approx(ro[1], rel=1e-3)


def test_residual_kahan_on_large_mesh(capi_mod, oracle_mod):
    # 98k tets: the compensated FP32 sums agree with the FP64 oracle
    sc = scenes.beam_twist()
    g, o = make_pair(sc, capi_mod, oracle_mod)
    dt = sc.frame_dt / sc.substeps
    xg, xo = sweeps(g, o, oracle_mod, dt, 1)
    g.set_predicted(0, xo)
    r, e = g.residual(dt)
    ro = np.zeros(3)
    o.L.orc_residual(o.h, dt, ro)
    assert r == pytest.approx(ro[0], rel=1e-3)
    assert e == pytest.approx(ro[1], rel=1e-3)


def test_invalid_arguments(capi_mod):
    import ctypes as C
    L = capi_mod.load()
    h = C.c_void_p()
    p = capi_mod.default_params()
    assert L.sbs_gpu_create(C.byref(p), C.byref(h)) == capi_mod.SBS_OK
    x0 = np.zeros(12)
    x0[3], x0[7], x0[11] = 1, 1, 1
    tets_bad = np.array([0, 1, 2, 9], np.uint32)
    mat = capi_mod.Material(0, 1e5, 0.3, 1000)
    bid = C.c_int32()
    assert L.sbs_gpu_add_body(h, x0, None, 4, tets_bad, 1, C.byref(mat), None,
                              C.byref(bid)) == capi_mod.SBS_EINVAL
    assert L.sbs_gpu_step(h, 1 / 60, 1, 1) == capi_mod.SBS_ESTATE
    assert L.sbs_gpu_finalize(h) == capi_mod.SBS_ESTATE   # no bodies
    tets = np.array([0, 1, 2, 3], np.uint32)
    assert L.sbs_gpu_add_body(h, x0, None, 4, tets, 1, C.byref(mat), None,
                              C.byref(bid)) == capi_mod.SBS_OK
    assert L.sbs_gpu_pin_vertices(h, 5, tets, 1) == capi_mod.SBS_EINVAL
    assert L.sbs_gpu_finalize(h) == capi_mod.SBS_OK
    assert L.sbs_gpu_step(h, -1.0, 1, 1) == capi_mod.SBS_EINVAL
    xs, vs = np.zeros(12, np.float32), np.zeros(12, np.float32)
    assert L.sbs_gpu_get_state(h, 0, xs.ctypes.data, vs.ctypes.data) == capi_mod.SBS_OK
    xbad = np.full(12, np.nan, np.float32)
    vnew = np.ones(12, np.float32)
    assert L.sbs_gpu_set_state(h, 0, xbad.ctypes.data, vnew.ctypes.data) == capi_mod.SBS_EINVAL
    # a rejected call leaves positions and velocities as they were
    x2, v2 = np.zeros(12, np.float32), np.zeros(12, np.float32)
    assert L.sbs_gpu_get_state(h, 0, x2.ctypes.data, v2.ctypes.data) == capi_mod.SBS_OK
    assert np.array_equal(xs, x2) and np.array_equal(vs, v2)
    assert L.sbs_gpu_destroy(h) == capi_mod.SBS_OK


# --- cluster-resident mode -------------------------------------------------

@pytest.mark.parametrize("make", [lambda: scenes.beam_c1(),
                                  lambda: scenes.beam_twist(16, 4, 4, 0.05)])
def test_cluster_mode_one_frame(capi_mod, oracle_mod, make):
    sc = make()
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=capi_mod.EXEC_CLUSTER)
    assert g.stats().exec_mode == capi_mod.EXEC_CLUSTER
    g.step(1)
    o.step(1)
    err = float(np.abs(g.positions() - o.get()).max())
    assert err < 2 * noise_floor(sc, oracle_mod, 1) + 1e-7


def test_cluster_mode_contacts_and_residual(capi_mod, oracle_mod):
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), -0.15)
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=capi_mod.EXEC_CLUSTER)
    g.step(1)
    o.step(1)
    vg, _ = g.contacts()
    # the frame's contacts come from the identical initial state
    o2 = oracle_mod.Oracle(sc)
    vo, _ = o2.detect_contacts()
    assert np.array_equal(vg, vo)
    r, e = g.residual(sc.frame_dt)
    assert np.isfinite(r) and np.isfinite(e) and r > 0


def _batch(n=40, seed=5):
    sc = scenes.box_drop(n_bodies=n, seed=seed, min_cells=5, max_cells=11, arena=12.0,
                         body_contacts=False, iterations=6, substeps=1)
    return sc


def test_cluster_mode_batch_of_bodies(capi_mod, oracle_mod):
    sc = _batch()
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=capi_mod.EXEC_CLUSTER)
    order, off = g.tet_order()
    # colour segments are vertex-disjoint, whatever the grouping
    tets = np.concatenate([b.tets.astype(np.int64) + sum(len(bb.x0) for bb in sc.bodies[:i])
                           for i, b in enumerate(sc.bodies)])
    for c in range(len(off) - 1):
        v = tets[order[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)
    g.step(1)
    o.step(1)
    err = float(np.abs(g.positions() - o.get()).max())
    assert err < 2 * oracle_mod.noise_floor(sc, 1, order, off, n_seeds=2) + 1e-7


def test_cluster_mode_deterministic(capi_mod):
    sc = scenes.beam_twist(16, 4, 4, 0.05)
    a = capi_mod.Solver(sc, exec_mode=3)
    b = capi_mod.Solver(sc, exec_mode=3)
    a.step(4)
    b.step(4)
    assert np.array_equal(a.positions(), b.positions())


@pytest.mark.parametrize("make", [lambda: scenes.beam_twist(16, 4, 4, 0.05), lambda: _batch(24, seed=9)])
def test_cluster_staging_is_exact(capi_mod, make):
    """Tet records staged in shared memory one phase ahead (bulk async copies)
    and records read from global memory in the phase give identical bits."""
    sc = make()
    a = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_CLUSTER, stage_records=1)
    b = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_CLUSTER, stage_records=0)
    assert a.stats().cluster_phase_max_tets > 0
    a.step(3)
    b.step(3)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())


@pytest.mark.parametrize("mode", [1, 2])
def test_small_colour_merge_is_exact(capi_mod, mode):
    """A colour run across the grid or, among the merged small colours, by one
    CTA after the others: the merge threshold the autotuner picks does not
    change results.  The graph mode's two kernels agree to the bit; in the
    persistent kernel the tail phase inlines the projection at another site,
    where the compiler contracts multiply-adds differently, so one iteration
    agrees to a few ulps (which the sequential loop then amplifies, as any
    rounding difference)."""
    sc = scenes.beam_c1()
    a = capi_mod.Solver(sc, exec_mode=mode, tail_threshold=0)        # every colour across the grid
    b = capi_mod.Solver(sc, exec_mode=mode, tail_threshold=1 << 20)  # every colour in the one-CTA tail
    assert a.stats().n_tail_colours == 0
    assert b.stats().n_tail_colours == b.stats().n_colours
    if mode == 1:
        a.step(3)
        b.step(3)
        assert np.array_equal(a.positions(), b.positions())
        assert np.array_equal(a.velocities(), b.velocities())
    else:
        a.step(1, iterations=1)
        b.step(1, iterations=1)
        assert np.abs(a.positions() - b.positions()).max() < 1e-6 * sc.bbox_diag()


@pytest.mark.parametrize("kind", ["uniaxial", "compressed", "shear", "general"])
def test_snh_kernel_against_closed_form_stress(capi_mod, kind):
    """The GPU's stable Neo-Hookean projection against the closed-form
    Neo-Hookean stress (Macklin & Mueller 2021), independent of the oracle:
    one projection from zero multipliers moves vertex i by w dt^2 f_i (1 - c w
    + O(w^2)); two vertex masses m and 2m (Richardson) remove the O(w) term.
    FP32 positions limit the comparison to ~1e-3 of the largest force."""
    from test_oracle import REST, SNH_KAT_F, snh_closed_form_forces
    E, nu, dt = 1e5, 0.3, 1 / 60
    xrest = REST.copy()
    x = (xrest - xrest[3]) @ SNH_KAT_F[kind].T + xrest[3]
    f = snh_closed_form_forces(xrest, x, E, nu)
    scaled = []
    for m in (60.0, 120.0):
        b = scenes.Body(x0=xrest, tets=np.array([[0, 1, 2, 3]], np.uint32), model=scenes.MODEL_SNH, young=E,
                        poisson=nu, density=1000.0, x_init=x, mass=np.full(4, m))
        sc = scenes.Scene("one", [b], dt, 1, 1, 1, gravity=(0.0, 0.0, 0.0), ground=None)
        g = capi_mod.Solver(sc)
        xf = x.astype(np.float32)
        g.set_predicted(0, xf)
        g.solve(dt, 1)
        dx = g.get_predicted(0).astype(np.float64) - xf.astype(np.float64)
        g.close()
        scaled.append(dx * m / dt ** 2)
    extrapolated = 2 * scaled[1] - scaled[0]
    assert np.abs(scaled[1] - f).max() < 0.05 * np.abs(f).max()      # first order already close
    assert np.abs(extrapolated - f).max() < 3e-3 * np.abs(f).max()


def test_colour_size_cap(capi_mod, oracle_mod):
    """Scenes that run in the global modes only: colours are rebalanced into
    more classes so that none holds more tets than the cap (one per resident
    thread of the persistent kernel by default).  With a small cap: every
    class within it, vertex-disjoint, at least ceil(T / cap) classes, and one
    frame against the oracle replaying that sweep within twice its FP32 noise
    floor."""
    sc = _batch(24, seed=11)
    g0 = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_PERSISTENT, colour_size_cap=-1)
    _, off0 = g0.tet_order()
    g0.close()
    T = sc.n_tets
    cap = int(np.ceil(T / (len(off0) - 1) * 0.8))
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=capi_mod.EXEC_PERSISTENT, colour_size_cap=cap)
    order, off = g.tet_order()
    sizes = np.diff(off)
    assert len(sizes) >= -(-T // cap) > len(off0) - 1
    assert sizes.max() <= cap
    assert np.array_equal(np.sort(order), np.arange(T))
    tets = np.concatenate([b.tets.astype(np.int64) + sum(len(bb.x0) for bb in sc.bodies[:i])
                           for i, b in enumerate(sc.bodies)])
    for c in range(len(off) - 1):
        v = tets[order[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)
    g.step(1)
    o.step(1)
    err = float(np.abs(g.positions() - o.get()).max())
    assert err < 2 * oracle_mod.noise_floor(sc, 1, order, off, n_seeds=2) + 1e-7
