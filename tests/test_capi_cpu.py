"""C-ABI library without a GPU: it builds, loads, exports every declared
symbol, plans sweeps on the host, and fails loudly instead of falling back."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from sbs_gb300 import capi, scenes


def test_exports_every_declared_symbol():
    L = capi.load()
    names = capi.declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing


def test_nm_lists_declared_symbols():
    from sbs_gb300 import build
    out = subprocess.run(["nm", "-D", "--defined-only", str(build.LIB)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert set(capi.declared_symbols()) <= exported


def test_params_default_follow_reference_parameters():
    p = capi.default_params()
    # simulation_parameters.h:12-27
    assert p.compliance == 1e-4 and p.damping == 0.0 and p.collision_compliance == 1e-8
    assert tuple(p.gravity) == (0.0, -9.81, 0.0)
    # library-side defaults: automatic mode, finite-state checks and staged
    # tet records in the cluster mode
    assert p.exec_mode == capi.EXEC_AUTO and p.check_finite == 1 and p.stage_records == 1


def test_create_without_gpu_fails_loudly():
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = capi.load()
    h = C.c_void_p()
    p = capi.default_params()
    assert L.sbs_gpu_create(C.byref(p), C.byref(h)) == capi.SBS_ECUDA
    with pytest.raises(capi.SbsError):
        capi.Solver(scenes.beam_c1())


def test_plan_sweep_is_a_valid_colouring():
    for sc in (scenes.beam_c1(), scenes.beam_twist(16, 8, 8, 0.05)):
        order, off = capi.plan_sweep(sc)
        t = sc.bodies[0].tets
        assert np.array_equal(np.sort(order), np.arange(len(t)))
        sizes = np.diff(off)
        assert np.all(sizes[:-1] >= sizes[1:])          # colours by decreasing size
        for c in range(len(off) - 1):
            v = t[order[off[c]:off[c + 1]]].ravel()
            assert len(np.unique(v)) == len(v)


def test_plan_sweep_colour_count_98k_beam():
    order, off = capi.plan_sweep(scenes.beam_twist(lattice=False))
    # interior vertices of the 6-tet split touch 24 tets: at least 24 colours
    assert 24 <= len(off) - 1 <= 40
    # the grid's lattice colouring reaches the bound, 4096 tets per colour
    order, off = capi.plan_sweep(scenes.beam_twist())
    assert len(off) - 1 == 24 and np.all(np.diff(off) == 4096)
    t = scenes.beam_twist().bodies[0].tets
    for c in range(24):
        v = t[order[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)


@pytest.mark.parametrize("dims", [(9, 9, 9), (10, 7, 6), (13, 5, 9)])
def test_lattice_colouring_of_the_5tet_split(dims):
    """The periodic 34-colouring of bar_5tet (4 x 4 x 4-cube torus pattern):
    no two tets of a colour share a vertex on grids of any size (32 tets meet
    at a centre tet's vertex), and the planner uses it unless its own
    colouring of a small grid needs fewer colours."""
    x0, t = scenes.bar_5tet(*dims, 0.1)
    col = scenes.lattice_colours_5tet(*dims)
    assert len(col) == len(t) and len(np.unique(col)) == 34
    for c in range(34):
        v = t[col == c].ravel()
        assert len(np.unique(v)) == len(v)
    sc = scenes.Scene("b", [scenes.Body(x0=x0, tets=t, colours=col)], 1 / 60, 1, 1, 1)
    order, off = capi.plan_sweep(sc)
    assert 32 <= len(off) - 1 <= 34
    if len(off) - 1 == 34:
        # the classes are the lattice's own
        for c in range(34):
            assert len(np.unique(col[order[off[c]:off[c + 1]]])) == 1


def test_plan_sweep_rejects_a_bad_colouring():
    sc = scenes.beam_twist(8, 4, 4, 0.05)
    sc.bodies[0].colours = np.zeros(len(sc.bodies[0].tets), np.uint32)   # one colour: tets share vertices
    with pytest.raises(capi.SbsError):
        capi.plan_sweep(sc)


def test_plan_sweep_rejects_bad_indices():
    L = capi.load()
    x0 = np.zeros(12)
    tets = np.array([0, 1, 2, 7], np.uint32)
    n = C.c_uint32()
    assert L.sbs_gpu_plan_sweep(x0, 4, tets, 1, None, None, None, None, 0, C.byref(n)) == capi.SBS_EINVAL


def test_plan_sweep_reports_colour_overflow():
    """130 tets sharing one vertex need 130 colours; the planner allows 128."""
    n = 130
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    x0 = [[0.0, 0.0, 0.0]]
    tets = []
    for i, a in enumerate(ang):
        c, s_ = np.cos(a), np.sin(a)
        base = len(x0)
        x0 += [[c, s_, 0.0], [c * 1.1, s_ * 1.1, 0.1], [c, s_, 0.2]]
        tets.append([0, base, base + 1, base + 2])
    x0 = np.array(x0).ravel()
    tets = np.array(tets, np.uint32).ravel()
    L = capi.load()
    cnt = C.c_uint32()
    order = np.zeros(n, np.uint32)
    off = np.zeros(129, np.uint32)
    st = L.sbs_gpu_plan_sweep(x0, len(x0) // 3, tets, n, None, None, order.ctypes.data, off.ctypes.data, len(off),
                              C.byref(cnt))
    assert st == capi.SBS_ECOLOUR


def test_plan_sweep_multibody_scene_is_valid():
    sc = scenes.box_drop(n_bodies=12, min_cells=2, max_cells=6, arena=4.0)
    order, off = capi.plan_sweep(sc)
    t = np.concatenate([b.tets + o for b, o in zip(sc.bodies, np.cumsum([0] + [len(b.x0) for b in sc.bodies]))])
    assert np.array_equal(np.sort(order), np.arange(len(t)))
    for c in range(len(off) - 1):
        v = t[order[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)
    # 5-tet cubes: at most 32 tets meet at a vertex; the planner stays close
    assert len(off) - 1 <= 40


def test_golden_fixtures_reproduce(oracle_mod):
    from pathlib import Path
    from golden.make_golden import golden_scene, NAMES
    d = np.load(Path(__file__).parent / "golden" / "ref_meshes.npz")
    for name in NAMES:
        sc = golden_scene(d[f"{name}_x0"], d[f"{name}_tets"])
        o = oracle_mod.Oracle(sc)
        o.set_order(d[f"{name}_order"], d[f"{name}_offsets"])
        o.step(1)
        assert np.array_equal(o.get(), d[f"{name}_x1"])
        o.step(9)
        assert np.array_equal(o.get(), d[f"{name}_x10"])


def test_get_state_rejects_bad_output_buffers():
    """Output buffers are checked on the host before any library call."""
    class Fake(capi.Solver):
        def __init__(self):
            pass

        def _nv(self, body):
            return 4
    f = Fake()
    with pytest.raises(ValueError):
        f.get_state(-1, np.zeros(12, np.float64), None)
    with pytest.raises(ValueError):
        f.get_state(-1, np.zeros(11, np.float32), None)
    with pytest.raises(ValueError):
        f.get_state(-1, np.zeros((12, 2), np.float32)[:, 0], None)
