"""Visual-model sync: the boundary mesh numbering of tetrahedral_mesh_boundary_t
(src/physics/tetrahedral_mesh_boundary.cpp:76-120) and the vertex normals of
compute_normals (:122-145), as updated by tetrahedral_body_t::update_visual_model
(src/physics/tetrahedral_body.cpp:157-165)."""
from pathlib import Path

import numpy as np
import pytest

from sbs_gb300 import scenes

GOLDEN = Path(__file__).parent / "golden" / "ref_meshes.npz"
NAMES = ["tetrahedron", "2tets", "3tets", "cube_tet", "tet_bar_5x2x2", "bar_tet"]

# unit normals from FP32 positions against the FP64 oracle
NORMAL_TOL = 2e-5


def restated_visual_model(tets):
    """Independent restatement of the reference's numbering: faces of each tet
    in faces_copy order (topology.cpp:335-342), a face listed once at its first
    appearance with that winding, boundary = != 2 incident tets, surface
    vertices numbered by first appearance."""
    faces = []
    count = {}
    for t in np.asarray(tets, np.int64):
        for f in ((t[0], t[1], t[3]), (t[1], t[2], t[3]), (t[2], t[0], t[3]), (t[0], t[2], t[1])):
            key = tuple(sorted(f))
            if key not in count:
                faces.append(f)
                count[key] = 0
            count[key] += 1
    tris, vmap, local = [], [], {}
    for f in faces:
        if count[tuple(sorted(f))] == 2:
            continue
        tri = []
        for v in f:
            if v not in local:
                local[v] = len(vmap)
                vmap.append(v)
            tri.append(local[v])
        tris.append(tri)
    return np.array(tris, np.uint32).reshape(-1, 3), np.array(vmap, np.uint32)


def restated_normals(x, tris, vmap, prev=None):
    """compute_normals on positions x[vmap]: add each triangle's cross product
    to its corners in triangle order, then normalise nonzero normals."""
    n = np.zeros((len(vmap), 3)) if prev is None else prev.copy()
    p = x[vmap]
    for a, b, c in tris:
        cr = np.cross(p[b] - p[a], p[c] - p[a])
        n[a] += cr
        n[b] += cr
        n[c] += cr
    z = np.sqrt((n * n).sum(1))
    n[z > 0] /= z[z > 0, None]
    return n


def mesh_scenes():
    from golden.make_golden import golden_scene
    d = np.load(GOLDEN)
    out = [golden_scene(d[f"{k}_x0"], d[f"{k}_tets"]) for k in NAMES]
    out.append(scenes.beam_c1())
    return out


def test_oracle_mesh_matches_restatement(oracle_mod):
    for sc in mesh_scenes():
        o = oracle_mod.Oracle(sc)
        tris, vmap = o.surface_mesh(0)
        rt, rv = restated_visual_model(sc.bodies[0].tets)
        assert np.array_equal(tris, rt), sc.name
        assert np.array_equal(vmap, rv), sc.name


def test_boundary_is_closed_two_manifold(oracle_mod):
    for sc in mesh_scenes()[3:]:
        tris, vmap = oracle_mod.Oracle(sc).surface_mesh(0)
        e = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert (cnt == 2).all(), sc.name
        assert len(vmap) == len(np.unique(tris))


def test_oracle_normals_accumulate_like_reference(oracle_mod):
    sc = scenes.beam_c1()
    o = oracle_mod.Oracle(sc)
    tris, vmap = o.surface_mesh(0)
    # the body constructor's update, then one per frame, never cleared
    n = restated_normals(o.get(), tris, vmap)
    for _ in range(3):
        o.step(1)
        n = restated_normals(o.get(), tris, vmap, n)
        p, no = o.update_surface(0, True)
        assert np.allclose(p, o.get()[vmap], atol=0, rtol=0)
        assert np.abs(no - n).max() < 1e-12
    p, fresh = o.update_surface(0, False)
    assert np.abs(fresh - restated_normals(o.get(), tris, vmap)).max() < 1e-12


def small_boxes():
    return scenes.box_drop(n_bodies=3, min_cells=2, max_cells=4, arena=2.0, body_contacts=False)


@pytest.mark.gpu
def test_gpu_mesh_equals_oracle(capi_mod, oracle_mod):
    for sc in mesh_scenes() + [small_boxes()]:
        g = capi_mod.Solver(sc)
        o = oracle_mod.Oracle(sc)
        for b in range(len(sc.bodies)):
            gt, gv = g.surface_mesh(b)
            ot, ov = o.surface_mesh(b)
            assert np.array_equal(gt, ot) and np.array_equal(gv, ov), (sc.name, b)
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("make", [scenes.beam_c1, small_boxes])
def test_gpu_normals_match_oracle(capi_mod, oracle_mod, make):
    sc = make()
    g = capi_mod.Solver(sc)
    o = oracle_mod.Oracle(sc)
    offs = np.cumsum([0] + [len(b.x0) for b in sc.bodies])
    for frame in range(3):
        g.step(2)
        x = g.positions().astype(np.float64)
        o.set(oracle_mod.FIELD_X, x)
        for b in range(len(sc.bodies)):
            acc = frame < 2
            buf = g.update_surface(b, accumulate=acc)
            p, n = o.update_surface(b, acc)
            _, vmap = g.surface_mesh(b)
            assert np.array_equal(buf[:, :3], x[offs[b] + vmap].astype(np.float32))
            assert np.array_equal(p, x[offs[b] + vmap])
            assert np.abs(buf[:, 3:6] - n).max() < NORMAL_TOL, (frame, b)
            assert (buf[:, 6:] == 0).all()
    g.close()


@pytest.mark.gpu
def test_gpu_surface_device_buffer(capi_mod):
    torch = pytest.importorskip("torch")
    sc = scenes.beam_c1()
    a = capi_mod.Solver(sc)
    a.step(3)
    # same state, normals recomputed from zero: device and host paths agree
    host = a.update_surface(0, False)
    dev = torch.full((host.shape[0], 9), 7.0, dtype=torch.float32, device="cuda:0")
    a.update_surface(0, False, buffer=dev.data_ptr(), stride=9)
    d = dev.cpu().numpy()
    assert np.array_equal(d[:, :6], host[:, :6])
    assert (d[:, 6:] == 7.0).all()
    # host buffer with a wider stride: only the first six floats are written
    wide = np.full((host.shape[0], 12), -1.0, np.float32)
    a.update_surface(0, False, buffer=wide, stride=12)
    assert np.array_equal(wide[:, :6], host[:, :6])
    assert (wide[:, 6:] == -1.0).all()
    a.close()


@pytest.mark.gpu
def test_gpu_surface_errors(capi_mod):
    g = capi_mod.Solver(scenes.beam_c1())
    with pytest.raises(capi_mod.SbsError):
        g.update_surface(0, True, buffer=np.zeros((200, 9), np.float32), stride=5)
    with pytest.raises(capi_mod.SbsError):
        g.surface_mesh(1)
    g.close()
