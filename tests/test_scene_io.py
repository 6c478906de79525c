"""Scene ingestion: read_ply (src/io/ply.cpp) and load_scene
(src/io/load_scene.cpp:83-365) into the C ABI."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden" / "ref_meshes.npz"


def write_ply(path, x, tets=None, tris=None, fmt="ascii"):
    """A PLY in the layout the reference's meshes use (float x y z, list uchar int)."""
    head = ["ply", f"format {fmt} 1.0", f"element vertex {len(x)}",
            "property float x", "property float y", "property float z"]
    if tris is not None:
        head += [f"element face {len(tris)}", "property list uchar int indices"]
    if tets is not None:
        head += [f"element tet {len(tets)}", "property list uchar int indices"]
    head.append("end_header")
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            for p in x:
                f.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n".encode())
            for t in (tris if tris is not None else []):
                f.write(("3 " + " ".join(str(int(i)) for i in t) + "\n").encode())
            for t in (tets if tets is not None else []):
                f.write(("4 " + " ".join(str(int(i)) for i in t) + "\n").encode())
        else:
            e = "<" if fmt == "binary_little_endian" else ">"
            f.write(np.asarray(x, np.float32).astype(e + "f4").tobytes())
            for n, rows in ((3, tris), (4, tets)):
                for t in (rows if rows is not None else []):
                    f.write(np.uint8(n).tobytes() + np.asarray(t, e + "i4").tobytes())


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
def test_read_ply_tet_mesh(capi_mod, tmp_path, fmt):
    d = np.load(GOLDEN)
    x, t = d["bar_tet_x0"], d["bar_tet_tets"]
    p = tmp_path / "bar.ply"
    write_ply(p, x, tets=t, fmt=fmt)
    xr, fr, tr = capi_mod.read_ply(p)
    assert np.array_equal(xr, x.astype(np.float32))
    assert np.array_equal(tr, t)
    assert len(fr) == 0


def test_read_ply_triangles_and_errors(capi_mod, tmp_path):
    d = np.load(GOLDEN)
    p = tmp_path / "floor.ply"
    write_ply(p, d["xz_plane_verts"], tris=d["xz_plane_tris"])
    x, f, t = capi_mod.read_ply(p)
    assert np.array_equal(f, d["xz_plane_tris"]) and len(t) == 0
    bad = tmp_path / "bad.ply"
    write_ply(bad, d["xz_plane_verts"], tris=np.array([[0, 1, 9]]))
    with pytest.raises(capi_mod.SbsError):
        capi_mod.read_ply(bad)
    with pytest.raises(capi_mod.SbsError):
        capi_mod.read_ply(tmp_path / "missing.ply")


def rescale_translate(x, box=None, tr=None):
    """load_scene.cpp:11-81 on float positions."""
    x = np.asarray(x, np.float32).copy()
    if box is not None:
        lo = x.min(0).astype(np.float64)
        hi = x.max(0).astype(np.float64)
        for k in range(3):
            dk = hi[k] - lo[k]
            if abs(dk) >= 1e-8:
                x[:, k] = (box[0][k] + (box[1][k] - box[0][k]) * (x[:, k].astype(np.float64) - lo[k]) / dk
                           ).astype(np.float32)
    if tr is not None:
        x = (x + np.asarray(tr, np.float32)).astype(np.float32)
    return x


@pytest.mark.gpu
def test_load_scene(capi_mod, tmp_path):
    import ctypes as C
    d = np.load(GOLDEN)
    (tmp_path / "meshes").mkdir()
    (tmp_path / "scenes").mkdir()
    write_ply(tmp_path / "meshes" / "floor.ply", d["xz_plane_verts"], tris=d["xz_plane_tris"])
    write_ply(tmp_path / "meshes" / "bar.ply", d["bar_tet_x0"], tets=d["bar_tet_tets"], fmt="binary_little_endian")
    box = ((-0.5, -0.05, -0.05), (0.5, 0.05, 0.05))
    tr = (0.0, 0.1, 0.0)
    scene = {
        "lights": {"directional": {"direction": {"x": 0, "y": 0, "z": -1}}},
        "environment": [{"id": "floor", "geometry": {"type": "triangle mesh", "path": "../meshes/floor.ply"},
                         "box": {"min": {"x": -2, "y": 0, "z": -2}, "max": {"x": 2, "y": 0, "z": 2}},
                         "color": {"r": 100, "g": 100, "b": 100}, "collideable": True}],
        "objects": [{"id": "bar", "geometry": {"type": "tetrahedral mesh", "path": "../meshes/bar.ply"},
                     "physics": {"type": "soft", "mass": 900.0, "velocity": {"x": 0.0, "y": -2.0, "z": 0.0}},
                     "box": {"min": {"x": box[0][0], "y": box[0][1], "z": box[0][2]},
                             "max": {"x": box[1][0], "y": box[1][1], "z": box[1][2]}},
                     "translation": {"x": tr[0], "y": tr[1], "z": tr[2]},
                     "color": {"r": 255, "g": 255, "b": 0}, "collideable": True}],
    }
    path = tmp_path / "scenes" / "scene.json"
    path.write_text(json.dumps(scene, indent=2))
    L = capi_mod.load()
    prm = capi_mod.default_params(exec_mode=1)
    h = C.c_void_p()
    assert L.sbs_gpu_create(C.byref(prm), C.byref(h)) == 0
    mat = capi_mod.Material(0, 1e5, 0.3, 1000.0)
    first, n = C.c_int32(), C.c_int32()
    cells = np.array([8, 8, 8], np.uint32)
    assert L.sbs_gpu_load_scene(h, str(path).encode(), C.byref(mat), cells, 0.5, C.byref(first), C.byref(n)) == 0
    assert (first.value, n.value) == (0, 1)
    assert L.sbs_gpu_finalize(h) == 0
    nv = len(d["bar_tet_x0"])
    x = np.zeros(3 * nv, np.float32)
    v = np.zeros(3 * nv, np.float32)
    assert L.sbs_gpu_get_state(h, 0, x.ctypes.data, v.ctypes.data) == 0
    expect = rescale_translate(d["bar_tet_x0"], box, tr)
    assert np.array_equal(x.reshape(-1, 3), expect)
    assert np.allclose(v.reshape(-1, 3), [0.0, -2.0, 0.0])
    # the floor (y = 0 after its rescale) stops the falling bar
    for _ in range(30):
        assert L.sbs_gpu_step(h, 1.0 / 60.0, 1, 10) == 0
    assert L.sbs_gpu_get_state(h, 0, x.ctypes.data, None) == 0
    assert np.isfinite(x).all() and x.reshape(-1, 3)[:, 1].min() > -0.05
    L.sbs_gpu_destroy(h)


# The reference's own data files (data/scenes/scene1.json and the meshes it
# and the viewer use), copied unchanged under tests/golden/ref_data/.
REF_DATA = Path(__file__).parent / "golden" / "ref_data"


def test_reference_binary_and_ascii_cube_agree(capi_mod):
    """data/meshes/cube_bin.ply (binary little endian) and cube.ply (ascii)
    hold the same cube: 8 vertices, 12 triangles."""
    xa, fa, ta = capi_mod.read_ply(REF_DATA / "meshes" / "cube.ply")
    xb, fb, tb = capi_mod.read_ply(REF_DATA / "meshes" / "cube_bin.ply")
    assert xa.shape == (8, 3) and fa.shape == (12, 3) and len(ta) == 0
    assert np.array_equal(xa, xb) and np.array_equal(fa, fb) and len(tb) == 0
    assert set(np.unique(xa).tolist()) == {0.0, 1.0}     # the unit cube (colour properties skipped)


def test_reference_bar_mesh_parses_as_the_golden_fixture(capi_mod):
    d = np.load(GOLDEN)
    x, f, t = capi_mod.read_ply(REF_DATA / "meshes" / "bar_tet.ply")
    assert np.array_equal(x, d["bar_tet_x0"].astype(np.float32))
    assert np.array_equal(t, d["bar_tet_tets"]) and len(f) == 0


@pytest.mark.gpu
def test_load_reference_scene1(capi_mod):
    """data/scenes/scene1.json as the reference ships it: the floor mesh
    becomes a signed-distance environment, the bar a body rescaled into its
    box and translated (load_scene.cpp:11-81); it falls onto the floor."""
    import ctypes as C
    spec = json.loads((REF_DATA / "scenes" / "scene1.json").read_text())
    obj = spec["objects"][0]
    box = tuple(tuple(obj["box"][k][a] for a in "xyz") for k in ("min", "max"))
    tr = tuple(obj["translation"][a] for a in "xyz")
    L = capi_mod.load()
    prm = capi_mod.default_params(exec_mode=1)
    h = C.c_void_p()
    assert L.sbs_gpu_create(C.byref(prm), C.byref(h)) == 0
    mat = capi_mod.Material(0, 1e5, 0.3, 1000.0)
    first, n = C.c_int32(), C.c_int32()
    cells = np.array([8, 8, 8], np.uint32)
    path = str(REF_DATA / "scenes" / "scene1.json").encode()
    assert L.sbs_gpu_load_scene(h, path, C.byref(mat), cells, 0.5, C.byref(first), C.byref(n)) == 0
    assert (first.value, n.value) == (0, 1)
    assert L.sbs_gpu_finalize(h) == 0
    x0, _, _ = capi_mod.read_ply(REF_DATA / "meshes" / "bar_tet.ply")
    x = np.zeros(3 * len(x0), np.float32)
    assert L.sbs_gpu_get_state(h, 0, x.ctypes.data, None) == 0
    assert np.array_equal(x.reshape(-1, 3), rescale_translate(x0, box, tr))
    for _ in range(60):
        assert L.sbs_gpu_step(h, 1.0 / 60.0, 1, 10) == 0
    assert L.sbs_gpu_get_state(h, 0, x.ctypes.data, None) == 0
    y = x.reshape(-1, 3)[:, 1]
    assert np.isfinite(x).all() and y.min() > -0.05 and y.min() < 1.0   # fell, and rests on y = 0
    L.sbs_gpu_destroy(h)
