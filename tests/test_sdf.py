"""Environment bodies as signed-distance grids (what environment_body_t builds
with Discregrid, src/physics/environment_body.cpp:12-78, evaluated by
sdf_model_t::evaluate, src/physics/collision/sdf_model.cpp:66-75) and their
contacts (bvh_model.cpp:72-94: n = normalised gradient, q = p + |sd| n)."""
from pathlib import Path

import numpy as np
import pytest

from sbs_gb300 import scenes

GOLDEN = Path(__file__).parent / "golden" / "ref_meshes.npz"


def box_mesh(lo, hi):
    """Closed box, 12 triangles wound outward."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float64)
    t = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [3, 6, 2], [3, 7, 6], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]], np.uint32)
    return v, t


def box_sdf(p, lo, hi):
    """Exact signed distance to an axis-aligned box."""
    c = (np.asarray(lo) + np.asarray(hi)) / 2
    e = (np.asarray(hi) - np.asarray(lo)) / 2
    q = np.abs(p - c) - e
    outside = np.linalg.norm(np.maximum(q, 0), axis=-1)
    inside = np.minimum(np.max(q, axis=-1), 0)
    return outside + inside


def grid_nodes(lo, hi, cells):
    xs = [np.linspace(lo[k], hi[k], cells[k] + 1) for k in range(3)]
    z, y, x = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return np.stack([x, y, z], -1)


def test_mesh_sdf_matches_box_distance(capi_mod):
    blo, bhi = (-0.3, -0.2, -0.25), (0.4, 0.1, 0.35)
    v, t = box_mesh(blo, bhi)
    lo, hi, cells = (-1.0, -0.8, -0.9), (1.1, 0.9, 1.0), (14, 11, 13)
    g = capi_mod.sdf_from_mesh(v, t, lo, hi, cells)
    exact = box_sdf(grid_nodes(lo, hi, cells), blo, bhi)
    assert np.abs(g - exact).max() < 1e-6


def test_open_floor_mesh_sign(capi_mod):
    d = np.load(GOLDEN)
    v, t = d["xz_plane_verts"], d["xz_plane_tris"]
    lo, hi, cells = (-0.9, -0.5, -0.9), (0.9, 0.5, 0.9), (6, 10, 6)
    g = capi_mod.sdf_from_mesh(v, t, lo, hi, cells)
    y = grid_nodes(lo, hi, cells)[..., 1]
    # above the quad the distance is +y, below -y (face region of the quad)
    assert np.abs(g - y).max() < 1e-6


def linear_floor_grid(y0=0.0):
    """Grid sampling sd = y - y0 exactly (trilinear reproduces it)."""
    lo, cells = np.array([-1.0, -1.5, -1.0]), (4, 6, 4)
    sp = np.array([0.75, 0.5, 0.75])
    nodes = (cells[0] + 1, cells[1] + 1, cells[2] + 1)
    y = lo[1] + sp[1] * np.arange(nodes[1])
    vals = np.broadcast_to((y - y0)[None, :, None], (nodes[2], nodes[1], nodes[0])).astype(np.float32)
    return (vals.copy(), nodes, lo, sp)


def test_oracle_linear_grid_equals_plane(oracle_mod):
    # a grid sampling sd = y + 0.05 gives the contacts of the plane y = -0.05
    a = scenes.beam_c1()
    a.ground = ((0.0, 1.0, 0.0), -0.05)
    b = scenes.beam_c1()
    b.ground = None
    b.sdf_grids = [linear_floor_grid(0.05)]
    oa, ob = oracle_mod.Oracle(a), oracle_mod.Oracle(b)
    va, qa = oa.detect_contacts()
    vb, qb = ob.detect_contacts()
    assert len(va) > 0
    assert np.array_equal(va, vb)
    assert np.abs(qa - qb).max() < 1e-8   # float32 node values


@pytest.mark.gpu
def test_gpu_grid_contacts_match_oracle(capi_mod, oracle_mod):
    from conftest import make_pair
    blo, bhi = (-0.2, -1.0, -0.2), (1.2, 0.06, 0.5)   # a block the beam's underside sinks into
    v, t = box_mesh(blo, bhi)
    lo, hi, cells = (-0.4, -1.2, -0.4), (1.4, 0.4, 0.7), (36, 32, 22)
    vals = capi_mod.sdf_from_mesh(v, t, lo, hi, cells)
    sp = (np.asarray(hi) - np.asarray(lo)) / np.asarray(cells)
    sc = scenes.beam_c1()
    sc.ground = None
    sc.sdf_grids = [(vals, (cells[0] + 1, cells[1] + 1, cells[2] + 1), lo, sp)]
    for mode in (1, 2):
        g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=mode)
        g.detect_contacts()
        vg, qg = g.contacts()
        vo, qo = o.detect_contacts()
        assert len(vo) > 0
        assert np.array_equal(vg, vo)
        assert np.abs(qg - qo).max() < 1e-5
        # one frame through the grid contacts
        g.step(1)
        o.step(1)
        assert np.isfinite(g.positions()).all()
        g.close()


@pytest.mark.gpu
def test_gpu_environment_mesh_like_plane(capi_mod):
    """The reference's floor mesh through environment_body_t's constructor
    path gives the plane's contacts."""
    d = np.load(GOLDEN)
    fv = d["xz_plane_verts"] * np.array([3.0, 1.0, 3.0]) + np.array([0.5, 0.05, 0.15])
    ft = d["xz_plane_tris"]
    a = scenes.beam_c1()
    a.ground = ((0.0, 1.0, 0.0), -0.05)           # y = 0.05: cuts the beam's bottom layer
    ga = capi_mod.Solver(a, exec_mode=1)
    b = scenes.beam_c1()
    b.ground = None
    gb = capi_mod.Solver.__new__(capi_mod.Solver)
    # build b by hand to call sbs_gpu_add_environment_mesh before finalize
    import ctypes as C
    L = capi_mod.load()
    prm = capi_mod.default_params(exec_mode=1)
    h = C.c_void_p()
    assert L.sbs_gpu_create(C.byref(prm), C.byref(h)) == 0
    body = b.bodies[0]
    mat = capi_mod.Material(body.model, body.young, body.poisson, body.density)
    bid = C.c_int32()
    x0 = np.ascontiguousarray(body.x0, np.float64).ravel()
    xi = np.ascontiguousarray(body.x_init, np.float64).ravel()
    tets = np.ascontiguousarray(body.tets, np.uint32).ravel()
    assert L.sbs_gpu_add_body(h, x0, xi.ctypes.data, len(body.x0), tets, len(body.tets), C.byref(mat), None,
                              C.byref(bid)) == 0
    assert L.sbs_gpu_pin_vertices(h, bid, np.ascontiguousarray(body.pinned, np.uint32), len(body.pinned)) == 0
    dom_lo, dom_hi = np.array([-1.5, -0.3, -1.5]), np.array([2.5, 0.3, 2.0])
    cells = np.array([16, 24, 14], np.uint32)
    assert L.sbs_gpu_add_environment_mesh(h, np.ascontiguousarray(fv, np.float64).ravel(), len(fv),
                                          np.ascontiguousarray(ft, np.uint32).ravel(), len(ft), dom_lo, dom_hi,
                                          cells) == 0
    assert L.sbs_gpu_finalize(h) == 0
    gb.L, gb.h, gb.scene, gb.body_sizes = L, h, b, [len(body.x0)]
    ga.detect_contacts()
    gb.detect_contacts()
    va, qa = ga.contacts()
    vb, qb = gb.contacts()
    assert len(va) > 0
    assert np.array_equal(va, vb)
    assert np.abs(qa - qb).max() < 1e-5
    ga.close()
    gb.close()


@pytest.mark.gpu
def test_gpu_grid_rejects_cluster_and_bad_grids(capi_mod):
    sc = scenes.beam_c1()
    sc.ground = None
    sc.sdf_grids = [linear_floor_grid(0.05)]
    with pytest.raises(capi_mod.SbsError):
        capi_mod.Solver(sc, exec_mode=3)
    vals, nodes, lo, sp = linear_floor_grid(0.05)
    vals = vals.copy()
    vals[0, 0, 0] = np.nan
    sc.sdf_grids = [(vals, nodes, lo, sp)]
    with pytest.raises(capi_mod.SbsError):
        capi_mod.Solver(sc)


# ---- the cubic Lagrange grid (Discregrid's CubicLagrangeDiscreteGrid,
# environment_body.cpp:72-73): 32-node serendipity cells

def cubic_layout_points(lo, sp, cells):
    """Positions of the cubic grid's values in their layout: vertices, then
    the nodes at 1/3 and 2/3 of every x-, y- and z-edge."""
    nx, ny, nz = (c + 1 for c in cells)
    lo, sp = np.asarray(lo, float), np.asarray(sp, float)
    pts = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                pts.append((i, j, k))
    for ax, (mx, my, mz) in enumerate(((nx - 1, ny, nz), (nx, ny - 1, nz), (nx, ny, nz - 1))):
        for k in range(mz):
            for j in range(my):
                for i in range(mx):
                    for s in (1 / 3, 2 / 3):
                        q = [i, j, k]
                        q[ax] += s
                        pts.append(tuple(q))
    return lo + np.asarray(pts, float) * sp


def serendipity(values, lo, sp, cells, p):
    """Independent numpy restatement of the 32-node cell interpolant: value
    and gradient at p (p inside the grid)."""
    nx, ny, nz = (c + 1 for c in cells)
    u = (np.asarray(p, float) - lo) / sp
    c = np.minimum(np.floor(u).astype(int), np.asarray(cells) - 1)
    r = 2 * (u - c) - 1
    V = values
    bases = [nx * ny * nz]
    bases.append(bases[0] + 2 * (nx - 1) * ny * nz)
    bases.append(bases[1] + 2 * nx * (ny - 1) * nz)
    f, g = 0.0, np.zeros(3)
    for a in (0, 1):
        for b in (0, 1):
            for e in (0, 1):
                s = np.array([2 * a - 1, 2 * b - 1, 2 * e - 1], float)
                val = V[((c[2] + e) * ny + c[1] + b) * nx + c[0] + a]
                lin = 1 + r * s
                q = 9 * (r @ r) - 19
                f += val * lin.prod() * q / 64
                for k in range(3):
                    g[k] += val * (s[k] * np.prod(np.delete(lin, k)) * q + lin.prod() * 18 * r[k]) / 64
    for ax in range(3):
        o = [k for k in range(3) if k != ax]
        for b1 in (0, 1):
            for b2 in (0, 1):
                idx3 = list(c)
                idx3[o[0]] += b1
                idx3[o[1]] += b2
                i, j, k = idx3
                if ax == 0:
                    base = bases[0] + 2 * ((k * ny + j) * (nx - 1) + i)
                elif ax == 1:
                    base = bases[1] + 2 * ((k * (ny - 1) + j) * nx + i)
                else:
                    base = bases[2] + 2 * ((k * ny + j) * nx + i)
                s1, s2 = 2 * b1 - 1, 2 * b2 - 1
                for t, tt in ((0, -1 / 3), (1, 1 / 3)):
                    val = V[base + t] * 9 / 64
                    u_ = r[ax]
                    pu = (1 - u_ * u_) * (1 + 9 * u_ * tt)
                    p1, p2 = 1 + r[o[0]] * s1, 1 + r[o[1]] * s2
                    f += val * pu * p1 * p2
                    g[ax] += val * (-2 * u_ * (1 + 9 * u_ * tt) + (1 - u_ * u_) * 9 * tt) * p1 * p2
                    g[o[0]] += val * pu * s1 * p2
                    g[o[1]] += val * pu * p1 * s2
    return f, g * 2 / sp


def _cubic_scene(values, cells, lo, sp):
    sc = scenes.beam_c1()
    sc.ground = None
    sc.sdf_grids = [(values, cells, lo, sp, "cubic")]
    return sc


def test_oracle_cubic_grid_matches_numpy_restatement(oracle_mod):
    rng = np.random.default_rng(3)
    cells, lo, sp = (3, 4, 2), np.array([-0.3, -0.5, 0.1]), np.array([0.2, 0.15, 0.3])
    pts = cubic_layout_points(lo, sp, cells)
    vals = rng.normal(size=len(pts)).astype(np.float32)
    o = oracle_mod.Oracle(_cubic_scene(vals, cells, lo, sp))
    hi = lo + sp * np.asarray(cells)
    for p in rng.uniform(lo, hi, size=(200, 3)):
        sd, g = o.grid_eval(0, p)
        f, gr = serendipity(vals.astype(np.float64), lo, sp, cells, p)
        assert abs(sd - f) < 1e-12 and np.abs(g - gr).max() < 1e-10
    assert o.grid_eval(0, hi + 0.01) is None


def test_cubic_grid_reproduces_cubic_polynomials(oracle_mod):
    """The 32-node element interpolates every cubic polynomial exactly
    (value and gradient), the property of the cubic Lagrange grid."""
    rng = np.random.default_rng(4)
    mons = [(a, b, c) for a in range(4) for b in range(4) for c in range(4) if a + b + c <= 3]
    coef = rng.normal(size=len(mons))

    def f(p):
        return sum(k * p[..., 0] ** a * p[..., 1] ** b * p[..., 2] ** c for k, (a, b, c) in zip(coef, mons))

    def grad(p, h=1e-6):
        return np.array([(f(p + h * e) - f(p - h * e)) / (2 * h) for e in np.eye(3)])
    cells, lo, sp = (2, 3, 2), np.array([-0.4, -0.3, -0.2]), np.array([0.4, 0.2, 0.2])
    vals = f(cubic_layout_points(lo, sp, cells))
    hi = lo + sp * np.asarray(cells)
    for p in rng.uniform(lo, hi, size=(100, 3)):
        fp, gp = serendipity(vals, lo, sp, cells, p)
        assert abs(fp - f(p)) < 1e-12
        assert np.abs(gp - grad(p)).max() < 1e-6


def test_cubic_grid_of_sphere_and_box(capi_mod, oracle_mod):
    """Analytic signed distances through the cubic grid: a radius-1 sphere
    sampled at the nodes of 0.25 m cells interpolates to within 5e-4 of its
    distance in the shell 0.6 < r < 1.4, a fifth of the trilinear grid's
    error on the same vertices or less; a box mesh's cubic node values are
    its exact distance."""
    cells, lo = (12, 12, 12), np.array([-1.5, -1.5, -1.5])
    sp = np.full(3, 3.0 / 12)
    pts = cubic_layout_points(lo, sp, cells)
    sph = (np.linalg.norm(pts, axis=1) - 1.0).astype(np.float32)
    o = oracle_mod.Oracle(_cubic_scene(sph, cells, lo, sp))
    n = 13 ** 3
    lin = scenes.beam_c1()
    lin.ground = None
    lin.sdf_grids = [(sph[:n].reshape(13, 13, 13), (13, 13, 13), lo, sp)]
    o_lin = oracle_mod.Oracle(lin)
    rng = np.random.default_rng(5)
    q = rng.normal(size=(300, 3))
    q = q / np.linalg.norm(q, axis=1)[:, None] * rng.uniform(0.6, 1.4, size=(300, 1))
    exact = np.linalg.norm(q, axis=1) - 1.0
    err = max(abs(o.grid_eval(0, p)[0] - e) for p, e in zip(q, exact))
    err_lin = max(abs(o_lin.grid_eval(0, p)[0] - e) for p, e in zip(q, exact))
    assert err < 5e-4 and err < 0.2 * err_lin
    blo, bhi = (-0.3, -0.2, -0.25), (0.4, 0.1, 0.35)
    v, t = box_mesh(blo, bhi)
    glo, ghi, gcells = np.array([-1.0, -0.8, -0.9]), np.array([1.1, 0.9, 1.0]), (7, 6, 5)
    vals = capi_mod.sdf_cubic_from_mesh(v, t, glo, ghi, gcells)
    exact = box_sdf(cubic_layout_points(glo, (ghi - glo) / np.asarray(gcells), gcells), blo, bhi)
    assert np.abs(vals - exact).max() < 1e-6


@pytest.mark.gpu
def test_gpu_cubic_grid_contacts_match_oracle(capi_mod, oracle_mod):
    """Contacts of the beam against a cubic grid of a box the beam's
    underside sinks into: same vertices as the oracle, contact points (p +
    |sd| n, from the interpolant and its gradient) within 1e-5 m."""
    from conftest import make_pair
    blo, bhi = (-0.2, -1.0, -0.2), (1.2, 0.06, 0.5)
    v, t = box_mesh(blo, bhi)
    lo, hi, cells = np.array([-0.4, -1.2, -0.4]), np.array([1.4, 0.4, 0.7]), (18, 16, 11)
    vals = capi_mod.sdf_cubic_from_mesh(v, t, lo, hi, cells)
    sc = _cubic_scene(vals, cells, lo, (hi - lo) / np.asarray(cells))
    for mode in (1, 2):
        g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=mode)
        g.detect_contacts()
        vg, qg = g.contacts()
        vo, qo = o.detect_contacts()
        assert len(vo) > 0
        assert np.array_equal(vg, vo)
        assert np.abs(qg - qo).max() < 1e-5
        g.step(1)
        o.step(1)
        assert np.isfinite(g.positions()).all()
        g.close()
