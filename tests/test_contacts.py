"""Body-body contacts: the spatial-hash broad phase (integer cells from FP32
products) must give bit-identical candidate sets on CPU and GPU; the narrow
phase and the contact projection are checked against the FP64 oracle."""
import numpy as np
import pytest

from conftest import make_pair
from sbs_gb300 import scenes

CELL = 0.2


# generic offsets (no vertex of one box exactly on a face plane of the other,
# where FP32 and FP64 inside tests may legitimately disagree) and a shallow
# overlap, so penetrating vertices sit in tets with a boundary face
def overlapping_boxes(shift=(0.353, 0.121, 0.047), model=scenes.MODEL_STVK, n=4, body_contacts=1):
    xa, ta = scenes.bar_5tet(n + 1, n + 1, n + 1, 0.1)
    xb = xa + np.asarray(shift)
    bodies = [scenes.Body(x0=x, tets=ta, model=model, young=1e5, poisson=0.3, density=1000.0,
                          x_init=x.copy()) for x in (xa, xb)]
    return scenes.Scene("two-boxes", bodies, 1.0 / 60.0, 1, 5, 1, ground=((0.0, 1.0, 0.0), 5.0),
                        body_contacts=body_contacts, hash_cell=CELL)


def numpy_candidates(scene, xf, cell, self_contacts=False):
    """Independent restatement of the candidate definition in numpy."""
    inv_h = np.float32(1.0 / cell)
    offs = np.cumsum([0] + [len(b.x0) for b in scene.bodies])
    body_of_v = np.concatenate([np.full(len(b.x0), i) for i, b in enumerate(scene.bodies)])
    surf = np.concatenate([scenes.boundary_vertices(b.tets, len(b.x0)).astype(np.int64) + offs[i]
                           for i, b in enumerate(scene.bodies)])
    vc = np.floor(xf[surf] * inv_h).astype(np.int64)          # float32 product, then floor
    pairs = []
    t0 = 0
    for bi, b in enumerate(scene.bodies):
        t = b.tets.astype(np.int64) + offs[bi]
        faces = np.sort(np.concatenate([b.tets[:, [0, 1, 3]], b.tets[:, [1, 2, 3]],
                                        b.tets[:, [2, 0, 3]], b.tets[:, [0, 2, 1]]]), axis=1)
        _, inv, cnt = np.unique(faces, axis=0, return_inverse=True, return_counts=True)
        bnd = (cnt[inv.ravel()] == 1).reshape(4, -1).any(0)
        for k in np.nonzero(bnd)[0]:
            p = xf[t[k]]
            lo = np.floor(p.min(0) * inv_h).astype(np.int64)
            hi = np.floor(p.max(0) * inv_h).astype(np.int64)
            inside = np.all((vc >= lo) & (vc <= hi), axis=1)
            for v in surf[inside]:
                if v in t[k]:
                    continue
                if not self_contacts and body_of_v[v] == bi:
                    continue
                pairs.append((int(v) << 32) | (t0 + int(k)))
        t0 += len(b.tets)
    return np.array(sorted(pairs), np.uint64)


def positions32(scene):
    return np.concatenate([b.x_init for b in scene.bodies]).astype(np.float32)


@pytest.mark.parametrize("self_contacts", [False, True])
def test_oracle_hash_matches_numpy(oracle_mod, self_contacts):
    sc = overlapping_boxes()
    o = oracle_mod.Oracle(sc)
    xf = positions32(sc)
    a = oracle_mod.hash_candidates(o, xf, CELL, self_contacts)
    b = numpy_candidates(sc, xf, CELL, self_contacts)
    assert len(a) > 100
    assert np.array_equal(a, b)


def test_oracle_body_contacts_push_boxes_apart(oracle_mod):
    sc = overlapping_boxes()
    sc.gravity = (0.0, 0.0, 0.0)
    o = oracle_mod.Oracle(sc)
    o.detect_contacts()
    assert o.L.orc_n_body_contacts(o.h) > 0
    nv = len(sc.bodies[0].x0)

    def gap():
        x = o.get()
        return np.linalg.norm(x[:nv].mean(0) - x[nv:].mean(0))

    g0 = gap()
    o.step(10)
    assert gap() > g0 + 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("self_contacts", [1, 2])
def test_candidates_bit_exact(capi_mod, oracle_mod, self_contacts):
    sc = overlapping_boxes(body_contacts=self_contacts)
    g = capi_mod.Solver(sc, candidate_capacity=1 << 20)
    o = oracle_mod.Oracle(sc)
    rng = np.random.default_rng(3)
    for trial in range(3):
        xf = positions32(sc) + rng.uniform(-0.02, 0.02, size=(sc.n_verts, 3)).astype(np.float32)
        off = 0
        for b, n in enumerate(g.body_sizes):
            g.set_state(b, xf[off:off + n], np.zeros((n, 3)))
            off += n
        g.detect_contacts()
        cg = g.candidates()
        co = oracle_mod.hash_candidates(o, xf, CELL, self_contacts == 2)
        assert len(co) > 100
        assert np.array_equal(cg, co)


@pytest.mark.gpu
def test_body_contact_set_and_sweep(capi_mod, oracle_mod):
    sc = overlapping_boxes()
    g, o = make_pair(sc, capi_mod, oracle_mod)
    g.detect_contacts()
    vg, qg = g.contacts()
    vo, qo = o.detect_contacts()
    assert len(vo) > 3
    assert np.array_equal(vg, vo)
    assert np.abs(qg - qo).max() < 1e-5
    dt = sc.frame_dt
    o.L.orc_predict(o.h, dt)
    o.L.orc_solve(o.h, dt, 1)
    g.predict(dt)
    g.solve(dt, 1)
    x_g = np.concatenate([g.get_predicted(b) for b in range(2)])
    err = np.abs(x_g - o.get(oracle_mod.FIELD_XI)).max() / sc.bbox_diag()
    assert err < 2e-5


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 3])
def test_body_contacts_every_mode(capi_mod, oracle_mod, mode):
    sc = overlapping_boxes()
    g, o = make_pair(sc, capi_mod, oracle_mod, exec_mode=mode)
    g.step(1)
    o.step(1)
    assert g.stats().n_body_contacts == o.L.orc_n_body_contacts(o.h)
    order, off = g.tet_order()
    floor = oracle_mod.noise_floor(sc, 1, order, off, n_seeds=2)
    assert np.abs(g.positions() - o.get()).max() < 2 * floor + 1e-7


@pytest.mark.gpu
def test_box_drop_batch_runs(capi_mod):
    sc = scenes.box_drop(n_bodies=64, seed=9, min_cells=4, max_cells=9, arena=6.0,
                         iterations=10, substeps=2)
    g = capi_mod.Solver(sc)
    for _ in range(20):
        g.step(1)
    x = g.positions()
    assert np.all(np.isfinite(x))
    st = g.stats()
    assert st.frames == 20 and st.n_tets == sc.n_tets
