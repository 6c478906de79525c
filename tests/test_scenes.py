"""Scene generators: sizes of the named workloads and mesh validity (CPU)."""
import numpy as np
import pytest

from sbs_gb300 import scenes


def test_beam_450_counts():
    x0, tets = scenes.bar_5tet(11, 4, 4, 0.1)
    assert (len(x0), len(tets)) == (176, 450)


def test_beam_98k_counts():
    x0, tets = scenes.bar_6tet(65, 17, 17, 0.05)
    assert (len(x0), len(tets)) == (18785, 98304)


def test_block_2p6m_counts():
    # vertex count only (cheap): (128+1)(64+1)(64+1); tets 128*64*64*5
    assert 129 * 65 * 65 == 545025 and 128 * 64 * 64 * 5 == 2621440


@pytest.mark.parametrize("gen", [scenes.bar_5tet, scenes.bar_6tet])
def test_split_is_conforming_and_fills_volume(gen):
    x0, tets = gen(4, 3, 5, 0.5)
    vol = scenes.signed_volumes(x0, tets)
    assert np.all(np.abs(vol) > 1e-9)
    assert abs(np.abs(vol).sum() - (3 * 2 * 4) * 0.125) < 1e-9
    # every face is shared by at most two tets, interior faces by exactly two
    t = tets.astype(np.int64)
    faces = np.sort(np.concatenate([t[:, [0, 1, 3]], t[:, [1, 2, 3]], t[:, [2, 0, 3]],
                                    t[:, [0, 2, 1]]]), axis=1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert cnt.max() == 2
    n_boundary = (cnt == 1).sum()
    # boundary triangles of a 3x2x4 box: 2 per unit square of surface
    assert n_boundary == 2 * 2 * (3 * 2 + 2 * 4 + 3 * 4)


def test_first_cube_matches_reference_table():
    # get_simple_bar_model.cpp:90-113, cube (0,0,0) has even parity
    _, tets = scenes.bar_5tet(2, 2, 2)
    p = {0: 0, 1: 4, 2: 6, 3: 2, 4: 1, 5: 5, 6: 7, 7: 3}  # corner label -> vertex id
    want = [[3, 1, 4, 0], [6, 1, 3, 2], [4, 1, 6, 5], [6, 3, 4, 7], [3, 1, 6, 4]]
    assert tets.tolist() == [[p[c] for c in row] for row in want]


def test_lumped_mass_total():
    x0, tets = scenes.bar_5tet(11, 4, 4, 0.1)
    m = scenes.lumped_masses(x0, tets, 1000.0)
    assert abs(m.sum() - 1000.0 * 1.0 * 0.3 * 0.3) < 1e-9


def test_boundary_vertices_of_beam():
    x0, tets = scenes.bar_5tet(11, 4, 4, 0.1)
    b = scenes.boundary_vertices(tets, len(x0))
    # all vertices except the interior ones (i in 1..9, j in 1..2, k in 1..2)
    assert len(b) == 176 - 9 * 2 * 2


def test_jitter_is_seeded_and_frozen():
    x = np.zeros((10, 3))
    a = scenes.jitter(x, 1e-3, 7, frozen=np.array([0, 3]))
    b = scenes.jitter(x, 1e-3, 7, frozen=np.array([0, 3]))
    assert np.array_equal(a, b)
    assert np.all(a[[0, 3]] == 0) and np.abs(a).max() <= 1e-3


def test_warm_start_workloads():
    """The warm-start workloads build the scenes their configurations name."""
    from sbs_gb300 import warmstart
    sc = warmstart.batch_scene([1, 2], workload=warmstart.CANTILEVER)
    assert len(sc.bodies) == 2 and sc.substeps == 1 and sc.iterations == 30
    assert sc.bodies[0].tets.shape == (450, 4) and sc.bodies[0].ext_acc is not None
    sc = warmstart.batch_scene([7], workload=warmstart.BEAM98K)
    b = sc.bodies[0]
    assert b.tets.shape == (98304, 4) and b.model == scenes.MODEL_SNH
    assert sc.substeps == 4 and sc.iterations == 30
    assert len(b.pinned) in (17 * 17, 65 * 17)          # one face of the 64x16x16 grid
    # the box batch: one whole scene per seed
    with pytest.raises(ValueError):
        warmstart.batch_scene([1, 2], workload=warmstart.BOXES512)
    # seeds differ in force field and pinned face, deterministically
    a1 = warmstart.beam_trajectory_body(5)
    a2 = warmstart.beam_trajectory_body(5)
    a3 = warmstart.beam_trajectory_body(6)
    assert np.array_equal(a1.ext_acc, a2.ext_acc) and not np.array_equal(a1.ext_acc, a3.ext_acc)
