"""The FP64 CPU oracle: pinned against an independent numpy restatement and
analytic known answers of the reference's formulas (CPU only)."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from sbs_gb300 import scenes
from oracle import numpy_oracle


def rand_F(rng, kind):
    A = rng.normal(size=(3, 3))
    if kind == "neg":
        A[:, 0] *= -1 if np.linalg.det(A) > 0 else 1
    elif kind == "rank2":
        A[:, 2] = A[:, 0] * 0.3 - A[:, 1] * 1.7
    elif kind == "near_id":
        A = np.eye(3) + 1e-4 * A
    elif kind == "repeated":
        Q, _ = np.linalg.qr(A)
        A = Q @ np.diag([2.0, 2.0, 0.5]) @ np.linalg.qr(rng.normal(size=(3, 3)))[0]
    return A


@pytest.mark.parametrize("kind", ["gen", "neg", "rank2", "near_id", "repeated"])
def test_svd3_convention_and_reconstruction(oracle_mod, kind):
    rng = np.random.default_rng(11)
    for _ in range(50):
        F = rand_F(rng, kind)
        U, s, V = oracle_mod.svd3(F)
        assert np.all(s >= 0) and s[0] >= s[1] >= s[2]
        assert np.allclose(U @ np.diag(s) @ V.T, F, atol=1e-12)
        assert np.allclose(U.T @ U, np.eye(3), atol=1e-12)
        assert np.allclose(V.T @ V, np.eye(3), atol=1e-12)
        assert np.allclose(s, np.linalg.svd(F, compute_uv=False), atol=1e-12)


def _one_tet_sim(oracle_mod, xrest, x, E=1e5, nu=0.3, model=scenes.MODEL_STVK):
    b = scenes.Body(x0=xrest, tets=np.array([[0, 1, 2, 3]], np.uint32), model=model, young=E,
                    poisson=nu, density=1000.0, x_init=x)
    sc = scenes.Scene("one", [b], 1 / 60, 1, 1, 1, gravity=(0.0, 0.0, 0.0), ground=None)
    o = oracle_mod.Oracle(sc)
    o.set(oracle_mod.FIELD_XI, x)
    return o


def _psi(oracle_mod, o):
    psi = C.c_double()
    f = np.zeros(12)
    o.L.orc_tet_eval(o.h, 0, C.byref(psi), f)
    return psi.value, f.reshape(4, 3)


REST = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]) * 0.1


def test_stvk_rest_state_is_free(oracle_mod):
    o = _one_tet_sim(oracle_mod, REST, REST)
    psi, f = _psi(oracle_mod, o)
    assert abs(psi) < 1e-20 and np.abs(f).max() < 1e-12


@pytest.mark.parametrize("s", [1.1, 0.9, 0.6])
def test_stvk_uniform_stretch_known_answer(oracle_mod, s):
    # F = s I: Ehat = (s^2-1)/2 I, E = U Ehat V^T = Ehat (U = V),
    # psi = mu*3e^2 + lam/2*(3e)^2 (green_constraint.cpp:104-110)
    E, nu = 1e5, 0.3
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    o = _one_tet_sim(oracle_mod, REST, REST * s, E, nu)
    psi, f = _psi(oracle_mod, o)
    e = 0.5 * (max(s, 0.577) ** 2 - 1)
    assert psi == pytest.approx(mu * 3 * e * e + 0.5 * lam * 9 * e * e, rel=1e-12)
    assert np.allclose(f.sum(0), 0, atol=1e-12)


def test_stvk_inverted_clamps_third_singular_value(oracle_mod):
    # reflect through z: F = diag(1,1,-1), inverted -> sigma3 = -1 -> clamped to
    # 0.577 (green_constraint.cpp:92-102); U col 2 flipped so E = diag(0,0,e3)
    E, nu = 1e5, 0.3
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    x = REST.copy()
    x[:, 2] *= -1
    o = _one_tet_sim(oracle_mod, REST, x, E, nu)
    psi, _ = _psi(oracle_mod, o)
    e3 = 0.5 * (0.577 ** 2 - 1)
    # E = U Ehat V^T with the flipped u3: tr(E) = e3 (u3.v3) = e3 * 1 after the flip
    assert psi == pytest.approx(mu * e3 * e3 + 0.5 * lam * e3 * e3, rel=1e-10)


def test_snh_single_tet_stays_at_rest(oracle_mod):
    o = _one_tet_sim(oracle_mod, REST, REST, 1e6, 0.3, scenes.MODEL_SNH)
    sc = o.scene
    sc.iterations = 30
    o.step(1)
    assert np.abs(o.get() - REST).max() < 1e-15


def snh_closed_form_forces(xrest, x, E, nu):
    """Nodal elastic forces of one tet under the stable Neo-Hookean energy of
    Macklin & Mueller 2021, psi = mu/2 (tr(F^T F) - 3) + lam/2 (det F - a)^2
    with a = 1 + mu/lam, from its closed-form first Piola stress
    P = mu F + lam (det F - a) cof(F):  f_i = -|V0| (P Dm^-T) e_i for the
    first three vertices, f_4 = -(f_1 + f_2 + f_3).  Nothing here uses the
    solver's constraint split (C_D = |F|, C_H = det F - a) or its 2x2 solve."""
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    Dm = np.stack([xrest[i] - xrest[3] for i in range(3)], axis=1)
    Ds = np.stack([x[i] - x[3] for i in range(3)], axis=1)
    F = Ds @ np.linalg.inv(Dm)
    cof = np.stack([np.cross(F[:, 1], F[:, 2]), np.cross(F[:, 2], F[:, 0]), np.cross(F[:, 0], F[:, 1])], axis=1)
    P = mu * F + lam * (np.linalg.det(F) - (1 + mu / lam)) * cof
    H = -abs(np.linalg.det(Dm) / 6) * P @ np.linalg.inv(Dm).T
    return np.vstack([H.T, -H.sum(axis=1)])


SNH_KAT_F = {
    "uniaxial": np.diag([1.2, 0.95, 0.95]),
    "compressed": np.diag([0.85, 1.03, 1.04]),
    "shear": np.array([[1.0, 0.25, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]),
    "general": np.array([[1.1, 0.1, -0.05], [0.03, 0.92, 0.12], [-0.08, 0.02, 1.05]]),
}


@pytest.mark.parametrize("kind", list(SNH_KAT_F))
def test_snh_projection_against_closed_form_stress(oracle_mod, kind):
    """Known answer for the stable Neo-Hookean constraint pair: with heavy
    vertices (w -> 0) one projection from zero multipliers moves vertex i by
    w dt^2 f_i, f_i the elastic force of the closed-form Neo-Hookean stress
    (XPBD: dlambda_j -> -C_j / alpha~_j, dx_i = w sum_j grad_i C_j dlambda_j
    = -w dt^2 grad_i U).  This pins the constraint formulation (shared by the
    oracle and the GPU kernels) to the published energy."""
    E, nu = 1e5, 0.3
    xrest = REST + np.array([0.3, -0.2, 0.1])
    x = (xrest - xrest[3]) @ SNH_KAT_F[kind].T + xrest[3]
    m = 1e7                                    # w = 1e-7: the O(w) correction is ~1e-7 relative
    b = scenes.Body(x0=xrest, tets=np.array([[0, 1, 2, 3]], np.uint32), model=scenes.MODEL_SNH, young=E,
                    poisson=nu, density=1000.0, x_init=x, mass=np.full(4, m))
    dt = 1 / 60
    sc = scenes.Scene("one", [b], dt, 1, 1, 1, gravity=(0.0, 0.0, 0.0), ground=None)
    o = oracle_mod.Oracle(sc)
    o.set(oracle_mod.FIELD_XI, x)
    o.L.orc_solve(o.h, dt, 1)
    dx = o.get(oracle_mod.FIELD_XI) - x
    f = snh_closed_form_forces(xrest, x, E, nu)
    assert np.abs(f).max() > 1.0
    assert np.abs(dx * m / dt ** 2 - f).max() < 1e-6 * np.abs(f).max()


def test_oracle_matches_numpy_restatement_first_frame(oracle_mod):
    sc = scenes.beam_c1(frames=1)
    o = oracle_mod.Oracle(sc)
    n = numpy_oracle.NumpyXPBD(sc)
    assert np.allclose(o.masses(), np.where(n.m > 0, n.m, 0.0), atol=1e-14)
    assert np.array_equal(o.surface(), np.array(n.surface, np.uint32))
    o.step(1)
    n.step()
    assert np.abs(o.get() - n.x).max() < 1e-9


def test_oracle_matches_numpy_with_contacts_and_force_gravity(oracle_mod):
    sc = scenes.beam_c1(frames=1)
    sc.ground = ((0.0, 1.0, 0.0), -0.12)   # plane y = 0.12 cuts the beam
    sc.gravity_mode = 1
    o = oracle_mod.Oracle(sc)
    n = numpy_oracle.NumpyXPBD(sc)
    v, qn = o.detect_contacts()
    assert len(v) > 0
    x0 = sc.bodies[0].x_init
    expect = [i for i in n.surface if x0[i, 1] - 0.12 < 0]
    assert sorted(v.tolist()) == expect
    assert np.allclose(qn[:, 1], 0.12) and np.allclose(qn[:, 4], 1.0)
    # one Gauss-Seidel sweep (contacts first, then tets) from the same state:
    # the stiff contacts (alpha 1e-8) make whole frames diverge at rounding
    # level, one sweep stays comparable
    n.s = dataclasses.replace(sc, iterations=1)
    o.scene = n.s
    o.step(1)
    n.step()
    assert np.abs(o.get() - n.x).max() < 1e-9


def test_gravity_modes(oracle_mod):
    # one free-falling tet, no elastic response at rest: after one substep
    # v = g dt (acceleration mode) or g w dt (force mode, timestep.cpp:39-40)
    for mode in (0, 1):
        b = scenes.Body(x0=REST, tets=np.array([[0, 1, 2, 3]], np.uint32), young=1e5,
                        poisson=0.3, density=1000.0)
        sc = scenes.Scene("fall", [b], 0.01, 1, 5, 1, ground=None, gravity_mode=mode)
        o = oracle_mod.Oracle(sc)
        o.step(1)
        v = o.get(oracle_mod.FIELD_V)
        w = 1.0 / o.masses()
        want = -9.81 * 0.01 * (w if mode == 1 else np.ones(4))
        assert np.allclose(v[:, 1], want, rtol=1e-12)


def test_pinned_and_kinematic_vertices(oracle_mod):
    sc = scenes.beam_twist(8, 2, 2, 0.1, frames=3, substeps=2, iterations=5)
    o = oracle_mod.Oracle(sc)
    o.step(3)
    b = sc.bodies[0]
    x = o.get()
    assert np.array_equal(x[b.pinned], b.x0[b.pinned])
    t = 3 * sc.frame_dt
    c = np.array(b.kin_center)
    ang = b.kin_omega * t
    R = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
    want = (b.x0[b.kin_verts] - c) @ R.T + c
    assert np.abs(x[b.kin_verts] - want).max() < 1e-12


def greedy_colour_order(tets, n_verts):
    used = [set() for _ in range(n_verts)]
    col = []
    for t in tets:
        c = 0
        forb = set().union(*(used[v] for v in t))
        while c in forb:
            c += 1
        col.append(c)
        for v in t:
            used[v].add(c)
    col = np.array(col)
    order = np.argsort(col, kind="stable").astype(np.uint32)
    offsets = np.searchsorted(col[order], np.arange(col.max() + 2)).astype(np.uint32)
    return order, offsets


def test_colour_parallel_oracle_is_bit_identical(oracle_mod):
    sc = scenes.beam_twist(12, 3, 3, 0.05, frames=2, substeps=2, iterations=8)
    order, off = greedy_colour_order(sc.bodies[0].tets, sc.n_verts)
    a = oracle_mod.Oracle(sc)
    b = oracle_mod.Oracle(sc, threads=4)
    a.set_order(order, off)
    b.set_order(order, off)
    a.step(2)
    b.step(2)
    assert np.array_equal(a.get(), b.get())


def test_sweep_order_changes_result_but_not_physics(oracle_mod):
    # Gauss-Seidel depends on order: a permuted sweep gives a (slightly)
    # different iterate, which is why the oracle replays the GPU's order.
    sc = scenes.beam_c1(frames=1)
    a = oracle_mod.Oracle(sc)
    b = oracle_mod.Oracle(sc)
    order, off = greedy_colour_order(sc.bodies[0].tets, sc.n_verts)
    b.set_order(order, off)
    a.step(1)
    b.step(1)
    d = np.abs(a.get() - b.get()).max()
    assert 0 < d < 1e-3


def test_predictability_horizon_of_the_reference_loop(oracle_mod):
    """A 1e-12 m perturbation of one vertex grows to >= 1e-6 m within a few
    frames of the 450-tet beam: the sequential loop itself is sensitive to
    rounding, so FP32 and FP64 (or two FP64 codes with different rounding)
    cannot agree to 1e-4 of the diagonal over a long run.  Parity is therefore
    checked within this horizon plus on size-independent properties."""
    sc = scenes.beam_c1(frames=8)
    a = oracle_mod.Oracle(sc)
    b = oracle_mod.Oracle(sc)
    a.step(1)
    b.step(1)
    x = b.get()
    x[100] += 1e-12
    v = b.get(oracle_mod.FIELD_V)
    b.set(oracle_mod.FIELD_X, x)
    b.set(oracle_mod.FIELD_V, v)
    growth = []
    for _ in range(4):
        a.step(1)
        b.step(1)
        growth.append(np.abs(a.get() - b.get()).max())
    assert max(growth) > 1e-6
