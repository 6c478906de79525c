"""The benchmark configurations for their whole configured runs, checked by
properties that do not depend on the trajectory's chaotic detail (the FP64
oracle cannot follow these sizes for hundreds of frames; frame-by-frame
parity is in test_config_parity.py and test_multiframe_parity.py).

- 98,304-tet SNH twisting beam, 300 frames: finite state, no inverted tet,
  the pinned face at rest, the driven face on the analytic rotation.
- 2.6M-tet SNH block, 200 frames (dropped 0.5 m): finite, the block's volume
  within 1% of rest (nu = 0.48), at rest on the ground at the end (centroid
  at half its height, penetration below 5 cm), inverted tets only where it
  touches the ground (< 0.05%).
- 512 StVK boxes, 600 frames: finite state.  (The loop is unstable at these
  settings: small stiff boxes invert and are flung out of the arena; the FP64
  oracle shows the same jitter on a 16-box version.)
"""
import numpy as np
import pytest

from sbs_gb300 import scenes

pytestmark = pytest.mark.gpu


def signed_volumes(x, tets):
    t = tets.astype(np.int64)
    d = np.stack([x[t[:, 0]] - x[t[:, 3]], x[t[:, 1]] - x[t[:, 3]], x[t[:, 2]] - x[t[:, 3]]], axis=2)
    return np.linalg.det(d) / 6.0


def test_beam98k_300_frames(capi_mod):
    sc = scenes.beam_twist()
    b = sc.bodies[0]
    g = capi_mod.Solver(sc)
    V0 = signed_volumes(b.x0, b.tets)
    done = 0
    for f in (75, 150, 300):
        g.step(f - done)
        done = f
        x = g.positions().astype(np.float64)
        assert np.isfinite(x).all()
        V = signed_volumes(x, b.tets)
        assert np.all((V > 0) == (V0 > 0))
    assert np.abs(x[b.pinned] - b.x0[b.pinned]).max() < 1e-6
    ang = b.kin_omega * 300 * sc.frame_dt
    R = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
    c = np.array(b.kin_center)
    want = (b.x0[b.kin_verts] - c) @ R.T + c
    assert np.abs(x[b.kin_verts] - want).max() < 1e-5
    g.close()


def test_block2m_200_frames(capi_mod):
    sc = scenes.big_block()
    b = sc.bodies[0]
    g = capi_mod.Solver(sc)
    V0 = signed_volumes(b.x0, b.tets)
    height = b.x0[:, 1].max() - b.x0[:, 1].min()
    done = 0
    for f in (50, 100, 200):
        g.step(f - done)
        done = f
        x = g.positions().astype(np.float64)
        assert np.isfinite(x).all()
        V = signed_volumes(x, b.tets)
        assert abs(V.sum() / V0.sum() - 1.0) < 1e-2
        assert np.count_nonzero((V > 0) != (V0 > 0)) < 5e-4 * len(V0)
    assert x[:, 1].min() > -0.05
    assert abs(x[:, 1].mean() - 0.5 * height) < 0.05 * height
    g.close()


def test_boxes512_600_frames(capi_mod):
    sc = scenes.box_drop()
    g = capi_mod.Solver(sc)
    for _ in range(4):
        g.step(150)
        x, v = g.get_state(-1)
        assert np.isfinite(x).all() and np.isfinite(v).all()
    g.close()
