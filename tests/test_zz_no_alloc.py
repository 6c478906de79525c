"""sbs_gpu_plane_contacts_noalloc: the plane-contact detection for callers
that cannot allocate device memory (their own allocator or budget, stream
capture, real-time loops).  Called twice in a row through the C ABI on
device buffers the test owns, it must give the same contacts as the solver's
own detection (sbs_gpu_detect_contacts + sbs_gpu_get_contacts) on the same
positions: the same vertex set, contact points within 1e-6 m.

Collected last on purpose (file name), so a failure here never hides the
other tests; it runs the same alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from sbs_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_noalloc_plane_contacts_match_solver(capi_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = capi_mod.load()
    L.sbs_gpu_plane_contacts_noalloc.restype = C.c_int
    L.sbs_gpu_plane_contacts_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                                 np.ctypeslib.ndpointer(np.float64, flags="C"),
                                                 C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    sc = scenes.beam_c1()
    sc.ground = ((0.0, 1.0, 0.0), -0.15)          # plane y = 0.15 cuts the beam
    g = capi_mod.Solver(sc)
    g.step(2)                                     # a deformed state
    g.detect_contacts()
    v_ref, qn_ref = g.contacts()
    assert len(v_ref) > 0
    x = g.positions().astype(np.float32)           # global vertex order
    surf = g.surface()
    dev = torch.device("cuda", 0)
    d_x = torch.from_numpy(np.ascontiguousarray(x).ravel()).to(dev)
    d_s = torch.from_numpy(surf.astype(np.int32)).to(dev)
    n = np.asarray(sc.ground[0], np.float64)
    for call in range(2):
        d_v = torch.full((len(surf),), -1, dtype=torch.int32, device=dev)
        d_q = torch.zeros(3 * len(surf), dtype=torch.float32, device=dev)
        d_c = torch.zeros(1, dtype=torch.int32, device=dev)
        st = L.sbs_gpu_plane_contacts_noalloc(d_x.data_ptr(), len(x), d_s.data_ptr(), len(surf), n,
                                              sc.ground[1], d_v.data_ptr(), d_q.data_ptr(),
                                              d_c.data_ptr(), None)
        assert st == capi_mod.SBS_OK
        torch.cuda.synchronize()
        cnt = int(d_c.item())
        verts = d_v.cpu().numpy()[:cnt].astype(np.uint32)
        q = d_q.cpu().numpy()[:3 * cnt].reshape(-1, 3)
        order = np.argsort(verts)
        assert np.array_equal(verts[order], v_ref)
        assert np.abs(q[order] - qn_ref[:, :3]).max() < 1e-6
        # contacts come out in the order of the surface list
        pos = np.searchsorted(surf, verts)
        assert np.all(np.diff(pos) > 0)


def _bind(capi_mod):
    L = capi_mod.load()
    L.sbs_gpu_plane_contacts_noalloc.restype = C.c_int
    L.sbs_gpu_plane_contacts_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                                 np.ctypeslib.ndpointer(np.float64, flags="C"),
                                                 C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    return L


def _call(L, capi_mod, torch, d_x, n_verts, d_s, n_surf, normal, d):
    dev = d_x.device
    d_v = torch.full((max(1, n_surf),), -1, dtype=torch.int32, device=dev)
    d_q = torch.zeros(3 * max(1, n_surf), dtype=torch.float32, device=dev)
    d_c = torch.zeros(1, dtype=torch.int32, device=dev)
    st = L.sbs_gpu_plane_contacts_noalloc(d_x.data_ptr(), n_verts, d_s.data_ptr(), n_surf,
                                          np.asarray(normal, np.float64), d, d_v.data_ptr(), d_q.data_ptr(),
                                          d_c.data_ptr(), None)
    assert st == capi_mod.SBS_OK
    torch.cuda.synchronize()
    cnt = int(d_c.item())
    return d_v.cpu().numpy()[:cnt].astype(np.uint32), d_q.cpu().numpy()[:3 * cnt].reshape(-1, 3)


def test_noalloc_many_blocks_match_solver(capi_mod):
    """The 98k-tet beam's surface (about 5,000 vertices, 20 blocks of 256):
    the scan carries counts between its threads and the write adds each
    block's offset.  Same contacts as the solver's own detection."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = _bind(capi_mod)
    sc = scenes.beam_twist()
    sc.ground = ((0.0, 1.0, 0.0), -0.3)           # plane y = 0.3 cuts the beam's 0.8 m height
    g = capi_mod.Solver(sc)
    g.detect_contacts()                           # at the initial state, before any frame lifts the beam
    v_ref, qn_ref = g.contacts()
    surf = g.surface()
    assert len(surf) > 4 * 256 and len(v_ref) > 1000
    x = g.positions().astype(np.float32)
    g.close()
    dev = torch.device("cuda", 0)
    d_x = torch.from_numpy(np.ascontiguousarray(x).ravel()).to(dev)
    d_s = torch.from_numpy(surf.astype(np.int32)).to(dev)
    for _ in range(2):
        verts, q = _call(L, capi_mod, torch, d_x, len(x), d_s, len(surf), sc.ground[0], sc.ground[1])
        order = np.argsort(verts)
        assert np.array_equal(verts[order], v_ref)
        assert np.abs(q[order] - qn_ref[:, :3]).max() < 1e-6
        assert np.all(np.diff(np.searchsorted(surf, verts)) > 0)


@pytest.mark.parametrize("n_surf", [600_001, 1_048_576])
def test_noalloc_synthetic_surface_near_cap(capi_mod, n_surf):
    """A synthetic surface list of 2,344 and 4,096 blocks (every scan
    thread's group of four counts is used at the cap), with repeated ids and
    ids past the position buffer, against a host compaction in list order."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = _bind(capi_mod)
    rng = np.random.default_rng(n_surf)
    n_verts = 700_000
    x = rng.uniform(-1.0, 1.0, (n_verts, 3)).astype(np.float32)
    surf = rng.integers(0, n_verts + 5_000, n_surf).astype(np.uint32)   # some ids >= n_verts
    normal = np.array([0.3, 1.0, -0.2])
    dplane = 0.1
    nl = np.linalg.norm(normal)
    pf = (normal / nl).astype(np.float32)
    df = np.float32(dplane / nl)
    valid = surf < n_verts
    xs = x[np.where(valid, surf, 0)]
    sd = (pf[0] * xs[:, 0] + pf[1] * xs[:, 1]) + pf[2] * xs[:, 2] + df   # float32 like the kernel (up to FMA)
    hit = valid & (sd < 0)
    near = np.abs(sd) < 1e-6                                             # rounding may decide these
    dev = torch.device("cuda", 0)
    d_x = torch.from_numpy(x.ravel().copy()).to(dev)
    d_s = torch.from_numpy(surf.astype(np.int32)).to(dev)
    for _ in range(2):
        verts, q = _call(L, capi_mod, torch, d_x, n_verts, d_s, n_surf, normal, dplane)
        exp = surf[hit & ~near]
        got_mask = np.isin(verts, surf[near & valid], invert=True)
        assert np.array_equal(verts[got_mask], exp)
        assert len(verts) >= len(exp)
        assert np.all(verts < n_verts)
        xv = x[verts]
        ad = np.abs((xv * pf).sum(1) + df)
        assert np.abs(q - (xv + pf[None, :] * ad[:, None])).max() < 1e-5


def test_noalloc_rejects_oversize_and_null(capi_mod):
    L = capi_mod.load()
    L.sbs_gpu_plane_contacts_noalloc.restype = C.c_int
    n = np.array([0.0, 1.0, 0.0])
    buf = (C.c_uint8 * 64)()
    p = C.cast(buf, C.c_void_p)
    L.sbs_gpu_plane_contacts_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                                 np.ctypeslib.ndpointer(np.float64, flags="C"),
                                                 C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    too_many = 1_048_577
    assert L.sbs_gpu_plane_contacts_noalloc(p, 4, p, too_many, n, 0.0, p, p, p, None) == capi_mod.SBS_EINVAL
    assert L.sbs_gpu_plane_contacts_noalloc(None, 4, p, 1, n, 0.0, p, p, p, None) == capi_mod.SBS_EINVAL
