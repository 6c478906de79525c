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
