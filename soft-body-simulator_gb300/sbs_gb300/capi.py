"""ctypes binding of libsbs_gpu.so (declarations: include/sbs_gpu.h).

Raises ``SbsError`` on any non-OK status.  There is no CPU fallback: if the
library or a GPU is missing, loading or creating a solver fails loudly.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

from . import build as _build

SBS_OK, SBS_EINVAL, SBS_ECUDA, SBS_ETIMEOUT, SBS_ENAN, SBS_ESTATE, SBS_ENOMEM, SBS_ECOLOUR = range(8)
EXEC_AUTO, EXEC_GRAPH, EXEC_PERSISTENT, EXEC_CLUSTER, EXEC_WAVEFRONT = 0, 1, 2, 3, 4
GRAVITY_ACCELERATION, GRAVITY_FORCE = 0, 1

HEADER = _build.INCLUDE / "sbs_gpu.h"


class SbsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"sbs status {status}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("compliance", C.c_double), ("damping", C.c_double),
                ("collision_compliance", C.c_double), ("gravity", C.c_double * 3),
                ("gravity_mode", C.c_int32), ("device", C.c_int32), ("exec_mode", C.c_int32),
                ("block_size", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("tail_threshold", C.c_int32), ("body_contacts", C.c_int32),
                ("hash_cell", C.c_float), ("candidate_capacity", C.c_uint32),
                ("check_finite", C.c_int32), ("stage_records", C.c_int32), ("wait_limit_us", C.c_int32),
                ("colour_size_cap", C.c_int32)]


class WarmStats(C.Structure):
    _fields_ = [("warm_substeps", C.c_uint64), ("calibration_substeps", C.c_uint64), ("sweeps", C.c_uint64),
                ("fallbacks", C.c_uint64), ("capped", C.c_uint64), ("mean_residual_ratio", C.c_double),
                ("max_residual_ratio", C.c_double), ("last_target", C.c_double), ("last_residual", C.c_double)]


class Material(C.Structure):
    _fields_ = [("model", C.c_int32), ("young", C.c_double), ("poisson", C.c_double),
                ("density", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("projections", C.c_uint64),
                ("n_vertices", C.c_uint32), ("n_tets", C.c_uint32), ("n_colours", C.c_uint32),
                ("n_tail_colours", C.c_uint32), ("n_contacts", C.c_uint32),
                ("n_body_contacts", C.c_uint32), ("body_contact_overflow", C.c_uint32),
                ("exec_mode", C.c_int32), ("grid_ctas", C.c_int32), ("block_size", C.c_int32),
                ("residual", C.c_double), ("energy", C.c_double), ("last_frame_ms", C.c_double),
                ("kernel_launches", C.c_uint64), ("cluster_phase_max_tets", C.c_uint32)]


_lib = None


def declared_symbols() -> list[str]:
    """Function names declared in include/sbs_gpu.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(sbs_gpu_[a-z_0-9]+)\s*\(", text)))


def load(build: bool = True):
    """Loads (building first if stale) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    L = C.CDLL(str(path))
    P = C.c_void_p
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C")
    f64 = np.ctypeslib.ndpointer(np.float64, flags="C")
    u32 = np.ctypeslib.ndpointer(np.uint32, flags="C")
    sig = {
        "sbs_gpu_params_default": [C.POINTER(Params)],
        "sbs_gpu_create": [C.POINTER(Params), C.POINTER(P)],
        "sbs_gpu_add_body": [P, f64, C.c_void_p, C.c_uint32, u32, C.c_uint32, C.POINTER(Material),
                             C.c_void_p, C.POINTER(C.c_int32)],
        "sbs_gpu_pin_vertices": [P, C.c_int32, u32, C.c_uint32],
        "sbs_gpu_add_kinematic_rotation": [P, C.c_int32, u32, C.c_uint32, f64, f64, C.c_double],
        "sbs_gpu_set_external_acceleration": [P, C.c_int32, f32],
        "sbs_gpu_add_ground_plane": [P, f64, C.c_double],
        "sbs_gpu_finalize": [P],
        "sbs_gpu_step": [P, C.c_double, C.c_uint32, C.c_uint32],
        "sbs_gpu_step_timed": [P, C.c_double, C.c_uint32, C.c_uint32],
        "sbs_gpu_withhold_barrier_arrival": [P],
        "sbs_gpu_solve": [P, C.c_double, C.c_uint32],
        "sbs_gpu_predict": [P, C.c_double],
        "sbs_gpu_update_velocities": [P, C.c_double],
        "sbs_gpu_detect_contacts": [P],
        "sbs_gpu_residual": [P, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)],
        "sbs_gpu_set_state": [P, C.c_int32, C.c_void_p, C.c_void_p],
        "sbs_gpu_get_state": [P, C.c_int32, C.c_void_p, C.c_void_p],
        "sbs_gpu_get_predicted": [P, C.c_int32, f32],
        "sbs_gpu_set_predicted": [P, C.c_int32, f32],
        "sbs_gpu_get_tet_order": [P, C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_get_lambdas": [P, f32],
        "sbs_gpu_get_contacts": [P, C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_get_masses": [P, f32],
        "sbs_gpu_get_surface": [P, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_set_body_velocity": [P, C.c_int32, f64],
        "sbs_io_read_ply": [C.c_char_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_void_p, C.c_uint32,
                            C.POINTER(C.c_uint32), C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_load_scene": [P, C.c_char_p, C.POINTER(Material), u32, C.c_double, C.POINTER(C.c_int32),
                               C.POINTER(C.c_int32)],
        "sbs_gpu_add_sdf_grid": [P, C.c_void_p, u32, f64, f64],
        "sbs_gpu_add_sdf_grid_cubic": [P, C.c_void_p, u32, f64, f64],
        "sbs_gpu_sdf_cubic_from_mesh": [f64, C.c_uint32, u32, C.c_uint32, f64, f64, u32, C.c_void_p],
        "sbs_gpu_add_environment_mesh": [P, f64, C.c_uint32, u32, C.c_uint32, f64, f64, u32],
        "sbs_gpu_sdf_from_mesh": [f64, C.c_uint32, u32, C.c_uint32, f64, f64, u32, C.c_void_p],
        "sbs_gpu_add_distance_constraints": [P, C.c_void_p, C.c_uint32, C.c_double, C.c_double],
        "sbs_gpu_get_distance_order": [P, C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_get_distance_lambdas": [P, C.c_void_p],
        "sbs_gpu_get_surface_mesh": [P, C.c_int32, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_void_p,
                                     C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_update_surface": [P, C.c_int32, C.c_int32, C.c_void_p, C.c_uint32],
        "sbs_gpu_get_stats": [P, C.POINTER(Stats)],
        "sbs_gpu_destroy": [P],
        "sbs_gpu_plan_sweep": [f64, C.c_uint32, u32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)],
        "sbs_gpu_set_tet_colours": [P, C.c_int32, u32],
        "sbs_gpu_get_candidates": [P, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)],
        "sbs_gpu_set_warm_start": [P, C.c_void_p, C.c_uint32],
        "sbs_gpu_set_warm_judge": [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double],
        "sbs_gpu_get_warm_stats": [P, C.POINTER(WarmStats)],
        "sbs_gpu_warm_start_init": [P, C.c_double],
        "sbs_gpu_solve_ex": [P, C.c_double, C.c_uint32, C.c_int32],
        "sbs_gpu_get_features": [P, f32],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
    msig = {
        "sbs_mlp_create": [C.c_int32, C.c_uint64, C.POINTER(P)],
        "sbs_mlp_destroy": [P],
        "sbs_mlp_get_params": [P, f32p],
        "sbs_mlp_set_params": [P, f32p],
        "sbs_mlp_set_normalization": [P, f32p, f32p, f32p],
        "sbs_mlp_forward": [P, f32p, C.c_uint32, f32p],
        "sbs_mlp_forward_path": [P, f32p, C.c_uint32, f32p, C.c_int32],
        "sbs_mlp_forward_device": [P, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32, C.POINTER(C.c_float)],
        "sbs_mlp_loss_grad": [P, f32p, f32p, C.c_uint32, C.POINTER(C.c_float), C.c_void_p],
        "sbs_mlp_set_dataset": [P, f32p, f32p, C.c_uint32],
        "sbs_mlp_train": [P, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64, C.POINTER(C.c_float)],
        "sbs_mlp_set_gemm": [P, C.c_int32],
    }
    for name, args in msig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.sbs_mlp_param_count.restype = C.c_uint32
    L.sbs_mlp_last_error.argtypes = [P]
    L.sbs_mlp_last_error.restype = C.c_char_p
    L.sbs_gpu_status_string.argtypes = [C.c_int]
    L.sbs_gpu_status_string.restype = C.c_char_p
    L.sbs_gpu_last_error.argtypes = [P]
    L.sbs_gpu_last_error.restype = C.c_char_p
    _lib = L
    return L


def default_params(**kw) -> Params:
    L = load()
    p = Params()
    L.sbs_gpu_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "gravity":
            p.gravity = (C.c_double * 3)(*v)
        else:
            setattr(p, k, v)
    return p


def _ptr(a):
    return None if a is None else a.ctypes.data


def read_ply(path):
    """(positions float32 [V,3], triangles [F,3], tets [T,4]) of a PLY file."""
    L = load()
    nv, nf, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
    st = L.sbs_io_read_ply(str(path).encode(), None, 0, C.byref(nv), None, 0, C.byref(nf), None, 0, C.byref(nt))
    if st != SBS_OK:
        raise SbsError(st, f"cannot read {path}")
    x = np.zeros((nv.value, 3), np.float32)
    f = np.zeros((nf.value, 3), np.uint32)
    t = np.zeros((nt.value, 4), np.uint32)
    st = L.sbs_io_read_ply(str(path).encode(), x.ctypes.data, nv.value, C.byref(nv), f.ctypes.data, nf.value,
                           C.byref(nf), t.ctypes.data, nt.value, C.byref(nt))
    if st != SBS_OK:
        raise SbsError(st, f"cannot read {path}")
    return x, f, t


def sdf_from_mesh(verts, tris, lo, hi, cells) -> np.ndarray:
    """Host-only signed distance of a triangle mesh at the (cells+1) nodes per
    axis of the box [lo, hi]; returns float32 [nz, ny, nx]."""
    L = load()
    v = np.ascontiguousarray(verts, np.float64).ravel()
    t = np.ascontiguousarray(tris, np.uint32).ravel()
    c = np.ascontiguousarray(cells, np.uint32)
    out = np.zeros((int(c[2]) + 1) * (int(c[1]) + 1) * (int(c[0]) + 1), np.float32)
    st = L.sbs_gpu_sdf_from_mesh(v, len(v) // 3, t, len(t) // 3, np.asarray(lo, np.float64),
                                 np.asarray(hi, np.float64), c, out.ctypes.data)
    if st != SBS_OK:
        raise SbsError(st, "sbs_gpu_sdf_from_mesh failed")
    return out.reshape(int(c[2]) + 1, int(c[1]) + 1, int(c[0]) + 1)


def sdf_cubic_from_mesh(verts, tris, lo, hi, cells) -> np.ndarray:
    """Host-only values of the cubic Lagrange grid (layout of
    sbs_gpu_add_sdf_grid_cubic) of a triangle mesh over the box [lo, hi]."""
    L = load()
    v = np.ascontiguousarray(verts, np.float64).ravel()
    t = np.ascontiguousarray(tris, np.uint32).ravel()
    c = np.ascontiguousarray(cells, np.uint32)
    nx, ny, nz = (int(k) + 1 for k in c)
    n = nx * ny * nz + 2 * ((nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1))
    out = np.zeros(n, np.float32)
    st = L.sbs_gpu_sdf_cubic_from_mesh(v, len(v) // 3, t, len(t) // 3, np.asarray(lo, np.float64),
                                       np.asarray(hi, np.float64), c, out.ctypes.data)
    if st != SBS_OK:
        raise SbsError(st, "sbs_gpu_sdf_cubic_from_mesh failed")
    return out


def plan_sweep(scene):
    """Sweep order of a scene computed by the library's host code (no GPU):
    (order, offsets) with bodies concatenated in add order; the bodies'
    colourings (Body.colours) are used as sbs_gpu_finalize uses them."""
    L = load()
    x0 = np.ascontiguousarray(np.concatenate([b.x0 for b in scene.bodies]), np.float64).ravel()
    tets, models, hints, off = [], [], [], 0
    for b in scene.bodies:
        tets.append(b.tets.astype(np.uint32) + off)
        models.append(np.full(len(b.tets), b.model, np.int32))
        hints.append(np.full(len(b.tets), -1, np.int32) if getattr(b, "colours", None) is None
                     else np.asarray(b.colours, np.int32))
        off += len(b.x0)
    tets = np.ascontiguousarray(np.concatenate(tets), np.uint32).ravel()
    models = np.ascontiguousarray(np.concatenate(models), np.int32)
    hints = np.ascontiguousarray(np.concatenate(hints), np.int32)
    n = C.c_uint32()
    T = len(models)
    order = np.zeros(T, np.uint32)
    offsets = np.zeros(129, np.uint32)
    st = L.sbs_gpu_plan_sweep(x0, len(x0) // 3, tets, T, models.ctypes.data, hints.ctypes.data, order.ctypes.data,
                              offsets.ctypes.data, len(offsets), C.byref(n))
    if st != SBS_OK:
        raise SbsError(st, L.sbs_gpu_last_error(None).decode())
    return order, offsets[: n.value + 1].copy()


class Solver:
    """One GPU scene (an ``sbs_gpu`` handle) built from a scenes.Scene."""

    def __init__(self, scene, **param_overrides):
        L = load()
        self.L = L
        self.scene = scene
        kw = dict(compliance=scene.compliance, damping=scene.damping,
                  collision_compliance=scene.collision_compliance, gravity=scene.gravity,
                  gravity_mode=scene.gravity_mode, body_contacts=int(scene.body_contacts),
                  hash_cell=float(scene.hash_cell))
        kw.update(param_overrides)
        prm = default_params(**kw)
        h = C.c_void_p()
        self._check(L.sbs_gpu_create(C.byref(prm), C.byref(h)), None)
        self.h = h
        self.body_sizes = []
        for b in scene.bodies:
            x0 = np.ascontiguousarray(b.x0, np.float64).ravel()
            xi = None if b.x_init is None else np.ascontiguousarray(b.x_init, np.float64).ravel()
            tets = np.ascontiguousarray(b.tets, np.uint32).ravel()
            mat = Material(b.model, b.young, b.poisson, b.density)
            bid = C.c_int32()
            mass = None if b.mass is None else np.ascontiguousarray(b.mass, np.float64)
            self._check(L.sbs_gpu_add_body(h, x0, _ptr(xi), len(b.x0), tets, len(b.tets),
                                           C.byref(mat), _ptr(mass), C.byref(bid)))
            if getattr(b, "colours", None) is not None:
                self._check(L.sbs_gpu_set_tet_colours(h, bid, np.ascontiguousarray(b.colours, np.uint32)))
            if len(b.pinned):
                self._check(L.sbs_gpu_pin_vertices(h, bid, np.ascontiguousarray(b.pinned, np.uint32),
                                                   len(b.pinned)))
            if len(b.kin_verts):
                self._check(L.sbs_gpu_add_kinematic_rotation(
                    h, bid, np.ascontiguousarray(b.kin_verts, np.uint32), len(b.kin_verts),
                    np.asarray(b.kin_center, np.float64), np.asarray(b.kin_axis, np.float64),
                    b.kin_omega))
            if b.ext_acc is not None:
                self._check(L.sbs_gpu_set_external_acceleration(
                    h, bid, np.ascontiguousarray(b.ext_acc, np.float32).ravel()))
            self.body_sizes.append(len(b.x0))
        dist = getattr(scene, "distance", None)
        if dist is not None and len(dist):
            ids = np.ascontiguousarray(dist, np.uint32).ravel()
            self._check(L.sbs_gpu_add_distance_constraints(h, ids.ctypes.data, len(dist),
                                                           scene.distance_compliance, scene.distance_damping))
        if scene.ground is not None:
            n, d = scene.ground
            self._check(L.sbs_gpu_add_ground_plane(h, np.asarray(n, np.float64), d))
        for grid in getattr(scene, "sdf_grids", None) or []:
            values, dims, origin, spacing = grid[:4]
            add = L.sbs_gpu_add_sdf_grid_cubic if len(grid) > 4 and grid[4] == "cubic" else L.sbs_gpu_add_sdf_grid
            v = np.ascontiguousarray(values, np.float32).ravel()
            self._check(add(h, v.ctypes.data, np.ascontiguousarray(dims, np.uint32),
                            np.asarray(origin, np.float64), np.asarray(spacing, np.float64)))
        self._check(L.sbs_gpu_finalize(h))
        if any(b.v_init is not None for b in scene.bodies):
            for i, b in enumerate(scene.bodies):
                if b.v_init is not None:
                    self.set_state(i, None, b.v_init)

    def _check(self, status, h="self"):
        if status != SBS_OK:
            L = self.L
            handle = self.h if h == "self" and getattr(self, "h", None) else None
            msg = L.sbs_gpu_last_error(handle).decode()
            raise SbsError(status, f"{L.sbs_gpu_status_string(status).decode()}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.sbs_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping -----------------------------------------------------------
    def step(self, frames: int = 1, frame_dt=None, substeps=None, iterations=None):
        s = self.scene
        fdt = s.frame_dt if frame_dt is None else frame_dt
        sub = s.substeps if substeps is None else substeps
        its = s.iterations if iterations is None else iterations
        for _ in range(frames):
            self._check(self.L.sbs_gpu_step(self.h, fdt, sub, its))

    def step_timed(self, iterations=None) -> float:
        s = self.scene
        its = s.iterations if iterations is None else iterations
        self._check(self.L.sbs_gpu_step_timed(self.h, s.frame_dt, s.substeps, its))
        return self.stats().last_frame_ms

    def solve(self, dt: float, iterations: int):
        self._check(self.L.sbs_gpu_solve(self.h, dt, iterations))

    def predict(self, dt: float):
        self._check(self.L.sbs_gpu_predict(self.h, dt))

    def update_velocities(self, dt: float):
        self._check(self.L.sbs_gpu_update_velocities(self.h, dt))

    def detect_contacts(self):
        self._check(self.L.sbs_gpu_detect_contacts(self.h))

    def residual(self, dt: float):
        r, e = C.c_double(), C.c_double()
        self._check(self.L.sbs_gpu_residual(self.h, dt, C.byref(r), C.byref(e)))
        return r.value, e.value

    # -- state --------------------------------------------------------------
    def _nv(self, body: int) -> int:
        return self.scene.n_verts if body == -1 else self.body_sizes[body]

    def get_state(self, body: int = 0, out_x=None, out_v=None):
        """(x, v) of one body, or of the whole scene with body = -1.  out_x /
        out_v: contiguous float32 arrays of 3 * n values to write into (for
        example pinned host memory, which the copies reach directly)."""
        n = self._nv(body)

        def buf(out):
            if out is None:
                return np.zeros(3 * n, np.float32)
            if out.dtype != np.float32 or out.size != 3 * n or not out.flags.c_contiguous:
                raise ValueError("output buffers must be contiguous float32 of 3 * n_verts values")
            return out
        x = buf(out_x)
        v = buf(out_v)
        self._check(self.L.sbs_gpu_get_state(self.h, body, x.ctypes.data, v.ctypes.data))
        return x.reshape(-1, 3), v.reshape(-1, 3)

    def positions(self) -> np.ndarray:
        return self.get_state(-1)[0]

    def velocities(self) -> np.ndarray:
        return self.get_state(-1)[1]

    def set_state(self, body: int, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, np.float32).ravel()
        va = None if v is None else np.ascontiguousarray(v, np.float32).ravel()
        self._check(self.L.sbs_gpu_set_state(self.h, body, _ptr(xa), _ptr(va)))

    def get_predicted(self, body: int = 0) -> np.ndarray:
        x = np.zeros(3 * self._nv(body), np.float32)
        self._check(self.L.sbs_gpu_get_predicted(self.h, body, x))
        return x.reshape(-1, 3)

    def set_predicted(self, body: int, xi):
        self._check(self.L.sbs_gpu_set_predicted(self.h, body,
                                                 np.ascontiguousarray(xi, np.float32).ravel()))

    # -- introspection ------------------------------------------------------
    def tet_order(self):
        n = C.c_uint32()
        self._check(self.L.sbs_gpu_get_tet_order(self.h, None, None, 0, C.byref(n)))
        order = np.zeros(self.scene.n_tets, np.uint32)
        off = np.zeros(n.value + 1, np.uint32)
        self._check(self.L.sbs_gpu_get_tet_order(self.h, order.ctypes.data, off.ctypes.data,
                                                 len(off), C.byref(n)))
        return order, off

    def lambdas(self) -> np.ndarray:
        out = np.zeros(2 * self.scene.n_tets, np.float32)
        self._check(self.L.sbs_gpu_get_lambdas(self.h, out))
        return out.reshape(-1, 2)

    def contacts(self):
        n = C.c_uint32()
        self._check(self.L.sbs_gpu_get_contacts(self.h, None, None, 0, C.byref(n)))
        v = np.zeros(n.value, np.uint32)
        qn = np.zeros(6 * n.value, np.float32)
        self._check(self.L.sbs_gpu_get_contacts(self.h, v.ctypes.data, qn.ctypes.data, n.value,
                                                C.byref(n)))
        return v, qn.reshape(-1, 6)

    # -- learned warm start -------------------------------------------------
    def set_warm_start(self, mlp, fit_sweeps: int = 1):
        self._warm = mlp
        self._check(self.L.sbs_gpu_set_warm_start(self.h, None if mlp is None else mlp.h, fit_sweeps))

    def set_warm_judge(self, check_every: int, max_sweeps: int = 0, calibrate_every: int = 0,
                       fixed_target: float = 0.0):
        """The plain solver as judge of the warm-started substeps: sweeps in
        chunks of `check_every` until the plain residual target is reached
        (or `max_sweeps`), with a fallback to the plain start when the warm
        start's residual is not below the plain start's."""
        self._check(self.L.sbs_gpu_set_warm_judge(self.h, check_every, max_sweeps, calibrate_every, fixed_target))

    def warm_stats(self) -> WarmStats:
        st = WarmStats()
        self._check(self.L.sbs_gpu_get_warm_stats(self.h, C.byref(st)))
        return st

    def warm_start_init(self, dt: float):
        self._check(self.L.sbs_gpu_warm_start_init(self.h, dt))

    def solve_ex(self, dt: float, iterations: int, reset: bool):
        self._check(self.L.sbs_gpu_solve_ex(self.h, dt, iterations, 1 if reset else 0))

    def features(self) -> np.ndarray:
        out = np.zeros(16 * self.scene.n_verts, np.float32)
        self._check(self.L.sbs_gpu_get_features(self.h, out))
        return out.reshape(-1, 16)

    def predicted_all(self) -> np.ndarray:
        return self.get_predicted(-1)

    def candidates(self) -> np.ndarray:
        """Broad-phase (vertex << 32 | tet) pairs of the last detection, sorted."""
        n = C.c_uint64()
        self._check(self.L.sbs_gpu_get_candidates(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint64)
        self._check(self.L.sbs_gpu_get_candidates(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def inv_masses(self) -> np.ndarray:
        out = np.zeros(self.scene.n_verts, np.float32)
        self._check(self.L.sbs_gpu_get_masses(self.h, out))
        return out

    def surface(self) -> np.ndarray:
        n = C.c_uint32()
        self._check(self.L.sbs_gpu_get_surface(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint32)
        self._check(self.L.sbs_gpu_get_surface(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def distance_order(self):
        """(projection order of the distance constraints, colour offsets)."""
        n = C.c_uint32()
        self._check(self.L.sbs_gpu_get_distance_order(self.h, None, None, 0, C.byref(n)))
        dist = getattr(self.scene, "distance", None)
        order = np.zeros(0 if dist is None else len(dist), np.uint32)
        off = np.zeros(n.value + 1, np.uint32)
        self._check(self.L.sbs_gpu_get_distance_order(self.h, order.ctypes.data, off.ctypes.data, len(off),
                                                      C.byref(n)))
        return order, off

    def distance_lambdas(self) -> np.ndarray:
        dist = getattr(self.scene, "distance", None)
        out = np.zeros(0 if dist is None else len(dist), np.float32)
        if len(out):
            self._check(self.L.sbs_gpu_get_distance_lambdas(self.h, out.ctypes.data))
        return out

    def surface_mesh(self, body: int = 0):
        """Visual model of a body: (triangles [n_tri, 3] in surface-vertex
        ids, surface vertex -> body vertex map)."""
        nt, nv = C.c_uint32(), C.c_uint32()
        self._check(self.L.sbs_gpu_get_surface_mesh(self.h, body, None, 0, C.byref(nt), None, 0, C.byref(nv)))
        tris = np.zeros(3 * nt.value, np.uint32)
        vmap = np.zeros(nv.value, np.uint32)
        self._check(self.L.sbs_gpu_get_surface_mesh(self.h, body, tris.ctypes.data, nt.value, C.byref(nt),
                                                    vmap.ctypes.data, nv.value, C.byref(nv)))
        return tris.reshape(-1, 3), vmap

    def update_surface(self, body: int = 0, accumulate: bool = True, buffer=None, stride: int = 9):
        """One visual-model update.  `buffer`: None (returns a new host array
        [n_sv, stride], floats past the normal zero), a float32 host array
        to fill in place, or an int device pointer (written by the kernel)."""
        if buffer is None:
            nv = len(self.surface_mesh(body)[1])
            buffer = np.zeros((nv, stride), np.float32)
        ptr = buffer if isinstance(buffer, int) else buffer.ctypes.data
        self._check(self.L.sbs_gpu_update_surface(self.h, body, 1 if accumulate else 0, ptr, stride))
        return buffer

    def stats(self) -> Stats:
        st = Stats()
        self._check(self.L.sbs_gpu_get_stats(self.h, C.byref(st)))
        return st


class Mlp:
    """The warm-start MLP (sbs_mlp handle)."""

    def __init__(self, device: int = 0, seed: int = 0):
        L = load()
        self.L = L
        h = C.c_void_p()
        st = L.sbs_mlp_create(device, seed, C.byref(h))
        if st != SBS_OK:
            raise SbsError(st, "sbs_mlp_create failed")
        self.h = h
        self.n_params = int(L.sbs_mlp_param_count())

    def _check(self, st):
        if st != SBS_OK:
            raise SbsError(st, self.L.sbs_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.sbs_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(self.L.sbs_mlp_get_params(self.h, out))
        return out

    def set_params(self, p):
        self._check(self.L.sbs_mlp_set_params(self.h, np.ascontiguousarray(p, np.float32)))

    def set_normalization(self, mean, std, scale):
        self._check(self.L.sbs_mlp_set_normalization(
            self.h, np.ascontiguousarray(mean, np.float32), np.ascontiguousarray(std, np.float32),
            np.ascontiguousarray(scale, np.float32)))

    def forward(self, x, path: int = 0) -> np.ndarray:
        """Network output for rows x; path 0 = fused tcgen05 kernel, 1 = per-layer GEMMs."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((len(x), 3), np.float32)
        self._check(self.L.sbs_mlp_forward_path(self.h, x.ravel(), len(x), y.ravel(), path))
        return y

    def forward_device(self, x_ptr: int, n: int, y_ptr: int, path: int = 0) -> float:
        """Forward on device buffers (pointers of the network's device);
        returns the kernels' device time in ms."""
        ms = C.c_float()
        self._check(self.L.sbs_mlp_forward_device(self.h, x_ptr, n, y_ptr, path, C.byref(ms)))
        return ms.value

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float()
        g = np.zeros(self.n_params, np.float32)
        self._check(self.L.sbs_mlp_loss_grad(self.h, x.ravel(), t.ravel(), len(x), C.byref(loss),
                                             g.ctypes.data))
        return loss.value, g

    def set_dataset(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        self._check(self.L.sbs_mlp_set_dataset(self.h, x.ravel(), t.ravel(), len(x)))

    def train(self, steps: int, batch: int, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_float()
        self._check(self.L.sbs_mlp_train(self.h, steps, batch, lr, seed, C.byref(loss)))
        return loss.value

    GEMM_TC, GEMM_MMA_SYNC = 0, 1

    def set_gemm(self, engine: int):
        """Engine of the per-layer GEMMs: GEMM_TC (tcgen05, default) or GEMM_MMA_SYNC."""
        self._check(self.L.sbs_mlp_set_gemm(self.h, engine))
