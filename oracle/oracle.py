"""ctypes front end of the FP64 CPU oracle (oracle/xpbd_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py to check and time against.  The CUDA library never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "xpbd_oracle.cpp"
LIB = HERE / "liboracle_xpbd.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (OpenMP for the colour-parallel baseline)."""
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(SRC)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, D, U32, I = C.c_void_p, C.c_double, C.c_uint32, C.c_int
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        up = np.ctypeslib.ndpointer(np.uint32, flags="C")
        L.orc_create.restype = P
        L.orc_create.argtypes = [D, D, D, dp, I]
        L.orc_destroy.argtypes = [P]
        L.orc_set_threads.argtypes = [P, I]
        L.orc_add_body.restype = I
        L.orc_add_body.argtypes = [P, dp, C.c_void_p, U32, up, U32, I, D, D, D, C.c_void_p]
        L.orc_pin.argtypes = [P, I, up, U32]
        L.orc_add_kinematic_rotation.argtypes = [P, I, up, U32, dp, dp, D]
        L.orc_set_external_acceleration.argtypes = [P, I, dp]
        L.orc_add_ground_plane.argtypes = [P, dp, D]
        L.orc_add_sdf_grid.argtypes = [P, C.c_void_p, up, dp, dp]
        L.orc_add_sdf_grid_cubic.argtypes = [P, C.c_void_p, up, dp, dp]
        L.orc_grid_eval.restype = I
        L.orc_grid_eval.argtypes = [P, I, dp, dp]
        L.orc_set_tet_order.restype = I
        L.orc_plan_colours.restype = U32
        L.orc_plan_colours.argtypes = [P, up, up, U32]
        L.orc_set_tet_order.argtypes = [P, up, U32, C.c_void_p, U32]
        L.orc_step.argtypes = [P, D, U32, U32]
        L.orc_step_fast.argtypes = [P, D, U32, U32]
        L.orc_solve.argtypes = [P, D, U32]
        L.orc_predict.argtypes = [P, D]
        L.orc_finalize.argtypes = [P, D]
        L.orc_detect_contacts.argtypes = [P]
        L.orc_residual.argtypes = [P, D, dp]
        L.orc_set_record_history.argtypes = [P, I]
        L.orc_get_history.restype = U32
        L.orc_get_history.argtypes = [P, dp, U32]
        L.orc_get.argtypes = [P, I, dp]
        L.orc_set.argtypes = [P, I, dp]
        L.orc_get_masses.argtypes = [P, dp]
        L.orc_get_surface.restype = U32
        L.orc_get_surface.argtypes = [P, I, up, U32]
        L.orc_get_lambdas.argtypes = [P, dp]
        L.orc_add_distance.restype = I
        L.orc_add_distance.argtypes = [P, up, U32, D, D]
        L.orc_set_edge_order.restype = I
        L.orc_set_edge_order.argtypes = [P, up, U32, C.c_void_p, U32]
        L.orc_get_distance_lambdas.argtypes = [P, dp]
        L.orc_surface_mesh.argtypes = [P, I, C.c_void_p, U32, C.POINTER(U32), C.c_void_p, U32, C.POINTER(U32)]
        L.orc_update_surface.argtypes = [P, I, I, dp, dp]
        L.orc_get_contacts.restype = U32
        L.orc_get_contacts.argtypes = [P, up, dp, U32]
        L.orc_tet_eval.argtypes = [P, U32, C.POINTER(D), dp]
        L.orc_svd3.argtypes = [dp, dp, dp, dp]
        L.orc_time.restype = D
        L.orc_time.argtypes = [P]
        L.orc_projections.restype = C.c_uint64
        L.orc_projections.argtypes = [P]
        L.orc_n_contacts.restype = U32
        L.orc_n_contacts.argtypes = [P]
        L.orc_stats.argtypes = [P, dp]
        L.orc_set_body_contacts.argtypes = [P, I, D]
        L.orc_hash_candidates.restype = C.c_uint64
        L.orc_hash_candidates.argtypes = [P, np.ctypeslib.ndpointer(np.float32, flags="C"), D, I,
                                          C.c_void_p, C.c_uint64]
        L.orc_n_body_contacts.restype = U32
        L.orc_n_body_contacts.argtypes = [P]
        L.orc_time_frames.restype = D
        L.orc_time_frames.argtypes = [P, D, U32, U32, U32]
        _lib = L
    return _lib


FIELD_X, FIELD_XI, FIELD_V, FIELD_X0 = 0, 1, 2, 3


class Oracle:
    """One oracle simulation built from a ``sbs_gb300.scenes.Scene``."""

    def __init__(self, scene, threads: int = 1):
        L = lib()
        self.L = L
        self.scene = scene
        g = np.asarray(scene.gravity, np.float64)
        self.h = L.orc_create(scene.compliance, scene.damping,
                              scene.collision_compliance, g, scene.gravity_mode)
        L.orc_set_threads(self.h, threads)
        self.n_verts = 0
        self.n_tets = 0
        self.body_ranges = []
        for b in scene.bodies:
            x0 = np.ascontiguousarray(b.x0, np.float64).ravel()
            xi = None if b.x_init is None else \
                np.ascontiguousarray(b.x_init, np.float64).ravel()
            tets = np.ascontiguousarray(b.tets, np.uint32).ravel()
            mass = None if getattr(b, "mass", None) is None else \
                np.ascontiguousarray(b.mass, np.float64)
            self._mass_keep = mass
            bid = L.orc_add_body(self.h, x0,
                                 None if xi is None else xi.ctypes.data,
                                 len(b.x0), tets, len(b.tets), b.model,
                                 b.young, b.poisson, b.density,
                                 None if mass is None else mass.ctypes.data)
            if len(b.pinned):
                L.orc_pin(self.h, bid, np.ascontiguousarray(b.pinned, np.uint32),
                          len(b.pinned))
            if len(b.kin_verts):
                L.orc_add_kinematic_rotation(
                    self.h, bid, np.ascontiguousarray(b.kin_verts, np.uint32),
                    len(b.kin_verts), np.asarray(b.kin_center, np.float64),
                    np.asarray(b.kin_axis, np.float64), b.kin_omega)
            if b.ext_acc is not None:
                L.orc_set_external_acceleration(
                    self.h, bid, np.ascontiguousarray(b.ext_acc, np.float64).ravel())
            self.body_ranges.append((self.n_verts, len(b.x0)))
            self.n_verts += len(b.x0)
            self.n_tets += len(b.tets)
        dist = getattr(scene, "distance", None)
        if dist is not None and len(dist):
            ids = np.ascontiguousarray(dist, np.uint32).ravel()
            if L.orc_add_distance(self.h, ids, len(dist), scene.distance_compliance, scene.distance_damping):
                raise ValueError("bad distance constraint ids")
        if scene.ground is not None:
            n, d = scene.ground
            L.orc_add_ground_plane(self.h, np.asarray(n, np.float64), d)
        self._grids = []
        for grid in getattr(scene, "sdf_grids", None) or []:
            values, dims, origin, spacing = grid[:4]
            cubic = len(grid) > 4 and grid[4] == "cubic"
            v = np.ascontiguousarray(values, np.float32).ravel()
            self._grids.append(v)
            add = L.orc_add_sdf_grid_cubic if cubic else L.orc_add_sdf_grid
            add(self.h, v.ctypes.data, np.ascontiguousarray(dims, np.uint32),
                np.asarray(origin, np.float64), np.asarray(spacing, np.float64))
        if getattr(scene, "body_contacts", 0):
            cell = scene.hash_cell if scene.hash_cell > 0 else mean_edge_cell(scene)
            self.hash_cell = cell
            L.orc_set_body_contacts(self.h, int(scene.body_contacts), cell)
        if scene.bodies and scene.bodies[0].v_init is not None:
            v = np.concatenate([b.v_init if b.v_init is not None else np.zeros_like(b.x0)
                                for b in scene.bodies])
            self.set(FIELD_V, v)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def set_order(self, order: np.ndarray, offsets: np.ndarray | None = None):
        order = np.ascontiguousarray(order, np.uint32)
        if offsets is None:
            rc = self.L.orc_set_tet_order(self.h, order, len(order), None, 0)
        else:
            off = np.ascontiguousarray(offsets, np.uint32)
            self._off = off
            rc = self.L.orc_set_tet_order(self.h, order, len(order),
                                          off.ctypes.data, len(off) - 1)
        if rc:
            raise ValueError("bad tet order")

    def plan_colours(self):
        """The oracle's own colour-parallel plan (first-fit colouring in list
        order, colour-major): (order, offsets), without the CUDA library."""
        order = np.zeros(self.n_tets, np.uint32)
        cap = 4096
        offsets = np.zeros(cap, np.uint32)
        n = self.L.orc_plan_colours(self.h, order, offsets, cap)
        if n == 0 and self.n_tets:
            raise ValueError("more than 4095 colours")
        return order, offsets[: n + 1].copy()

    def set_edge_order(self, order: np.ndarray, offsets: np.ndarray | None = None):
        """Projection order (input indices, colour-major) of the distance
        constraints, which run after the tets in every sweep."""
        order = np.ascontiguousarray(order, np.uint32)
        off = None if offsets is None else np.ascontiguousarray(offsets, np.uint32)
        self._eoff = off
        rc = self.L.orc_set_edge_order(self.h, order, len(order), None if off is None else off.ctypes.data,
                                       0 if off is None else len(off) - 1)
        if rc:
            raise ValueError("bad edge order")

    def distance_lambdas(self) -> np.ndarray:
        dist = getattr(self.scene, "distance", None)
        n = 0 if dist is None else len(dist)
        out = np.zeros(n)
        if n:
            self.L.orc_get_distance_lambdas(self.h, out)
        return out

    def step(self, frames: int = 1, fast: bool = False):
        s = self.scene
        f = self.L.orc_step_fast if fast else self.L.orc_step
        for _ in range(frames):
            f(self.h, s.frame_dt, s.substeps, s.iterations)

    def get(self, field: int = FIELD_X) -> np.ndarray:
        out = np.zeros(self.n_verts * 3)
        self.L.orc_get(self.h, field, out)
        return out.reshape(-1, 3)

    def set(self, field: int, x: np.ndarray):
        self.L.orc_set(self.h, field, np.ascontiguousarray(x, np.float64).ravel())

    def masses(self) -> np.ndarray:
        out = np.zeros(self.n_verts)
        self.L.orc_get_masses(self.h, out)
        return out

    def surface(self, body: int = 0) -> np.ndarray:
        n = self.L.orc_get_surface(self.h, body, np.zeros(0, np.uint32), 0)
        out = np.zeros(n, np.uint32)
        self.L.orc_get_surface(self.h, body, out, n)
        return out

    def surface_mesh(self, body: int = 0):
        """(triangles [n_tri, 3] of surface-local ids, surface vertex -> body
        vertex map) of the body's visual model."""
        nt, nv = C.c_uint32(), C.c_uint32()
        self.L.orc_surface_mesh(self.h, body, None, 0, C.byref(nt), None, 0, C.byref(nv))
        tris = np.zeros(3 * nt.value, np.uint32)
        vmap = np.zeros(nv.value, np.uint32)
        self.L.orc_surface_mesh(self.h, body, tris.ctypes.data, nt.value, C.byref(nt), vmap.ctypes.data,
                                nv.value, C.byref(nv))
        return tris.reshape(-1, 3), vmap

    def update_surface(self, body: int = 0, accumulate: bool = True):
        """One visual-model update; returns (positions, normals) [n_sv, 3]."""
        _, vmap = self.surface_mesh(body)
        pos = np.zeros(3 * len(vmap))
        nrm = np.zeros(3 * len(vmap))
        self.L.orc_update_surface(self.h, body, 1 if accumulate else 0, pos, nrm)
        return pos.reshape(-1, 3), nrm.reshape(-1, 3)

    def lambdas(self) -> np.ndarray:
        out = np.zeros(self.n_tets * 2)
        self.L.orc_get_lambdas(self.h, out)
        return out.reshape(-1, 2)

    def detect_contacts(self):
        self.L.orc_detect_contacts(self.h)
        n = self.L.orc_get_contacts(self.h, np.zeros(0, np.uint32), np.zeros(0), 0)
        v = np.zeros(n, np.uint32)
        qn = np.zeros(6 * n)
        self.L.orc_get_contacts(self.h, v, qn, n)
        return v, qn.reshape(-1, 6)

    def stats(self) -> dict:
        out = np.zeros(4)
        self.L.orc_stats(self.h, out)
        return {"residual": out[0], "energy": out[1], "residual_elastic": out[2],
                "residual_contact": out[3],
                "projections": int(self.L.orc_projections(self.h)),
                "contacts": int(self.L.orc_n_contacts(self.h))}

    def grid_eval(self, grid: int, p):
        """(signed distance, gradient) of environment grid `grid` at p, or
        None outside it."""
        out = np.zeros(4)
        if not self.L.orc_grid_eval(self.h, grid, np.ascontiguousarray(p, np.float64), out):
            return None
        return out[0], out[1:]

    def time_frames(self, n: int) -> float:
        s = self.scene
        return self.L.orc_time_frames(self.h, s.frame_dt, s.substeps, s.iterations, n)


def mean_edge_cell(scene) -> float:
    """2 x the mean edge length of the rest meshes (the default hash cell)."""
    tot, cnt = 0.0, 0
    for b in scene.bodies:
        t = b.tets.astype(np.int64)
        for a, c in ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)):
            tot += np.linalg.norm(b.x0[t[:, a]] - b.x0[t[:, c]], axis=1).sum()
            cnt += len(t)
    return 2.0 * tot / cnt


def hash_candidates(o: "Oracle", xf: np.ndarray, cell: float, self_contacts: bool = False):
    """Broad-phase candidate pairs (vertex << 32 | tet) of the CPU hash for
    float32 positions xf [V,3] (add order), sorted."""
    xf = np.ascontiguousarray(xf, np.float32).ravel()
    n = o.L.orc_hash_candidates(o.h, xf, cell, int(self_contacts), None, 0)
    out = np.zeros(n, np.uint64)
    o.L.orc_hash_candidates(o.h, xf, cell, int(self_contacts), out.ctypes.data, n)
    return out


def nudged_oracle(scene, order=None, offsets=None, seed: int = 0, threads: int = 1) -> "Oracle":
    """An oracle whose initial positions are rounded to FP32 and then moved
    one ulp up or down per coordinate (seeded): the smallest perturbation an
    FP32 implementation makes to the initial state."""
    b = Oracle(scene, threads=threads)
    if order is not None:
        b.set_order(order, offsets)
    x = b.get()
    rng = np.random.default_rng(seed)
    x32 = x.astype(np.float32)
    toward = np.where(rng.random(x.shape) < 0.5, -np.inf, np.inf).astype(np.float32)
    b.set(FIELD_X, np.nextafter(x32, toward).astype(np.float64))
    return b


def noise_floor(scene, frames: int, order=None, offsets=None, seed: int = 0, threads: int = 1,
                n_seeds: int = 1) -> float:
    """Max position deviation after `frames` between the oracle and oracles
    restarted from FP32-rounded initial positions nudged by one ulp (seeds
    seed .. seed + n_seeds - 1; the largest deviation counts).  It measures
    how far rounding at FP32 level alone carries the sequential loop, the
    yardstick for multi-frame FP32-vs-FP64 comparisons.  `threads` > 1 runs
    the colour-parallel sweep, bit-identical to the sequential one."""
    a = Oracle(scene, threads=threads)
    if order is not None:
        a.set_order(order, offsets)
    a.step(frames)
    xa = a.get()
    worst = 0.0
    for k in range(n_seeds):
        b = nudged_oracle(scene, order, offsets, seed + k, threads)
        b.step(frames)
        worst = max(worst, float(np.abs(xa - b.get()).max()))
    return worst


def sync_state(src: "Oracle", dst_oracle: "Oracle | None" = None):
    """FP32-rounded positions and velocities of `src` (also written back)."""
    x = src.get().astype(np.float32).astype(np.float64)
    v = src.get(FIELD_V).astype(np.float32).astype(np.float64)
    src.set(FIELD_X, x)
    src.set(FIELD_V, v)
    return x, v


def svd3(F: np.ndarray):
    U = np.zeros(9)
    s = np.zeros(3)
    V = np.zeros(9)
    lib().orc_svd3(np.ascontiguousarray(F, np.float64).ravel(), U, s, V)
    return U.reshape(3, 3), s, V.reshape(3, 3)
