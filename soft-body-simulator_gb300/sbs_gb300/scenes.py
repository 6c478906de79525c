"""Synthetic tetrahedral scenes for the XPBD hot path.

Every generator returns plain numpy arrays (float64 positions, uint32 tets) so
the same input feeds the CUDA library (through the C ABI) and the FP64 CPU
oracle.  Nothing here touches a GPU.

* ``bar_5tet`` restates the reference's ``get_simple_bar_model``
  (src/geometry/get_simple_bar_model.cpp:6-122): ``width x height x depth``
  *vertices* at unit spacing, vertex ``(i, j, k)`` at row
  ``i*height*depth + j*depth + k``, five tets per cube with the split chosen by
  the parity of ``i + j + k``.
* ``bar_6tet`` is the Freudenthal/Kuhn split (six tets per cube around the
  ``p0 -> p6`` diagonal); the reference has no such generator.
* ``lumped_masses`` gives every vertex a quarter of the mass of each incident
  tet (the reference gives every particle mass 1, src/physics/particle.cpp:7).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MODEL_STVK = 0
MODEL_SNH = 1


def _corner_ids(width: int, height: int, depth: int):
    """Vertex ids of the 8 corners of every cube, in the reference's p0..p7
    labelling (get_simple_bar_model.cpp:34-51), cubes in (i, j, k) order."""
    i, j, k = np.meshgrid(np.arange(width - 1), np.arange(height - 1),
                          np.arange(depth - 1), indexing="ij")
    i = i.ravel().astype(np.int64)
    j = j.ravel().astype(np.int64)
    k = k.ravel().astype(np.int64)
    hd = height * depth

    def vid(a, b, c):
        return a * hd + b * depth + c

    p = np.stack([
        vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
        vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1),
        vid(i, j + 1, k + 1)], axis=1)
    return p, (i + j + k) % 2


def bar_vertices(width: int, height: int, depth: int, spacing: float = 1.0):
    """Grid vertices, row-major in (i, j, k) as get_simple_bar_model.cpp:11-24."""
    i, j, k = np.meshgrid(np.arange(width), np.arange(height), np.arange(depth),
                          indexing="ij")
    x = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    return x * spacing


def bar_5tet(width: int, height: int, depth: int, spacing: float = 1.0):
    """Five tets per cube, split alternating with cube parity.

    Restates get_simple_bar_model.cpp:26-117 (odd parity -> first table,
    even parity -> second table), tet order cube-major, five per cube.
    Returns ``(x0 [V,3] float64, tets [T,4] uint32)``.
    """
    p, parity = _corner_ids(width, height, depth)
    odd = np.array([[1, 0, 5, 2], [5, 2, 7, 6], [7, 0, 5, 4], [2, 0, 7, 3],
                    [5, 0, 7, 2]])
    even = np.array([[3, 1, 4, 0], [6, 1, 3, 2], [4, 1, 6, 5], [6, 3, 4, 7],
                     [3, 1, 6, 4]])
    table = np.where(parity[:, None, None] == 1, odd[None], even[None])
    tets = np.take_along_axis(p[:, None, :].repeat(5, axis=1), table, axis=2)
    return bar_vertices(width, height, depth, spacing), \
        tets.reshape(-1, 4).astype(np.uint32)


def bar_6tet(width: int, height: int, depth: int, spacing: float = 1.0):
    """Six tets per cube (Freudenthal/Kuhn), every cube split the same way.

    For each permutation (a, b, c) of the axes the tet walks p0 -> p0+e_a ->
    p0+e_a+e_b -> p6.  Conforming across cubes because all cubes share the
    same diagonal direction.
    """
    p, _ = _corner_ids(width, height, depth)
    # corner label of offset (dx, dy, dz) in the p0..p7 scheme
    lab = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3,
           (0, 0, 1): 4, (1, 0, 1): 5, (1, 1, 1): 6, (0, 1, 1): 7}
    rows = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        o = [0, 0, 0]
        walk = [lab[tuple(o)]]
        for ax in perm:
            o[ax] = 1
            walk.append(lab[tuple(o)])
        rows.append(walk)
    table = np.array(rows)
    tets = p[:, table]  # [cubes, 6, 4]
    return bar_vertices(width, height, depth, spacing), \
        tets.reshape(-1, 4).astype(np.uint32)


def lattice_colours_6tet(width: int, height: int, depth: int) -> np.ndarray:
    """A 24-colouring of bar_6tet's tets (same arguments, in vertices):
    colour = 4 * (the tet's axis permutation, 0..5) + (i + j + k) mod 4 for
    the tet of cube (i, j, k).  Tets of one permutation in two cubes share a
    vertex only if the cubes' offset is a difference of two corners of that
    permutation's walk p0 -> p0+e_a -> p0+e_a+e_b -> p6, whose coordinate
    sums are +-1, +-2 or +-3, never 0 mod 4; so a colour class shares no
    vertex.  24 tets meet at an interior vertex, so 24 colours is the
    minimum; the library's greedy colourings need 28 on the 98k-tet beam."""
    i, j, k = np.meshgrid(np.arange(width - 1), np.arange(height - 1), np.arange(depth - 1), indexing="ij")
    lat = ((i + j + k) % 4).ravel()
    return (4 * np.arange(6)[None, :] + lat[:, None]).ravel().astype(np.uint32)


# A 34-colouring of bar_5tet's tets on the 4 x 4 x 4-cube torus (cubes
# (i, j, k) mod 4, five tets each in bar_5tet's order), found by TabuCol
# (Hertz & de Werra 1987) for this project.  Any two tets of a grid that share
# a vertex also share it on the torus, so the pattern repeated over any grid
# is a valid colouring.  Every colour holds 9 or 10 of the torus's 320 tets.
_COLOURS_5TET_P4 = np.array([
    27, 2, 9, 4, 24, 12, 31, 14, 10, 0, 33, 24, 32, 12, 29, 16, 22, 1, 10, 18,
    7, 8, 11, 31, 25, 16, 21, 22, 20, 18, 11, 7, 28, 19, 25, 30, 23, 13, 32, 0,
    30, 2, 29, 17, 33, 10, 31, 24, 14, 32, 29, 30, 5, 33, 12, 22, 27, 18, 1, 16,
    15, 19, 22, 28, 8, 11, 6, 9, 15, 16, 25, 11, 0, 2, 26, 14, 7, 29, 25, 31,
    6, 19, 26, 30, 3, 23, 1, 22, 28, 5, 19, 20, 1, 21, 8, 14, 31, 23, 4, 33,
    17, 12, 32, 20, 15, 6, 16, 33, 13, 14, 2, 0, 27, 6, 17, 26, 14, 5, 19, 9,
    11, 7, 4, 26, 24, 3, 5, 9, 28, 23, 1, 2, 15, 8, 4, 21, 23, 3, 6, 28,
    12, 17, 27, 21, 0, 25, 7, 20, 30, 13, 3, 27, 24, 17, 18, 13, 5, 20, 10, 32,
    24, 11, 14, 20, 10, 29, 24, 9, 4, 32, 26, 10, 4, 29, 30, 28, 8, 7, 16, 22,
    21, 8, 27, 1, 28, 31, 0, 13, 18, 25, 15, 24, 7, 12, 11, 18, 33, 0, 13, 25,
    19, 14, 17, 10, 30, 33, 32, 21, 22, 29, 10, 14, 20, 30, 31, 32, 18, 22, 16, 29,
    4, 18, 8, 31, 2, 15, 11, 16, 33, 12, 17, 2, 11, 6, 0, 25, 12, 33, 15, 9,
    29, 33, 1, 16, 26, 5, 17, 3, 7, 23, 8, 5, 19, 1, 13, 27, 9, 21, 6, 17,
    3, 5, 19, 2, 12, 15, 27, 30, 22, 9, 26, 4, 21, 3, 2, 14, 15, 23, 31, 20,
    4, 0, 26, 9, 6, 28, 3, 23, 19, 1, 17, 13, 8, 5, 6, 27, 26, 11, 7, 10,
    5, 32, 21, 25, 13, 7, 18, 27, 31, 20, 21, 28, 4, 15, 22, 24, 20, 19, 3, 23,
], dtype=np.uint32).reshape(4, 4, 4, 5)


def lattice_colours_5tet(width: int, height: int, depth: int) -> np.ndarray:
    """A 34-colouring of bar_5tet's tets (same arguments, in vertices): the
    torus pattern _COLOURS_5TET_P4 repeated with period 4 cubes.  32 tets meet
    at the vertices the centre tets use, so 32 colours is the bound; the
    library's greedy colourings need 36 on the 2.6M-tet block."""
    i, j, k = np.meshgrid(np.arange(width - 1), np.arange(height - 1), np.arange(depth - 1), indexing="ij")
    return _COLOURS_5TET_P4[i.ravel() % 4, j.ravel() % 4, k.ravel() % 4].ravel().astype(np.uint32)


def signed_volumes(x: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """V = det([x1-x4, x2-x4, x3-x4]) / 6 (green_constraint.cpp:160-173)."""
    t = tets.astype(np.int64)
    d = np.stack([x[t[:, 0]] - x[t[:, 3]], x[t[:, 1]] - x[t[:, 3]],
                  x[t[:, 2]] - x[t[:, 3]]], axis=2)
    return np.linalg.det(d) / 6.0


def lumped_masses(x0: np.ndarray, tets: np.ndarray, density: float) -> np.ndarray:
    """m_v = sum over incident tets of density * |V0| / 4."""
    vol = np.abs(signed_volumes(x0, tets))
    m = np.zeros(len(x0))
    for c in range(4):
        np.add.at(m, tets[:, c].astype(np.int64), density * vol / 4.0)
    return m


def boundary_vertices(tets: np.ndarray, n_verts: int) -> np.ndarray:
    """Vertices on boundary triangles (faces with != 2 incident tets).

    Faces follow tetrahedron_t::faces_copy (src/physics/topology.cpp:335-342),
    deduplicated by their sorted vertex triple as triangle_t::operator<
    (topology.cpp:245-254) does; boundary rule from
    tetrahedral_mesh_boundary.cpp:86-90.  Returned sorted ascending.
    """
    t = tets.astype(np.int64)
    faces = np.concatenate([t[:, [0, 1, 3]], t[:, [1, 2, 3]], t[:, [2, 0, 3]],
                            t[:, [0, 2, 1]]])
    faces = np.sort(faces, axis=1)
    key = (faces[:, 0] * n_verts + faces[:, 1]) * n_verts + faces[:, 2]
    uniq, cnt = np.unique(key, return_counts=True)
    bkey = uniq[cnt != 2]
    verts = np.unique(np.stack([bkey // (n_verts * n_verts),
                                (bkey // n_verts) % n_verts,
                                bkey % n_verts], axis=1))
    return verts.astype(np.uint32)


def boundary_triangles(tets: np.ndarray, n_verts: int) -> np.ndarray:
    """Boundary triangles (faces with one incident tet), outward winding.

    The winding is taken from the owning tet's face so that the normal of
    ``(b - a) x (c - a)`` points out of a positively oriented tet.
    """
    t = tets.astype(np.int64)
    faces = np.concatenate([t[:, [0, 1, 3]], t[:, [1, 2, 3]], t[:, [2, 0, 3]],
                            t[:, [0, 2, 1]]])
    s = np.sort(faces, axis=1)
    key = (s[:, 0] * n_verts + s[:, 1]) * n_verts + s[:, 2]
    _, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
    keep = cnt[inv] == 1
    return faces[keep].astype(np.uint32)


def jitter(x: np.ndarray, amplitude: float, seed: int,
           frozen: np.ndarray | None = None) -> np.ndarray:
    """Uniform +-amplitude jitter from a seeded PCG64 stream; ``frozen``
    vertex ids keep their rest position."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(-amplitude, amplitude, size=x.shape)
    if frozen is not None and len(frozen):
        d[np.asarray(frozen, dtype=np.int64)] = 0.0
    return x + d


@dataclass
class Body:
    """One tetrahedral body: rest shape, initial state and material."""
    x0: np.ndarray                  # [V,3] rest positions (float64)
    tets: np.ndarray                # [T,4] uint32
    model: int = MODEL_STVK
    young: float = 1e6
    poisson: float = 0.3
    density: float = 1000.0
    x_init: np.ndarray | None = None  # [V,3] initial positions (defaults to x0)
    v_init: np.ndarray | None = None  # [V,3] initial velocities (defaults to 0)
    pinned: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    kin_verts: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    kin_center: tuple = (0.0, 0.0, 0.0)
    kin_axis: tuple = (1.0, 0.0, 0.0)
    kin_omega: float = 0.0
    ext_acc: np.ndarray | None = None  # [V,3] external acceleration field
    mass: np.ndarray | None = None     # [V] per-vertex masses (None: lumped from density)
    colours: np.ndarray | None = None  # [T] a colouring for the sweep order (None: the library's own)


@dataclass
class Scene:
    """A set of bodies plus the solver settings of one workload."""
    name: str
    bodies: list
    frame_dt: float = 1.0 / 60.0
    substeps: int = 1
    iterations: int = 10
    frames: int = 1
    compliance: float = 1e-4          # simulation_parameters.h:12
    damping: float = 0.0              # simulation_parameters.h:13
    collision_compliance: float = 1e-8  # simulation_parameters.h:26
    gravity: tuple = (0.0, -9.81, 0.0)
    gravity_mode: int = 0             # 0: acceleration, 1: force on m (reference)
    # distance_constraint_t (distance_constraint.cpp:8-53): rows (b1, b2, v1, v2)
    distance: list | None = None
    distance_compliance: float = 0.0
    distance_damping: float = 0.0
    ground: tuple | None = ((0.0, 1.0, 0.0), 1.0)  # (n, d): n.x + d = 0
    # signed-distance grids of environment bodies: (values [nz, ny, nx] float32,
    # nodes (nx, ny, nz), origin, spacing)
    sdf_grids: list | None = None
    body_contacts: bool = False
    hash_cell: float = 0.0

    @property
    def n_tets(self) -> int:
        return sum(len(b.tets) for b in self.bodies)

    @property
    def n_verts(self) -> int:
        return sum(len(b.x0) for b in self.bodies)

    def bbox_diag(self) -> float:
        x = np.concatenate([b.x_init if b.x_init is not None else b.x0
                            for b in self.bodies])
        return float(np.linalg.norm(x.max(0) - x.min(0)))


def beam_c1(seed: int = 1, frames: int = 120, iterations: int = 10) -> Scene:
    """Cantilever of 10x3x3 cubes of 0.1 m, 5 tets each (450 tets, 176
    vertices); StVK E 1e5 / nu 0.45 / rho 1000; x=0 face pinned; ground y=-1;
    dt 1/60, 1 substep, 10 iterations; +-1e-3 m jitter on unpinned vertices."""
    x0, tets = bar_5tet(11, 4, 4, 0.1)
    pinned = np.nonzero(np.isclose(x0[:, 0], 0.0))[0].astype(np.uint32)
    b = Body(x0=x0, tets=tets, model=MODEL_STVK, young=1e5, poisson=0.45,
             density=1000.0, x_init=jitter(x0, 1e-3, seed, pinned), pinned=pinned)
    return Scene("beam-450-stvk", [b], 1.0 / 60.0, 1, iterations, frames,
                 ground=((0.0, 1.0, 0.0), 1.0))


def beam_twist(nx: int = 64, ny: int = 16, nz: int = 16, h: float = 0.05,
               seed: int = 2, frames: int = 300, substeps: int = 4,
               iterations: int = 30, omega: float = 1.0, lattice: bool = True) -> Scene:
    """Twisting beam: nx x ny x nz cubes of h metres, 6 tets each, stable
    Neo-Hookean E 1e6 / nu 0.49 / rho 1000; x=0 face pinned, x=max face turned
    about the beam's x axis at ``omega`` rad/s; +-1e-4 m jitter.  The default
    sizes are the 98,304-tet / 18,785-vertex beam.  lattice: the body carries
    the grid's 24-colouring (lattice_colours_6tet) for the sweep order."""
    x0, tets = bar_6tet(nx + 1, ny + 1, nz + 1, h)
    xmax = nx * h
    pinned = np.nonzero(np.isclose(x0[:, 0], 0.0))[0].astype(np.uint32)
    kin = np.nonzero(np.isclose(x0[:, 0], xmax))[0].astype(np.uint32)
    frozen = np.concatenate([pinned, kin])
    center = (xmax, ny * h / 2.0, nz * h / 2.0)
    b = Body(x0=x0, tets=tets, model=MODEL_SNH, young=1e6, poisson=0.49,
             density=1000.0, x_init=jitter(x0, 1e-4, seed, frozen),
             pinned=pinned, kin_verts=kin, kin_center=center,
             kin_axis=(1.0, 0.0, 0.0), kin_omega=omega,
             colours=lattice_colours_6tet(nx + 1, ny + 1, nz + 1) if lattice else None)
    return Scene(f"beam-{len(tets)}-snh-twist", [b], 1.0 / 60.0, substeps,
                 iterations, frames, ground=((0.0, 1.0, 0.0), 1.0))


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation from a uniform unit quaternion (Shoemake)."""
    u1, u2, u3 = rng.uniform(size=3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2),
                  math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3),
                  math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def box_drop(n_bodies: int = 512, seed: int = 3, cell: float = 0.05,
             min_cells: int = 4, max_cells: int = 24, arena: float = 20.0,
             frames: int = 600, substeps: int = 2, iterations: int = 20,
             model: int = MODEL_STVK, body_contacts: bool = True,
             young: tuple = (1e4, 1e6)) -> Scene:
    """Batch of box bodies dropped onto the ground.

    Cells per axis are floor(log-uniform[min_cells, max_cells]), 5 tets per
    cube; E log-uniform [young[0], young[1]] (1e4..1e6 Pa by default), nu
    U(0.3, 0.49); drop height U(1, 10) m; uniform random rotation; centres on
    a jittered grid over the arena.
    """
    rng = np.random.default_rng(seed)
    bodies = []
    side = int(math.ceil(math.sqrt(n_bodies)))
    pitch = arena / side
    edge_sum, edge_n = 0.0, 0
    for b in range(n_bodies):
        n = [int(math.floor(math.exp(rng.uniform(math.log(min_cells),
                                                  math.log(max_cells)))))
             for _ in range(3)]
        n = [min(max(v, min_cells), max_cells) for v in n]
        young_b = math.exp(rng.uniform(math.log(young[0]), math.log(young[1])))
        nu = rng.uniform(0.3, 0.49)
        height = rng.uniform(1.0, 10.0)
        rot = random_rotation(rng)
        gx, gz = b % side, b // side
        cx = -arena / 2 + (gx + 0.5) * pitch + rng.uniform(-0.1, 0.1) * pitch
        cz = -arena / 2 + (gz + 0.5) * pitch + rng.uniform(-0.1, 0.1) * pitch
        x0, tets = bar_5tet(n[0] + 1, n[1] + 1, n[2] + 1, cell)
        x0 = x0 - x0.mean(0)
        x0 = x0 @ rot.T + np.array([cx, height, cz])
        bodies.append(Body(x0=x0, tets=tets, model=model, young=young_b,
                           poisson=nu, density=1000.0, x_init=x0.copy()))
        edge_sum += cell * (n[0] * 1.0)
        edge_n += n[0]
    # mean edge of the 5-tet split: 12 cube edges (h) + 6 face diagonals (h*sqrt2)
    # per cube, with face diagonals shared by two cubes -> use h*(12+6*sqrt2)/18
    mean_edge = cell * (12 + 6 * math.sqrt(2)) / 18.0
    return Scene(f"box-drop-{n_bodies}", bodies, 1.0 / 60.0, substeps,
                 iterations, frames, ground=((0.0, 1.0, 0.0), 0.0),
                 body_contacts=body_contacts, hash_cell=2.0 * mean_edge)


def hanging_block(alpha: float = 1e-7, beta: float = 0.0, frames: int = 60, iterations: int = 20) -> Scene:
    """Distance constraints: a 4x2x2-cube StVK cantilever (pinned at x = 0)
    with a 2x2x2-cube block hanging 0.2 m below its free end on four springs
    (bottom corners of the end face to the block's top corners), plus four
    springs inside the cantilever (diagonals across its top face)."""
    xa, ta = bar_5tet(5, 3, 3, 0.1)
    xb, tb = bar_5tet(3, 3, 3, 0.1)
    xb = xb + np.array([0.2, -0.4, 0.0])
    pin = np.nonzero(np.isclose(xa[:, 0], 0.0))[0].astype(np.uint32)

    def at(x, p):
        return int(np.argmin(((x - np.asarray(p)) ** 2).sum(1)))

    dist = []
    for z in (0.0, 0.2):
        for xe in (0.4,):
            dist.append((0, 1, at(xa, (xe, 0.0, z)), at(xb, (0.4, -0.2, z))))
            dist.append((0, 1, at(xa, (xe - 0.2, 0.0, z)), at(xb, (0.2, -0.2, z))))
    for x0 in (0.0, 0.2):
        dist.append((0, 0, at(xa, (x0, 0.2, 0.0)), at(xa, (x0 + 0.2, 0.2, 0.2))))
        dist.append((0, 0, at(xa, (x0, 0.2, 0.2)), at(xa, (x0 + 0.2, 0.2, 0.0))))
    a = Body(x0=xa, tets=ta, model=MODEL_STVK, young=1e5, poisson=0.45, density=1000.0, pinned=pin)
    b = Body(x0=xb, tets=tb, model=MODEL_STVK, young=1e5, poisson=0.45, density=1000.0)
    return Scene("hanging-block-springs", [a, b], 1.0 / 60.0, 1, iterations, frames,
                 distance=np.array(dist, np.uint32), distance_compliance=alpha, distance_damping=beta,
                 ground=((0.0, 1.0, 0.0), 2.0))


def big_block(nx: int = 128, ny: int = 64, nz: int = 64, h: float = 0.02,
              frames: int = 200, substeps: int = 4, iterations: int = 30,
              drop: float = 0.5, lattice: bool = False) -> Scene:
    """Large SNH block (default 2,621,440 tets / 545,025 vertices), E 5e5,
    nu 0.48, dropped onto the ground from ``drop`` metres, with self contacts
    (vertex against the block's own surface triangles, spatial hash).
    lattice: carry the periodic 34-colouring (lattice_colours_5tet) as the
    body's colouring."""
    x0, tets = bar_5tet(nx + 1, ny + 1, nz + 1, h)
    x0 = x0 + np.array([0.0, drop, 0.0])
    b = Body(x0=x0, tets=tets, model=MODEL_SNH, young=5e5, poisson=0.48,
             density=1000.0, x_init=x0.copy(),
             colours=lattice_colours_5tet(nx + 1, ny + 1, nz + 1) if lattice else None)
    return Scene(f"block-{len(tets)}-snh", [b], 1.0 / 60.0, substeps,
                 iterations, frames, ground=((0.0, 1.0, 0.0), 0.0), body_contacts=2)


def body_force_field(x0: np.ndarray, seed: int, length: float,
                     amp_max: float = 50.0, max_cycles: float = 4.0):
    """Sum of three sinusoidal acceleration fields (N/kg) over the rest shape:
    sum_m A_m d_m sin(k_m . x + phi_m), A ~ U(0, amp_max), |k| up to
    max_cycles cycles per ``length``, d_m a random unit direction."""
    rng = np.random.default_rng(seed)
    acc = np.zeros_like(x0)
    for _ in range(3):
        a = rng.uniform(0.0, amp_max)
        kdir = rng.normal(size=3)
        kdir /= np.linalg.norm(kdir)
        kmag = rng.uniform(0.0, max_cycles) * 2 * math.pi / length
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        phi = rng.uniform(0, 2 * math.pi)
        acc += a * np.sin(x0 @ (kdir * kmag) + phi)[:, None] * d[None, :]
    return acc
