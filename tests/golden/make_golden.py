"""Generates tests/golden/ref_meshes.npz from the reference's PLY meshes.

Reads the ascii tetrahedral meshes of Q-Minh/soft-body-simulator
(data/meshes/{tetrahedron,2tets,3tets,cube_tet,tet_bar_5x2x2,bar_tet}.ply, the
only fixtures the reference ships; element `tet` with `property list uchar int
indices`, parsed as src/io/ply.cpp:616-640 does) and stores, per mesh:
  <name>_x0     rest positions (float64)
  <name>_tets   tets (uint32)
  <name>_order  the Gauss-Seidel sweep order used (tet ids, colour-major, from
                the library's host planner when the file was made),
  <name>_offsets its colour offsets,
  <name>_x1     FP64 oracle positions after one frame of the golden scenario
                in that order, and
  <name>_x10    after ten frames;
and the reference's floor triangle mesh (data/meshes/xz_plane.ply, the
environment of data/scenes/scene1.json) as xz_plane_verts / xz_plane_tris.
Golden scenario: positions scaled by 0.1, vertices with minimal x pinned,
StVK E 1e5 / nu 0.3 / rho 1000, compliance 1e-4, gravity -9.81 (acceleration),
ground plane y = -0.05, dt 1/60, 1 substep, 10 iterations.

Usage: python tests/golden/make_golden.py /path/to/reference/data/meshes
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "soft-body-simulator_gb300"))
sys.path.insert(0, str(ROOT))

NAMES = ["tetrahedron", "2tets", "3tets", "cube_tet", "tet_bar_5x2x2", "bar_tet"]


def read_ply_tets(path: Path):
    lines = path.read_text().splitlines()
    nv = nt = 0
    i = 0
    while lines[i].strip() != "end_header":
        tok = lines[i].split()
        if tok[:2] == ["element", "vertex"]:
            nv = int(tok[2])
        if tok[:2] == ["element", "tet"]:
            nt = int(tok[2])
        i += 1
    i += 1
    x = np.array([[float(t) for t in lines[i + k].split()[:3]] for k in range(nv)])
    i += nv
    tets = []
    for k in range(nt):
        tok = [int(t) for t in lines[i + k].split()]
        assert tok[0] == 4
        tets.append(tok[1:5])
    return x, np.array(tets, np.uint32)


def read_ply_faces(path: Path):
    """Vertices and triangle faces of an ascii PLY (element face, list uchar int)."""
    lines = path.read_text().splitlines()
    nv = nf = 0
    i = 0
    while lines[i].strip() != "end_header":
        tok = lines[i].split()
        if tok[:2] == ["element", "vertex"]:
            nv = int(tok[2])
        if tok[:2] == ["element", "face"]:
            nf = int(tok[2])
        i += 1
    i += 1
    x = np.array([[float(t) for t in lines[i + k].split()[:3]] for k in range(nv)])
    i += nv
    f = []
    for k in range(nf):
        tok = [int(t) for t in lines[i + k].split()]
        assert tok[0] == 3
        f.append(tok[1:4])
    return x, np.array(f, np.uint32)


def golden_scene(x0, tets):
    from sbs_gb300 import scenes
    x0 = x0 * 0.1
    pinned = np.nonzero(np.isclose(x0[:, 0], x0[:, 0].min()))[0].astype(np.uint32)
    b = scenes.Body(x0=x0, tets=tets, model=scenes.MODEL_STVK, young=1e5, poisson=0.3,
                    density=1000.0, x_init=x0.copy(), pinned=pinned)
    return scenes.Scene("golden", [b], 1.0 / 60.0, 1, 10, 10,
                        ground=((0.0, 1.0, 0.0), 0.05))


def main(meshdir: Path):
    from oracle import oracle
    from sbs_gb300 import capi
    out = {}
    for name in NAMES:
        x0, tets = read_ply_tets(meshdir / f"{name}.ply")
        sc = golden_scene(x0, tets)
        order, off = capi.plan_sweep(sc)
        o = oracle.Oracle(sc)
        o.set_order(order, off)
        o.step(1)
        x1 = o.get().copy()
        o.step(9)
        out[f"{name}_x0"] = x0
        out[f"{name}_tets"] = tets
        out[f"{name}_order"] = np.asarray(order, np.uint32)
        out[f"{name}_offsets"] = np.asarray(off, np.uint32)
        out[f"{name}_x1"] = x1
        out[f"{name}_x10"] = o.get().copy()
    fx, ff = read_ply_faces(meshdir / "xz_plane.ply")
    out["xz_plane_verts"] = fx
    out["xz_plane_tris"] = ff
    np.savez_compressed(HERE / "ref_meshes.npz", **out)
    print("wrote", HERE / "ref_meshes.npz")


if __name__ == "__main__":
    main(Path(sys.argv[1]))
