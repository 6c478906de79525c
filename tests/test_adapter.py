"""The header-only C++ drop-in (include/sbs_gpu_timestep.hpp): it compiles
against the C ABI (CPU), and on a GPU its frames equal the Python binding's
frames on the same scene, with the oracle's sweep as the yardstick."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "adapter_demo.cpp"


def build_demo(tmp_path):
    from sbs_gb300 import build
    lib = build.build()
    exe = tmp_path / "adapter_demo"
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(SRC),
                    "-L", str(lib.parent), "-lsbs_gpu", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)],
                   check=True)
    return exe


def test_adapter_compiles(tmp_path):
    assert build_demo(tmp_path).exists()


def demo_scene():
    from sbs_gb300 import scenes
    x0 = scenes.bar_vertices(4, 2, 2, 0.1)
    _, tets = scenes.bar_5tet(4, 2, 2, 0.1)
    mass = np.where(np.isclose(x0[:, 0], 0.0), 0.0, 0.25)
    b = scenes.Body(x0=x0, tets=tets, model=scenes.MODEL_STVK, young=1e5, poisson=0.3,
                    density=1000.0, x_init=x0.copy(), mass=mass)
    return scenes.Scene("adapter-demo", [b], 1.0 / 60.0, 1, 10, 30, ground=((0.0, 1.0, 0.0), 1.0))


@pytest.mark.gpu
def test_adapter_matches_binding(tmp_path, capi_mod):
    exe = build_demo(tmp_path)
    out = subprocess.run([str(exe), "30"], capture_output=True, text=True, check=True).stdout
    x_demo = np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])
    sc = demo_scene()
    g = capi_mod.Solver(sc)
    for _ in range(30):
        x, v = g.get_state(0)
        g.set_state(0, x, v)
        g.step(1)
    x_py = g.positions()
    assert x_demo.shape == x_py.shape
    assert np.all(np.isfinite(x_demo))
    assert np.abs(x_demo - x_py).max() < 1e-6
    pinned = np.isclose(sc.bodies[0].x0[:, 0], 0.0)
    assert np.array_equal(x_demo[pinned].astype(np.float32), sc.bodies[0].x0[pinned].astype(np.float32))
