import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT / "soft-body-simulator_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libsbs_gpu.so kernels)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def capi_mod():
    from sbs_gb300 import capi
    capi.load()
    return capi


def make_pair(scene, capi, oracle, **kw):
    """GPU solver and FP64 oracle running the same sweep order."""
    g = capi.Solver(scene, **kw)
    order, off = g.tet_order()
    o = oracle.Oracle(scene)
    o.set_order(order, off)
    if getattr(scene, "distance", None) is not None and len(scene.distance):
        eo, eoff = g.distance_order()
        o.set_edge_order(eo, eoff)
    return g, o
