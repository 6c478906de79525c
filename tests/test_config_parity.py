"""FP64-oracle error of every benchmark configuration, one frame from the
configuration's initial state: the GPU (default mode, through the C ABI)
against the oracle replaying the GPU's sweep order, with the oracle's own
FP32 noise floor beside it.

The sequential Gauss-Seidel loop amplifies rounding differences by x3-30
per sweep, so no FP32 run can track the FP64 oracle to a fixed bound over
many frames; the yardstick is the spread between the oracle and the oracle
restarted from FP32-rounded initial positions (oracle.noise_floor, the
larger of two nudge seeds).  The GPU must stay within 2x of it.  Run with -s to see the per-configuration
errors (max vertex error / bounding-box diagonal).
"""
import os

import numpy as np
import pytest

from conftest import make_pair
from sbs_gb300 import scenes

pytestmark = pytest.mark.gpu

CONFIGS = {
    "beam-450-stvk": scenes.beam_c1,
    "beam-98304-snh-twist": scenes.beam_twist,
    "box-drop-512": scenes.box_drop,
    "block-2621440-snh": scenes.big_block,
}


@pytest.mark.parametrize("name", list(CONFIGS))
def test_config_one_frame_vs_oracle(capi_mod, oracle_mod, name):
    sc = CONFIGS[name]()
    threads = max(1, min(16, os.cpu_count() or 1))
    g, o = make_pair(sc, capi_mod, oracle_mod)
    order, off = g.tet_order()   # the oracle replays this order (make_pair)
    o.L.orc_set_threads(o.h, threads)
    g.step(1)
    o.step(1)
    x = g.positions()
    assert np.all(np.isfinite(x))
    diag = sc.bbox_diag()
    err = float(np.abs(x - o.get()).max())
    floor = oracle_mod.noise_floor(sc, 1, order, off, threads=threads, n_seeds=2)
    mode = ["auto", "graph", "persistent", "cluster", "wavefront"][g.stats().exec_mode]
    print(f"\n{name}: mode {mode}, GPU vs FP64 oracle {err / diag:.3e} x diag, "
          f"oracle FP32 noise floor {floor / diag:.3e} x diag, ratio {err / max(floor, 1e-30):.2f}")
    assert err < 2 * floor + 1e-6 * diag
