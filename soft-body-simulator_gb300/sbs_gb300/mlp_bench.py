"""Throughput of the warm-start network's forward pass on the GPU.

    python -m sbs_gb300.mlp_bench [--rows 545025] [--reps 20]

Times both implementations on device-resident rows (CUDA events on the
network's stream, after warm-up): the fused tcgen05 kernel (path 0) and the
per-layer mma.sync GEMMs (path 1).  Prints one JSON line with ms per call,
rows/s and TFLOP/s (70,400 FLOP per row).
"""
from __future__ import annotations

import argparse
import json

import numpy as np

FLOP_PER_ROW = 2 * (16 * 128 + 2 * 128 * 128 + 128 * 3)


def main():
    import torch
    from . import capi
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=545025)   # vertices of the 2.6M-tet block
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args()
    m = capi.Mlp(device=0, seed=1)
    rng = np.random.default_rng(0)
    x = torch.from_numpy(rng.normal(size=(args.rows, 16)).astype(np.float32)).cuda()
    y = torch.empty((args.rows, 3), dtype=torch.float32, device="cuda")
    out = {"rows": args.rows, "flop_per_row": FLOP_PER_ROW}
    for path, name in ((0, "tcgen05_fused"), (1, "mma_sync_layers")):
        for _ in range(3):
            m.forward_device(x.data_ptr(), args.rows, y.data_ptr(), path)
        ms = sorted(m.forward_device(x.data_ptr(), args.rows, y.data_ptr(), path) for _ in range(args.reps))
        med = ms[len(ms) // 2]
        out[name] = {"ms": med, "rows_per_s": args.rows / (med * 1e-3),
                     "tflops": args.rows * FLOP_PER_ROW / (med * 1e-3) / 1e12}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
