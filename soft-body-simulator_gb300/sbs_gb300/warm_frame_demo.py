"""Steps warm-started frames of the 98,304-tet beam (carry start, cluster
mode, 12 sweeps per substep) with an untrained network, the kernel mix of a
warm-started frame being independent of the weights; prints the device time
of each timed frame.  Used to list a warm-started frame's kernel launches
(python -m sbs_gb300.warm_frame_demo [frames])."""
import sys

import numpy as np

from . import capi, warmstart


def main(frames: int = 3):
    sc = warmstart.batch_scene([60000], None, warmstart.BEAM98K)
    g = capi.Solver(sc, exec_mode=capi.EXEC_CLUSTER)   # fixed: a profiler distorts the autotuner's timings
    g.step(2)                                   # plain frames
    m = capi.Mlp(device=0, seed=1)
    m.set_normalization(np.zeros(16, np.float32), np.ones(16, np.float32), np.full(3, 1e-4, np.float32))
    g.set_warm_start(m, 0)
    g.step(2, iterations=12)                    # warm-started frames (and their graph capture)
    for _ in range(frames):
        print(f"warm-started frame: {g.step_timed(iterations=12):.3f} ms")
    g.set_warm_start(None)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 3)
