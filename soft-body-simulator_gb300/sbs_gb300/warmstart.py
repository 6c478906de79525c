"""Learned warm start: training data from the plain solver, GPU training,
and evaluation by Gauss-Seidel iterations to reach the plain residual.

The workload is the 450-tet cantilever (10x3x3 cubes of 0.1 m, StVK E 1e5,
nu 0.45, rho 1000), 1 substep of 1/60 s, 30 plain iterations, under seeded
random body-force fields (three sinusoids, amplitude U(0, 50) N/kg, wave
vectors up to 4 cycles per beam length) and a random pinned face.  Many
trajectories run as independent bodies of one solver handle.
"""
from __future__ import annotations

import math

import numpy as np

from . import capi, scenes

FACES = ("x0", "x1", "y0", "y1", "z0", "z1")


def beam_trajectory_body(seed: int):
    """One C1 beam with its own force field and pinned face."""
    x0, tets = scenes.bar_5tet(11, 4, 4, 0.1)
    rng = np.random.default_rng(seed)
    face = FACES[rng.integers(0, 6)]
    ax = "xyz".index(face[0])
    val = x0[:, ax].min() if face[1] == "0" else x0[:, ax].max()
    pinned = np.nonzero(np.isclose(x0[:, ax], val))[0].astype(np.uint32)
    acc = scenes.body_force_field(x0, seed + 7919, length=1.0, amp_max=50.0, max_cycles=4.0)
    xi = scenes.jitter(x0, 1e-3, seed + 104729, pinned)
    return scenes.Body(x0=x0, tets=tets, model=scenes.MODEL_STVK, young=1e5, poisson=0.45,
                       density=1000.0, x_init=xi, pinned=pinned, ext_acc=acc)


def batch_scene(seeds, iterations: int = 30) -> scenes.Scene:
    return scenes.Scene("beam450-batch", [beam_trajectory_body(s) for s in seeds], 1.0 / 60.0, 1,
                        iterations, 60, ground=((0.0, 1.0, 0.0), 1.0))


def generate(seeds, frames: int = 60, iterations: int = 30, exec_mode: int = 1):
    """Runs the plain solver on the trajectories `seeds` and returns
    (features [N,16], targets [N,3]): per substep and vertex, the features at
    the predicted state and the part of the displacement the 30-iteration
    solve applied that the previous substep's displacement (features 3:6)
    does not already give."""
    sc = batch_scene(seeds, iterations)
    g = capi.Solver(sc, exec_mode=exec_mode)
    dt = sc.frame_dt
    X, Y = [], []
    for f in range(frames):
        g.detect_contacts()
        g.predict(dt)
        feat = g.features()
        xp = g.predicted_all()
        g.solve(dt, iterations)
        X.append(feat)
        Y.append(g.predicted_all() - xp - feat[:, 3:6])
        g.update_velocities(dt)
    g.close()
    return np.concatenate(X).astype(np.float32), np.concatenate(Y).astype(np.float32)


def fit(X, Y, steps: int = 20000, batch: int = 65536, lr: float = 1e-3, seed: int = 0, device: int = 0,
        chunk: int = 1000):
    """Trains a fresh network with Adam on the GPU; returns (mlp, losses)."""
    m = capi.Mlp(device=device, seed=seed)
    mean = X.mean(0)
    std = X.std(0)
    std[std < 1e-8] = 1.0
    scale = Y.std(0) + 1e-12
    m.set_normalization(mean, std, scale)
    m.set_dataset(X, Y)
    losses = []
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        losses.append(m.train(k, min(batch, len(X)), lr, seed=seed + done))
        done += k
    return m, losses


def residual_after(g, dt):
    return g.residual(dt)[0]


def _plain_frame(g, dt, iterations):
    """One frame of the plain solver that also records the prediction, so
    the next substep knows its previous solve displacement."""
    g.detect_contacts()
    g.predict(dt)
    g.features()
    g.solve(dt, iterations)
    g.update_velocities(dt)


def evaluate(mlp, seeds, frame: int = 20, iterations: int = 30, max_iters: int = 60, exec_mode: int = 1,
             fit_sweeps: int = 1):
    """For each held-out trajectory, two handles advance `frame` plain frames
    in lockstep (identical states); then one runs plain sweeps (residual
    r_plain[k] after k sweeps) and the other the warm start (fit sweeps, then
    sweeps continuing from the fitted multipliers).  The warm start is
    discarded, and the plain start used, when its residual after the fit
    exceeds r_plain[1]; otherwise `iterations` is the number of sweeps (fit
    sweeps included) it needs to reach r_plain[iterations].  Returns a list of
    dicts."""
    out = []
    for s in seeds:
        sc = batch_scene([s], iterations)
        a = capi.Solver(sc, exec_mode=exec_mode)
        b = capi.Solver(sc, exec_mode=exec_mode)
        dt = sc.frame_dt
        for _ in range(frame):
            _plain_frame(a, dt, iterations)
            _plain_frame(b, dt, iterations)
        same = bool(np.array_equal(a.get_state(0)[0], b.get_state(0)[0]))
        a.detect_contacts()
        a.predict(dt)
        a.features()
        r_plain = [None]
        for k in range(1, iterations + 1):
            a.solve_ex(dt, 1, k == 1)
            r_plain.append(residual_after(a, dt))
        target = r_plain[iterations]
        b.detect_contacts()
        b.predict(dt)
        b.set_warm_start(mlp, fit_sweeps)
        b.warm_start_init(dt)
        r_fit = residual_after(b, dt)
        used, fallback, r_end = iterations, True, target
        if r_fit <= r_plain[1]:
            k, r = fit_sweeps, r_fit
            while r > target and k < max_iters:
                b.solve_ex(dt, 1, False)
                k += 1
                r = residual_after(b, dt)
            if r <= target and k <= iterations:
                used, fallback, r_end = k, False, r
        b.set_warm_start(None)
        out.append({"seed": int(s), "same_start": same, "r_plain": float(target), "r_plain_1": float(r_plain[1]),
                    "r_fit": float(r_fit), "iterations": int(used), "fallback": bool(fallback),
                    "r_end": float(r_end)})
        a.close()
        b.close()
    return out
