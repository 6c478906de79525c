"""Learned warm start: training data from the plain solver, GPU training,
and evaluation by Gauss-Seidel iterations to reach the plain residual.

Two workloads, both under seeded random body-force fields (three sinusoids,
amplitude U(0, 50) N/kg, wave vectors up to 4 cycles per beam length) and a
random pinned face, many trajectories running as independent bodies of one
solver handle:

* ``CANTILEVER``: the 450-tet beam (10x3x3 cubes of 0.1 m, 5 tets each,
  StVK E 1e5, nu 0.45, rho 1000), 1 substep of 1/60 s, 30 plain iterations;
* ``BEAM98K``: the 98,304-tet beam (64x16x16 cubes of 0.05 m, 6 tets each,
  stable Neo-Hookean E 1e6, nu 0.49, rho 1000), 4 substeps x 30 plain
  iterations per 1/60 s frame.

``TWIST98K`` is the 98,304-tet beam of the benchmark (x=0 face pinned, x=max
face turned about the beam's axis) with a per-trajectory turning rate
U(0.5, 1.5) rad/s and jitter seed, no body force: the trajectories a network
for that scene is trained on.  Its sweep order is the library's own greedy
colouring (28 colours): on the grid's lattice colouring (24 colours) the
solve displacement left after the previous substep's is harder to predict
per vertex (normalised training loss 0.51 against 0.30).  Trained networks are saved as .npz files
(parameters and the input/output normalisation, ``save_network``) and loaded
with ``load_network``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable

import numpy as np

from . import capi, scenes

FACES = ("x0", "x1", "y0", "y1", "z0", "z1")


def _trajectory_body(seed: int, x0, tets, model: int, young: float, poisson: float, length: float,
                     jitter: float):
    """A beam with its own force field and pinned face."""
    rng = np.random.default_rng(seed)
    face = FACES[rng.integers(0, 6)]
    ax = "xyz".index(face[0])
    val = x0[:, ax].min() if face[1] == "0" else x0[:, ax].max()
    pinned = np.nonzero(np.isclose(x0[:, ax], val))[0].astype(np.uint32)
    acc = scenes.body_force_field(x0, seed + 7919, length=length, amp_max=50.0, max_cycles=4.0)
    xi = scenes.jitter(x0, jitter, seed + 104729, pinned)
    return scenes.Body(x0=x0, tets=tets, model=model, young=young, poisson=poisson,
                       density=1000.0, x_init=xi, pinned=pinned, ext_acc=acc)


def beam_trajectory_body(seed: int):
    """One 450-tet cantilever trajectory."""
    x0, tets = scenes.bar_5tet(11, 4, 4, 0.1)
    return _trajectory_body(seed, x0, tets, scenes.MODEL_STVK, 1e5, 0.45, 1.0, 1e-3)


def beam98k_trajectory_body(seed: int):
    """One 98,304-tet beam trajectory."""
    x0, tets = scenes.bar_6tet(65, 17, 17, 0.05)
    return _trajectory_body(seed, x0, tets, scenes.MODEL_SNH, 1e6, 0.49, 3.2, 1e-4)


def twist98k_trajectory_body(seed: int):
    """One twisting-beam trajectory (the benchmark scene's body with its own
    turning rate and jitter)."""
    rng = np.random.default_rng(seed)
    omega = float(rng.uniform(0.5, 1.5))
    return scenes.beam_twist(seed=seed + 104729, omega=omega, lattice=False).bodies[0]


@dataclass(frozen=True)
class Workload:
    name: str
    make_body: Callable | None    # seed -> one trajectory body (None: make_scene)
    substeps: int
    iterations: int
    frame_dt: float = 1.0 / 60.0
    make_scene: Callable | None = None   # seed -> a whole scene (one trajectory)


def block_initial_state(x0: np.ndarray, seed: int):
    """One trajectory of the 2.6M-tet block: the rest shape turned by a
    random rotation of up to 0.3 rad about a random axis through its centre,
    its lowest point raised to U(0.1, 1.0) m above the ground, and a random
    initial velocity (horizontal U(-1, 1) m/s per axis, vertical U(-2, 0)).
    Returns (positions, velocities)."""
    rng = np.random.default_rng(seed)
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = rng.uniform(0.0, 0.3)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
    c = x0.mean(0)
    x = (x0 - c) @ R.T + c
    x[:, 1] += rng.uniform(0.1, 1.0) - x[:, 1].min()
    v = np.zeros_like(x)
    v[:] = [rng.uniform(-1, 1), rng.uniform(-2, 0), rng.uniform(-1, 1)]
    return x, v


def generate_resets(scene: scenes.Scene, make_state, seeds, frames: int, keep: float, seed: int = 0,
                    exec_mode: int = 0):
    """As generate, for one large body whose trajectories differ only in
    their initial state: one handle, the state replaced (set_state) at the
    start of each trajectory, so the scene is built and coloured once."""
    g = capi.Solver(scene, exec_mode=exec_mode)
    dt = scene.frame_dt / scene.substeps
    rng = np.random.default_rng(seed)
    x0 = scene.bodies[0].x0
    X, Y = [], []
    for s in seeds:
        x, v = make_state(x0, s)
        g.set_state(-1, x, v)
        for _ in range(frames):
            g.detect_contacts()
            for _ in range(scene.substeps):
                g.predict(dt)
                feat = g.features()
                xp = g.predicted_all()
                g.solve(dt, scene.iterations)
                y = g.predicted_all() - xp - feat[:, 3:6]
                sel = rng.random(len(feat)) < keep
                X.append(feat[sel].astype(np.float32))
                Y.append(y[sel].astype(np.float32))
                g.update_velocities(dt)
    g.close()
    return np.concatenate(X), np.concatenate(Y)


def block_judged(mlp, frames: int = 20, lead_frames: int = 5, check_every: int = 3, calibrate_every: int = 5,
                 exec_mode: int = 0):
    """The 2.6M-tet block as configured (dropped 0.5 m): plain frames and
    judged warm-started frames (as judged_rate) from the same start, timed."""
    sc = scenes.big_block()
    out = {}
    for judged in (False, True):
        g = capi.Solver(sc, exec_mode=exec_mode)
        g.step(lead_frames)
        if judged:
            g.set_warm_start(mlp, 0)
            g.set_warm_judge(check_every, 0, calibrate_every, 0.0)
        ms = [g.step_timed() for _ in range(frames)]
        out["judged" if judged else "plain"] = {"ms_per_frame": float(np.mean(ms)), "frame_ms": ms,
                                                "exec_mode": int(g.stats().exec_mode)}
        if judged:
            st = g.warm_stats()
            out["judged"].update({"warm_substeps": int(st.warm_substeps),
                                  "calibration_substeps": int(st.calibration_substeps),
                                  "mean_sweeps_per_warm_substep": st.sweeps / max(1, st.warm_substeps),
                                  "fallbacks": int(st.fallbacks), "capped": int(st.capped),
                                  "mean_residual_ratio": st.mean_residual_ratio,
                                  "max_residual_ratio": st.max_residual_ratio})
            g.set_warm_start(None)
        g.close()
    out["frames_per_s_ratio"] = out["plain"]["ms_per_frame"] / out["judged"]["ms_per_frame"]
    out["check_every"], out["calibrate_every"] = check_every, calibrate_every
    return out


def main_block(argv=None):
    """The 2.6M-tet block's learned warm start: trajectories of the block from
    random initial states (block_initial_state), a network trained on them,
    and judged frames of the configured drop against plain ones; one JSON
    line (python -m sbs_gb300.warmstart block ...)."""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--frames", type=int, default=10)
    ap.add_argument("--keep", type=float, default=1.0 / 32)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--judge-frames", type=int, default=20)
    ap.add_argument("--judge-check", type=int, default=3)
    ap.add_argument("--judge-calibrate", type=int, default=5)
    ap.add_argument("--save", default="")
    args = ap.parse_args(argv)
    sc = scenes.big_block()
    t0 = time.perf_counter()
    X, Y = generate_resets(sc, block_initial_state, list(range(5000, 5000 + args.train_seeds)), args.frames,
                           args.keep)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    m, losses = fit(X, Y, steps=args.steps, batch=args.batch, lr=1e-3, seed=1)
    t_fit = time.perf_counter() - t0
    if args.save:
        save_network(m, args.save, workload="block2m", train_trajectories=args.train_seeds, frames=args.frames,
                     keep=args.keep, steps=args.steps, loss_first=losses[0], loss_last=losses[-1])
    line = {"workload": "block2m", "train_trajectories": args.train_seeds, "frames": args.frames,
            "samples": int(len(X)), "generate_s": t_gen, "train_steps": args.steps, "train_s": t_fit,
            "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
            "judged": block_judged(m, frames=args.judge_frames, check_every=args.judge_check,
                                   calibrate_every=args.judge_calibrate)}
    print(json.dumps(line))


def _box_scene(seed: int) -> scenes.Scene:
    return scenes.box_drop(seed=seed)


CANTILEVER = Workload("beam450", beam_trajectory_body, 1, 30)
BEAM98K = Workload("beam98k", beam98k_trajectory_body, 4, 30)
TWIST98K = Workload("twist98k", twist98k_trajectory_body, 4, 30)
# the batch of 512 boxes (StVK, body-body contacts, 2 substeps x 20
# iterations); a trajectory is a whole scene of 512 bodies
BOXES512 = Workload("boxes512", None, 2, 20, make_scene=_box_scene)


def batch_scene(seeds, iterations: int | None = None, workload: Workload = CANTILEVER) -> scenes.Scene:
    it = workload.iterations if iterations is None else iterations
    if workload.make_scene is not None:
        if len(seeds) != 1:
            raise ValueError(f"{workload.name}: one scene per seed")
        import dataclasses
        sc = workload.make_scene(seeds[0])
        return dataclasses.replace(sc, iterations=it, substeps=workload.substeps, frame_dt=workload.frame_dt)
    return scenes.Scene(f"{workload.name}-batch", [workload.make_body(s) for s in seeds], workload.frame_dt,
                        workload.substeps, it, 60, ground=((0.0, 1.0, 0.0), 1.0))


def generate(seeds, frames: int = 60, iterations: int | None = None, exec_mode: int = 1,
             workload: Workload = CANTILEVER, keep: float = 1.0, seed: int = 0):
    """Runs the plain solver on the trajectories `seeds` and returns
    (features [N,16], targets [N,3]): per substep and vertex, the features at
    the predicted state and the part of the displacement the plain solve
    applied that the previous substep's displacement (features 3:6) does not
    already give.  keep < 1 keeps that random fraction of the vertices of
    each substep (bounds the data of large bodies)."""
    sc = batch_scene(seeds, iterations, workload)
    g = capi.Solver(sc, exec_mode=exec_mode)
    dt = sc.frame_dt / sc.substeps
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for f in range(frames):
        g.detect_contacts()
        for _ in range(sc.substeps):
            g.predict(dt)
            feat = g.features()
            xp = g.predicted_all()
            g.solve(dt, sc.iterations)
            y = g.predicted_all() - xp - feat[:, 3:6]
            if keep < 1.0:
                sel = rng.random(len(feat)) < keep
                feat, y = feat[sel], y[sel]
            X.append(feat.astype(np.float32))
            Y.append(y.astype(np.float32))
            g.update_velocities(dt)
    g.close()
    return np.concatenate(X), np.concatenate(Y)


def fit(X, Y, steps: int = 20000, batch: int = 65536, lr: float = 1e-3, seed: int = 0, device: int = 0,
        chunk: int = 1000):
    """Trains a fresh network with Adam on the GPU; returns (mlp, losses)."""
    m = capi.Mlp(device=device, seed=seed)
    mean = X.mean(0)
    std = X.std(0)
    std[std < 1e-8] = 1.0
    scale = Y.std(0) + 1e-12
    m.set_normalization(mean, std, scale)
    m.normalization = (mean.astype(np.float32), std.astype(np.float32), scale.astype(np.float32))
    m.set_dataset(X, Y)
    losses = []
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        losses.append(m.train(k, min(batch, len(X)), lr, seed=seed + done))
        done += k
    return m, losses


def save_network(m, path, **meta):
    """Parameters and normalisation of a trained network (fit) as .npz."""
    mean, std, scale = m.normalization
    np.savez(path, params=m.params(), mean=mean, std=std, scale=scale,
             **{k: np.asarray(v) for k, v in meta.items()})


def load_network(path, device: int = 0):
    """A network saved by save_network, on `device`."""
    d = np.load(path)
    m = capi.Mlp(device=device, seed=0)
    m.set_params(d["params"].astype(np.float32))
    m.set_normalization(d["mean"].astype(np.float32), d["std"].astype(np.float32), d["scale"].astype(np.float32))
    m.normalization = (d["mean"], d["std"], d["scale"])
    return m


def judged_rate(mlp, seeds, frames: int = 30, lead_frames: int = 5, check_every: int = 3,
                calibrate_every: int = 10, workload: Workload = CANTILEVER, exec_mode: int = 0):
    """Frames per second at equal residual with the plain solver as judge.
    Per held-out trajectory a plain handle and a judged warm-started handle
    (sbs_gpu_set_warm_judge: sweeps in chunks of `check_every` until the
    plain residual target, fallback to the plain start, a plain calibration
    frame every `calibrate_every` frames) advance `lead_frames` plain frames,
    then step `frames` timed frames each (the judged handle's calibration
    frames included).  Returns mean device times per frame, their ratio and
    the judge's totals."""
    plain_ms, warm_ms = [], []
    tot = {"warm_substeps": 0, "calibration_substeps": 0, "sweeps": 0, "fallbacks": 0, "capped": 0}
    ratio_sum, ratio_max = 0.0, 0.0
    for s in seeds:
        sc = batch_scene([s], None, workload)
        a = capi.Solver(sc, exec_mode=exec_mode)
        a.step(lead_frames)
        plain_ms += [a.step_timed() for _ in range(frames)]
        a.close()
        b = capi.Solver(sc, exec_mode=exec_mode)
        b.step(lead_frames)
        b.set_warm_start(mlp, 0)
        b.set_warm_judge(check_every, 0, calibrate_every, 0.0)
        warm_ms += [b.step_timed() for _ in range(frames)]
        st = b.warm_stats()
        for k in tot:
            tot[k] += int(getattr(st, k))
        ratio_sum += st.mean_residual_ratio * st.warm_substeps
        ratio_max = max(ratio_max, st.max_residual_ratio)
        b.set_warm_start(None)
        b.close()
    pm, wm = float(np.mean(plain_ms)), float(np.mean(warm_ms))
    return {"plain_ms_per_frame": pm, "judged_ms_per_frame": wm, "frames_per_s_ratio": pm / wm,
            "frames": len(warm_ms), "check_every": check_every, "calibrate_every": calibrate_every,
            "mean_sweeps_per_warm_substep": tot["sweeps"] / max(1, tot["warm_substeps"]),
            "plain_sweeps": sc.iterations,
            "mean_residual_ratio": ratio_sum / max(1, tot["warm_substeps"]), "max_residual_ratio": ratio_max,
            **tot}


def residual_after(g, dt):
    return g.residual(dt)[0]


def _plain_frame(g, sc):
    """One frame of the plain solver that also records the predictions, so
    every substep knows its previous solve displacement."""
    dt = sc.frame_dt / sc.substeps
    g.detect_contacts()
    for _ in range(sc.substeps):
        g.predict(dt)
        g.features()
        g.solve(dt, sc.iterations)
        g.update_velocities(dt)


def evaluate(mlp, seeds, frame: int = 20, iterations: int | None = None, max_iters: int = 60,
             exec_mode: int = 1, fit_sweeps: int = 1, workload: Workload = CANTILEVER):
    """For each held-out trajectory, two handles advance `frame` plain frames
    in lockstep (identical states); then, on the first substep of the next
    frame, one runs plain sweeps (residual r_plain[k] after k sweeps) and the
    other the warm start (fit sweeps, then sweeps continuing from the fitted
    multipliers; fit_sweeps = 0: the carry start).  The warm start is
    discarded, and the plain start used, when its residual after the fit
    exceeds the plain start's after as many sweeps (r_plain[0]: at the
    prediction, with zero multipliers); otherwise `iterations` is the number
    of sweeps (fit sweeps included) it needs to reach r_plain[iterations].
    Returns a list of dicts."""
    out = []
    for s in seeds:
        sc = batch_scene([s], iterations, workload)
        it = sc.iterations
        a = capi.Solver(sc, exec_mode=exec_mode)
        b = capi.Solver(sc, exec_mode=exec_mode)
        dt = sc.frame_dt / sc.substeps
        for _ in range(frame):
            _plain_frame(a, sc)
            _plain_frame(b, sc)
        same = bool(np.array_equal(a.get_state(0)[0], b.get_state(0)[0]))
        a.detect_contacts()
        a.predict(dt)
        a.features()
        r_plain = [residual_after(a, dt)]
        for k in range(1, it + 1):
            a.solve_ex(dt, 1, k == 1)
            r_plain.append(residual_after(a, dt))
        target = r_plain[it]
        b.detect_contacts()
        b.predict(dt)
        b.set_warm_start(mlp, fit_sweeps)
        b.warm_start_init(dt)
        r_fit = residual_after(b, dt)
        used, fallback, r_end = it, True, target
        if r_fit <= r_plain[min(fit_sweeps, it)]:
            k, r = fit_sweeps, r_fit
            while r > target and k < max_iters:
                b.solve_ex(dt, 1, False)
                k += 1
                r = residual_after(b, dt)
            if r <= target and k <= it:
                used, fallback, r_end = k, False, r
        b.set_warm_start(None)
        out.append({"seed": int(s), "same_start": same, "r_plain": float(target), "r_plain_1": float(r_plain[1]),
                    "r_fit": float(r_fit), "iterations": int(used), "fallback": bool(fallback),
                    "r_end": float(r_end)})
        a.close()
        b.close()
    return out


def frame_rate(mlp, seeds, k_list, frames: int = 30, lead_frames: int = 20, fit_sweeps: int = 0,
               workload: Workload = CANTILEVER):
    """Frames per second against residual: per held-out trajectory a plain
    handle (default execution mode, the workload's iterations) and, for each
    k in `k_list`, a warm-started one (default mode too, k iterations per
    substep, its frames captured as CUDA graphs) advance `lead_frames` plain frames; a warm
    handle then runs one untimed warm-started frame (so every substep knows
    its predecessor's displacement), and each handle steps `frames` timed
    frames.  The trajectories part ways, so the comparison is statistical:
    median device time per frame and median residual after a frame, over all
    frames and trajectories."""
    plain_ms, plain_r = [], []
    warm_ms = {k: [] for k in k_list}
    warm_r = {k: [] for k in k_list}
    for s in seeds:
        sc = batch_scene([s], None, workload)
        dt = sc.frame_dt / sc.substeps
        a = capi.Solver(sc)
        a.step(lead_frames + 1)
        for _ in range(frames):
            plain_ms.append(a.step_timed())
            plain_r.append(a.residual(dt)[0])
        a.close()
        for k in k_list:
            b = capi.Solver(sc)
            b.step(lead_frames)
            b.set_warm_start(mlp, fit_sweeps)
            b.step(1, iterations=k)
            for _ in range(frames):
                warm_ms[k].append(b.step_timed(iterations=k))
                warm_r[k].append(b.residual(dt)[0])
            b.set_warm_start(None)
            b.close()
    pm, pr = float(np.median(plain_ms)), float(np.median(plain_r))
    out = {"plain_iterations": sc.iterations, "frames": len(plain_ms), "plain_ms_per_frame": pm,
           "plain_residual_median": pr, "warm": {}}
    for k in k_list:
        wm, wr = float(np.median(warm_ms[k])), float(np.median(warm_r[k]))
        out["warm"][str(k)] = {"ms_per_frame": wm, "residual_median": wr, "frames_per_s_ratio": pm / wm,
                               "residual_ratio": wr / pr}
    return out


def main(argv=None):
    """Generate, train and evaluate one warm-start experiment; prints one
    JSON line (python -m sbs_gb300.warmstart --workload beam98k ...)."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="beam450", choices=["beam450", "beam98k", "twist98k", "boxes512"])
    ap.add_argument("--train-seeds", type=int, default=256, help="training trajectories")
    ap.add_argument("--bodies-per-handle", type=int, default=64, help="trajectories run as one handle's bodies")
    ap.add_argument("--frames", type=int, default=60)
    ap.add_argument("--keep", type=float, default=1.0, help="fraction of vertices kept per substep")
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--eval-seeds", type=int, default=40)
    ap.add_argument("--eval-frame", type=int, default=20)
    ap.add_argument("--fit-sweeps", default="0,2,3", help="0: carry the previous multipliers")
    ap.add_argument("--rate-k", default="",
                    help="comma list: also time frames with these warm-started iterations per substep")
    ap.add_argument("--rate-seeds", type=int, default=4)
    ap.add_argument("--rate-frames", type=int, default=30)
    ap.add_argument("--judge-seeds", type=int, default=0,
                    help="also time judged warm-started frames against plain ones on this many trajectories")
    ap.add_argument("--judge-check", type=int, default=3, help="sweeps between the judge's residual checks")
    ap.add_argument("--judge-calibrate", type=int, default=10, help="a plain calibration frame every N frames")
    ap.add_argument("--save", default="", help="write the trained network to this .npz file")
    args = ap.parse_args(argv)
    wl = {"beam450": CANTILEVER, "beam98k": BEAM98K, "twist98k": TWIST98K, "boxes512": BOXES512}[args.workload]
    if wl.make_scene is not None:
        args.bodies_per_handle = 1
    t0 = time.perf_counter()
    Xs, Ys = [], []
    seeds = list(range(1000, 1000 + args.train_seeds))
    for i in range(0, len(seeds), args.bodies_per_handle):
        X, Y = generate(seeds[i:i + args.bodies_per_handle], frames=args.frames, workload=wl, keep=args.keep,
                        seed=i)
        Xs.append(X)
        Ys.append(Y)
    X, Y = np.concatenate(Xs), np.concatenate(Ys)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    m, losses = fit(X, Y, steps=args.steps, batch=args.batch, lr=1e-3, seed=1)
    t_fit = time.perf_counter() - t0
    line = {"workload": wl.name, "substeps": wl.substeps, "plain_iterations": wl.iterations,
            "train_trajectories": args.train_seeds, "frames": args.frames, "samples": int(len(X)),
            "generate_s": t_gen, "train_steps": args.steps, "train_s": t_fit,
            "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "eval": {}}
    eval_seeds = list(range(50000, 50000 + args.eval_seeds))
    for fs in [int(v) for v in args.fit_sweeps.split(",")]:
        res = evaluate(m, eval_seeds, frame=args.eval_frame, fit_sweeps=fs, workload=wl)
        its = np.array([r["iterations"] for r in res])
        line["eval"][f"fit_{fs}"] = {"mean_iterations": float(its.mean()),
                                     "fallbacks": int(sum(r["fallback"] for r in res)),
                                     "same_start": all(r["same_start"] for r in res),
                                     "sweep_fraction": float(its.mean() / wl.iterations)}
    if args.save:
        save_network(m, args.save, workload=wl.name, train_trajectories=args.train_seeds, frames=args.frames,
                     keep=args.keep, steps=args.steps, loss_first=losses[0], loss_last=losses[-1])
    if args.judge_seeds:
        line["judged"] = judged_rate(m, list(range(60000, 60000 + args.judge_seeds)), frames=args.rate_frames,
                                     lead_frames=args.eval_frame, check_every=args.judge_check,
                                     calibrate_every=args.judge_calibrate, workload=wl)
    if args.rate_k:
        line["frame_rate"] = frame_rate(m, list(range(60000, 60000 + args.rate_seeds)),
                                        [int(v) for v in args.rate_k.split(",")], frames=args.rate_frames,
                                        lead_frames=args.eval_frame, workload=wl)
    # the previous-displacement guess alone (network output zero)
    m.set_params(np.zeros(m.n_params, np.float32))
    for fs in [int(v) for v in args.fit_sweeps.split(",")]:
        res = evaluate(m, eval_seeds, frame=args.eval_frame, fit_sweeps=fs, workload=wl)
        line["eval"][f"prev_displacement_only_fit_{fs}"] = {
            "mean_iterations": float(np.mean([r["iterations"] for r in res])),
            "fallbacks": int(sum(r["fallback"] for r in res))}
    print(json.dumps(line))


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "block":
        main_block(sys.argv[2:])
    else:
        main()
