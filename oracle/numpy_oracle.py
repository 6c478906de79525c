"""Independent numpy restatement of the reference's XPBD step (small cases).

TEST INFRASTRUCTURE ONLY.  It exists to cross-check the C++ oracle: it is
written separately, loops over constraints in pure Python and uses LAPACK's
SVD (numpy.linalg.svd, singular values >= 0 in decreasing order, the same
convention as Eigen's JacobiSVD) instead of the oracle's Jacobi SVD.

Restated from (Q-Minh/soft-body-simulator):
  timestep_t::step               src/physics/timestep.cpp:20-70
  gauss_seidel_solver_t::solve   src/physics/gauss_seidel_solver.cpp:8-37
  green_constraint_t             src/physics/xpbd/green_constraint.cpp:11-173
  collision_constraint_t         src/physics/xpbd/collision_constraint.cpp:21-48
  plane contact rule             src/physics/collision/bvh_model.cpp:72-94
"""
from __future__ import annotations

import numpy as np


def _stvk_eval(xs, DmInv, V0, mu, lam):
    x1, x2, x3, x4 = xs
    Vs = np.linalg.det(np.stack([x1 - x4, x2 - x4, x3 - x4], 1)) / 6.0
    inverted = (Vs >= 0.0) != (V0 >= 0.0)
    F = np.stack([x1 - x4, x2 - x4, x3 - x4], 1) @ DmInv
    U, s, Vt = np.linalg.svd(F)
    U = U.copy()
    s = s.copy()
    if inverted:
        s[2] = -s[2]
        U[:, 2] = -U[:, 2]
    s = np.maximum(s, 0.577)
    Ehat = np.diag(0.5 * (s * s - 1.0))
    Phat = np.diag(s) @ (2.0 * mu * Ehat + lam * np.trace(Ehat) * np.eye(3))
    E = U @ Ehat @ Vt
    psi = mu * np.sum(E * E) + 0.5 * lam * np.trace(E) ** 2
    P = U @ Phat @ Vt
    H = -abs(V0) * P @ DmInv.T
    f = [H[:, 0], H[:, 1], H[:, 2]]
    f.append(-(f[0] + f[1] + f[2]))
    return psi, f


class NumpyXPBD:
    """StVK-only restatement with plane contacts, gravity in either mode."""

    def __init__(self, scene):
        assert len(scene.bodies) == 1
        b = scene.bodies[0]
        self.s = scene
        self.x0 = b.x0.astype(np.float64)
        x = (b.x_init if b.x_init is not None else b.x0).astype(np.float64)
        self.x = x.copy()
        self.xn = x.copy()
        self.xi = x.copy()
        self.v = np.zeros_like(x)
        self.tets = b.tets.astype(np.int64)
        vol = []
        self.DmInv = []
        for t in self.tets:
            Dm = np.stack([self.x0[t[0]] - self.x0[t[3]], self.x0[t[1]] - self.x0[t[3]],
                           self.x0[t[2]] - self.x0[t[3]]], 1)
            self.DmInv.append(np.linalg.inv(Dm))
            vol.append(np.linalg.det(Dm) / 6.0)
        self.V0 = np.array(vol)
        self.m = np.zeros(len(x))
        for t, v in zip(self.tets, self.V0):
            for k in range(4):
                self.m[t[k]] += b.density * abs(v) / 4.0
        self.m[np.asarray(b.pinned, np.int64)] = 0.0
        self.w = np.where(self.m > 0, 1.0 / np.where(self.m > 0, self.m, 1.0), 0.0)
        self.mu = b.young / (2.0 * (1.0 + b.poisson))
        self.lam = b.young * b.poisson / ((1.0 + b.poisson) * (1.0 - 2.0 * b.poisson))
        self.order = np.arange(len(self.tets))
        # boundary vertices: faces with != 2 incident tets
        from collections import Counter
        faces = Counter()
        for t in self.tets:
            for f in ((t[0], t[1], t[3]), (t[1], t[2], t[3]), (t[2], t[0], t[3]),
                      (t[0], t[2], t[1])):
                faces[tuple(sorted(f))] += 1
        self.surface = sorted({v for f, c in faces.items() if c != 2 for v in f})

    def step(self):
        s = self.s
        dt = s.frame_dt / s.substeps
        at_c = s.collision_compliance / dt ** 2
        contacts = []
        if s.ground is not None:
            n = np.asarray(s.ground[0], float)
            ln = np.linalg.norm(n)
            n, d = n / ln, s.ground[1] / ln
            for vi in self.surface:
                sd = n @ self.x[vi] + d
                if sd < 0:
                    contacts.append([vi, self.x[vi] + abs(sd) * n, n, 0.0])
        g = np.asarray(s.gravity, float)
        for _ in range(s.substeps):
            f = g[None, :] if s.gravity_mode == 1 else g[None, :] * self.m[:, None]
            self.v = self.v + f * self.w[:, None] * dt
            self.xi = self.x + self.v * dt
            lagr = np.zeros(len(self.tets))
            for c in contacts:
                c[3] = 0.0
            at = s.compliance / dt ** 2
            bt = s.damping * dt ** 2
            gamma = at * bt / dt
            for _ in range(s.iterations):
                for c in contacts:
                    vi, q, n, l = c
                    C = (self.xi[vi] - q) @ n
                    if C >= 0:
                        continue
                    dl = -(C + at_c * l) / (self.w[vi] + at_c)
                    c[3] = l + dl
                    self.xi[vi] = self.xi[vi] + self.w[vi] * n * dl
                for k in self.order:
                    t = self.tets[k]
                    psi, fs = _stvk_eval([self.xi[t[i]] for i in range(4)], self.DmInv[k],
                                         self.V0[k], self.mu, self.lam)
                    S = sum(self.w[t[i]] * fs[i] @ fs[i] for i in range(4))
                    if S < 1e-20:
                        continue
                    C = abs(self.V0[k]) * psi
                    gd = sum(fs[i] @ (self.xi[t[i]] - self.xn[t[i]]) for i in range(4))
                    dl = (-(C + at * lagr[k]) + gamma * gd) / ((1 + gamma) * S + at)
                    lagr[k] += dl
                    for i in range(4):
                        self.xi[t[i]] = self.xi[t[i]] - self.w[t[i]] * fs[i] * dl
            self.x = self.xi.copy()
            self.v = (self.x - self.xn) / dt
            self.xn = self.x.copy()
        self.lagrange = lagr
