"""The warm-start evaluation protocol on a simulated solver (CPU): sweeps are
counted to the plain solver's residual after `iterations` sweeps, fit sweeps
included, and a start whose residual exceeds the plain start's after as many
sweeps is discarded (counted as `iterations`)."""
import math

import pytest

from sbs_gb300 import warmstart


class FakeScene:
    frame_dt = 1.0 / 60.0
    substeps = 1
    iterations = 30


class FakeSolver:
    """Residual r0 * rate^k after k sweeps; the warm start begins at r_warm
    after its fit sweeps and then converges at the same rate."""
    r_plain0 = 2.0
    r_warm = 0.5
    rate = 0.8

    def __init__(self, sc, exec_mode=1):
        self.r = self.r_plain0
        self.warm = None

    def detect_contacts(self):
        pass

    def predict(self, dt):
        self.r = self.r_plain0

    def features(self):
        return None

    def solve(self, dt, iterations):
        pass

    def update_velocities(self, dt):
        pass

    def get_state(self, body):
        return ([0.0], [0.0])

    def solve_ex(self, dt, k, reset):
        self.r *= self.rate ** k

    def residual(self, dt):
        return self.r, 0.0

    def set_warm_start(self, mlp, fit_sweeps=1):
        self.warm = fit_sweeps

    def warm_start_init(self, dt):
        self.r = self.r_warm

    def close(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(warmstart.capi, "Solver", FakeSolver)
    monkeypatch.setattr(warmstart, "batch_scene", lambda seeds, iterations=None, workload=None: FakeScene())
    return FakeSolver


def expected_sweeps(fit, r_warm, r0=2.0, rate=0.8, its=30):
    target = r0 * rate ** its
    return fit + math.ceil(math.log(target / r_warm) / math.log(rate) - 1e-9)


@pytest.mark.parametrize("fit", [0, 2])
def test_counts_sweeps_to_the_plain_residual(fake, fit):
    res = warmstart.evaluate(None, [1], frame=1, iterations=30, fit_sweeps=fit)
    r = res[0]
    assert not r["fallback"] and r["same_start"]
    assert r["iterations"] == expected_sweeps(fit, FakeSolver.r_warm)
    assert r["r_end"] <= r["r_plain"]


def test_start_worse_than_plain_is_discarded(fake, monkeypatch):
    monkeypatch.setattr(FakeSolver, "r_warm", 3.0)       # above the plain start's 2.0
    r = warmstart.evaluate(None, [1], frame=1, iterations=30, fit_sweeps=0)[0]
    assert r["fallback"] and r["iterations"] == 30


def test_fit_sweeps_compared_with_as_many_plain_sweeps(fake, monkeypatch):
    # after 2 fit sweeps the warm start must beat the plain start after 2
    # sweeps (2.0 * 0.8^2 = 1.28), not the plain start itself
    monkeypatch.setattr(FakeSolver, "r_warm", 1.5)
    r = warmstart.evaluate(None, [1], frame=1, iterations=30, fit_sweeps=2)[0]
    assert r["fallback"]
    r = warmstart.evaluate(None, [1], frame=1, iterations=30, fit_sweeps=0)[0]
    assert not r["fallback"]


def test_never_more_than_the_plain_sweeps(fake, monkeypatch):
    # a start barely better than the plain one cannot use more sweeps than plain
    monkeypatch.setattr(FakeSolver, "r_warm", 1.99)
    r = warmstart.evaluate(None, [1], frame=1, iterations=30, fit_sweeps=2)[0]
    assert r["iterations"] <= 30
