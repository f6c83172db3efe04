"""Host logic of adjoint.rollout without a GPU: checkpoint segmentation and the
state/collider snapshot round trip, on a stand-in solver."""
import ctypes as C

import torch

from mpm_engine_gb300 import _abi, adjoint


class FakeSolver:
    def __init__(self, n=5):
        self._t = {"x": torch.zeros(n, 3), "v": torch.zeros(n, 3), "C": torch.zeros(n, 3, 3),
                   "F_trial": torch.eye(3).repeat(n, 1, 1), "L": torch.zeros(n, 3, 3),
                   "yield_stress": torch.zeros(n), "mu": torch.ones(n), "lam": torch.ones(n), "Jp": torch.ones(n)}
        self._cols = [_abi.Collider()]
        self._cols_dirty = False
        self._time = 0.0
        self.steps = []
        self.synced = 0

    def _pull_colliders(self):
        pass

    def _sync_engine(self):
        self.synced += 1

    def step(self, dt, k):
        self.steps.append(k)
        self._time += dt * k
        self._t["x"] += 1.0
        self._cols[0].point[0] += 1.0


def test_segments_cover_the_rollout():
    s = FakeSolver()
    ckpts = adjoint._forward(s, 0.5, 45, 20)
    assert s.steps == [20, 20, 5]
    assert [c[1] for c in ckpts] == [20, 20, 5]
    assert [c[0][2] for c in ckpts] == [0.0, 10.0, 20.0]
    assert all(c[2] is None for c in ckpts)   # replayed backwards: no kept states


def test_snapshot_restores_state_colliders_and_clock():
    s = FakeSolver()
    snap = adjoint._snapshot(s)
    s.step(0.1, 3)
    adjoint._restore(s, snap)
    assert float(s._t["x"].abs().max()) == 0.0
    assert s._cols[0].point[0] == 0.0 and s._time == 0.0
    assert s._cols_dirty and s.synced == 1
    # the snapshot owns copies: later changes to the solver do not reach it
    s._cols[0].point[0] = 7.0
    assert snap[1][0].point[0] == 0.0
    assert C.sizeof(snap[1][0]) == C.sizeof(_abi.Collider)


def test_collider_only_snapshot_restores_clock_and_colliders():
    s = FakeSolver()
    snap = adjoint._snapshot(s, particles=False)
    assert snap[0] is None
    s.step(0.1, 3)
    adjoint._restore(s, snap)
    assert float(s._t["x"].abs().max()) == 1.0   # particles untouched
    assert s._cols[0].point[0] == 0.0 and s._time == 0.0


def test_state_bytes():
    assert adjoint.state_bytes(50_000, 400) == 37 * 4 * 50_000 * 400


def test_mu_lam_is_the_reference_formula():
    mu, lam = adjoint.mu_lam(torch.tensor(1.0e5), torch.tensor(0.3))
    assert abs(float(mu) - 1.0e5 / 2.6) < 1e-2
    assert abs(float(lam) - 1.0e5 * 0.3 / (1.3 * 0.4)) < 1e-1
