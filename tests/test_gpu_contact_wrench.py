"""Device stress-integral wrench (Solver.contact_wrench) against the reference's
box_contact_wrench (coupling/wrench.py:15-46) restated in numpy over the same
x, cauchy() and vol(): a granular heap pressed by a plate (the press workload,
scaled down)."""
import numpy as np
import pytest

from scenes_lib import MATERIALS, make

pytestmark = pytest.mark.gpu


def _press(Solver):
    rng = np.random.default_rng(0)
    ng, lim = 48, 0.4
    dx = lim / ng
    h = dx / 2
    ax = np.arange(0.12, 0.28, h)
    pts = np.stack(np.meshgrid(ax, ax, np.arange(3 * dx + h / 2, 0.12, h), indexing="ij"), -1).reshape(-1, 3)
    pts = (pts + rng.uniform(-0.25 * h, 0.25 * h, pts.shape)).astype(np.float32)
    s = make(Solver, ng, lim).load_particles(pts, np.full(len(pts), h ** 3, np.float32))
    s.set_material(MATERIALS["mu_i"]())
    s.add_plane((0, 0, 3 * dx), (0, 0, 1), "sticky")
    s.add_domain_walls()
    top = float(pts[:, 2].max())
    center = (0.2, 0.2, top + dx)
    half = (0.05, 0.05, dx)
    s.add_box(center, half, velocity=(0.0, 0.0, -0.2))
    return s, center, half, dx


@pytest.mark.parametrize("compressive", [True, False])
def test_contact_wrench_matches_reference_formula(cuda, oracle_lib, compressive):
    from mpm_engine_gb300 import Solver
    s, center, half, dx = _press(Solver)
    checked = 0
    for tick in range(6):
        s.step(2e-5, 25)
        c = (center[0], center[1], center[2] - 0.2 * 2e-5 * 25 * (tick + 1))
        for layer in (None, 3.0):
            got = s.contact_wrench(c, half, layer_cells=layer, dx=dx if layer else None, compressive_only=compressive)
            want = oracle_lib.box_contact_wrench(s.x().astype(np.float64), s.cauchy().astype(np.float64),
                                                 s.vol().astype(np.float64), c, half, layer_cells=layer,
                                                 dx=dx if layer else None, compressive_only=compressive)
            assert got["n_contact"] == want["n_contact"]
            if want["n_contact"]:
                checked += 1
                scale = np.abs(want["force"]).max() + 1e-12
                assert np.abs(got["force"] - want["force"]).max() <= 1e-5 * scale
                tscale = np.abs(want["torque"]).max() + 1e-12
                assert np.abs(got["torque"] - want["torque"]).max() <= 1e-5 * tscale + 1e-9 * scale
    assert checked >= 4, "the plate never reached the heap"


def test_contact_wrench_inversion_policy(cuda):
    from mpm_engine_gb300 import Solver
    s, center, half, dx = _press(Solver)
    F = s.F()
    F[0] = -np.eye(3, dtype=np.float32)
    s._t["F"].copy_(__import__("torch").from_numpy(F))
    s.inversion_policy = "raise"
    with pytest.raises(RuntimeError, match="non-positive det"):
        s.contact_wrench(center, half)
    s.inversion_policy = "warn"
    with pytest.warns(RuntimeWarning, match="inverted"):
        s.contact_wrench(center, half)


def test_device_cauchy_and_volume_match_reference_formula(cuda):
    """Solver.cauchy()/vol() now computed on the device (core/solver.py:559-598)."""
    from mpm_engine_gb300 import Solver
    s, center, half, dx = _press(Solver)
    s.step(2e-5, 50)
    F, S = s.F().astype(np.float64), s.stress().astype(np.float64)
    J = np.linalg.det(F)
    want_c = S / np.clip(np.abs(J), 1e-9, None)[:, None, None]
    want_v = s._vol0.astype(np.float64) * np.abs(J)
    got_c, got_v = s.cauchy(), s.vol()
    assert np.abs(got_c - want_c).max() <= 1e-5 * np.abs(want_c).max()
    np.testing.assert_allclose(got_v, want_v, rtol=1e-5)
    F32 = s.F()
    F32[3] = -np.eye(3, dtype=np.float32)
    s._t["F"].copy_(__import__("torch").from_numpy(F32))
    s.inversion_policy = "nan"
    v = s.vol()
    assert np.isnan(v[3]) and np.isfinite(np.delete(v, 3)).all()
    s.inversion_policy = "raise"
    with pytest.raises(RuntimeError, match="non-positive det"):
        s.cauchy()
