"""The CPU oracle against the reference's own physics gates and pipeline
invariants (restated from the reference suite; its Warp tests cannot run here).

Sources: tests/test_engine.py:51-73,101-107 (free fall, volume, settling),
tests/test_fused_pipeline.py:59-75 (fused == split bitwise),
tests/test_pour.py:39-57 (a static cup reads the water's weight),
tests/test_material_review_fixes.py:51-60 (von Mises hardening evolves yield).
"""
import numpy as np
import pytest

from mpm_engine_gb300 import GlassProfile
from scenes_lib import blob_scene, free_blob, water_in_cup


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib.OracleSolver


def test_free_fall_momentum(O):
    s = free_blob(O)
    dt, n = 2.0e-5, 100
    s.step(dt, n)
    vz = float(s.v()[:, 2].mean())
    expect = -9.81 * dt * n
    assert abs(vz - expect) < 0.05 * abs(expect)
    assert abs(float(s.v()[:, 0].mean())) < 0.02 * abs(expect)


def test_volume_conserved_in_free_fall(O):
    s = free_blob(O)
    s.step(2.0e-5, 5)
    F0 = float(np.abs(np.linalg.det(s.F())).mean())
    s.step(2.0e-5, 200)
    F1 = float(np.abs(np.linalg.det(s.F())).mean())
    assert abs(F1 - 1.0) < 5e-3
    assert abs(F1 - F0) / F0 < 5e-3


@pytest.mark.parametrize("key", ["newtonian", "jelly", "metal", "mu_i", "sand"])
def test_fused_bitwise_equals_split(O, key):
    """Oracle-internal invariant: the fused schedule equals the three-pass one bit for bit."""
    out = []
    for fused in (False, True):
        s, _ = blob_scene(O, key, fused=fused, n=600)
        for _ in range(3):
            s.step(2.0e-4, 6)
        out.append((s.x().copy(), s.v().copy(), s.F().copy(), s.a["stress"].copy()))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_fused_bitwise_with_moving_cup_wrench(O):
    res = []
    for fused in (False, True):
        s, h = blob_scene(O, "newtonian", fused=fused, cup=True, n=600)
        for _ in range(3):
            s.reset_wrench(h)
            s.step(2.0e-4, 6)
        res.append((s.x().copy(), s.wrench_of(h, 2.0e-4 * 6)))
    assert np.array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1]["force"], res[1][1]["force"])
    np.testing.assert_array_equal(res[0][1]["torque"], res[1][1]["torque"])


def test_static_cup_reads_weight(O):
    s, cup_pos, vol, h = water_in_cup(O, n_grid=24, grid_lim=0.35, fill=0.4)
    cup = s.add_cup(GlassProfile(), cup_pos, (1.0, 0.0, 0.0, 0.0), friction=0.05)
    m_water = float(1000.0 * vol.sum())
    dt = 5.0e-5
    fz = []
    for _ in range(4):
        s.reset_wrench(cup)
        s.step(dt, 250)
        fz.append(s.wrench_of(cup, dt * 250)["force"][2])
    f_settled = float(np.mean(fz[-2:]))
    assert abs(f_settled + 9.81 * m_water) < 0.15 * 9.81 * m_water


def test_von_mises_hardening_evolves_yield(O):
    s, h = blob_scene(O, "metal_hardening", box=True, n=800)
    y0 = s.a["yield_stress"].copy()
    for _ in range(4):
        s.step(2.0e-4, 10)
    assert (s.a["yield_stress"] > y0).any()


def test_svd_reconstructs_and_orders(oracle_lib):
    rng = np.random.default_rng(3)
    for _ in range(200):
        F = (np.eye(3) + 0.3 * rng.standard_normal((3, 3))).astype(np.float32)
        if rng.random() < 0.2:
            F[:, 2] *= -1  # reflections: sigma_3 carries the sign
        U, s, V = oracle_lib.svd3(F)
        np.testing.assert_allclose(U @ np.diag(s) @ V.T, F, atol=2e-6)
        assert np.linalg.det(U) > 0.99 and np.linalg.det(V) > 0.99
        assert s[0] >= s[1] >= abs(s[2]) - 1e-7
        np.testing.assert_allclose(np.abs(s), np.linalg.svd(F.astype(np.float64))[1], rtol=2e-6, atol=1e-7)


def test_own_sin_cos_acos_match_libm(oracle_lib):
    """The oracle's written-out sin, cos and acos (the rotation modifier's; the
    deterministic GPU passes state the same operations) against the host's libm, in
    double over the angles and cosines the modifier forms, and rounded to float."""
    rng = np.random.default_rng(11)
    th = np.concatenate([rng.uniform(-np.pi, np.pi, 200000),
                         [0.0, np.pi, -np.pi, np.pi / 2, -np.pi / 2, np.pi / 4, 1e-9, -3e-5]])
    c = np.concatenate([rng.uniform(-1.0, 1.0, 200000), [-1.0, -0.5, 0.0, 0.5, 1.0, 1.0 - 1e-12, -1.0 + 1e-9]])
    for kind, x, ref in (("sin", th, np.sin(th)), ("cos", th, np.cos(th)), ("acos", c, np.arccos(c))):
        got = oracle_lib.trig(x, kind)
        err = np.abs(got - ref)
        assert err.max() < 1e-15, (kind, float(err.max()), float(x[np.argmax(err)]))
        differ = np.float32(got) != np.float32(ref)
        assert differ.mean() < 1e-4, (kind, int(differ.sum()))
    assert np.isnan(oracle_lib.trig(np.array([1.5, np.nan]), "acos")).all()
    assert np.isnan(oracle_lib.trig(np.array([np.inf, np.nan]), "sin")).all()


@pytest.mark.parametrize("fused", [True, False])
def test_interleaved_oracle_instances_do_not_interact(O, fused):
    """The oracle library keeps one grid for every instance (each substep clears the box
    it touches before use). Two copies of a scene stepped alternately, with a third,
    different scene stepping in between, end bit-identical to a copy stepped alone:
    tests that hold several oracles at once compare clean runs."""
    alone, _ = blob_scene(O, "newtonian", fused=fused, v0=True)
    for _ in range(4):
        alone.step(2.0e-4, 3)
    a, _ = blob_scene(O, "newtonian", fused=fused, v0=True)
    b, _ = blob_scene(O, "newtonian", fused=fused, v0=True)
    other, _ = blob_scene(O, "jelly", fused=not fused, n=800, cup=True)
    for _ in range(4):
        a.step(2.0e-4, 3)
        other.step(1.0e-4, 5)
        b.step(2.0e-4, 3)
    for s in (a, b):
        np.testing.assert_array_equal(s.a["x"], alone.a["x"])
        np.testing.assert_array_equal(s.a["v"], alone.a["v"])
