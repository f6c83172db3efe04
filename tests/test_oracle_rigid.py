"""Rigid bodies and particle modifiers in the CPU oracle (the reference's split
pipeline tail, mpm_solver_warp.py:1338-1367, and its pre-P2G operations,
:1182-1196): physical gates that need no GPU."""
import numpy as np
import pytest

from mpm_engine_gb300 import elastic
from scenes_lib import blob, make, rigid_scene, set_rigid_motion


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib.OracleSolver


def test_rigid_body_free_fall_is_exact_and_keeps_its_shape(O):
    s, n_w = rigid_scene(O, water=False)
    set_rigid_motion(s, n_w, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    x0 = s.x().copy()
    dt, n = 1.0e-4, 30
    s.step(dt, n)
    st = s.rigid_state(0)
    assert abs(st["v"][2] - (-9.81 * dt * n)) < 1e-3 * 9.81 * dt * n
    assert np.abs(st["omega"]).max() < 1e-3
    np.testing.assert_allclose(st["R"], np.eye(3), atol=1e-5)
    d = s.x() - x0                          # every particle moved with the body
    assert np.abs(d - d.mean(axis=0)).max() < 1e-5


def test_rigid_body_bounces_off_a_restitution_surface(O):
    s, _ = rigid_scene(O, water=False, restitution=0.5, height=0.09)
    floor = 3 * 0.4 / 32
    vz = []
    for _ in range(40):
        s.step(1.0e-4, 10)
        vz.append(float(s.rigid_state(0)["v"][2]))
        assert s.x()[:, 2].min() > floor - 1e-3      # never through the floor
    assert min(vz) < -0.9 and max(vz[vz.index(min(vz)):]) > 0.05   # falling, then moving up after contact


def test_rigid_body_orientation_stays_orthonormal(O):
    s, _ = rigid_scene(O, water=True)
    for _ in range(5):
        s.step(1.0e-4, 10)
    R = s.rigid_state(0)["R"]
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-5)
    assert abs(np.linalg.det(R) - 1.0) < 1e-5


def test_impulse_adds_its_momentum_only_inside_its_window(O):
    pts, vol = blob(n=800)
    s = make(O, 32, 0.4, fused=True).load_particles(pts, vol)
    s.set_material(elastic(E=1e4, nu=0.3, density=1000.0), g=[0.0, 0.0, 0.0])
    dt = 1.0e-4
    sel = np.abs(pts - np.float32(0.2)).max(axis=1) < np.float32(0.03)
    s.add_impulse_on_particles((0.0, 0.0, 2.0e-3), dt, point=(0.2, 0.2, 0.2), size=(0.03, 0.03, 0.03), num_dt=3,
                               start_time=2 * dt)
    s.step(dt, 8)
    p = (s.a["mass"][:, None].astype(np.float64) * s.v()).sum(axis=0)
    expect = 3 * dt * 2.0e-3 * sel.sum()
    assert abs(p[2] - expect) < 1e-3 * expect and np.abs(p[:2]).max() < 1e-4 * expect


def test_translation_modifier_holds_its_particles(O):
    pts, vol = blob(n=800)
    s = make(O, 32, 0.4, fused=True).load_particles(pts, vol)
    s.set_material(elastic(E=1e4, nu=0.3, density=1000.0), g=[0.0, 0.0, 0.0])
    s.enforce_particle_velocity_translation((0.2, 0.2, 0.2), (0.02, 0.02, 0.02), (0.0, 0.5, 0.0), 0.0, 1.0)
    s.step(1.0e-4, 20)
    # the whole blob is dragged toward +y by the enforced core
    assert s.v()[:, 1].mean() > 0.05
