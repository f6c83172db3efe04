"""Mesh-SDF colliders on the CUDA engine.

These tests cover the reference's SDF collider suite (tests/test_sdf_collider.py:20-126),
restated on the GPU:
- a fluid stays inside a cup built from its mesh;
- the cup's reaction equals the contained weight within 25 %;
- tilting the cup carries the fluid;
- a band wider than the SDF margin is refused;
- pose jumps and velocities that sweep past the band warn of tunnelling.

A per-substep parity run against the oracle adds a thrown, spinning blob landing on a
moving, turning mesh cup: particle fields within 1e-5 relative per substep, the
wrench within 1e-4.
"""
import functools

import numpy as np
import pytest

from test_gpu_parity import assert_close, rel_err

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=1)
def _cup_sdf():
    """The reference's test cup: inner radius 4 cm, 8 mm walls, 9 cm tall, 1 cm
    base, 40 segments, voxelised at 48^3 with a 4-cell margin."""
    from mpm_engine_gb300.meshfield import build_sdf, make_cup_mesh
    v, f = make_cup_mesh(inner_radius=0.04, wall_thickness=0.008, height=0.09, base_thickness=0.01, n_theta=40)
    return build_sdf(v, f, res=48, margin_cells=4, interior_probe=np.array([0.044, 0.0, 0.04]))


def _fill_cavity(center, dx, radius=0.030, z_lo=0.015, z_hi=0.05):
    h = dx / 2
    ax = np.arange(-radius, radius, h)
    X, Y, Z = np.meshgrid(ax, ax, np.arange(z_lo, z_hi, h), indexing="ij")
    keep = (X ** 2 + Y ** 2) < radius ** 2
    pts = np.stack([X[keep], Y[keep], Z[keep]], -1) + np.asarray(center)
    return pts.astype(np.float32), np.full(len(pts), h ** 3, np.float32)


def _cup_solver(eta=5.0, fused=True):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    grid = GridConfig(n_grid=48, grid_lim=0.4)
    center = np.array([0.2, 0.2, 0.06])
    pts, vol = _fill_cavity(center, grid.dx)
    s = Solver(grid=grid, fused=fused).load_particles(pts, vol)
    s.set_material(newtonian(eta=eta, density=1000.0, bulk_modulus=5.0e5))
    h = s.add_sdf_collider(_cup_sdf(), center=center, surface="separable", friction=0.3)
    return s, h, center, float(vol.sum() * 1000.0)


def test_fluid_stays_contained_in_the_cup(cuda):
    s, h, center, _ = _cup_solver()
    z0 = float(s.x()[:, 2].min())
    for _ in range(30):
        s.step(2.0e-4, substeps=5)
    x = s.x()
    assert x[:, 2].min() > center[2] - 0.01, "fluid leaked below the cup base"
    assert abs(float(x[:, 2].min()) - z0) < 0.03
    assert s.inverted_count() == 0


def test_reaction_equals_the_contained_weight(cuda):
    s, h, _, mass = _cup_solver()
    dt, fz = 2.0e-4, []
    for it in range(30):
        s.reset_sdf_force(h)
        s.step(dt, substeps=5)
        if it >= 15:
            fz.append(float(s.sdf_wrench(h, dt * 5)["force"][2]))
    weight = mass * 9.81
    assert abs(abs(float(np.mean(fz))) - weight) < 0.25 * weight, (np.mean(fz), weight)


def test_turning_cup_carries_the_fluid(cuda):
    s, h, _, _ = _cup_solver(eta=2.0)
    for _ in range(10):
        s.step(2.0e-4, substeps=5)
    x0 = float(s.x()[:, 0].mean())
    s.set_sdf_pose(h, omega=(0.0, 8.0, 0.0))
    for _ in range(80):
        s.step(2.0e-4, substeps=5)
    assert float(s.x()[:, 0].mean()) - x0 > 0.004
    assert s.inverted_count() == 0


def test_band_wider_than_the_margin_is_refused(cuda):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    grid = GridConfig(n_grid=48, grid_lim=0.4)
    center = np.array([0.2, 0.2, 0.06])
    pts, vol = _fill_cavity(center, grid.dx, radius=0.01, z_lo=0.02, z_hi=0.03)
    s = Solver(grid=grid).load_particles(pts, vol)
    s.set_material(newtonian(eta=5.0, density=1000.0, bulk_modulus=5.0e5))
    with pytest.raises(ValueError, match="margin"):
        s.add_sdf_collider(_cup_sdf(), center=center, band=0.05)


def test_pose_jump_and_fast_velocity_warn_of_tunnelling(cuda):
    s, h, center, _ = _cup_solver()
    with pytest.warns(RuntimeWarning, match="tunnel"):
        s.set_sdf_pose(h, center=(center[0] + 0.1, center[1], center[2]))
    s, h, _, _ = _cup_solver()
    s.set_sdf_pose(h, velocity=(50.0, 0.0, 0.0))      # 10 mm a substep against a ~8 mm band
    with pytest.warns(RuntimeWarning, match="tunnel"):
        s.step(2.0e-4, substeps=1)


@pytest.mark.parametrize("fused", [True, False])
def test_mesh_cup_parity_with_oracle(cuda, oracle_lib, fused):
    """A thrown, spinning jelly blob landing in a mesh cup that translates and
    turns: GPU against the oracle, substep by substep, and the cup's wrench."""
    from mpm_engine_gb300 import GridConfig, Solver, elastic
    from scenes_lib import spin_velocity
    grid = GridConfig(n_grid=48, grid_lim=0.4)
    center = np.array([0.2, 0.2, 0.06])
    pts, vol = _fill_cavity(center, grid.dx, z_lo=0.03, z_hi=0.06)
    s = Solver(grid=grid, fused=fused).load_particles(pts, vol)
    s.set_material(elastic(E=5.0e4, nu=0.3, density=1000.0))
    s.set_v(spin_velocity(pts, lin=(0.1, 0.0, -0.5), omega=(0.0, 0.0, 4.0)))
    h = s.add_sdf_collider(_cup_sdf(), center=center, quat=(0.0, 0.0, float(np.sin(0.1)), float(np.cos(0.1))),
                           velocity=(0.05, 0.0, 0.0), omega=(0.0, 0.0, 1.0), surface="separable", friction=0.3)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), 48, 0.4, fused=fused)
    dt = 2.0e-4
    for t in range(6):
        s.reset_sdf_force(h)
        o.reset_wrench(h)
        s.step(dt, 4)
        o.step(dt, 4)
        assert_close(s, o, 4 * (t + 1) * 1e-5, f"mesh cup tick {t}")
        wg, wo = s.sdf_wrench(h, dt * 4), o.wrench_of(h, dt * 4)
        assert rel_err(wg["force"], wo["force"], 1e-9) < 1e-4, (wg["force"], wo["force"])
