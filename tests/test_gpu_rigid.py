"""Rigid bodies and particle modifiers on the GPU against the CPU oracle.

The engine runs them inside its fused tick (rigid particles deposit after their
body moves; modifiers act inside the particle pass); the oracle runs the
reference's split pipeline (core/solver.py:440-453 sends these scenes there). The
two orders are the same computation, so they agree to float rounding: per tick
within 1e-5 relative per substep, as the other parity tests.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_close
from scenes_lib import blob, make, rigid_scene

pytestmark = pytest.mark.gpu

DT, SUB = 1.0e-4, 10


def _pair(cuda, oracle_lib, **kw):
    from mpm_engine_gb300 import Solver
    s, n_w = rigid_scene(Solver, **kw)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    return s, o


def _rigid_close(s, o, tol, what):
    a, b = s.rigid_state(0), o.rigid_state(0)
    for k in ("com", "v", "omega", "R"):
        scale = np.abs(b[k]).max() + (1e-6 if k != "omega" else 1e-4)
        err = float(np.abs(np.asarray(a[k], np.float64) - b[k]).max() / scale)
        assert err <= tol, f"{what}: rigid {k} relative error {err:.3g} > {tol}"


@pytest.mark.parametrize("water,resort", [(False, False), (True, False), (True, True)])
def test_rigid_body_matches_oracle(cuda, oracle_lib, water, resort):
    """A tilted cube thrown, spinning, at a restitution floor (alone: 12 ticks, into
    the floor with the deepest-corner impulse) or into a water slab (6 ticks:
    two-way coupling through the grid, the cube pushing the fluid); with `resort`,
    the working copy is sorted again at substeps 3 and 6 of each tick, and the list
    of rigid rows is rebuilt after each re-sort."""
    s, o = _pair(cuda, oracle_lib, water=water)
    if resort:
        from mpm_engine_gb300.autotune import set_solver_resort
        set_solver_resort(s, 3)
    for t in range(6 if water else 12):
        s.step(DT, SUB)
        o.step(DT, SUB)
        tol = 1e-5 * SUB * (t + 1)
        _rigid_close(s, o, tol, f"tick {t}")
        assert_close(s, o, tol, f"tick {t}")
    assert o.rigid_state(0)["v"][2] > -0.9       # the floor impulse or the water slowed the fall


def test_rigid_fused_equals_split_on_gpu(cuda):
    from mpm_engine_gb300 import Solver
    out = []
    for fused in (True, False):
        s, _ = rigid_scene(Solver, water=True, fused=fused)
        for _ in range(4):
            s.step(DT, SUB)
        out.append((s.x(), s.v(), s.rigid_state(0)))
    np.testing.assert_allclose(out[0][0], out[1][0], rtol=0, atol=1e-5 * 0.4)
    for k in ("com", "v", "R"):
        np.testing.assert_allclose(out[0][2][k], out[1][2][k], rtol=1e-4, atol=1e-6)


def test_rigid_body_api_and_reference_views(cuda):
    """The MPM_Simulator_WARP views scripts read (tests/test_vehicle.py:84-97)."""
    from mpm_engine_gb300 import Solver
    s, n_w = rigid_scene(Solver, water=True)
    assert s._sim.n_rigid_bodies == 1
    m = float(s._t["mass"][n_w:].sum())
    np.testing.assert_allclose(s._sim.rigid_mass.numpy()[0], m, rtol=1e-5)
    st = s.rigid_state()
    np.testing.assert_allclose(st["R"], np.eye(3), atol=1e-7)
    np.testing.assert_allclose(s._sim.rigid_x_cm.numpy()[0], st["com"])
    s.step(DT, SUB)
    R = s.rigid_state()["R"]
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-5)
    with pytest.raises(IndexError):
        s.rigid_state(1)


@pytest.mark.parametrize("resort", [False, True])
def test_particle_modifiers_match_oracle(cuda, oracle_lib, resort):
    """An impulse (active 3 substeps), a held translation and a rotating cylinder on
    one jelly blob, GPU fused tick against the oracle's split pipeline; with
    `resort`, the working copy (modifier masks included) is sorted again at
    substeps 3 and 6 of each tick."""
    from mpm_engine_gb300 import Solver, elastic
    from mpm_engine_gb300.autotune import set_solver_resort
    pts, vol = blob(n=3000, lo=0.12, size=0.12)
    s = make(Solver, 40, 0.4).load_particles(pts, vol)
    if resort:
        set_solver_resort(s, 3)
    s.set_material(elastic(E=2e4, nu=0.3, density=1000.0))
    s.add_domain_walls()
    s.add_impulse_on_particles((0.0, 0.0, 5.0e-4), DT, point=(0.15, 0.15, 0.15), size=(0.03, 0.03, 0.03), num_dt=3,
                               start_time=2 * DT)
    s.enforce_particle_velocity_translation((0.22, 0.22, 0.22), (0.015, 0.015, 0.015), (0.0, 0.3, 0.0), 0.0, 1.0)
    s.enforce_particle_velocity_rotation((0.18, 0.18, 0.18), (0.3, 0.2, 1.0), (0.02, 0.025), 4.0, 0.1, 5 * DT, 1.0)
    assert len(s._sim.pre_p2g_operations) == 1 and len(s._sim.particle_velocity_modifiers) == 2
    o = oracle_lib.OracleSolver.from_state(s.export_state(), 40, 0.4)
    for t in range(4):
        s.step(DT, SUB)
        o.step(DT, SUB)
        assert_close(s, o, 1e-5 * SUB * (t + 1), f"tick {t}")
    assert abs(float(s.v()[:, 1].mean())) > 1e-3     # the translation drags the blob


def test_rigid_body_survives_particle_sorting(cuda):
    """sort_interval permutes rigid_id, x_ref and mod_mask with the other particle
    arrays: the body moves as without sorting (to the order of float atomics)."""
    from mpm_engine_gb300 import Solver
    out = []
    for sort in (0, 1):
        s, _ = rigid_scene(Solver, water=True)
        s.sort_interval = sort
        for _ in range(4):
            s.step(DT, SUB)
        out.append(s.rigid_state(0))
    for k in ("com", "v", "R"):
        np.testing.assert_allclose(out[1][k], out[0][k], rtol=1e-4, atol=1e-5)


def test_rigid_scenes_in_a_batch(cuda):
    """Two rigid scenes in one BatchSolver graph step like each scene alone."""
    from mpm_engine_gb300 import BatchSolver, Solver
    alone = []
    for restitution in (0.3, 0.6):
        s, _ = rigid_scene(Solver, water=False, restitution=restitution)
        for _ in range(8):
            s.step(DT, SUB)
        alone.append(s.rigid_state(0))
    scenes = [rigid_scene(Solver, water=False, restitution=e)[0] for e in (0.3, 0.6)]
    b = BatchSolver(scenes)
    for _ in range(8):
        b.step(DT, SUB)
    for s, ref in zip(scenes, alone):
        st = s.rigid_state(0)
        for k in ("com", "v", "R"):
            np.testing.assert_allclose(st[k], ref[k], rtol=1e-4, atol=1e-5)
