"""CPIC thin-boundary (CDF) colliders on the CUDA engine, through the C ABI,
against the CPU oracle.

Stamps are decided on identical host-integrated poses with per-operation fp32
rounding on both sides, so node tag and distance grids must agree bit for bit.
Particle fields follow the engine's parity contract (1e-5 relative per substep,
composed over k substeps); the per-lane reaction (float64 on the device, fp32 in
the oracle) within 1e-3 of its largest component. Reference gates restated:
tests/test_cdf_transfers.py:43-67 (the dam holds), tests/test_cdf_collider.py:73-86
(guards), tests/test_cdf_stamp_skip.py:73-80 (a static pose stamps once).
"""
import numpy as np
import pytest

from mpm_engine_gb300.geometry import sheet_cdf
from scenes_lib import CDF_DX, CDF_LIM, CDF_NG, cdf_solver, cdf_water, set_velocity, spin_velocity
from test_gpu_parity import assert_close, rel_err

pytestmark = pytest.mark.gpu

DT, SUB = 2e-4, 10


def _pair(oracle_lib, build, fused=True):
    from mpm_engine_gb300 import Solver
    s = build(Solver, fused)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), CDF_NG, CDF_LIM, fused=fused)
    return s, o


def _shelf(cls, fused):
    """Water thrown down, spinning, onto a static horizontal sheet; its lowest layer
    starts within one stencil of the sheet, so deposits are blocked from the start."""
    pos = cdf_water(0.14, 0.26, 0.14, 0.26, 0.2025, 0.25)
    s = cdf_solver(cls, pos, g=(0.0, 0.0, -9.81), fused=fused)
    set_velocity(s, spin_velocity(pos, lin=(0.1, 0.0, -0.6), omega=(0.0, 0.0, 4.0)))
    s.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.20), friction=0.3)
    return s


def _sweep(cls, fused):
    """A tilted vertical sheet translating and turning into a resting block."""
    pos = cdf_water(0.22, 0.30, 0.14, 0.26, 3 * CDF_DX, 3 * CDF_DX + 0.08)
    s = cdf_solver(cls, pos, fused=fused)
    half = 0.5 * np.deg2rad(10.0)
    quat = (0.0, 0.0, float(np.sin(half)), float(np.cos(half)))
    s.add_cdf_collider(sheet_cdf("x"), center=(0.18, 0.2, 0.2), quat=quat, velocity=(0.8, 0.0, 0.0),
                       omega=(0.0, 0.0, 0.6), surface="slip")
    return s


def _check_grids(s, o, what):
    tg, dg, ng = s.cdf_grids()
    to, do, no = o.cdf_grids()
    assert ng == no, f"{what}: {ng} stamps on the GPU, {no} in the oracle"
    assert np.array_equal(tg, to), f"{what}: {int((tg != to).sum())} node tags differ"
    assert np.array_equal(dg, do), f"{what}: owner distances differ"


def _check_tags(s, o, what):
    pt = s._t["cdf_tag"].cpu().numpy()
    frac = float((pt != o.a["cdf_tag"]).mean())
    assert frac <= 1e-3, f"{what}: {frac:.4%} of particle tags differ"


@pytest.mark.parametrize("fused", [True, False])
def test_shelf_parity(cuda, oracle_lib, fused):
    s, o = _pair(oracle_lib, _shelf, fused)
    _shelf_ticks(s, o)


def test_shelf_parity_with_resorts(cuda, oracle_lib):
    """The shelf with the working copy sorted again every 3 substeps of each
    10-substep fused tick (at substeps 3 and 6; one at 9 would leave less than half an
    interval). The CPIC scan a particle caches at its scatter for the next gather
    moves with its row, so the bounds are those without re-sorts."""
    from mpm_engine_gb300.autotune import set_solver_resort
    s, o = _pair(oracle_lib, _shelf, True)
    set_solver_resort(s, 3)
    _shelf_ticks(s, o)
    # the static sheet stamps no more: a tick's launches differ by the two re-sorts,
    # each a key pass, two radix passes of three kernels (15 key bits at 32^3) and a
    # permute
    counts = []
    for every in (0, 3):
        set_solver_resort(s, every)
        launches = s.launch_count()
        s.step(DT, SUB)
        counts.append(s.launch_count() - launches)
    assert counts[1] - counts[0] == 2 * 8, counts


def _shelf_ticks(s, o):
    k = 0
    for tick in range(6):
        s.reset_cdf_wrench()
        o.reset_cdf_wrench()
        s.step(DT, SUB)
        o.step(DT, SUB)
        k += SUB
        assert_close(s, o, k * 1e-5, f"shelf tick {tick}")
        _check_grids(s, o, f"shelf tick {tick}")
        _check_tags(s, o, f"shelf tick {tick}")
        wg, wo = s.cdf_wrench(0, DT * SUB), o.cdf_wrench(0, DT * SUB)
        # every tick blocks deposits (the water lands, then rebounds off the sheet)
        assert np.abs(wg["force"]).max() > 0.0, f"tick {tick}: no blocked deposits"
        if tick == 0:
            assert wg["force"][2] < 0.0, "the landing water presses down on the sheet"
        for key in ("force", "torque"):
            assert rel_err(wg[key], wo[key], 1e-9) < 1e-3, (tick, key, wg[key], wo[key])


@pytest.mark.parametrize("fused", [True, False])
def test_moving_turning_sheet_parity(cuda, oracle_lib, fused):
    s, o = _pair(oracle_lib, _sweep, fused)
    k = 0
    for tick in range(4):
        s.step(DT, SUB)
        o.step(DT, SUB)
        k += SUB
        assert_close(s, o, k * 1e-5, f"sweep tick {tick}")
        _check_grids(s, o, f"sweep tick {tick}")
        _check_tags(s, o, f"sweep tick {tick}")
    s._pull_cdf()
    o._pull_cdf()
    for a, b in zip(s._cdf, o.cdf_lanes):
        assert list(a.center) == list(b.center) and list(a.quat) == list(b.quat)
    assert s._cdf[0].center[0] > 0.18 + 0.8 * k * DT * 0.99


def test_zero_thickness_dam_holds(cuda):
    from mpm_engine_gb300 import Solver
    pos = cdf_water(0.10, 0.16, 0.12, 0.28, 3 * CDF_DX, 3 * CDF_DX + 0.08)
    s = cdf_solver(Solver, pos)
    x_wall = 0.20
    s.add_cdf_collider(sheet_cdf("x"), center=(x_wall, 0.2, 0.2))
    v = s.v()
    v[:, 0] += 1.0
    s.set_v(v)
    crossed, near = 0, False
    for _ in range(30):
        s.step(DT, SUB)
        x = s.x()
        crossed = max(crossed, int((x[:, 0] > x_wall).sum()))
        near = near or bool((x[:, 0] > x_wall - 1.5 * CDF_DX).any())
    assert near and crossed == 0, (near, crossed)


def test_static_pose_stamps_once_and_sort_keeps_tags(cuda):
    from mpm_engine_gb300 import Solver
    s = _shelf(Solver, True)
    for _ in range(5):
        s.step(DT, SUB)
    assert s.cdf_grids()[2] == 1
    tags = s._t["cdf_tag"].cpu().numpy().copy()
    x = s.x().copy()
    assert (tags != 0).any()
    assert s._sort_particles()
    perm = s._t["perm"].cpu().numpy()[: len(x)]
    assert np.array_equal(s.x(), x[perm])
    assert np.array_equal(s._t["cdf_tag"].cpu().numpy(), tags[perm])


def test_guards_and_api(cuda):
    from mpm_engine_gb300 import BatchSolver, GridConfig, Solver
    s = cdf_solver(Solver, cdf_water(0.08, 0.14, 0.08, 0.14, 0.08, 0.14))
    cdf = sheet_cdf("z", size=0.3, band_cells=6.0)
    with pytest.raises(ValueError, match="runtime band"):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2), band=10.0)
    with pytest.warns(RuntimeWarning, match="below 1.5 dx"):
        h = s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2), band=0.5 * CDF_DX)
    with pytest.warns(RuntimeWarning, match="jumped the surface"):
        s.set_cdf_pose(h, center=(0.2, 0.2, 0.35))
    for _ in range(3):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2))
    with pytest.raises(ValueError, match="at most"):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2))
    with pytest.raises(NotImplementedError):
        BatchSolver([s]).step(DT, 1)
    s.step(DT, 2)
    s.reset_cdf_wrench()
    assert np.all(s.cdf_wrench(0, DT)["force"] == 0.0)
    pos = cdf_water(0.10, 0.14, 0.10, 0.14, 0.10, 0.14)
    p = Solver(grid=GridConfig(n_grid=CDF_NG, grid_lim=CDF_LIM), periodic_x=True)
    p.load_particles(pos, np.full(len(pos), 1e-7, np.float32))
    with pytest.raises(NotImplementedError):
        p.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2))


def test_fast_sheet_warns_on_band_sweep(cuda):
    from mpm_engine_gb300 import Solver
    s = cdf_solver(Solver, cdf_water(0.14, 0.20, 0.14, 0.26, 3 * CDF_DX, 3 * CDF_DX + 0.05))
    band = 2.0 * CDF_DX
    s.add_cdf_collider(sheet_cdf("x"), center=(0.3, 0.2, 0.2), velocity=(2.0 * band / DT, 0.0, 0.0))
    with pytest.warns(RuntimeWarning, match="sweeps"):
        s.step(DT, 1)


def test_cdf_pour_holds_and_matches_oracle(cuda, oracle_lib):
    """The pour with both glasses as CPIC sheets (examples/pour_franka.py:278-286) at
    96^3: the tilting source glass restamps every substep; tags stay bit-exact with
    the oracle and the honey stays in the glass. Thousands of particles here read
    ghost velocities, whose normalised gradients, capped Coulomb impulse and
    separation push pass rounding through non-smooth operations, so particle fields
    are held to 2e-5 relative per substep (composed) rather than 1e-5."""
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.glass import GlassProfile
    from mpm_engine_gb300.scenes import POUR_SOURCE, pour_scene
    s, src, rcv, traj, S, dt = pour_scene(Solver, n_grid=96, glass="cdf")
    o = oracle_lib.OracleSolver.from_state(s.export_state(), 96, 0.7)
    o.threads = 16
    # the same pose command on both sides, so their lane bookkeeping stays identical;
    # the trajectory then continues from there (a jump back would teleport the sheet)
    t0 = 0.15
    c, q, v, w = traj.command(t0, 1.0 / 60.0)
    for solver in (s, o):
        solver.set_cdf_pose(src, center=c, quat=(q[1], q[2], q[3], q[0]), velocity=v, omega=w)
    k = 0
    for _ in range(2):
        s.step(dt, 10)
        o.step(dt, 10)
        k += 10
        assert_close(s, o, k * 2e-5, f"cdf pour after {k} substeps")
        _check_grids(s, o, f"cdf pour after {k} substeps")
    for i in range(1, 7):
        c, q, v, w = traj.command(t0 + i / 60.0, 1.0 / 60.0)
        s.set_cdf_pose(src, center=c, quat=(q[1], q[2], q[3], q[0]), velocity=v, omega=w)
        s.step(dt, S)
    prof = GlassProfile()
    x = s.x() - np.asarray(POUR_SOURCE)
    r = np.hypot(x[:, 0], x[:, 1])
    inside = r < prof.inner_radius - 2 * 0.7 / 96
    assert np.isfinite(x).all()
    assert (x[inside, 2] > prof.inner_floor_z - 1.5 * 0.7 / 96).all(), "honey leaked through the glass floor"


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("moving", [False, True])
def test_block_mask_skip_changes_nothing(cuda, fused, moving):
    """The block-mask early-out of the CPIC scan (tests/test_cdf_mask.py:37-75): a
    column on a sheet plus a blob far from any sheet, stepped with the early-out on
    and with every particle scanning its stencil (model.cdf_mask_off = 1). The skip
    is exact; two GPU runs agree to float-atomic rounding."""
    from mpm_engine_gb300 import Solver
    out = []
    for off in (0, 1):
        pos = np.concatenate([cdf_water(0.14, 0.26, 0.14, 0.26, 0.21, 0.27),
                              cdf_water(0.06, 0.12, 0.06, 0.12, 0.08, 0.14)])
        s = cdf_solver(Solver, pos, g=(0.0, 0.0, -9.81), fused=fused)
        h = s.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.20), friction=0.3)
        s._sim.mpm_model.cdf_mask_off = off
        assert s._sim.mpm_model.cdf_mask_off == off
        if moving:
            s.set_cdf_pose(h, velocity=(0.0, 0.0, 0.01))
        for _ in range(8 if moving else 5):
            s.step(DT, SUB)
        out.append((s.x(), s.v()))
    np.testing.assert_allclose(out[1][0], out[0][0], rtol=1e-5, atol=1e-6)
    vs = float(np.abs(out[0][1]).max())
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=0, atol=1e-4 * vs + 1e-7)
