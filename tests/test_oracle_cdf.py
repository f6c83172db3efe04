"""CPIC thin-boundary (CDF) colliders on the CPU oracle: the reference's own CDF
gates restated (its Warp tests cannot run here).

Sources: tests/test_cdf_geometry.py:40-57 (sheet distance, side and rim),
tests/test_cdf_collider.py:40-104 (stamp bits against the analytic plane, guards,
an inert collider changes nothing), tests/test_cdf_transfers.py:43-167 (the
zero-thickness dam holds, the shelf reads a fraction of the weight, a moving wall
sweeps without leaks), tests/test_cdf_fused.py:42-52 (fused == split bitwise),
tests/test_cdf_stamp_skip.py:73-80 (a static pose stamps once).
"""
import numpy as np
import pytest

from mpm_engine_gb300.geometry import load_cdf, save_cdf, sheet_cdf
from scenes_lib import CDF_DX, cdf_solver, cdf_water, set_velocity

DT, SUB = 2e-4, 10


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib.OracleSolver


def _lookup(cdf, pts):
    idx = np.clip(np.rint((pts - cdf.origin) / cdf.cell).astype(int), 0, cdf.res - 1)
    snapped = cdf.origin + idx * cdf.cell
    return cdf.values[idx[:, 0], idx[:, 1], idx[:, 2]], cdf.valid[idx[:, 0], idx[:, 1], idx[:, 2]], snapped


def test_sheet_signed_distance_and_rim(tmp_path):
    cdf = sheet_cdf("z", size=1.0, res=48)
    h = cdf.cell
    for z in (h, -h, 2 * h, -2 * h):
        d, ok, snapped = _lookup(cdf, np.array([[0.0, 0.0, z], [-0.1, 0.1, z]]))
        assert np.all(ok == 1.0)
        assert np.allclose(d, snapped[:, 2], atol=0.15 * h)
    _, ok, _ = _lookup(cdf, np.array([[-0.5, 0.0, h], [-0.5 - 0.5 * h, 0.0, 0.0]]))
    assert np.all(ok == 0.0), "rim neighbourhood must be invalid"
    _, ok, _ = _lookup(cdf, np.array([[0.0, 0.0, 10 * h]]))
    assert np.all(ok == 0.0)
    save_cdf(cdf, tmp_path / "sheet.npz")
    c = load_cdf(tmp_path / "sheet.npz")
    assert np.array_equal(cdf.values, c.values) and c.band == cdf.band


def test_stamp_bits_match_analytic_plane(O):
    rng = np.random.default_rng(0)
    pos = (np.full((8, 3), 0.2) + rng.uniform(0, 0.01, (8, 3))).astype(np.float32)
    s = cdf_solver(O, pos, fused=False, floor=False)
    z0 = 0.2
    h = s.add_cdf_collider(sheet_cdf("z", size=0.3, band_cells=6.0), center=(0.2, 0.2, z0), band=2.5 * CDF_DX)
    assert h == 0
    s.step(1e-4, 1)
    tag, d, stamps = s.cdf_grids()
    assert stamps == 1
    k0 = int(round(z0 / CDF_DX))
    ij = np.arange(int(0.15 / CDF_DX), int(0.25 / CDF_DX))
    above = tag[np.ix_(ij, ij, [k0 + 1, k0 + 2])]
    below = tag[np.ix_(ij, ij, [k0 - 1, k0 - 2])]
    assert np.all(above & 1) and np.all(above & 2)
    assert np.all(below & 1) and np.all(below & 2 == 0)
    assert np.all(tag[np.ix_(ij, ij, [k0 + 5, k0 - 5])] == 0), "beyond the band untagged"
    assert np.all(tag[int(0.05 / CDF_DX), ij, k0 + 1] == 0), "rim tube untagged"
    assert np.allclose(d[np.ix_(ij, ij, [k0 + 1])], CDF_DX, atol=0.1 * CDF_DX)


def test_guards(O):
    s = cdf_solver(O, cdf_water(0.08, 0.14, 0.08, 0.14, 0.08, 0.14))
    cdf = sheet_cdf("z", size=0.3, band_cells=6.0)
    with pytest.raises(ValueError, match="runtime band"):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2), band=10.0)
    with pytest.warns(RuntimeWarning, match="below 1.5 dx"):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2), band=0.5 * CDF_DX)
    for _ in range(3):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2))
    with pytest.raises(ValueError, match="at most"):
        s.add_cdf_collider(cdf, center=(0.2, 0.2, 0.2))


@pytest.mark.parametrize("fused", [False, True])
def test_inert_collider_is_bitwise_invisible(O, fused):
    pos = cdf_water(0.08, 0.14, 0.08, 0.14, 0.08, 0.14)
    a = cdf_solver(O, pos, fused=fused)
    b = cdf_solver(O, pos, fused=fused)
    b.add_cdf_collider(sheet_cdf("z", size=0.3, band_cells=6.0), center=(0.30, 0.30, 0.30))
    for _ in range(4):
        a.step(DT, SUB)
        b.step(DT, SUB)
    assert np.array_equal(a.x(), b.x()) and np.array_equal(a.v(), b.v()) and np.array_equal(a.F(), b.F())


def test_zero_thickness_dam_holds(O):
    pos = cdf_water(0.10, 0.16, 0.12, 0.28, 3 * CDF_DX, 3 * CDF_DX + 0.08)
    s = cdf_solver(O, pos)
    s.threads = 8
    x_wall = 0.20
    s.add_cdf_collider(sheet_cdf("x"), center=(x_wall, 0.2, 0.2))
    v = s.v().copy()
    v[:, 0] += 1.0
    set_velocity(s, v)
    crossed, near = 0, False
    for _ in range(30):
        s.step(DT, SUB)
        x = s.x()
        crossed = max(crossed, int((x[:, 0] > x_wall).sum()))
        near = near or bool((x[:, 0] > x_wall - 1.5 * CDF_DX).any())
    assert near, "the slab never reached the wall"
    assert crossed == 0, f"{crossed} particles crossed the thin wall"


def test_shelf_reads_a_scaled_fraction_of_the_weight(O):
    pos = cdf_water(0.14, 0.26, 0.14, 0.26, 0.21, 0.29)
    s = cdf_solver(O, pos, g=(0.0, 0.0, -9.81))
    s.threads = 8
    h = s.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.20))
    weight = float(len(pos) * (CDF_DX / 2) ** 3 * 1000.0 * 9.81)
    for _ in range(120):
        s.step(DT, SUB)
    s.model.grid_v_damping_scale = 0.999
    forces = []
    for _ in range(40):
        s.reset_cdf_wrench()
        s.step(DT, SUB)
        forces.append(s.cdf_wrench(h, DT * SUB)["force"][2])
    f = float(np.mean(forces))
    assert f < 0.0, "the material presses down on the shelf"
    assert 0.15 * weight < -f < 0.6 * weight, f"{f:.3f} N vs weight {weight:.3f} N"
    assert float(s.x()[:, 2].min()) > 0.20 - 1.5 * CDF_DX, "material fell through the shelf"


def test_moving_wall_sweeps_without_leaks(O):
    pos = cdf_water(0.22, 0.30, 0.14, 0.26, 3 * CDF_DX, 3 * CDF_DX + 0.08)
    s = cdf_solver(O, pos)
    s.threads = 8
    x0, v_wall = 0.18, 1.0
    s.add_cdf_collider(sheet_cdf("x"), center=(x0, 0.2, 0.2), velocity=(v_wall, 0.0, 0.0))
    t = 0.0
    for _ in range(40):
        s.step(DT, SUB)
        t += DT * SUB
        wall_x = x0 + v_wall * t
        behind = int((s.x()[:, 0] < wall_x - 1.5 * CDF_DX).sum())
        assert behind == 0, f"{behind} particles tunnelled behind the moving wall"
    assert wall_x > 0.25


def _fused_split_scene(O, fused, vel, omega=(0.0, 0.0, 0.0)):
    pos = cdf_water(0.14, 0.26, 0.14, 0.26, 0.21, 0.28)
    s = cdf_solver(O, pos, g=(0.0, 0.0, -9.81), fused=fused)
    s.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.20), velocity=vel, omega=omega)
    return s


@pytest.mark.parametrize("moving", [False, True])
def test_cdf_fused_matches_split_bitwise(O, moving):
    vel = (0.0, 0.0, 0.01) if moving else (0.0, 0.0, 0.0)
    a = _fused_split_scene(O, False, vel)
    b = _fused_split_scene(O, True, vel)
    for _ in range(8):
        a.step(DT, SUB)
        b.step(DT, SUB)
    for name in ("x", "v", "F"):
        assert np.array_equal(getattr(a, name)(), getattr(b, name)()), name
    assert np.array_equal(a.a["stress"], b.a["stress"])


def test_static_pose_stamps_once(O):
    for fused in (False, True):
        s = _fused_split_scene(O, fused, (0.0, 0.0, 0.0))
        for _ in range(5):
            s.step(DT, SUB)
        assert s.cdf_grids()[2] == 1
        m = _fused_split_scene(O, fused, (0.0, 0.0, 0.01))
        for _ in range(2):
            m.step(DT, SUB)
        assert m.cdf_grids()[2] == 2 * SUB
