"""Hooks of MPM_Simulator_WARP that scripts and the reference's tests reach through
Solver._sim, restated from the reference suite: tests/test_cuda_graph.py:37-48
(graph replay), tests/test_restricted_launch.py:50-64 (launch boxes),
tests/test_cdf_collider.py:40-75 (stamp bits of a sheet built from its mesh) and
tests/test_cdf_stamp_skip.py:35-95 (the static-lane stamp skip). The reference runs
these on its CPU backend and asserts bitwise equality between runs; float atomics
make GPU runs agree to rounding instead, so those checks take a 1e-6 bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sphere_scene(use_graph):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    from mpm_engine_gb300.geometry import analytic_sdf
    grid = GridConfig(n_grid=64, grid_lim=0.4)
    h = grid.dx / 2
    ax = np.arange(-0.03 + h / 2, 0.03, h)
    pts = (np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3) + (0.2, 0.2, 0.165)).astype(np.float32)
    s = Solver(grid=grid, fused=False).load_particles(pts, np.full(len(pts), h ** 3, np.float32))
    s.set_material(newtonian(eta=5.0, density=1000.0, bulk_modulus=5.0e5))
    s.add_plane((0, 0, 3 * grid.dx), (0, 0, 1), "slip", friction=0.2)
    h = s.add_sdf_collider(analytic_sdf("sphere", radius=0.04), center=(0.2, 0.2, 0.09), surface="separable",
                           friction=0.3)
    s._sim.use_cuda_graph = use_graph
    return s, h


def test_graph_matches_live(cuda):
    sa, ha = _sphere_scene(True)
    sb, hb = _sphere_scene(False)
    dt = 5.0e-5   # under the acoustic limit 0.3 dx / sqrt(K / rho) = 8.4e-5 s
    for _ in range(20):
        sa.step(dt, substeps=4)
        sb.step(dt, substeps=4)
    assert sa._sim._graph_A is not None, "graph capture never engaged"
    assert sb._sim._graph_A is None
    assert np.isfinite(sa.x()).all()
    np.testing.assert_allclose(sa.x(), sb.x(), rtol=1e-5, atol=1e-6)
    wa, wb = sa.sdf_wrench(ha, dt * 4), sb.sdf_wrench(hb, dt * 4)
    np.testing.assert_allclose(wa["force"], wb["force"], rtol=1e-3, atol=1e-5)


def test_collider_outside_domain_has_no_launch_box(cuda):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    from mpm_engine_gb300.geometry import analytic_sdf
    grid = GridConfig(n_grid=48, grid_lim=0.4)
    pts = (np.random.default_rng(1).uniform(-0.03, 0.03, (2000, 3)) + 0.2).astype(np.float32)
    s = Solver(grid=grid).load_particles(pts, np.full(len(pts), 1e-8, np.float32))
    s.set_material(newtonian(eta=5.0, density=1000.0, bulk_modulus=5.0e5))
    s.add_plane((0, 0, 3 * grid.dx), (0, 0, 1), "slip", friction=0.2)
    s.add_sdf_collider(analytic_sdf("sphere", radius=0.04), center=(5.0, 5.0, 5.0), surface="separable")
    assert s._sim.collider_aabbs[-1]() is None, "a far-away collider reaches no node"
    assert s._sim.collider_aabbs[0]() is not None    # the floor plane spans the grid
    s.step(2.0e-4, substeps=2)
    assert np.isfinite(s.x()).all()


def _mesh_sheet_cdf(size=0.3, res=64):
    """Horizontal square sheet at z = 0, normals +z, built from its two triangles."""
    from mpm_engine_gb300.meshfield import build_surface_cdf
    v = np.array([[-size / 2, -size / 2, 0], [size / 2, -size / 2, 0], [size / 2, size / 2, 0],
                  [-size / 2, size / 2, 0]], dtype=float)
    f = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int64)
    return build_surface_cdf(v, f, res=res, band_cells=6.0)


def test_stamp_bits_match_analytic_plane(cuda):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    g = GridConfig(n_grid=32, grid_lim=0.4)
    s = Solver(grid=g, fused=False)
    s.load_particles(np.full((8, 3), 0.2, np.float32) +
                     np.random.default_rng(0).uniform(0, 0.01, (8, 3)).astype(np.float32),
                     np.full(8, (g.dx / 2) ** 3, np.float32))
    s.set_material(newtonian(eta=0.2, density=1000.0, bulk_modulus=5.0e4))
    z0 = 0.2
    h = s.add_cdf_collider(_mesh_sheet_cdf(), center=(0.2, 0.2, z0), band=2.5 * g.dx)
    assert h == 0
    s._sim._stamp_cdf(1e-4, "cuda")
    tag = s._sim.mpm_state.grid_cdf_tag.numpy()
    k0 = z0 / g.dx
    ij = np.arange(int(0.15 / g.dx), int(0.25 / g.dx))
    above = tag[np.ix_(ij, ij, [int(k0 + 1), int(k0 + 2)])]
    below = tag[np.ix_(ij, ij, [int(k0 - 1), int(k0 - 2)])]
    assert np.all(above & 1) and np.all(above & 2), "valid and side bits above the sheet"
    assert np.all(below & 1) and np.all(below & 2 == 0), "valid bit, side bit clear below"
    far = tag[np.ix_(ij, ij, [int(k0 + 5), int(k0 - 5)])]
    assert np.all(far == 0), "beyond the band untagged"
    assert np.all(tag[int(0.05 / g.dx), ij, int(k0 + 1)] == 0), "rim tube untagged"
    d = s._sim.mpm_state.grid_cdf_d.numpy()
    zs = int(k0 + 1) * g.dx - z0
    assert np.allclose(d[np.ix_(ij, ij, [int(k0 + 1)])], abs(zs), atol=0.1 * g.dx)


def _shelf_run(fused, force, ticks=5, sub=10, dt=2e-4):
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    from mpm_engine_gb300.geometry import sheet_cdf
    g = GridConfig(n_grid=32, grid_lim=0.4)
    hp = g.dx / 2
    ax = np.arange(0.14 + hp / 2, 0.26, hp)
    az = np.arange(0.21 + hp / 2, 0.27, hp)
    pos = np.stack(np.meshgrid(ax, ax, az, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    s = Solver(grid=g, fused=fused).load_particles(pos, np.full(len(pos), hp ** 3, np.float32))
    s.set_material(newtonian(eta=0.5, density=1000.0, bulk_modulus=5.0e4), g=[0.0, 0.0, -9.81])
    s.add_plane((0, 0, 3 * g.dx), (0, 0, 1), "slip")
    s.add_domain_walls()
    s.add_cdf_collider(sheet_cdf("z", size=0.5), center=(0.2, 0.2, 0.20), friction=0.3)
    s._sim._cdf_force_stamp = force
    for _ in range(ticks):
        s.step(dt, sub)
    return s.x(), s.v(), s._sim._cdf_stamp_count


@pytest.mark.parametrize("fused", [False, True])
def test_static_shelf_stamps_once_and_forcing_changes_nothing(cuda, fused):
    x_skip, v_skip, n_skip = _shelf_run(fused, force=False)
    x_all, v_all, n_all = _shelf_run(fused, force=True)
    assert n_skip == 1, f"a static pose stamps once, got {n_skip}"
    assert n_all == 5 * 10
    np.testing.assert_allclose(x_all, x_skip, rtol=0, atol=1e-6)
    np.testing.assert_allclose(v_all, v_skip, rtol=0, atol=1e-6 + 1e-5 * float(np.abs(v_skip).max()))
