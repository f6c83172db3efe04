"""Mesh -> field builders on the GPU against the oracle and against the reference's
own outputs (tests/golden/mesh_fields.npz, from tests/golden/make_mesh_fields.py)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import mesh_oracle

pytestmark = pytest.mark.gpu
G = np.load(Path(__file__).resolve().parent / "golden" / "mesh_fields.npz")


def test_nearest_sample_is_exact(cuda):
    """Index and float64 distance identical to the brute-force oracle, on the field
    grid and on scattered points, including duplicated samples (ties go to the
    lowest index)."""
    from mpm_engine_gb300 import meshfield
    v, f = meshfield.make_cup_mesh(n_theta=24)
    origin, cell, _ = meshfield.field_grid(v, 28, 3.0)
    s = meshfield.surface_samples(v, f, 0.4 * cell)
    s = np.concatenate([s, s[::7]])                        # exact duplicates at higher indices
    d, i = meshfield.nearest_samples(s, grid=(origin, cell, 28))
    do, io = mesh_oracle.nearest_sample(meshfield.grid_points(origin, cell, 28), s)
    np.testing.assert_array_equal(d, do)
    np.testing.assert_array_equal(i, io)
    rng = np.random.default_rng(5)
    pts = rng.uniform(v.min(0) - 0.05, v.max(0) + 0.05, size=(2000, 3))
    pts[:50] = s[rng.integers(0, len(s), 50)]             # queries on samples: distance 0
    d, i = meshfield.nearest_samples(s, points=pts)
    do, io = mesh_oracle.nearest_sample(pts, s)
    np.testing.assert_array_equal(d, do)
    np.testing.assert_array_equal(i, io)
    assert (d[:50] == 0.0).all()


def test_winding_numbers(cuda):
    from mpm_engine_gb300 import meshfield
    v, f = meshfield.make_cup_mesh(n_theta=24)
    rng = np.random.default_rng(6)
    pts = rng.uniform(v.min(0) - 0.02, v.max(0) + 0.02, size=(3000, 3))
    ref = mesh_oracle.winding_number(pts, v, f)
    fast = meshfield.winding_numbers(v, f, points=pts)
    exact = meshfield.winding_numbers(v, f, points=pts, precise=True)
    np.testing.assert_allclose(exact, ref, rtol=0, atol=1e-12)
    np.testing.assert_allclose(fast, ref, rtol=0, atol=1e-4)
    # the inside decision is the float64 one everywhere
    assert ((fast > 0.5) == (ref > 0.5)).all() and ((fast < -0.5) == (ref < -0.5)).all()
    np.testing.assert_allclose(meshfield.winding_numbers(G["cup_v"], G["cup_f"], points=G["pts"], precise=True),
                               G["wn"], rtol=0, atol=1e-12)


def test_triangle_distance(cuda):
    from mpm_engine_gb300 import meshfield
    np.testing.assert_allclose(meshfield.triangle_distance(G["cup_v"], G["cup_f"], points=G["pts"]), G["tri"],
                               rtol=1e-12, atol=1e-15)
    v, f = meshfield.make_cup_mesh(n_theta=20)
    origin, cell, _ = meshfield.field_grid(v, 20, 2.0)
    got = meshfield.triangle_distance(v, f, grid=(origin, cell, 20))
    ref = mesh_oracle.triangle_distance(meshfield.grid_points(origin, cell, 20), v, f)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("tag, kw", [("sdf_kd", {}), ("sdf_ex", {"method": "exact"}),
                                     ("sdf_probe", {"interior_probe": (0.0, 0.0, 0.01)})])
def test_build_sdf_matches_reference(cuda, tag, kw):
    """scipy path (samples), no-scipy path (exact) and an explicit probe, against the
    reference's build_sdf on the same mesh and grid."""
    from mpm_engine_gb300 import meshfield
    sdf = meshfield.build_sdf(G["cup_v"], G["cup_f"], res=int(G["res"]), margin_cells=float(G["margin"]), **kw)
    np.testing.assert_array_equal(sdf.origin, G[f"{tag}_origin"])
    assert sdf.cell == float(G[f"{tag}_cell"])
    tol = 0.0 if tag != "sdf_ex" else 1e-13
    np.testing.assert_allclose(sdf.values, G[f"{tag}_values"], rtol=tol, atol=tol)
    np.testing.assert_allclose(sdf.grads, G[f"{tag}_grads"], rtol=1e-12, atol=1e-11)
    assert abs(sdf.sdf_max - float(G[f"{tag}_sdf_max"])) <= 1e-13


@pytest.mark.parametrize("tag", ["cdf_kd", "cdf_bf"])
def test_build_surface_cdf_matches_reference(cuda, tag):
    from mpm_engine_gb300 import meshfield
    cdf = meshfield.build_surface_cdf(G["open_v"], G["open_f"], res=int(G["res"]), band_cells=float(G["band_cells"]),
                                      margin_cells=float(G["margin"]))
    np.testing.assert_array_equal(cdf.values, G[f"{tag}_values"])
    np.testing.assert_array_equal(cdf.valid, G[f"{tag}_valid"])
    np.testing.assert_array_equal(cdf.origin, G[f"{tag}_origin"])
    assert cdf.cell == float(G[f"{tag}_cell"]) and cdf.band == float(G[f"{tag}_band"])


def test_built_cdf_drives_a_collider(cuda, tmp_path):
    """A glass CDF built from its open mid-surface mesh loads into a Solver as a CPIC
    collider, holds water falling onto its floor, and round-trips the reference's
    cache format. The band is 4 CDF cells (9 mm, over 2 dx), as CPIC needs it
    wider than 1.5 grid cells."""
    from mpm_engine_gb300 import GridConfig, Solver, meshfield, newtonian
    v, f = meshfield.revolve_profile_open([(0.0, 0.004), (0.031, 0.004), (0.033, 0.006), (0.033, 0.07)], n_theta=32)
    cdf = meshfield.build_surface_cdf_cached(v, f, res=40, band_cells=4.0, margin_cells=5.0, cache_dir=tmp_path)
    again = meshfield.build_surface_cdf_cached(v, f, res=40, band_cells=4.0, margin_cells=5.0, cache_dir=tmp_path)
    np.testing.assert_array_equal(cdf.values, again.values)
    assert len(list(tmp_path.glob("cdf_*.npz"))) == 1
    rng = np.random.default_rng(0)
    pos = (rng.uniform(-0.02, 0.02, size=(2000, 3)) + (0.2, 0.2, 0.095)).astype(np.float32)
    s = Solver(grid=GridConfig(96, 0.4)).load_particles(pos, np.full(len(pos), 2e-8, np.float32))
    s.set_material(newtonian(eta=0.5, density=1000.0, bulk_modulus=2e4))
    s.add_domain_walls()
    s.add_cdf_collider(cdf, (0.2, 0.2, 0.05))
    s.set_v(np.tile(np.array([0.0, 0.0, -1.0], np.float32), (len(pos), 1)))
    s.step(1e-4, 400)                 # free fall would take the lowest particles to z = 0.027
    x = s.x()
    assert np.isfinite(x).all()
    assert x[:, 2].min() > 0.05       # held on the glass floor sheet (z = 0.054 in the scene)
