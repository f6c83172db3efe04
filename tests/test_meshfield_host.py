"""Mesh -> field builders without a GPU: the procedural meshes and the samplers
reproduce the reference's arrays exactly, and the oracle of the device searches is
pinned against the reference's own outputs (tests/golden/make_mesh_fields.py)."""
from pathlib import Path

import numpy as np
import pytest

from mpm_engine_gb300 import meshfield
from oracle import mesh_oracle

G = np.load(Path(__file__).resolve().parent / "golden" / "mesh_fields.npz")


def test_procedural_meshes_match_reference():
    v, f = meshfield.make_cup_mesh(n_theta=12)
    np.testing.assert_array_equal(v, G["cup_v"])
    np.testing.assert_array_equal(f, G["cup_f"])
    v, f = meshfield.revolve_profile_open(G["open_profile"], n_theta=12)
    np.testing.assert_array_equal(v, G["open_v"])
    np.testing.assert_array_equal(f, G["open_f"])
    v, f = meshfield.revolve_profile([(0.0, 0.0), (0.02, 0.0), (0.02, 0.03), (0.0, 0.03)], n_theta=10)
    np.testing.assert_array_equal(v, G["closed_v"])
    np.testing.assert_array_equal(f, G["closed_f"])


def test_samplers_match_reference_bit_for_bit():
    sp = float(G["spacing"])
    np.testing.assert_array_equal(meshfield.surface_samples(G["cup_v"], G["cup_f"], sp), G["samples_all"])
    s, fid = meshfield.surface_samples(G["open_v"], G["open_f"], sp, with_faces=True)
    np.testing.assert_array_equal(s, G["samples_face"])
    np.testing.assert_array_equal(fid, G["samples_fid"])
    np.testing.assert_array_equal(meshfield.boundary_samples(G["open_v"], G["open_f"], sp), G["rim"])
    assert meshfield.boundary_samples(G["cup_v"], G["cup_f"], sp).shape == (0, 3)   # closed mesh


def test_oracle_winding_and_exact_distance_match_reference():
    np.testing.assert_allclose(mesh_oracle.winding_number(G["pts"], G["cup_v"], G["cup_f"]), G["wn"],
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(mesh_oracle.triangle_distance(G["pts"], G["cup_v"], G["cup_f"]), G["tri"],
                               rtol=1e-12, atol=1e-15)


def test_oracle_nearest_reproduces_reference_cdf_distances():
    """The CDF values are side * nearest-sample distance; the oracle's distances
    equal the reference's (cKDTree and brute force) to the last bit."""
    origin, cell, res = G["cdf_kd_origin"], float(G["cdf_kd_cell"]), int(G["res"])
    pts = meshfield.grid_points(origin, cell, res)
    s, _ = meshfield.surface_samples(G["open_v"], G["open_f"], 0.4 * cell, with_faces=True)
    d, _ = mesh_oracle.nearest_sample(pts, s)
    np.testing.assert_array_equal(d, np.abs(G["cdf_kd_values"]).ravel())
    np.testing.assert_array_equal(d, np.abs(G["cdf_bf_values"]).ravel())


def test_oracle_nearest_reproduces_reference_sdf_magnitudes():
    """build_sdf's magnitudes are the nearest-sample distances (vertices first, then
    the face lattices); the oracle's equal the reference's cKDTree query bit for bit."""
    origin, cell, res = G["sdf_kd_origin"], float(G["sdf_kd_cell"]), int(G["res"])
    s = meshfield.surface_samples(G["cup_v"], G["cup_f"], 0.4 * cell)
    d, _ = mesh_oracle.nearest_sample(meshfield.grid_points(origin, cell, res), s)
    np.testing.assert_array_equal(d, np.abs(G["sdf_kd_values"]).ravel())
    np.testing.assert_array_equal(d, np.abs(G["sdf_probe_values"]).ravel())


def test_field_grid_matches_reference():
    origin, cell, _ = meshfield.field_grid(G["cup_v"], int(G["res"]), float(G["margin"]))
    np.testing.assert_array_equal(origin, G["sdf_kd_origin"])
    assert cell == float(G["sdf_kd_cell"])


def test_builders_refuse_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        meshfield.build_sdf(G["cup_v"], G["cup_f"], res=8, margin_cells=1.0)
