"""Host glass helpers of mpm_engine_gb300.glass against the reference's outputs
(golden/glass_tools.npz, written by golden/make_glass_tools.py from
src/warpmpm/colliders/glass.py). Quaternions, signed distances, masks and the
projection out of the solid are float64 on both sides and agree to rounding; masks
and projection counts exactly; the render mesh line for line below its header
comment."""
from pathlib import Path

import numpy as np

from mpm_engine_gb300 import glass as g

D = np.load(Path(__file__).resolve().parent / "golden" / "glass_tools.npz")


def test_quaternion_helpers():
    got = np.stack([g.quat_from_mat(m) for m in D["mats"]])
    np.testing.assert_allclose(got, D["quat_from_mat"], rtol=0, atol=1e-14)
    np.testing.assert_array_equal(np.stack([g.quat_conj(q) for q in D["quats"]]), D["quat_conj"])


def test_posed_glass_sdf_and_masks():
    pts, pos, quat, prof = D["pts"], D["pos"], D["quat"], g.GlassProfile()
    np.testing.assert_allclose(g.glass_sdf(pts, pos, quat, prof), D["glass_sdf"], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(g.cavity_mask(pts, pos, quat, prof), D["cavity_mask"])
    np.testing.assert_array_equal(g.cavity_mask(pts, pos, quat, prof, pad=0.004, brim_clearance=0.01),
                                  D["cavity_mask_pad"])
    np.testing.assert_array_equal(g.solid_mask(pts, pos, quat, prof), D["solid_mask"])
    np.testing.assert_array_equal(g.solid_mask(pts, pos, quat, prof, tol=0.002), D["solid_mask_tol"])


def test_project_out_of_solid():
    pts, v, pos, quat, prof = D["pts"], D["v"], D["pos"], D["quat"], g.GlassProfile()
    for tag, sv in (("static", None), ("moving", (np.array([0.1, -0.05, 0.02]), np.array([0.0, 1.5, -0.4])))):
        xn, vn, nb = g.project_out_of_solid(pts, v, pos, quat, prof, clearance=0.001, solid_velocity=sv)
        assert nb == int(D[f"proj_{tag}_n"]) > 0
        np.testing.assert_allclose(xn, D[f"proj_{tag}_x"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(vn, D[f"proj_{tag}_v"], rtol=0, atol=1e-12)
        assert not g.solid_mask(xn, pos, quat, prof, tol=1e-9).any()
    x0 = pts.copy()
    g.project_out_of_solid(pts, v, pos, quat, prof)
    np.testing.assert_array_equal(pts, x0)               # inputs untouched
