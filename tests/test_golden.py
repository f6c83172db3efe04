"""Host logic and oracle pinned against fixtures generated from the reference's own
modules (tests/golden/make_golden.py): glass SDF, cup fill, material mapping, sort keys."""
import json
from pathlib import Path

import numpy as np
import pytest

from mpm_engine_gb300 import glass, materials

G = Path(__file__).resolve().parent / "golden"


def test_glass_sdf_matches_reference_float64():
    d = np.load(G / "glass_sdf.npz")
    np.testing.assert_array_equal(glass.glass_sdf_local(d["points"], glass.GlassProfile()), d["sdf_default"])
    thin = glass.GlassProfile(outer_radius=0.06, inner_radius=0.05, height=0.16, base_thickness=0.02,
                              fillet_radius=0.006)
    np.testing.assert_array_equal(glass.glass_sdf_local(d["points"], thin), d["sdf_thin"])
    np.testing.assert_array_equal(glass.GlassProfile().inner_radius_at_z(np.linspace(-0.12, 0.12, 101)),
                                  d["inner_radius_at_z"])


def test_oracle_glass_sdf_fp32_within_rounding(oracle_lib):
    """The collider kernels' fp32 SDF (oracle restatement) against the reference's float64 twin."""
    import ctypes as C
    from mpm_engine_gb300 import host
    d = np.load(G / "glass_sdf.npz")
    p = glass.GlassProfile()
    rec = host.cup_collider((0, 0, 0), np.eye(3), outer_radius=p.outer_radius, inner_radius=p.inner_radius,
                            half_height=p.half_height, inner_floor_z=p.inner_floor_z, fillet_radius=p.fillet_radius)
    lib = oracle_lib.load()
    pts = d["points"].astype(np.float32)
    out = np.array([lib.gbmpm_oracle_glass_sdf(C.byref(rec), pts[i].ctypes.data) for i in range(len(pts))])
    np.testing.assert_allclose(out, d["sdf_default"], atol=2e-7)


def test_cup_fill_pour_geometry_is_the_reference_340k():
    d = np.load(G / "cup_fill.npz")
    for tag, n_grid in (("n192", 192), ("n96", 96)):
        pos, vol = glass.cup_fill(glass.GlassProfile(), 0.7 / n_grid / 2, fill_fraction=0.80)
        assert len(pos) == int(d[f"{tag}_count"])
        np.testing.assert_array_equal(pos[:16], d[f"{tag}_head"])
        np.testing.assert_array_equal(pos[-16:], d[f"{tag}_tail"])
        np.testing.assert_allclose(pos.astype(np.float64).sum(0), d[f"{tag}_sum"], rtol=0, atol=1e-9)
        assert vol[0] == d[f"{tag}_vol"][0]
    assert int(d["n192_count"]) == 340489
    pos, _ = glass.cup_fill(glass.GlassProfile(), 0.7 / 96 / 2, fill_fraction=0.80)
    np.testing.assert_array_equal(pos, d["n96_pos"])


def test_material_resolve_matches_reference():
    ref = json.loads((G / "materials.json").read_text())
    cases = {
        "newtonian": materials.newtonian(eta=10.0, density=1420.0, bulk_modulus=9.0e5),
        "bingham": materials.newtonian(eta=40.0).with_yield(200.0),
        "herschel_bulkley": materials.newtonian(eta=0.0, density=1400.0).with_yield(50.0).with_powerlaw(K=20.0, n=0.6),
        "granular": materials.granular(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1e6, nu=0.3),
        "granular_phi": materials.granular(mu_s=0.38).with_dilatancy(phi_init=0.58, chi=0.25),
        "elastic": materials.elastic(E=2e5, nu=0.25, density=1100.0),
        "vonmises": materials.vonmises(E=5e5, nu=0.3, yield_stress=2e3),
        "vonmises_hard": materials.vonmises(E=5e5, nu=0.3, yield_stress=2e3, hardening_xi=0.5),
        "tabulated": materials.tabulated_viscous([5.0, 3.0, 1.5, 1.0], smin=-1.0, smax=2.0),
    }
    for k, m in cases.items():
        name, params = m.resolve()
        assert name == ref["resolve"][k]["name"], k
        assert json.loads(json.dumps(params)) == ref["resolve"][k]["params"], k
    bad = {"tab_short": materials.tabulated_viscous([1.0]), "tab_neg": materials.tabulated_viscous([1.0, -1.0]),
           "tab_range": materials.tabulated_viscous([1.0, 2.0], smin=2.0, smax=1.0)}
    for k, m in bad.items():
        with pytest.raises(ValueError) as e:
            m.resolve()
        assert str(e.value) == ref["errors"][k]


def test_oracle_sort_keys_and_stable_permutation(oracle_lib):
    d = np.load(G / "sort_keys.npz")
    moved, perm, keys = oracle_lib.sort_perm(d["x"], float(d["dx"]), int(d["n_grid"]))
    assert moved
    np.testing.assert_array_equal(keys, d["keys"])
    np.testing.assert_array_equal(perm, d["perm"])
    moved2, _, _ = oracle_lib.sort_perm(d["x"][d["perm"]], float(d["dx"]), int(d["n_grid"]))
    assert not moved2  # already ordered: the reference skips the permutation
