"""Generate the golden fixtures in this folder from the reference's own Python modules.

Run in a checkout where the reference (kks32/mpm-engine) is available:

    python tests/golden/make_golden.py /path/to/mpm-engine

The glass geometry (src/warpmpm/colliders/glass.py) and the material mapping
(src/warpmpm/materials/__init__.py) are pure numpy / Python, so they are
imported directly from their files (the package __init__ pulls in Warp, which is
not needed here). The block-sort keys are produced by the reference's formula
(src/warpmpm/core/solver.py:458-465), evaluated here in numpy on seeded
positions because that module imports Warp.
"""
from __future__ import annotations

import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def _load(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def main(ref_root: str) -> None:
    root = Path(ref_root)
    glass = _load(root / "src/warpmpm/colliders/glass.py", "ref_glass")
    mats = _load(root / "src/warpmpm/materials/__init__.py", "ref_materials")

    # 1. revolved glass SDF on seeded points around the default and a thin profile
    rng = np.random.default_rng(1234)
    pts = rng.uniform(-0.13, 0.13, size=(4000, 3))
    pts[:1000, 2] = rng.uniform(-0.13, -0.02, size=1000)       # denser sampling near the floor fillet
    prof_b = glass.GlassProfile(outer_radius=0.06, inner_radius=0.05, height=0.16, base_thickness=0.02,
                                fillet_radius=0.006)
    np.savez_compressed(OUT / "glass_sdf.npz", points=pts,
                        sdf_default=glass.glass_sdf_local(pts, glass.GlassProfile()),
                        sdf_thin=glass.glass_sdf_local(pts, prof_b),
                        inner_radius_at_z=glass.GlassProfile().inner_radius_at_z(np.linspace(-0.12, 0.12, 101)))

    # 2. the 340k-particle pour fill: GlassProfile() at 80 % on 192^3 / grid_lim 0.7 (h = dx/2),
    #    plus a coarse 96^3 fill kept whole
    out = {}
    for tag, n_grid in (("n192", 192), ("n96", 96)):
        h = 0.7 / n_grid / 2
        pos, vol = glass.cup_fill(glass.GlassProfile(), h, fill_fraction=0.80)
        out[f"{tag}_count"] = np.int64(len(pos))
        out[f"{tag}_sum"] = pos.astype(np.float64).sum(axis=0)
        out[f"{tag}_head"] = pos[:16]
        out[f"{tag}_tail"] = pos[-16:]
        out[f"{tag}_vol"] = vol[:1]
        if n_grid == 96:
            out["n96_pos"] = pos
    np.savez_compressed(OUT / "cup_fill.npz", **out)

    # 3. Material.resolve() of the factories and modifiers
    cases = {
        "newtonian": mats.newtonian(eta=10.0, density=1420.0, bulk_modulus=9.0e5),
        "bingham": mats.newtonian(eta=40.0).with_yield(200.0),
        "herschel_bulkley": mats.newtonian(eta=0.0, density=1400.0).with_yield(50.0).with_powerlaw(K=20.0, n=0.6),
        "granular": mats.granular(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1e6, nu=0.3),
        "granular_phi": mats.granular(mu_s=0.38).with_dilatancy(phi_init=0.58, chi=0.25),
        "elastic": mats.elastic(E=2e5, nu=0.25, density=1100.0),
        "vonmises": mats.vonmises(E=5e5, nu=0.3, yield_stress=2e3),
        "vonmises_hard": mats.vonmises(E=5e5, nu=0.3, yield_stress=2e3, hardening_xi=0.5),
        "tabulated": mats.tabulated_viscous([5.0, 3.0, 1.5, 1.0], smin=-1.0, smax=2.0),
    }
    res = {}
    for k, m in cases.items():
        name, params = m.resolve()
        res[k] = {"name": name, "params": params}
    errors = {}
    for k, m in {"tab_short": mats.tabulated_viscous([1.0]), "tab_neg": mats.tabulated_viscous([1.0, -1.0]),
                 "tab_range": mats.tabulated_viscous([1.0, 2.0], smin=2.0, smax=1.0)}.items():
        try:
            m.resolve()
            errors[k] = None
        except ValueError as e:
            errors[k] = str(e)
    (OUT / "materials.json").write_text(json.dumps({"resolve": res, "errors": errors}, indent=1, sort_keys=True))

    # 4. block-sort keys and stable permutation (solver.py:458-465 formula)
    rng = np.random.default_rng(7)
    n_grid, lim = 64, 0.4
    dx = lim / n_grid
    x = rng.uniform(2 * dx, lim - 3 * dx, size=(5000, 3)).astype(np.float32)
    x[100:200] = x[100]                                         # ties must keep index order
    base = (np.floor(x / dx - 0.5).astype(np.int64)) >> 2
    nb = (n_grid >> 2) + 2
    keys = (base[:, 0] * nb + base[:, 1]) * nb + base[:, 2]
    perm = np.argsort(keys, kind="stable")
    np.savez_compressed(OUT / "sort_keys.npz", x=x, dx=dx, n_grid=n_grid, keys=keys, perm=perm)
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <reference checkout root>")
    main(sys.argv[1])
