"""Generate glass_tools.npz: outputs of the reference's host glass helpers
(src/warpmpm/colliders/glass.py) on seeded inputs, for tests/test_glass_tools_host.py.
The module is pure numpy and is loaded from its file, so Warp is not needed.

    python tests/golden/make_glass_tools.py <reference_root>
"""
from __future__ import annotations

import importlib.util
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
    g = _load(Path(ref_root) / "src/warpmpm/colliders/glass.py", "ref_glass")
    rng = np.random.default_rng(77)
    out = {}
    # rotations: random, plus the half turns and near half turns that take each branch
    quats = rng.normal(size=(40, 4))
    quats /= np.linalg.norm(quats, axis=1, keepdims=True)
    extra = [g.quat_from_axis_angle(ax, a) for ax in np.eye(3) for a in (np.pi, np.pi - 1e-3, 0.3)]
    quats = np.vstack([quats, np.asarray(extra)])
    mats = np.stack([g.quat_to_mat(q) for q in quats])
    out["mats"] = mats
    out["quat_from_mat"] = np.stack([g.quat_from_mat(m) for m in mats])
    out["quats"] = quats
    out["quat_conj"] = np.stack([g.quat_conj(q) for q in quats])
    # a posed glass: SDF and masks on points around it
    prof = g.GlassProfile()
    pos = np.array([0.3, 0.4, 0.2])
    quat = g.quat_from_axis_angle([0.3, 1.0, 0.1], 0.7)
    pts = pos + rng.uniform(-0.14, 0.14, size=(2000, 3))
    out["pos"], out["quat"], out["pts"] = pos, quat, pts
    out["glass_sdf"] = g.glass_sdf(pts, pos, quat, prof)
    out["cavity_mask"] = g.cavity_mask(pts, pos, quat, prof)
    out["cavity_mask_pad"] = g.cavity_mask(pts, pos, quat, prof, pad=0.004, brim_clearance=0.01)
    out["solid_mask"] = g.solid_mask(pts, pos, quat, prof)
    out["solid_mask_tol"] = g.solid_mask(pts, pos, quat, prof, tol=0.002)
    # projection out of the solid: static wall and a moving, spinning wall
    v = rng.normal(scale=0.3, size=pts.shape)
    out["v"] = v
    for tag, sv in (("static", None), ("moving", (np.array([0.1, -0.05, 0.02]), np.array([0.0, 1.5, -0.4])))):
        xn, vn, nb = g.project_out_of_solid(pts, v, pos, quat, prof, clearance=0.001, solid_velocity=sv)
        out[f"proj_{tag}_x"], out[f"proj_{tag}_v"], out[f"proj_{tag}_n"] = xn, vn, np.int64(nb)
    np.savez_compressed(OUT / "glass_tools.npz", **out)
    print(OUT / "glass_tools.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <reference checkout root>")
    main(sys.argv[1])
