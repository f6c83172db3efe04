"""Generate tests/golden/mesh_fields.npz from the reference's mesh -> field builders.

Run in a checkout where the reference (kks32/mpm-engine) is available:

    python tests/golden/make_mesh_fields.py /path/to/mpm-engine

src/warpmpm/geometry/mesh_sdf.py is numpy-only (scipy optional), so it is imported
from its file (the package __init__ pulls in Warp). Both of its distance paths are
recorded: with scipy (cKDTree over surface samples, the default) and without it
(exact point-triangle distance for build_sdf, brute-force nearest sample for
build_surface_cdf), the latter by hiding scipy.spatial during the call.
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


def _without_scipy(fn, *args, **kw):
    saved = sys.modules.get("scipy.spatial", None)
    had = "scipy.spatial" in sys.modules
    sys.modules["scipy.spatial"] = None          # `from scipy.spatial import ...` now raises ImportError
    try:
        return fn(*args, **kw)
    finally:
        if had:
            sys.modules["scipy.spatial"] = saved
        else:
            del sys.modules["scipy.spatial"]


# the open glass mid-surface used here: floor from the axis, then the wall up to the rim
OPEN_PROFILE = [(0.0, 0.004), (0.031, 0.004), (0.033, 0.006), (0.033, 0.07)]
RES, MARGIN, BAND = 16, 3.0, 2.5


def main(ref_root: str) -> None:
    m = _load(Path(ref_root) / "src/warpmpm/geometry/mesh_sdf.py", "ref_mesh_sdf")
    cup_v, cup_f = m.make_cup_mesh(n_theta=12)
    open_v, open_f = m.revolve_profile_open(OPEN_PROFILE, n_theta=12)
    closed_v, closed_f = m.revolve_profile([(0.0, 0.0), (0.02, 0.0), (0.02, 0.03), (0.0, 0.03)], n_theta=10)
    spacing = 0.0031
    s_all = m._sample_surface(cup_v, cup_f, spacing)
    s_face, s_fid = m._sample_surface_with_faces(open_v, open_f, spacing)
    rim = m._boundary_loop_samples(open_v, open_f, spacing)
    rng = np.random.default_rng(2024)
    lo, hi = cup_v.min(axis=0), cup_v.max(axis=0)
    pts = rng.uniform(lo - 0.01, hi + 0.01, size=(300, 3))
    a, b, c = cup_v[cup_f[:, 0]], cup_v[cup_f[:, 1]], cup_v[cup_f[:, 2]]
    wn = m._winding_number(pts, cup_v, cup_f)
    tri = m._point_triangle_distance_exact(pts, a, b, c)

    sdf_kd = m.build_sdf(cup_v, cup_f, res=RES, margin_cells=MARGIN)
    sdf_ex = _without_scipy(m.build_sdf, cup_v, cup_f, res=RES, margin_cells=MARGIN)
    probe = np.array([0.0, 0.0, 0.01])
    sdf_probe = m.build_sdf(cup_v, cup_f, res=RES, margin_cells=MARGIN, interior_probe=probe)
    cdf_kd = m.build_surface_cdf(open_v, open_f, res=RES, band_cells=BAND, margin_cells=MARGIN)
    cdf_bf = _without_scipy(m.build_surface_cdf, open_v, open_f, res=RES, band_cells=BAND, margin_cells=MARGIN)

    out = dict(cup_v=cup_v, cup_f=cup_f, open_v=open_v, open_f=open_f, closed_v=closed_v, closed_f=closed_f,
               open_profile=np.asarray(OPEN_PROFILE), spacing=spacing, samples_all=s_all, samples_face=s_face,
               samples_fid=s_fid, rim=rim, pts=pts, wn=wn, tri=tri, res=RES, margin=MARGIN, band_cells=BAND,
               probe=probe)
    for tag, f in (("sdf_kd", sdf_kd), ("sdf_ex", sdf_ex), ("sdf_probe", sdf_probe)):
        out[f"{tag}_values"] = f.values
        out[f"{tag}_grads"] = f.grads
        out[f"{tag}_origin"] = f.origin
        out[f"{tag}_cell"] = f.cell
        out[f"{tag}_sdf_max"] = f.sdf_max
    for tag, f in (("cdf_kd", cdf_kd), ("cdf_bf", cdf_bf)):
        out[f"{tag}_values"] = f.values
        out[f"{tag}_valid"] = f.valid
        out[f"{tag}_origin"] = f.origin
        out[f"{tag}_cell"] = f.cell
        out[f"{tag}_band"] = f.band
    np.savez_compressed(OUT / "mesh_fields.npz", **out)
    print("wrote", OUT / "mesh_fields.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <reference checkout root>")
    main(sys.argv[1])
