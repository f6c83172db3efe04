"""Signed-distance-field data format for mesh colliders.

`SDFData` has the fields of warpmpm.geometry.SDFData (src/warpmpm/geometry/mesh_sdf.py:25-44)
and the same npz cache format (save_sdf / load_sdf, :538-548), so fields built by
the reference's host builders load here unchanged. The mesh -> SDF builder itself
(winding numbers, point-triangle distances) is host preprocessing outside the
simulation step; `analytic_sdf` builds fields of simple shapes for tests.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np


@dataclass
class SDFData:
    values: np.ndarray      # [res,res,res] signed distance (m), negative inside
    grads: np.ndarray       # [res,res,res,3] outward gradient
    origin: np.ndarray      # body-frame coordinate of voxel (0,0,0)
    cell: float             # metres per voxel
    sdf_max: float

    @property
    def res(self) -> int:
        return int(self.values.shape[0])


def save_sdf(sdf: SDFData, path) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, values=sdf.values, grads=sdf.grads, origin=sdf.origin, cell=sdf.cell,
                        sdf_max=sdf.sdf_max)


def load_sdf(path) -> SDFData:
    d = np.load(path)
    return SDFData(values=d["values"], grads=d["grads"], origin=d["origin"], cell=float(d["cell"]),
                   sdf_max=float(d["sdf_max"]))


def analytic_sdf(kind: str, res: int = 48, half_extent=(0.05, 0.05, 0.05), radius: float = 0.05,
                 margin: float = 0.02) -> SDFData:
    """Voxel SDF of a box (half extents) or sphere (radius) centred at the body origin,
    with a numerical outward gradient."""
    ext = (max(half_extent) if kind == "box" else radius) + margin
    origin = np.full(3, -ext)
    cell = 2.0 * ext / (res - 1)
    ax = origin[0] + cell * np.arange(res)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    P = np.stack([X, Y, Z], axis=-1)
    if kind == "sphere":
        vals = np.linalg.norm(P, axis=-1) - radius
    elif kind == "box":
        q = np.abs(P) - np.asarray(half_extent)
        vals = np.linalg.norm(np.maximum(q, 0.0), axis=-1) + np.minimum(q.max(-1), 0.0)
    else:
        raise ValueError(f"unknown analytic sdf kind {kind!r}")
    grads = np.stack(np.gradient(vals, cell), axis=-1)
    return SDFData(values=vals, grads=grads, origin=origin, cell=float(cell), sdf_max=float(vals.max()))


__all__ = ["SDFData", "analytic_sdf", "load_sdf", "save_sdf"]
