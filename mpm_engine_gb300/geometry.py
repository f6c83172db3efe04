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


@dataclass
class CDFData:
    """Side-signed distance field around an OPEN oriented sheet for CPIC colliders
    (warpmpm.geometry.CDFData, src/warpmpm/geometry/mesh_sdf.py:47-76)."""
    values: np.ndarray      # [res,res,res] signed distance to the sheet (m)
    valid: np.ndarray       # [res,res,res] 1 where distance and side are trustworthy
    origin: np.ndarray
    cell: float
    band: float             # metres from the sheet within which valid can be 1

    @property
    def res(self) -> int:
        return int(self.values.shape[0])


def save_cdf(cdf: CDFData, path) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, values=cdf.values, valid=cdf.valid, origin=cdf.origin, cell=cdf.cell, band=cdf.band)


def load_cdf(path) -> CDFData:
    d = np.load(path)
    return CDFData(values=d["values"], valid=d["valid"], origin=d["origin"], cell=float(d["cell"]),
                   band=float(d["band"]))


def sheet_cdf(normal: str = "z", size: float = 0.5, res: int = 64, band_cells: float = 3.0,
              margin_cells: float = 4.0) -> CDFData:
    """CDF of a square sheet of edge `size` through the body origin with normal +x or +z,
    on the grid build_surface_cdf uses (mesh_sdf.py:412-480): distance to the sheet,
    side from its normal, valid within `band` of the sheet and farther than `band`
    from its open rim."""
    span = float(size)
    cell = span / (res - 1 - 2 * margin_cells)
    band = band_cells * cell
    L = cell * (res - 1)
    origin = np.full(3, -0.5 * L)
    ax = origin[0] + cell * np.arange(res)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    if normal == "x":
        dn, u, v = X, Y, Z
    elif normal == "z":
        dn, u, v = Z, X, Y
    else:
        raise ValueError("normal must be 'x' or 'z'")
    h = 0.5 * size
    # distance to the square patch and to its rim (the patch boundary)
    du = np.maximum(np.abs(u) - h, 0.0)
    dv = np.maximum(np.abs(v) - h, 0.0)
    dist = np.sqrt(dn * dn + du * du + dv * dv)
    side = np.where(dn >= 0.0, 1.0, -1.0)
    eu = np.abs(np.abs(u) - h)
    ev = np.abs(np.abs(v) - h)
    inside_u = np.abs(u) <= h
    inside_v = np.abs(v) <= h
    rim_u = np.sqrt(dn * dn + eu * eu + np.where(inside_v, 0.0, dv * dv))   # distance to the u = +-h edges
    rim_v = np.sqrt(dn * dn + ev * ev + np.where(inside_u, 0.0, du * du))
    rim = np.minimum(rim_u, rim_v)
    valid = ((dist <= band) & (rim > band)).astype(np.float64)
    return CDFData(values=side * dist, valid=valid, origin=origin, cell=float(cell), band=float(band))


def revolved_open_cdf(profile_rz, res: int = 96, band_cells: float = 3.0, margin_cells: float = 4.0) -> CDFData:
    """CDF of the open surface of revolution of an (r, z) polyline about the z axis,
    on the grid build_surface_cdf uses for its revolved mesh (mesh_sdf.py:412-480):
    exact distance to the surface (the distance in the meridian plane), side from
    the normal of the nearest segment (the tangent turned +90 degrees in (r, z), so
    a profile traced floor-then-wall gives +1 inside the cavity), valid within
    `band` of the surface and farther than `band` from the open rim (the last
    polyline vertex; the first lies on the axis)."""
    P = np.asarray(profile_rz, dtype=np.float64)
    rmax = float(P[:, 0].max())
    zmin, zmax = float(P[:, 1].min()), float(P[:, 1].max())
    span = max(2.0 * rmax, zmax - zmin)
    cell = span / (res - 1 - 2 * margin_cells)
    band = band_cells * cell
    L = cell * (res - 1)
    center = np.array([0.0, 0.0, 0.5 * (zmin + zmax)])
    origin = center - 0.5 * L
    ax = [origin[d] + cell * np.arange(res) for d in range(3)]
    X, Y, Z = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
    R = np.sqrt(X * X + Y * Y)
    best = np.full(R.shape, np.inf)
    side = np.ones(R.shape)
    for a, b in zip(P[:-1], P[1:]):
        t = b - a
        tl2 = float(t @ t)
        u = np.clip(((R - a[0]) * t[0] + (Z - a[1]) * t[1]) / tl2, 0.0, 1.0)
        cr, cz = a[0] + u * t[0], a[1] + u * t[1]
        d = np.sqrt((R - cr) ** 2 + (Z - cz) ** 2)
        n = np.array([-t[1], t[0]]) / np.sqrt(tl2)
        s_seg = np.where((R - cr) * n[0] + (Z - cz) * n[1] >= 0.0, 1.0, -1.0)
        closer = d < best
        best = np.where(closer, d, best)
        side = np.where(closer, s_seg, side)
    rim = np.sqrt((R - P[-1, 0]) ** 2 + (Z - P[-1, 1]) ** 2)
    valid = ((best <= band) & (rim > band)).astype(np.float64)
    return CDFData(values=side * best, valid=valid, origin=origin, cell=float(cell), band=float(band))


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


__all__ = ["CDFData", "SDFData", "analytic_sdf", "load_cdf", "load_sdf", "revolved_open_cdf", "save_cdf", "save_sdf",
           "sheet_cdf"]
