"""Oracle (test infrastructure only) for the mesh -> field searches: a float64 numpy
restatement of the reference's algorithms in src/warpmpm/geometry/mesh_sdf.py, used
by tests to check gbmpm_field_nearest, gbmpm_field_winding and
gbmpm_field_tri_distance. Pinned against tests/golden/mesh_fields.npz, which the
reference's own functions produced (tests/golden/make_mesh_fields.py). Nothing in
the product imports this module.
"""
from __future__ import annotations

import numpy as np


def nearest_sample(points, samples, chunk: int = 1024):
    """Brute-force nearest sample (build_surface_cdf's numpy path, mesh_sdf.py:455-466):
    distance sqrt((dx^2 + dy^2) + dz^2) with the terms added left to right, and the
    first index of the smallest rounded distance."""
    p = np.asarray(points, dtype=np.float64)
    s = np.asarray(samples, dtype=np.float64)
    dist = np.empty(len(p))
    idx = np.empty(len(p), dtype=np.int64)
    for a in range(0, len(p), chunk):
        d = p[a:a + chunk, None, :] - s[None]
        d2 = d[..., 0] * d[..., 0]
        d2 = d2 + d[..., 1] * d[..., 1]
        d2 = d2 + d[..., 2] * d[..., 2]
        r = np.sqrt(d2)
        idx[a:a + chunk] = r.argmin(axis=1)
        dist[a:a + chunk] = r.min(axis=1)
    return dist, idx


def winding_number(points, verts, faces, chunk: int = 512):
    """Generalized winding number (mesh_sdf.py:210-233): sum over faces of the
    Van Oosterom-Strackee solid angle 2 atan2(num, den), divided by 4 pi."""
    p_all = np.asarray(points, dtype=np.float64)
    v = np.asarray(verts, dtype=np.float64)
    f = np.asarray(faces, dtype=np.int64)
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    out = np.empty(len(p_all))
    for s in range(0, len(p_all), chunk):
        p = p_all[s:s + chunk][:, None, :]
        A, B, Cc = a[None] - p, b[None] - p, c[None] - p
        la, lb, lc = (np.sqrt((X * X).sum(axis=2)) for X in (A, B, Cc))
        num = (A * np.cross(B, Cc)).sum(axis=2)
        den = la * lb * lc + (A * B).sum(axis=2) * lc + (B * Cc).sum(axis=2) * la + (Cc * A).sum(axis=2) * lb
        out[s:s + chunk] = (2.0 * np.arctan2(num, den)).sum(axis=1) / (4.0 * np.pi)
    return out


def triangle_distance(points, verts, faces, chunk: int = 512):
    """Exact distance to the nearest triangle (mesh_sdf.py:236-289): closest point by
    barycentric region, vertex and edge regions overriding the interior in the order
    A, B, C, AB, AC, BC."""
    p_all = np.asarray(points, dtype=np.float64)
    v = np.asarray(verts, dtype=np.float64)
    f = np.asarray(faces, dtype=np.int64)
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    ab, ac = b - a, c - a
    out = np.empty(len(p_all))
    for s in range(0, len(p_all), chunk):
        p = p_all[s:s + chunk][:, None, :]
        ap, bp, cp = p - a[None], p - b[None], p - c[None]
        d1, d2 = (ap * ab).sum(2), (ap * ac).sum(2)
        d3, d4 = (bp * ab).sum(2), (bp * ac).sum(2)
        d5, d6 = (cp * ab).sum(2), (cp * ac).sum(2)
        va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
        den = va + vb + vc
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = np.where(np.abs(den) > 1e-30, 1.0 / den, 0.0)
            t_ab = np.where(np.abs(d1 - d3) > 1e-30, d1 / (d1 - d3), 0.0)
            t_ac = np.where(np.abs(d2 - d6) > 1e-30, d2 / (d2 - d6), 0.0)
            e = (d4 - d3) + (d5 - d6)
            t_bc = np.where(np.abs(e) > 1e-30, (d4 - d3) / e, 0.0)
        vv, ww = vb * inv, vc * inv
        for cond, nv, nw in (((d1 <= 0) & (d2 <= 0), 0.0, 0.0),
                             ((d3 >= 0) & (d4 <= d3), 1.0, 0.0),
                             ((d6 >= 0) & (d5 <= d6), 0.0, 1.0),
                             ((vc <= 0) & (d1 >= 0) & (d3 <= 0), t_ab, 0.0),
                             ((vb <= 0) & (d2 >= 0) & (d6 <= 0), 0.0, t_ac),
                             ((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), 1.0 - t_bc, t_bc)):
            vv = np.where(cond, nv, vv)
            ww = np.where(cond, nw, ww)
        closest = a[None] + vv[..., None] * ab[None] + ww[..., None] * ac[None]
        out[s:s + chunk] = np.sqrt(((p - closest) ** 2).sum(axis=2)).min(axis=1)
    return out
