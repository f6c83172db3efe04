"""Mesh -> distance fields with the searches on the GPU.

The drop-in for warpmpm.geometry.mesh_sdf's builders (src/warpmpm/geometry/mesh_sdf.py):
`build_sdf` voxelizes a watertight mesh into an SDFData (signed distance, negative
inside, plus its gradient) and `build_surface_cdf` an open oriented sheet into a
CDFData (side-signed distance plus validity), with the reference's grids, sampling
and formulas. The O(grid nodes x surface elements) work runs on the device through
libgbmpm (gbmpm_field_nearest, gbmpm_field_winding, gbmpm_field_tri_distance):

- distance magnitude: the nearest of dense surface samples 0.4 cells apart, which
  is what the reference computes with scipy's cKDTree (its default); the GPU search
  is an exact nearest neighbour in float64, so values match it to the last bit up to
  ties. `method="exact"` takes the exact distance to the triangles instead, the
  reference's path when scipy is absent;
- sign: the generalized winding number with the reference's interior-probe rule;
- the CDF side: the sign of the offset from the nearest sample along its face's
  normal; validity: within the band of the sheet and farther than the band from
  its open rim.

The procedural meshes (`revolve_profile`, `revolve_profile_open`, `make_cup_mesh`)
and the samplers produce the reference's vertices, faces and samples in the same
order (the nearest-sample tie rule depends on that order). Cached variants use the
reference's cache keys and npz formats, so caches written by either load in both.
"""
from __future__ import annotations

import ctypes as C
import hashlib
from pathlib import Path

import numpy as np

from . import _abi
from .geometry import CDFData, SDFData, load_cdf, load_sdf, save_cdf, save_sdf

_AXIS_EPS = 1e-9


# ---------------------------------------------------------------- procedural meshes
def _rings(profile, n_theta: int):
    th = np.linspace(0.0, 2.0 * np.pi, n_theta, endpoint=False)
    ct, st = np.cos(th), np.sin(th)
    verts, rings = [], []
    for r, z in np.asarray(profile, dtype=float):
        if r <= _AXIS_EPS:                          # a ring on the axis collapses to one vertex
            rings.append([len(verts)] * n_theta)
            verts.append((0.0, 0.0, float(z)))
        else:
            base = len(verts)
            verts.extend((float(r) * ct[j], float(r) * st[j], float(z)) for j in range(n_theta))
            rings.append(list(range(base, base + n_theta)))
    return verts, rings


def _stitch(rings, pairs, n_theta: int):
    faces = []
    for i, i2 in pairs:
        lo, hi = rings[i], rings[i2]
        for j in range(n_theta):
            j2 = (j + 1) % n_theta
            a, b, c, d = lo[j], lo[j2], hi[j2], hi[j]
            if a == b and c == d:
                continue
            if a == b:                               # fan from an axis vertex
                faces.append((a, c, d))
            elif c == d:
                faces.append((a, b, c))
            else:
                faces.append((a, b, c))
                faces.append((a, c, d))
    return faces


def revolve_profile(profile_rz, n_theta: int = 64):
    """Watertight solid of revolution of a closed (r, z) polygon about z
    (mesh_sdf.py:86-129): uniform winding, axis vertices shared, caps as fans."""
    verts, rings = _rings(profile_rz, n_theta)
    P = len(rings)
    faces = _stitch(rings, [(i, (i + 1) % P) for i in range(P)], n_theta)
    return np.asarray(verts, dtype=float), np.asarray(faces, dtype=np.int64)


def revolve_profile_open(profile_rz, n_theta: int = 64):
    """Open surface of revolution of an (r, z) polyline (mesh_sdf.py:132-172): no
    closing segment, no caps; face normals point to one side of the sheet."""
    verts, rings = _rings(profile_rz, n_theta)
    faces = _stitch(rings, [(i, i + 1) for i in range(len(rings) - 1)], n_theta)
    return np.asarray(verts, dtype=float), np.asarray(faces, dtype=np.int64)


def make_cup_mesh(inner_radius: float = 0.035, wall_thickness: float = 0.006, height: float = 0.085,
                  base_thickness: float = 0.008, n_theta: int = 64):
    """Watertight open-top cup, base at z = 0 (mesh_sdf.py:175-205)."""
    r_out = inner_radius + wall_thickness
    profile = [(0.0, 0.0), (r_out, 0.0), (r_out, height), (inner_radius, height), (inner_radius, base_thickness),
               (0.0, base_thickness)]
    return revolve_profile(profile, n_theta=n_theta)


# ---------------------------------------------------------------- surface samples
def _face_corners(verts, faces):
    v = np.asarray(verts, dtype=float)
    f = np.asarray(faces, dtype=np.int64)
    return v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]


def surface_samples(verts, faces, spacing: float, include_verts: bool = True, with_faces: bool = False):
    """Barycentric lattice samples on every face, about `spacing` apart
    (_sample_surface, mesh_sdf.py:292-311; with_faces: _sample_surface_with_faces,
    :367-390, which has no vertex block). A face of side ~ n * spacing gets the
    (n+1)^2 lattice u, v in linspace(0, 1, n+1) with u + v <= 1; a face smaller
    than the spacing gets its centroid. Faces of equal n are evaluated together and
    written at their place in face order."""
    a, b, c = _face_corners(verts, faces)
    nf = len(a)
    areas = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    step = max(spacing, 1e-9)
    n = np.array([int(max(1, np.ceil(np.sqrt(areas[i]) / step))) for i in range(nf)], dtype=np.int64)
    patterns = {}
    for k in np.unique(n):
        if k <= 1:
            continue
        u, w = np.meshgrid(np.linspace(0, 1, k + 1), np.linspace(0, 1, k + 1), indexing="ij")
        u, w = u.ravel(), w.ravel()
        keep = (u + w) <= 1.0
        patterns[int(k)] = (u[keep], w[keep])
    count = np.array([1 if k <= 1 else len(patterns[int(k)][0]) for k in n], dtype=np.int64)
    start = np.concatenate([[0], np.cumsum(count)[:-1]])
    out = np.empty((int(count.sum()), 3))
    fid = np.empty(len(out), dtype=np.int64)
    for k in np.unique(n):
        sel = np.nonzero(n == k)[0]
        if k <= 1:
            out[start[sel]] = (a[sel] + b[sel] + c[sel]) / 3.0
            fid[start[sel]] = sel
            continue
        u, w = patterns[int(k)]
        block = a[sel][:, None, :] + u[None, :, None] * (b[sel] - a[sel])[:, None, :] + \
            w[None, :, None] * (c[sel] - a[sel])[:, None, :]
        rows = start[sel][:, None] + np.arange(len(u))[None, :]
        out[rows.ravel()] = block.reshape(-1, 3)
        fid[rows.ravel()] = np.repeat(sel, len(u))
    if include_verts and not with_faces:
        out = np.concatenate([np.asarray(verts, dtype=float), out], axis=0)
    return (out, fid) if with_faces else out


def boundary_samples(verts, faces, spacing: float):
    """Samples along the open boundary: the edges with one incident face, in the
    sorted order of their vertex pairs, at least two points each
    (_boundary_loop_samples, mesh_sdf.py:393-409). (0, 3) for a closed mesh."""
    f = np.asarray(faces, dtype=np.int64)
    v = np.asarray(verts, dtype=float)
    edges = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    uniq, counts = np.unique(edges, axis=0, return_counts=True)
    open_edges = uniq[counts == 1]
    if len(open_edges) == 0:
        return np.zeros((0, 3))
    pts = []
    for i0, i1 in open_edges:
        p0, p1 = v[i0], v[i1]
        k = int(max(2, np.ceil(np.linalg.norm(p1 - p0) / max(spacing, 1e-9)) + 1))
        t = np.linspace(0.0, 1.0, k)[:, None]
        pts.append(p0[None] * (1 - t) + p1[None] * t)
    return np.concatenate(pts, axis=0)


# ---------------------------------------------------------------- device searches
def _torch():
    import torch
    return torch


def _device(device):
    torch = _torch()
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda" or not torch.cuda.is_available():
        raise RuntimeError("the mesh field builders run on a CUDA device; none is available")
    return dev


def _points(points, grid, dev):
    """FieldPoints for explicit points [n][3] or grid = (origin, cell, res); keeps the
    device copy alive with the record."""
    torch = _torch()
    rec = _abi.FieldPoints()
    if grid is not None:
        origin, cell, res = grid
        rec.points = None
        rec.n = 0
        for a in range(3):
            rec.origin[a] = float(origin[a])
        rec.cell = float(cell)
        rec.res = int(res)
        return rec, None, int(res) ** 3
    t = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3), device=dev)
    rec.points = t.data_ptr()
    rec.n = t.shape[0]
    rec.cell = 1.0
    rec.res = 0
    return rec, t, t.shape[0]


def _call(name, *args):
    lib = _abi.load()
    _abi.check(getattr(lib, name)(*args), name)


def nearest_samples(samples, points=None, grid=None, device=None):
    """Per query point the nearest sample: (distance float64, index int64), numpy.
    Query points are `points` [n][3] or the grid (origin, cell, res)."""
    torch = _torch()
    dev = _device(device)
    rec, keep, n = _points(points, grid, dev)
    s = torch.as_tensor(np.ascontiguousarray(samples, dtype=np.float64).reshape(-1, 3), device=dev)
    dist = torch.empty(n, dtype=torch.float64, device=dev)
    idx = torch.empty(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call("gbmpm_field_nearest", C.byref(rec), s.data_ptr(), s.shape[0], dist.data_ptr(), idx.data_ptr(), stream)
    return dist.cpu().numpy(), idx.cpu().numpy()


def _faces_tensor(verts, faces, dev):
    a, b, c = _face_corners(verts, faces)
    return _torch().as_tensor(np.ascontiguousarray(np.stack([a, b, c], axis=1)), device=dev)


def winding_numbers(verts, faces, points=None, grid=None, precise: bool = False, device=None):
    """Generalized winding number of each query point (_winding_number,
    mesh_sdf.py:210-233). float32-summed away from the +-0.5 threshold unless
    `precise`."""
    torch = _torch()
    dev = _device(device)
    rec, keep, n = _points(points, grid, dev)
    tri = _faces_tensor(verts, faces, dev)
    wn = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call("gbmpm_field_winding", C.byref(rec), tri.data_ptr(), tri.shape[0], 1 if precise else 0, wn.data_ptr(),
          stream)
    return wn.cpu().numpy()


def triangle_distance(verts, faces, points=None, grid=None, device=None):
    """Exact distance from each query point to the nearest face
    (_point_triangle_distance_exact, mesh_sdf.py:236-289)."""
    torch = _torch()
    dev = _device(device)
    rec, keep, n = _points(points, grid, dev)
    tri = _faces_tensor(verts, faces, dev)
    dist = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call("gbmpm_field_tri_distance", C.byref(rec), tri.data_ptr(), tri.shape[0], dist.data_ptr(), stream)
    return dist.cpu().numpy()


# ---------------------------------------------------------------- builders
def field_grid(verts, res: int, margin_cells: float):
    """The builders' cubic grid: `res` nodes across the bounding box's longest side
    plus `margin_cells` on each side, centred on the box (mesh_sdf.py:339-346).
    Returns (origin, cell, centre)."""
    v = np.asarray(verts, dtype=float)
    lo, hi = v.min(axis=0), v.max(axis=0)
    center = 0.5 * (lo + hi)
    span = float((hi - lo).max())
    cell = span / (res - 1 - 2 * margin_cells)
    origin = center - 0.5 * (cell * (res - 1))
    return origin, cell, center


def grid_points(origin, cell, res: int):
    axes = [origin[d] + cell * np.arange(res) for d in range(3)]
    X, Y, Z = np.meshgrid(axes[0], axes[1], axes[2], indexing="ij")
    return np.stack([X, Y, Z], axis=-1).reshape(-1, 3)


def build_sdf(verts, faces, res: int = 64, margin_cells: float = 4.0, interior_probe=None,
              method: str = "samples", device=None) -> SDFData:
    """Voxelize a watertight mesh into an SDFData (build_sdf, mesh_sdf.py:329-364).

    method "samples": distance to the nearest surface sample (the reference with
    scipy); "exact": exact distance to the faces (the reference without scipy)."""
    verts = np.asarray(verts, dtype=float)
    faces = np.asarray(faces, dtype=np.int64)
    origin, cell, center = field_grid(verts, res, margin_cells)
    grid = (origin, cell, res)
    if method == "samples":
        unsigned, _ = nearest_samples(surface_samples(verts, faces, 0.4 * cell), grid=grid, device=device)
    elif method == "exact":
        unsigned = triangle_distance(verts, faces, grid=grid, device=device)
    else:
        raise ValueError("method must be 'samples' or 'exact'")
    wn = winding_numbers(verts, faces, grid=grid, device=device)
    probe = center if interior_probe is None else np.asarray(interior_probe, dtype=float)
    w_probe = winding_numbers(verts, faces, points=probe[None], precise=True, device=device)[0]
    inside = (wn * np.sign(w_probe)) > 0.5 if abs(w_probe) > 0.1 else (np.abs(wn) > 0.5)
    signed = np.where(inside, -unsigned, unsigned).reshape(res, res, res)
    grads = np.stack(np.gradient(signed, cell, edge_order=2), axis=-1)
    return SDFData(values=signed.astype(np.float64), grads=grads.astype(np.float64),
                   origin=origin.astype(np.float64), cell=float(cell), sdf_max=float(np.abs(signed).max()))


def build_surface_cdf(verts, faces, res: int = 64, band_cells: float = 3.0, margin_cells: float = 4.0,
                      device=None) -> CDFData:
    """Voxelize an open oriented sheet into a CDFData (build_surface_cdf,
    mesh_sdf.py:412-480): distance to the nearest surface sample, side from that
    sample's face normal, valid within the band and farther than the band from the
    open rim."""
    verts = np.asarray(verts, dtype=float)
    faces = np.asarray(faces, dtype=np.int64)
    origin, cell, _ = field_grid(verts, res, margin_cells)
    band = band_cells * cell
    grid = (origin, cell, res)
    a, b, c = _face_corners(verts, faces)
    normals = np.cross(b - a, c - a)
    normals /= np.maximum(np.linalg.norm(normals, axis=1, keepdims=True), 1e-30)
    samples, sample_face = surface_samples(verts, faces, 0.4 * cell, with_faces=True)
    rim = boundary_samples(verts, faces, 0.4 * cell)
    dist, idx = nearest_samples(samples, grid=grid, device=device)
    rim_dist = nearest_samples(rim, grid=grid, device=device)[0] if len(rim) else np.full(len(dist), np.inf)
    pts = grid_points(origin, cell, res)
    side = np.sign(np.einsum("ij,ij->i", pts - samples[idx], normals[sample_face[idx]]))
    side[side == 0.0] = 1.0
    signed = (side * dist).reshape(res, res, res)
    valid = ((dist <= band) & (rim_dist > band)).astype(np.float64).reshape(res, res, res)
    return CDFData(values=signed.astype(np.float64), valid=valid, origin=origin.astype(np.float64), cell=float(cell),
                   band=float(band))


# ---------------------------------------------------------------- caches (the reference's keys)
_SDF_CACHE_VERSION = 2
_CDF_CACHE_VERSION = 1


def _sdf_key(verts, faces, res, margin_cells, interior_probe=None) -> str:
    v64 = np.ascontiguousarray(verts, dtype=np.float64)
    probe = 0.5 * (v64.min(axis=0) + v64.max(axis=0)) if interior_probe is None else \
        np.asarray(interior_probe, dtype=np.float64)
    if probe.shape != (3,) or not np.isfinite(probe).all():
        raise ValueError(f"interior_probe must be a finite 3-vector, got {probe}")
    h = hashlib.sha1()
    for arr in (np.array([_SDF_CACHE_VERSION], dtype=np.int64), v64, np.ascontiguousarray(faces, dtype=np.int64),
                np.array([res, margin_cells], dtype=np.float64), np.ascontiguousarray(probe, dtype=np.float64)):
        h.update(arr.tobytes())
    return h.hexdigest()[:16]


def build_sdf_cached(verts, faces, res: int = 64, margin_cells: float = 4.0, cache_dir=None, interior_probe=None,
                     device=None) -> SDFData:
    """build_sdf with the reference's versioned npz cache (mesh_sdf.py:502-563)."""
    if cache_dir is None:
        return build_sdf(verts, faces, res, margin_cells, interior_probe, device=device)
    path = Path(cache_dir) / f"sdf_{_sdf_key(verts, faces, res, margin_cells, interior_probe)}.npz"
    if path.exists():
        return load_sdf(path)
    sdf = build_sdf(verts, faces, res, margin_cells, interior_probe, device=device)
    save_sdf(sdf, path)
    return sdf


def build_surface_cdf_cached(verts, faces, res: int = 64, band_cells: float = 3.0, margin_cells: float = 4.0,
                             cache_dir=None, device=None) -> CDFData:
    """build_surface_cdf with the reference's versioned npz cache (mesh_sdf.py:498-519)."""
    if cache_dir is None:
        return build_surface_cdf(verts, faces, res, band_cells, margin_cells, device=device)
    h = hashlib.sha1()
    for arr in (np.array([_CDF_CACHE_VERSION], dtype=np.int64), np.ascontiguousarray(verts, dtype=np.float64),
                np.ascontiguousarray(faces, dtype=np.int64),
                np.array([res, band_cells, margin_cells], dtype=np.float64)):
        h.update(arr.tobytes())
    path = Path(cache_dir) / f"cdf_{h.hexdigest()[:16]}.npz"
    if path.exists():
        return load_cdf(path)
    cdf = build_surface_cdf(verts, faces, res, band_cells, margin_cells, device=device)
    save_cdf(cdf, path)
    return cdf


__all__ = ["boundary_samples", "build_sdf", "build_sdf_cached", "build_surface_cdf", "build_surface_cdf_cached",
           "field_grid", "grid_points", "make_cup_mesh", "nearest_samples", "revolve_profile", "revolve_profile_open",
           "surface_samples", "triangle_distance", "winding_numbers"]
