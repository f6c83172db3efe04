"""Open-top glass geometry: profile, signed distance, fill lattice, quaternion helpers.

Same public behaviour as warpmpm.colliders.glass (src/warpmpm/colliders/glass.py):
`GlassProfile` (defaults 0.089 m outer radius, 0.020 m wall, 0.24 m height, 0.050 m
base, 0.012 m fillet), the revolved SDF `glass_sdf_local` that the cup collider
kernel evaluates, and `cup_fill`, whose jittered lattice defines the 340,489-particle
pour at 192^3 / grid_lim 0.7. The host helpers that pour scripts use around the step
are here too: `glass_sdf` at a pose, `cavity_mask` (liquid held), `solid_mask`
(leak audit), `project_out_of_solid` and the quaternion conversions. Quaternions here are w x y z.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def quat_to_mat(q) -> np.ndarray:
    """Rotation matrix (float64) of a w x y z quaternion."""
    w, x, y, z = (float(c) for c in q)
    return np.array([
        [1.0 - 2.0 * (y * y + z * z), 2.0 * (x * y - z * w), 2.0 * (x * z + y * w)],
        [2.0 * (x * y + z * w), 1.0 - 2.0 * (x * x + z * z), 2.0 * (y * z - x * w)],
        [2.0 * (x * z - y * w), 2.0 * (y * z + x * w), 1.0 - 2.0 * (x * x + y * y)],
    ], dtype=np.float64)


def quat_mul(a, b) -> np.ndarray:
    aw, ax, ay, az = (float(c) for c in a)
    bw, bx, by, bz = (float(c) for c in b)
    return np.array([aw * bw - ax * bx - ay * by - az * bz,
                     aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw], dtype=np.float64)


def quat_conj(q) -> np.ndarray:
    """Conjugate (the inverse rotation for a unit quaternion), w x y z."""
    w, x, y, z = (float(c) for c in q)
    return np.array([w, -x, -y, -z], dtype=np.float64)


def quat_from_mat(m) -> np.ndarray:
    """Unit w x y z quaternion of a rotation matrix. Shepperd's method: take the
    square root of whichever of 1 + trace and 1 + 2 m_ii - trace is largest (the
    best-conditioned component), then the other three components from the
    off-diagonal sums and differences."""
    m = np.asarray(m, dtype=np.float64)
    t = float(m[0, 0] + m[1, 1] + m[2, 2])
    if t > 0.0:
        k = 0
    elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
        k = 1
    elif m[1, 1] > m[2, 2]:
        k = 2
    else:
        k = 3
    if k == 0:
        r = 2.0 * np.sqrt(t + 1.0)
        q = [0.25 * r, (m[2, 1] - m[1, 2]) / r, (m[0, 2] - m[2, 0]) / r, (m[1, 0] - m[0, 1]) / r]
    elif k == 1:
        r = 2.0 * np.sqrt(max(1.0 + m[0, 0] - m[1, 1] - m[2, 2], 1e-12))
        q = [(m[2, 1] - m[1, 2]) / r, 0.25 * r, (m[0, 1] + m[1, 0]) / r, (m[0, 2] + m[2, 0]) / r]
    elif k == 2:
        r = 2.0 * np.sqrt(max(1.0 + m[1, 1] - m[0, 0] - m[2, 2], 1e-12))
        q = [(m[0, 2] - m[2, 0]) / r, (m[0, 1] + m[1, 0]) / r, 0.25 * r, (m[1, 2] + m[2, 1]) / r]
    else:
        r = 2.0 * np.sqrt(max(1.0 + m[2, 2] - m[0, 0] - m[1, 1], 1e-12))
        q = [(m[1, 0] - m[0, 1]) / r, (m[0, 2] + m[2, 0]) / r, (m[1, 2] + m[2, 1]) / r, 0.25 * r]
    q = np.asarray(q, dtype=np.float64)
    return q / np.linalg.norm(q)


def quat_from_axis_angle(axis, angle: float) -> np.ndarray:
    a = np.asarray(axis, dtype=np.float64)
    a = a / max(float(np.linalg.norm(a)), 1e-12)
    h = 0.5 * float(angle)
    return np.concatenate([[np.cos(h)], np.sin(h) * a])


def angular_velocity_between(q0, q1, dt: float) -> np.ndarray:
    """World-frame angular velocity taking w x y z quaternion q0 to q1 over dt."""
    d = quat_mul(np.asarray(q1, dtype=np.float64), np.array([q0[0], -q0[1], -q0[2], -q0[3]], dtype=np.float64))
    d = d / np.linalg.norm(d)
    if d[0] < 0.0:
        d = -d
    s = float(np.linalg.norm(d[1:]))
    if s < 1e-9:
        return np.zeros(3)
    return d[1:] / s * (2.0 * np.arctan2(s, float(d[0])) / dt)


def world_to_local(points, pos, quat) -> np.ndarray:
    return (np.asarray(points, dtype=np.float64) - np.asarray(pos, dtype=np.float64)) @ quat_to_mat(quat)


@dataclass(frozen=True)
class GlassProfile:
    outer_radius: float = 0.089
    inner_radius: float = 0.069
    height: float = 0.24
    base_thickness: float = 0.050
    fillet_radius: float = 0.012

    def __post_init__(self):
        if not 0.0 < self.inner_radius < self.outer_radius:
            raise ValueError("need 0 < inner_radius < outer_radius")
        if not 0.0 < self.base_thickness < self.height:
            raise ValueError("need 0 < base_thickness < height")
        if not 0.0 <= self.fillet_radius < self.inner_radius:
            raise ValueError("need 0 <= fillet_radius < inner_radius")

    @property
    def half_height(self) -> float:
        return 0.5 * self.height

    @property
    def inner_floor_z(self) -> float:
        return self.base_thickness - 0.5 * self.height

    @property
    def rim_z(self) -> float:
        return 0.5 * self.height

    @property
    def wall_thickness(self) -> float:
        return self.outer_radius - self.inner_radius

    def inner_radius_at_z(self, z) -> np.ndarray:
        """Cavity radius against local z, including the quarter-circle floor fillet."""
        z = np.asarray(z, dtype=np.float64)
        fr = self.fillet_radius
        r = np.full_like(z, self.inner_radius)
        if fr > 0.0:
            zc = self.inner_floor_z + fr
            in_fillet = (z >= self.inner_floor_z) & (z < zc)
            dz = z[in_fillet] - zc
            r[in_fillet] = self.inner_radius - fr + np.sqrt(np.maximum(fr * fr - dz * dz, 0.0))
            r = np.where(z < self.inner_floor_z, self.inner_radius - fr, r)
        return r


def _capped_cylinder(r, z, radius, z0, z1):
    zc, hh = 0.5 * (z0 + z1), 0.5 * (z1 - z0)
    dr = r - radius
    dz = np.abs(z - zc) - hh
    a, b = np.maximum(dr, 0.0), np.maximum(dz, 0.0)
    return np.sqrt(a * a + b * b) + np.minimum(np.maximum(dr, dz), 0.0)


def glass_sdf_local(points_local, profile: GlassProfile):
    """Signed distance (float64, negative inside the glass material) in the local frame:
    outer capped cylinder minus the fillet-dilated, rim-extended cavity cylinder."""
    p = np.asarray(points_local, dtype=np.float64)
    r = np.linalg.norm(p[..., :2], axis=-1)
    z = p[..., 2]
    fr = profile.fillet_radius
    outer = _capped_cylinder(r, z, profile.outer_radius, -profile.half_height, profile.half_height)
    cavity = _capped_cylinder(r, z, profile.inner_radius - fr, profile.inner_floor_z + fr,
                              profile.half_height + profile.outer_radius) - fr
    return np.maximum(outer, -cavity)


def glass_sdf(points_world, pos, quat, profile: GlassProfile):
    """glass_sdf_local of world points for the glass at (pos, w x y z quat)."""
    return glass_sdf_local(world_to_local(points_world, pos, quat), profile)


def cavity_mask(points_world, pos, quat, profile: GlassProfile, pad: float = 0.0,
                brim_clearance: float = 0.0) -> np.ndarray:
    """Points held in the open cavity: within the cavity radius at their height (plus
    `pad`), at or above the floor (1 mm slack) and at most `brim_clearance` below the
    rim (colliders/glass.py:218-230)."""
    loc = world_to_local(points_world, pos, quat)
    r = np.hypot(loc[:, 0], loc[:, 1])
    z = loc[:, 2]
    return (r < profile.inner_radius_at_z(z) + pad) & (z >= profile.inner_floor_z - 1e-3) & \
        (z <= profile.rim_z - brim_clearance)


def solid_mask(points_world, pos, quat, profile: GlassProfile, tol: float = 0.0) -> np.ndarray:
    """Points embedded in the glass material deeper than `tol`."""
    return glass_sdf(points_world, pos, quat, profile) < -tol


def project_out_of_solid(x, v, pos, quat, profile: GlassProfile, clearance: float = 0.0, solid_velocity=None):
    """Moves every point embedded in the glass out along the SDF gradient (central
    differences, step 1e-5 m) to `clearance` outside the surface. It then removes the
    inward normal part of its velocity relative to the wall, whose velocity is
    v_lin + omega x (x - pos) when `solid_velocity` = (v_lin, omega) is given, else
    zero (colliders/glass.py:238-290). Returns (x_new, v_new, number moved); the
    inputs are not modified."""
    x = np.array(x, dtype=np.float64)
    v = np.array(v, dtype=np.float64)
    d = glass_sdf(x, pos, quat, profile)
    bad = d < 0.0
    nb = int(bad.sum())
    if nb == 0:
        return x, v, 0
    R = quat_to_mat(quat)
    p0 = np.asarray(pos, dtype=np.float64)
    loc = world_to_local(x[bad], pos, quat)
    eps = 1e-5
    g = np.empty_like(loc)
    for a in range(3):
        e = np.zeros(3)
        e[a] = eps
        g[:, a] = glass_sdf_local(loc + e, profile) - glass_sdf_local(loc - e, profile)
    n = g / np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-12)
    x[bad] = (loc + (clearance - d[bad])[:, None] * n) @ R.T + p0
    nw = n @ R.T
    if solid_velocity is None:
        vw = np.zeros((nb, 3))
    else:
        vl, om = (np.asarray(c, dtype=np.float64) for c in solid_velocity)
        vw = vl + np.cross(om, x[bad] - p0)
    rel = v[bad] - vw
    vn = np.einsum("ij,ij->i", rel, nw)
    v[bad] = vw + rel - nw * np.minimum(vn, 0.0)[:, None]
    return x, v, nb


def cup_fill(profile: GlassProfile, h: float, fill_fraction: float = 0.80, clearance: float | None = None,
             floor_clearance: float | None = None, brim_clearance: float = 0.006, seed: int = 0):
    """Jittered lattice (spacing h, +-h/4 uniform jitter from default_rng(seed)) filling
    the cavity to `fill_fraction` of its usable height. Returns local-frame
    (pos[N,3] float32, vol[N] float32)."""
    clearance = h if clearance is None else clearance
    floor_clearance = h if floor_clearance is None else floor_clearance
    usable = profile.rim_z - profile.inner_floor_z - brim_clearance - floor_clearance
    fill_h = fill_fraction * usable
    if fill_h <= 0:
        raise ValueError("fill height is non-positive; check clearances")
    z0 = profile.inner_floor_z + floor_clearance
    r_max = profile.inner_radius - clearance
    xs = np.arange(-r_max + 0.5 * h, r_max, h)
    zs = np.arange(z0 + 0.5 * h, z0 + fill_h, h)
    lattice = np.stack(np.meshgrid(xs, xs, zs, indexing="ij"), axis=-1).reshape(-1, 3)
    lattice = lattice + np.random.default_rng(seed).uniform(-0.25 * h, 0.25 * h, size=lattice.shape)
    rad = np.linalg.norm(lattice[:, :2], axis=1)
    z = lattice[:, 2]
    keep = (rad < profile.inner_radius_at_z(z) - clearance) & (z >= z0) & (z <= z0 + fill_h)
    pos = lattice[keep].astype(np.float32)
    return pos, np.full(len(pos), h ** 3, dtype=np.float32)


__all__ = ["GlassProfile", "angular_velocity_between", "cup_fill", "glass_sdf_local", "quat_from_axis_angle", "quat_mul", "quat_to_mat",
           "world_to_local"]


def glass_cavity_profile(profile: GlassProfile | None = None) -> np.ndarray:
    """Open (r, z) polyline of the glass cavity surface, floor disk then inner wall
    up to the rim (glass_cavity_profile, colliders/glass.py:162-183): the CPIC sheet
    traces the cavity so CDF and SDF contact geometry coincide."""
    p = GlassProfile() if profile is None else profile
    return np.array([(0.0, p.inner_floor_z), (p.inner_radius, p.inner_floor_z), (p.inner_radius, p.rim_z)])


def glass_cdf(dx: float, profile: GlassProfile | None = None, res: int = 96):
    """The glass as a CDF collider field, with a built band wide enough for a runtime
    band of 2 dx (examples/pour_franka.py:249-262). The field's margin around the
    surface is widened to cover the band: with the recipe's fixed 4-cell margin a
    coarse grid's band reaches past the field below the glass floor, nodes there are
    never tagged and material seeps through."""
    from .geometry import revolved_open_cdf
    prof = glass_cavity_profile(profile)
    span = max(2.0 * float(prof[:, 0].max()), float(prof[:, 1].max() - prof[:, 1].min()))
    margin = 4.0
    for _ in range(3):
        cell = span / (res - 1 - 2 * margin)
        band_cells = max(3.0, float(np.ceil(2.2 * dx / cell)))
        margin = max(4.0, band_cells + 1.0)
    cell = span / (res - 1 - 2 * margin)
    band_cells = max(3.0, float(np.ceil(2.2 * dx / cell)))
    return revolved_open_cdf(prof, res=res, band_cells=band_cells, margin_cells=margin)

