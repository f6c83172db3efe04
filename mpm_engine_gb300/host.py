"""Host-side construction of the engine's model and collider records.

These are the parameter conventions of warpmpm's MPM_Simulator_WARP, restated
as plain functions over the ctypes records of include/gbmpm.h so they can be
tested without a GPU: per-type material tables (mpm_solver_warp.py:236-274),
set_parameters_dict (:634-800), set_parameters_for_particles (:1700-1783) and
the collider constructors (:1880-2285, 2287-2380, 2621-2814).
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi
from .materials import material_id

F32 = np.float32


def f32(x) -> float:
    """Round a Python float to fp32, as storing it in a Warp struct or array does."""
    return float(np.float32(x))


def friction_alpha(angle_deg: float) -> float:
    """Drucker-Prager alpha from a friction angle (mpm_solver_warp.py:286-293): warp's
    Python-scope sin/sqrt evaluate in fp32, the rest in float64, stored as fp32."""
    sin_phi = float(np.sin(np.float32(angle_deg / 180.0 * 3.14159265)))
    return f32(float(np.sqrt(np.float32(2.0 / 3.0))) * 2.0 * sin_phi / (3.0 - sin_phi))


def default_model(n_grid: int, grid_lim: float) -> _abi.Model:
    """Model record as MPM_Simulator_WARP.initialize leaves it (mpm_solver_warp.py:218-299)."""
    m = _abi.Model()
    m.n_grid = int(n_grid)
    m.grid_lim = f32(grid_lim)
    m.dx = f32(grid_lim / n_grid)
    m.inv_dx = f32(float(n_grid / grid_lim))
    m.gravity[:] = (0.0, 0.0, 0.0)
    m.rpic_damping = 0.0
    m.grid_v_damping_scale = 1.1
    m.periodic_x = 0
    m.update_cov_with_F = 0
    m.material_mask = 1  # every particle starts as jelly (id 0)
    alpha = friction_alpha(25.0)
    for i in range(_abi.MAX_MATERIALS):
        m.alpha[i] = alpha
        m.softening[i] = 0.1
        m.muI_I0[i] = 1.0
        m.muI_d[i] = 1.0
        m.muI_rho_s[i] = 1.0
        m.muI_phi_init[i] = 1.0
    m.eta_table_n = 2
    m.eta_table_smin = -1.0
    m.eta_table_smax = 2.0
    return m


# parameter key -> per-type table field of the model record
TYPE_TABLE_KEYS = {
    "E": "E", "nu": "nu", "bulk_modulus": "bulk", "hardening": "hardening", "xi": "xi",
    "plastic_viscosity": "plastic_viscosity", "softening": "softening",
    "mu_s": "muI_mu_s", "delta_mu": "muI_delta_mu", "I0": "muI_I0", "grain_diameter": "muI_d",
    "grain_density": "muI_rho_s", "phi_init": "muI_phi_init", "phi_chi": "muI_phi_chi",
}


def apply_type_params(m: _abi.Model, mat_id: int, params: dict) -> None:
    """Per-type entries of set_parameters_dict / set_parameters_for_particles."""
    for key, field in TYPE_TABLE_KEYS.items():
        if key in params:
            getattr(m, field)[mat_id] = f32(float(params[key]))
    if "friction_angle" in params:
        m.alpha[mat_id] = friction_alpha(float(params["friction_angle"]))


def mu_lam_from_E_nu_f32(E: np.ndarray, nu: np.ndarray):
    """compute_mu_lam_from_E_nu (mpm_utils.py:583-588) in fp32."""
    E = np.asarray(E, dtype=F32)
    nu = np.asarray(nu, dtype=F32)
    one, two = F32(1.0), F32(2.0)
    mu = E / (two * (one + nu))
    lam = E * nu / ((one + nu) * (one - two * nu))
    return mu.astype(F32), lam.astype(F32)


def _vec(dst, vals) -> None:
    for i, v in enumerate(vals):
        dst[i] = f32(float(v))


def plane_collider(point, normal, surface: str = "sticky", friction: float = 0.0,
                   start_time: float = 0.0, end_time: float = 999.0) -> _abi.Collider:
    """add_surface_collider (mpm_solver_warp.py:1880-1920)."""
    if surface == "sticky" and friction != 0:
        raise ValueError("friction must be 0 on sticky surfaces.")
    s32 = float(np.sqrt(np.float32(float(sum(float(x) ** 2 for x in normal)))))
    scale = 1.0 / s32
    c = _abi.Collider()
    c.kind = _abi.COLLIDER_PLANE
    c.surface_type = {"sticky": 0, "slip": 1, "cut": 11}.get(surface, 2)
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    _vec(c.point, point)
    _vec(c.normal, [scale * float(x) for x in normal])
    c.friction = f32(friction)
    return c


def box_collider(point, size, velocity, start_time: float = 0.0, end_time: float = 999.0,
                 reset: int = 0) -> _abi.Collider:
    """set_velocity_on_cuboid (mpm_solver_warp.py:2028-2106)."""
    c = _abi.Collider()
    c.kind = _abi.COLLIDER_BOX
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    _vec(c.point, point)
    _vec(c.size, size)
    _vec(c.velocity, velocity)
    c.reset = int(reset)
    return c


def set_rotation(c: _abi.Collider, rot) -> None:
    r = np.asarray(rot, dtype=np.float64).reshape(3, 3)
    for i in range(9):
        c.rot64[i] = float(r.flat[i])
        c.rot[i] = f32(float(r.flat[i]))


def cup_collider(point, rot, velocity=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0), outer_radius=0.089,
                 inner_radius=0.069, half_height=0.12, inner_floor_z=-0.07, fillet_radius=0.012,
                 friction=0.0, sticky_depth=0.0, contact_band=0.0, start_time=0.0,
                 end_time=999.0) -> _abi.Collider:
    """add_revolved_sdf_collider (mpm_solver_warp.py:2121-2159)."""
    c = _abi.Collider()
    c.kind = _abi.COLLIDER_CUP
    _vec(c.point, point)
    set_rotation(c, rot)
    _vec(c.velocity, velocity)
    _vec(c.omega, omega)
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    c.friction = f32(friction)
    c.outer_radius, c.inner_radius = f32(outer_radius), f32(inner_radius)
    c.half_height, c.inner_floor_z, c.fillet_radius = f32(half_height), f32(inner_floor_z), f32(fillet_radius)
    c.sticky_depth, c.contact_band = f32(sticky_depth), f32(contact_band)
    return c


def walls_collider(start_time: float = 0.0, end_time: float = 999.0) -> _abi.Collider:
    """add_bounding_box (mpm_solver_warp.py:2287-2380): one record covers the six shells."""
    c = _abi.Collider()
    c.kind = _abi.COLLIDER_WALLS
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    return c


SDF_SURFACES = {"sticky": 0, "slip": 1, "separable": 2}


def sdf_boundary_min(values: np.ndarray) -> float:
    """Smallest stored distance on the six faces of the SDF box (mpm_solver_warp.py:2636-2638)."""
    v = np.asarray(values)
    return float(min(v[0].min(), v[-1].min(), v[:, 0, :].min(), v[:, -1, :].min(), v[:, :, 0].min(),
                     v[:, :, -1].min()))


def sdf_r_max(origin, cell: float, res: int) -> float:
    """Largest lever arm from the body origin to a corner of the SDF box (:2646-2652)."""
    ext = (res - 1) * float(cell)
    corners = np.array([[float(origin[0]) + a * ext, float(origin[1]) + b * ext, float(origin[2]) + c * ext]
                        for a in (0, 1) for b in (0, 1) for c in (0, 1)])
    return float(np.linalg.norm(corners, axis=1).max())


def sdf_collider(val_ptr: int, grad_ptr: int, res: int, origin, cell, center, quat, velocity, omega,
                 band: float, surface_id: int, friction: float, start_time: float,
                 end_time: float) -> _abi.Collider:
    """add_sdf_collider's parameter record (mpm_solver_warp.py:2657-2677)."""
    c = _abi.Collider()
    c.kind = _abi.COLLIDER_SDF
    c.sdf_val, c.sdf_grad, c.sdf_res = val_ptr, grad_ptr, int(res)
    _vec(c.sdf_origin, origin)
    c.sdf_cell = f32(cell)
    _vec(c.point, center)
    _vec(c.quat, quat)
    _vec(c.velocity, velocity)
    _vec(c.omega, omega)
    c.band = f32(band)
    c.surface_type = int(surface_id)
    c.friction = f32(friction)
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    return c


def cdf_lane(values_ptr: int, valid_ptr: int, res: int, origin, cell, center, quat, velocity, omega,
             band: float, surface_id: int, friction: float, start_time: float, end_time: float) -> _abi.Cdf:
    """CDFCollider record of add_cdf_collider (mpm_solver_warp.py:2853-2869)."""
    c = _abi.Cdf()
    c.values, c.valid, c.res = values_ptr, valid_ptr, int(res)
    c.surface_type = int(surface_id)
    _vec(c.origin, origin)
    c.cell = f32(cell)
    _vec(c.center, center)
    _vec(c.quat, quat)
    _vec(c.velocity, velocity)
    _vec(c.omega, omega)
    c.band = f32(band)
    c.friction = f32(friction)
    c.start_time, c.end_time = f32(start_time), f32(end_time)
    return c


def cdf_band(built_band: float, dx: float, band=None) -> float:
    """Runtime band rules of add_cdf_collider (mpm_solver_warp.py:2833-2849)."""
    import warnings
    if band is None:
        band = min(float(built_band), 2.0 * float(dx))
    if band > float(built_band) + 1e-12:
        raise ValueError(f"runtime band ({band * 1e3:.1f} mm) exceeds the band the field was built with "
                         f"({float(built_band) * 1e3:.1f} mm); rebuild the CDF with a larger band_cells.")
    if band < 1.5 * float(dx):
        warnings.warn(f"CDF band ({band * 1e3:.1f} mm) is below 1.5 dx ({1.5 * dx * 1e3:.1f} mm): straddling "
                      f"particle-node pairs can go untagged and the wall can leak.", RuntimeWarning, stacklevel=3)
    return float(band)


def grid_guard_message(lo: float, hi: float, lim: float, dx: float) -> str:
    """Text of the edge-guard RuntimeError (core/solver.py:508-512)."""
    return (f"particles within 2 cells of the grid edge (x in [{lo:.4f}, {hi:.4f}] m, domain [0, {lim}] m, "
            f"dx={dx:.4f}): the P2G stencil would write out of bounds. Enlarge grid_lim or add a "
            f"bounding box / wall collider.")


def material_mask_bit(name) -> int:
    return 1 << material_id(name)


def is_finite_number(x) -> bool:
    return isinstance(x, (int, float)) and math.isfinite(float(x))


# ---- rigid bodies and particle modifiers ----------------------------------------
def rigid_bodies(x, mass, material, rigid_id):
    """Bodies of the material-8 particles grouped by rigid_id (finalize_rigid_bodies,
    mpm_solver_warp.py:834-879): mass, centre of mass (float32 sums as the reference
    forms them), body-frame inverse inertia (float64 sum, inverted, stored float32),
    identity orientation, at rest; plus each rigid particle's body-frame position
    x - x_cm. Returns (list of _abi.RigidBody, x_ref float32 [n][3])."""
    x = np.asarray(x, np.float32)
    m = np.asarray(mass, np.float32)
    rigid = np.asarray(material) == 8
    rid = np.asarray(rigid_id)
    x_ref = np.zeros_like(x)
    if not rigid.any():
        return [], x_ref
    out = []
    for b in range(int(rid[rigid].max()) + 1):
        idx = np.nonzero(rigid & (rid == b))[0]
        if len(idx) == 0:
            raise ValueError(f"rigid body {b} has no particles (obj_id values must be 0 .. n-1)")
        mb = m[idx]
        M = np.float32(mb.sum())
        com = ((x[idx] * mb[:, None]).sum(axis=0) / M).astype(np.float32)
        r = (x[idx] - com).astype(np.float32)
        x_ref[idx] = r
        r64, m64 = r.astype(np.float64), mb.astype(np.float64)
        inertia = np.eye(3) * (m64 * (r64 * r64).sum(axis=1)).sum() - np.einsum("p,pi,pj->ij", m64, r64, r64)
        inv = np.linalg.inv(inertia).astype(np.float32)
        rec = _abi.RigidBody()
        rec.x_cm[:] = tuple(float(c) for c in com)
        rec.R[:] = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
        rec.mass = float(M)
        rec.inv_inertia[:] = tuple(float(c) for c in inv.reshape(-1))
        out.append(rec)
    return out, x_ref


def rigid_surface(point, normal, friction, restitution, start_time=0.0, end_time=999.0):
    """add_surface_collider's rigid contact record (mpm_solver_warp.py:1880-1927)."""
    n = np.asarray(normal, dtype=np.float64)
    n = n / np.sqrt((n * n).sum())
    rec = _abi.RigidSurface()
    rec.point[:] = tuple(float(c) for c in point)
    rec.normal[:] = tuple(float(c) for c in n)
    rec.friction, rec.restitution = float(friction), float(restitution)
    rec.start_time, rec.end_time = float(start_time), float(end_time)
    return rec


def impulse_modifier(force, dt, num_dt, start_time):
    """add_impulse_on_particles (mpm_solver_warp.py:2385-2427): active for num_dt
    substeps from start_time."""
    rec = _abi.Modifier()
    rec.kind = 0
    rec.start_time = float(start_time)
    rec.end_time = float(start_time + dt * num_dt)
    rec.vec[:] = tuple(float(c) for c in force)
    return rec


def translation_modifier(velocity, start_time, end_time):
    """enforce_particle_velocity_translation (mpm_solver_warp.py:2431-2469)."""
    rec = _abi.Modifier()
    rec.kind = 1
    rec.start_time, rec.end_time = float(start_time), float(end_time)
    rec.vec[:] = tuple(float(c) for c in velocity)
    return rec


def rotation_modifier(point, normal, rotation_scale, translation_scale, start_time, end_time):
    """enforce_particle_velocity_rotation (mpm_solver_warp.py:2475-2539): the unit axis
    and the two horizontal axes the reference derives from (1, 1, 1) (or
    (0.72, 0.37, -0.67) when that is nearly along the axis), in float32."""
    n = np.asarray(normal, dtype=np.float32)
    n = (n * np.float32(1.0 / np.sqrt(np.float32((n.astype(np.float64) ** 2).sum())))).astype(np.float32)
    h1 = np.array([1.0, 1.0, 1.0], np.float32)
    if abs(float(np.dot(n, h1))) < 0.01:
        h1 = np.array([0.72, 0.37, -0.67], np.float32)
    h1 = (h1 - np.float32(np.dot(h1, n)) * n).astype(np.float32)
    h1 = (h1 * np.float32(1.0 / np.linalg.norm(h1))).astype(np.float32)
    h2 = np.cross(h1, n).astype(np.float32)
    rec = _abi.Modifier()
    rec.kind = 2
    rec.start_time, rec.end_time = float(start_time), float(end_time)
    rec.point[:] = tuple(float(c) for c in point)
    rec.normal[:] = tuple(float(c) for c in n)
    rec.axis1[:] = tuple(float(c) for c in h1)
    rec.axis2[:] = tuple(float(c) for c in h2)
    rec.rotation_scale, rec.translation_scale = float(rotation_scale), float(translation_scale)
    return rec


def box_mask(x, point, size):
    """Particles with |x - point| < size on every axis (the modifiers' box selection,
    mpm_utils.py:1321-1345)."""
    x = np.asarray(x, np.float32)
    return (np.abs(x - np.asarray(point, np.float32)) < np.asarray(size, np.float32)).all(axis=1)


def cylinder_mask(x, point, unit_normal, half_height, radius):
    """Particles inside the cylinder about the axis (mpm_utils.py:1349-1362)."""
    x = np.asarray(x, np.float32)
    n = np.asarray(unit_normal, np.float32)
    off = x - np.asarray(point, np.float32)
    along = off @ n
    horiz = np.linalg.norm(off - along[:, None] * n, axis=1)
    return (np.abs(along) < np.float32(half_height)) & (horiz < np.float32(radius))
