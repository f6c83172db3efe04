"""Small scenes shared by the oracle physics gates and the GPU parity tests.

Each builder takes a solver class with the warpmpm.Solver surface
(mpm_engine_gb300.Solver or oracle.oracle.OracleSolver) and returns the loaded
scene plus whatever the test reads back.
"""
from __future__ import annotations

import numpy as np

from mpm_engine_gb300 import GlassProfile, GridConfig, cup_fill, newtonian
from mpm_engine_gb300.materials import elastic, granular, tabulated_viscous, vonmises
from mpm_engine_gb300.scenes import block, dough

SMALL_CUP = GlassProfile(outer_radius=0.05, inner_radius=0.04, height=0.12, base_thickness=0.02,
                         fillet_radius=0.006)


def make(cls, n_grid, grid_lim, **kw):
    """Instantiate either solver flavour with the same grid."""
    if cls.__name__ == "OracleSolver":
        return cls(n_grid=n_grid, grid_lim=grid_lim, fused=kw.get("fused", True),
                   periodic_x=kw.get("periodic_x", False))
    return cls(grid=GridConfig(n_grid=n_grid, grid_lim=grid_lim), **kw)


def blob(n=2000, seed=0, lo=0.15, size=0.10):
    rng = np.random.default_rng(seed)
    pts = (rng.random((n, 3), dtype=np.float32) * size + lo).astype(np.float32)
    return pts, np.full(n, 1.0e-7, np.float32)


MATERIALS = {
    "newtonian": lambda: newtonian(eta=2.0, density=1000.0, bulk_modulus=2.0e5),
    "herschel_bulkley": lambda: newtonian(eta=0.0, density=1400.0, bulk_modulus=2.0e5).with_yield(50.0)
    .with_powerlaw(K=20.0, n=0.6),
    "bingham": lambda: dough(),
    "jelly": lambda: elastic(E=5.0e4, nu=0.3, density=800.0),
    "metal": lambda: vonmises(E=1.0e5, nu=0.3, yield_stress=2.0e3, density=1200.0),
    "metal_hardening": lambda: vonmises(E=1.0e5, nu=0.3, yield_stress=5.0e2, hardening_xi=0.5, density=1200.0),
    "mu_i": lambda: granular(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1e5, nu=0.3),
    "mu_i_phi": lambda: granular(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1e5, nu=0.3)
    .with_dilatancy(phi_init=0.6, chi=0.2),
    "tabulated": lambda: tabulated_viscous([8.0, 4.0, 2.0, 1.0, 0.5], smin=-1.0, smax=2.0, bulk_modulus=2.0e5),
    "sand": "sand",
    "water": "fluid",
    "plasticine": "plasticine",
}

# extra per-type parameters for the fork names used as plain strings
NAME_PARAMS = {
    "sand": dict(E=1.0e5, nu=0.3, density=1600.0, friction_angle=30.0),
    "fluid": dict(density=1000.0, bulk_modulus=2.0e5),
    "plasticine": dict(E=1.0e5, nu=0.3, density=1200.0, yield_stress=1.0e3, softening=0.1, hardening=0.0),
}


# laws named by engine name and per-type parameters, compared outside the
# all-materials sweep: tabulated mu(I) (id 13, mpm_utils.py:327-407), whose friction
# coefficient is a table over log10 I
EXTRA_MATERIALS = {
    "tabulated_mu_i": ("tabulated_mu_i", dict(E=1.0e5, nu=0.3, density=2500.0, eta_table=[0.38, 0.45, 0.55, 0.64],
                                               eta_table_smin=-4.0, eta_table_smax=0.0, grain_diameter=1.0e-3,
                                               grain_density=2650.0)),
}


def spin_velocity(pts, lin=(0.3, 0.1, -0.4), omega=(0.0, 1.0, 3.0)):
    """A translating, spinning initial velocity field v0 = lin + omega x (x - centroid)."""
    c = pts.mean(axis=0)
    return (np.asarray(lin, np.float32) + np.cross(np.asarray(omega, np.float32), pts - c)).astype(np.float32)


def blob_scene(cls, material_key, n_grid=48, grid_lim=0.4, fused=True, cup=False, box=False, n=2000, v0=False,
               cov=None, cov_mode="step", **kw):
    """A blob on a separable floor with domain walls (the fused-pipeline test
    scene, tests/test_fused_pipeline.py:27-56), optionally thrown with a spinning
    initial velocity, with a moving cup or a descending plate, optionally carrying a
    per-particle covariance (load_particles' cov and cov_mode)."""
    pts, vol = blob(n=n)
    s = make(cls, n_grid, grid_lim, fused=fused, **kw)
    s = s.load_particles(pts, vol) if cov is None else s.load_particles(pts, vol, cov=cov, cov_mode=cov_mode)
    if v0:
        vel = spin_velocity(pts)
        if cls.__name__ == "OracleSolver":
            s.a["v"][:] = vel
        else:
            s.set_v(vel)
    mat = MATERIALS[material_key] if material_key in MATERIALS else EXTRA_MATERIALS[material_key]
    if isinstance(mat, tuple):
        s.set_material(mat[0], **mat[1])
    elif isinstance(mat, str):
        s.set_material(mat, **NAME_PARAMS[mat])
    else:
        s.set_material(mat())
    dx = grid_lim / n_grid
    s.add_plane((0, 0, 3 * dx), (0, 0, 1), "separate", friction=0.3)
    s.add_domain_walls()
    h = None
    if cup:
        h = s.add_cup(SMALL_CUP, np.array([0.2, 0.2, 3 * dx + 0.001]))
        s.set_cup(h, center=np.array([0.2, 0.2, 3 * dx + 0.001]), quat=(1.0, 0.0, 0.0, 0.0),
                  velocity=(0.02, 0.0, 0.0), omega=(0.0, 0.0, 0.3))
    if box:
        h = s.add_box((0.2, 0.2, 0.27), (0.08, 0.08, 0.01), velocity=(0.0, 0.0, -0.5))
    return s, h


def water_in_cup(cls, n_grid=40, grid_lim=0.35, fill=0.5):
    """A cup of water on the floor (tests/test_pour.py:25-37)."""
    dx = grid_lim / n_grid
    h = dx / 2
    pos_local, vol = cup_fill(GlassProfile(), h, fill_fraction=fill)
    cup_pos = np.array([0.5 * grid_lim, 0.5 * grid_lim, 0.16])
    s = make(cls, n_grid, grid_lim).load_particles((pos_local + cup_pos).astype(np.float32), vol)
    s.set_material(newtonian(eta=1.0e-3, density=1000.0, bulk_modulus=9.0e5))
    s.add_plane((0, 0, 3 * dx), (0, 0, 1), "separate", friction=0.3)
    s.add_domain_walls()
    return s, cup_pos, vol, h


def dam_break(cls, n_grid=32, grid_lim=1.0, hi=(0.4, 0.6, 0.95)):
    """Dam-break fill at 8 particles per cell with six sticky planes 3 dx inside the
    faces plus domain walls, Newtonian water (eta 1e-2, rho 1000, K 1e4)."""
    from mpm_engine_gb300.scenes import dam_break_lattice
    pos, vol = dam_break_lattice(n_grid, grid_lim, hi=hi)
    s = make(cls, n_grid, grid_lim).load_particles(pos, vol)
    s.set_material(newtonian(eta=1.0e-2, density=1000.0, bulk_modulus=1.0e4), g=[0.0, 0.0, -9.8])
    add_sticky_box(s, n_grid, grid_lim)
    s.add_domain_walls()
    return s


def add_sticky_box(s, n_grid, grid_lim):
    dx = grid_lim / n_grid
    lo, hi = 3 * dx, grid_lim - 3 * dx
    for axis in range(3):
        p = [0.0, 0.0, 0.0]
        nrm = [0.0, 0.0, 0.0]
        p[axis], nrm[axis] = lo, 1.0
        s.add_plane(tuple(p), tuple(nrm), "sticky")
        p[axis], nrm[axis] = hi, -1.0
        s.add_plane(tuple(p), tuple(nrm), "sticky")


def free_blob(cls, n_grid=40):
    grid = GridConfig(n_grid=n_grid, grid_lim=0.4)
    pos, vol, _ = block(grid, size=(0.08, 0.05, 0.05), ppc=2)
    pos[:, 2] += grid.grid_lim * 0.5 - pos[:, 2].mean()
    s = make(cls, n_grid, 0.4).load_particles(pos, vol)
    s.set_material(dough())
    return s


# ---- CPIC (CDF) scenes: a 32^3 grid over 0.4 m, water at 2 particles per cell
# edge (tests/test_cdf_transfers.py:14-40)
CDF_NG, CDF_LIM = 32, 0.4
CDF_DX = CDF_LIM / CDF_NG


def cdf_water(x0, x1, y0, y1, z0, z1):
    hp = CDF_DX / 2
    ax = [np.arange(a + hp / 2, b, hp) for a, b in ((x0, x1), (y0, y1), (z0, z1))]
    return np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)


def cdf_solver(cls, pos, g=(0.0, 0.0, 0.0), fused=True, floor=True):
    s = make(cls, CDF_NG, CDF_LIM, fused=fused).load_particles(pos, np.full(len(pos), (CDF_DX / 2) ** 3,
                                                                             np.float32))
    s.set_material(newtonian(eta=0.5, density=1000.0, bulk_modulus=5.0e4), g=list(g))
    if floor:
        s.add_plane((0, 0, 3 * CDF_DX), (0, 0, 1), "slip")
    s.add_domain_walls()
    return s


def set_velocity(s, vel):
    if type(s).__name__ == "OracleSolver":
        s.a["v"][:] = vel
    else:
        s.set_v(vel)


def tilted_cube(center, edge, spacing, ax=0.5, ay=0.35):
    """Lattice points of a cube rotated by ax about x then ay about y (radians), so
    its lowest point is one corner."""
    k = np.arange(int(round(edge / spacing))) * spacing
    k = k - k.mean()
    p = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3)
    cx, sx, cy, sy = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    return (p @ (Ry @ Rx).T + np.asarray(center)).astype(np.float32)


def rigid_scene(cls, water=True, fused=True, restitution=0.3, n_grid=32, grid_lim=0.4, height=None):
    """A tilted rigid cube (obj_id 0, density 500) thrown, spinning, at a slip floor
    that is also a restitution surface, optionally above a water slab, inside
    domain walls (the two-way coupling of warpmpm.vehicle at test scale)."""
    dx = grid_lim / n_grid
    h = dx / 2
    floor = 3 * dx
    cube = tilted_cube((0.2, 0.2, floor + (height if height is not None else (0.09 if water else 0.05))), 0.06, h)
    parts = [cube]
    if water:
        ax = np.arange(0.08, 0.32, h)
        w = np.stack(np.meshgrid(ax, ax, np.arange(floor + 0.5 * h, floor + 0.04, h), indexing="ij"), -1)
        w = w.reshape(-1, 3) + np.random.default_rng(1).uniform(-0.2 * h, 0.2 * h, (w.size // 3, 3))
        parts.insert(0, w.astype(np.float32))
    pos = np.concatenate(parts).astype(np.float32)
    n_w = len(pos) - len(cube)
    s = make(cls, n_grid, grid_lim, fused=fused).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(newtonian(eta=0.5, density=1000.0, bulk_modulus=4.0e4))
    s.set_material_range(n_w, len(pos), "rigid", obj_id=0, density=500.0)
    s.finalize_rigid_bodies()
    s.add_plane((0, 0, floor), (0, 0, 1), "slip", friction=0.2, restitution=restitution)
    s.add_domain_walls()
    set_rigid_motion(s, n_w, (0.3, -0.1, -1.0), (0.0, 2.0, 1.0))
    return s, n_w


def set_rigid_motion(s, n_w, v_cm, omega):
    """Body velocity and the matching particle velocities v_cm + omega x r: the
    body's own velocity alone is replaced by its particles' momentum at the first
    substep (the rigid tail gathers it from the grid they deposit to)."""
    s.set_rigid_body_velocity(0, v_cm, omega)
    x = np.asarray(s.x(), np.float64)
    com = np.asarray(s.rigid_state(0)["com"], np.float64)
    v = np.array(s.v(), np.float32)
    v[n_w:] = (np.asarray(v_cm) + np.cross(np.asarray(omega), x[n_w:] - com)).astype(np.float32)
    if hasattr(s, "set_v"):
        s.set_v(v)
    else:
        s.a["v"][:] = v
