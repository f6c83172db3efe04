"""Scene builders used by tests and benchmarks (warpmpm.scenes, src/warpmpm/scenes.py:10-34),
plus the synthetic workloads the benchmark runs (dam break, pour)."""
from __future__ import annotations

import numpy as np

from .materials import Material, newtonian


def dough(eta: float = 40.0, tau_y: float = 200.0) -> Material:
    """Bingham preset of the squeeze-flow study: newtonian(eta) with a yield stress."""
    return newtonian(eta=eta, density=1000.0).with_yield(tau_y)


def block(grid, size=(0.12, 0.05, 0.06), center=None, ppc: int = 2, seed: int = 0):
    """Jittered particle box resting 3 cells above the domain floor.
    Returns (pos[N,3] float32, vol[N] float32, floor_z)."""
    dx = grid.dx
    floor = 3 * dx
    h = dx / ppc
    cx = grid.grid_lim * 0.5 if center is None else center[0]
    cy = grid.grid_lim * 0.5 if center is None else center[1]
    sx, sy, sz = size
    axes = (np.arange(cx - 0.5 * sx + 0.5 * h, cx + 0.5 * sx, h),
            np.arange(cy - 0.5 * sy + 0.5 * h, cy + 0.5 * sy, h),
            np.arange(floor + 0.5 * h, floor + sz, h))
    pts = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
    pts = pts + np.random.default_rng(seed).uniform(-0.25 * h, 0.25 * h, size=pts.shape)
    pos = pts.astype(np.float32)
    return pos, np.full(len(pos), h ** 3, dtype=np.float32), floor


def dam_break_lattice(n_grid: int = 64, grid_lim: float = 1.0, lo=(0.05, 0.05, 0.05), hi=(0.4, 0.6, 0.95),
                      seed: int = 0):
    """Dam-break fill: 8 particles per cell (spacing dx/2) over the box [lo, hi] with
    +-h/4 seeded jitter. At 64^3 on the unit cube this is 362,250 particles."""
    dx = grid_lim / n_grid
    h = 0.5 * dx
    axes = [np.arange(lo[a] + 0.5 * h, hi[a], h) for a in range(3)]
    pts = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
    pts = pts + np.random.default_rng(seed).uniform(-0.25 * h, 0.25 * h, size=pts.shape)
    pos = pts.astype(np.float32)
    return pos, np.full(len(pos), h ** 3, dtype=np.float32)


# ---- the 340,489-particle pour (examples/pour_franka.py:73-116, 266-291, 341-365) ----
POUR_GRID_LIM = 0.7
POUR_SOURCE = (0.22, 0.50, 0.34)       # source glass centre in the MPM domain (scripted stand-in for the arm)
POUR_RECEIVER = (0.46, 0.38, 0.14)     # receiver glass resting on the floor
POUR_FLOOR_Z = 0.02
HONEY = dict(eta=10.0, density=1420.0, bulk_modulus=9.0e5)


def pour_substeps(liq: dict, dx: float, dt_tick: float = 1.0 / 60.0, cfl: float = 0.28) -> int:
    """Acoustic CFL plus the explicit-viscosity bound (examples/pour_franka.py:98-110)."""
    c = float(np.sqrt(1.1 * liq["bulk_modulus"] / liq["density"]))
    acoustic = c / (cfl * dx)
    viscous = 6.0 * liq["eta"] / (liq["density"] * dx * dx)
    return int(np.ceil(dt_tick * max(acoustic, viscous)))


class PourTrajectory:
    """Scripted source-glass pose: upright, then a smoothstep tilt of `angle_deg`
    over `duration` s toward the receiver, then hold (w x y z quaternions)."""

    def __init__(self, angle_deg: float = 115.0, start: float = 0.1, duration: float = 1.2):
        from .glass import quat_from_axis_angle
        d = np.array(POUR_RECEIVER[:2]) - np.array(POUR_SOURCE[:2])
        self.axis = np.array([-d[1], d[0], 0.0]) / np.linalg.norm(d)   # z x d: tips the rim toward d
        self.angle, self.start, self.duration = np.deg2rad(angle_deg), start, duration
        self._q = quat_from_axis_angle

    def quat(self, t: float):
        u = min(max((t - self.start) / self.duration, 0.0), 1.0)
        return self._q(self.axis, self.angle * u * u * (3.0 - 2.0 * u))

    def command(self, t: float, dt_tick: float):
        """(center, quat, velocity, omega) for the control tick starting at t."""
        from .glass import angular_velocity_between
        q0, q1 = self.quat(t), self.quat(t + dt_tick)
        return POUR_SOURCE, q0, (0.0, 0.0, 0.0), angular_velocity_between(q0, q1, dt_tick)


def pour_scene(solver_cls, n_grid: int = 192, material=None, glass: str = "cup", **solver_kw):
    """The reference pour geometry: default GlassProfile filled to 80 % with cup_fill at
    h = dx/2 (340,489 particles at 192^3, grid_lim 0.7), a separable floor (mu 0.3),
    domain walls, a source and a receiver glass (friction 0.05), as revolved-SDF cups
    or, with glass="cdf", as CPIC sheets of the cavity (examples/pour_franka.py:266-291).
    Returns (solver, source handle, receiver handle, trajectory, substeps per 1/60 s
    frame, dt)."""
    from .glass import GlassProfile, cup_fill, glass_cdf
    from .solver import GridConfig
    prof = GlassProfile()
    grid = GridConfig(n_grid=n_grid, grid_lim=POUR_GRID_LIM)
    pos_local, vol = cup_fill(prof, grid.dx / 2, fill_fraction=0.80)
    pos = (pos_local + np.asarray(POUR_SOURCE)).astype(np.float32)
    s = solver_cls(grid=grid, **solver_kw).load_particles(pos, vol)
    s.set_material(material if material is not None else newtonian(**HONEY))
    s.add_plane((0, 0, POUR_FLOOR_Z), (0, 0, 1), "separate", friction=0.3)
    s.add_domain_walls()
    traj = PourTrajectory()
    if glass == "cdf":
        cdf = glass_cdf(grid.dx, prof)
        q = traj.quat(0.0)
        src = s.add_cdf_collider(cdf, POUR_SOURCE, quat=(q[1], q[2], q[3], q[0]), friction=0.05)
        rcv = s.add_cdf_collider(cdf, POUR_RECEIVER, friction=0.05)
    else:
        src = s.add_cup(prof, POUR_SOURCE, tuple(traj.quat(0.0)), friction=0.05)
        rcv = s.add_cup(prof, POUR_RECEIVER, (1.0, 0.0, 0.0, 0.0), friction=0.05)
    substeps = pour_substeps(HONEY, grid.dx)
    return s, src, rcv, traj, substeps, (1.0 / 60.0) / substeps


# ---- granular press: a seeded random-height heap of mu(I) grains under a plate ----------
PRESS_GRANULAR = dict(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1.0e6, nu=0.3)


def press_heap(n_grid: int = 256, grid_lim: float = 1.0, seed: int = 0):
    """Heap of grains at 8 particles per cell (spacing dx/2, +-h/4 seeded jitter) over
    the square footprint [0.25, 0.75]^2 x grid_lim, standing on the floor 3 cells up.
    Its height at (x, y) is 0.06 grid_lim plus a seeded smooth field of amplitude
    0.025 grid_lim (six random plane waves), so the plate meets the peaks first. At
    256^3 on the unit cube this is about 2.0 M particles. Returns (pos, vol, floor_z)."""
    dx = grid_lim / n_grid
    h = 0.5 * dx
    floor = 3 * dx
    rng = np.random.default_rng(seed)
    k = rng.uniform(1.0, 4.0, (6, 2)) * (2.0 * np.pi / (0.5 * grid_lim)) * rng.choice([-1.0, 1.0], (6, 2))
    phase = rng.uniform(0.0, 2.0 * np.pi, 6)
    ax = np.arange(0.25 * grid_lim + 0.5 * h, 0.75 * grid_lim, h)
    X, Y = np.meshgrid(ax, ax, indexing="ij")
    field = sum(np.cos(k[i, 0] * X + k[i, 1] * Y + phase[i]) for i in range(6)) / np.sqrt(6.0)
    height = grid_lim * (0.06 + 0.025 * np.clip(field, -1.5, 1.5) / 1.5)
    layers = np.floor(height / h).astype(np.int64)
    reps = layers.reshape(-1)
    xy = np.repeat(np.stack([X.reshape(-1), Y.reshape(-1)], -1), reps, axis=0)
    z = floor + 0.5 * h + h * (np.arange(reps.sum()) - np.repeat(np.cumsum(reps) - reps, reps))
    pts = np.concatenate([xy, z[:, None]], axis=1)
    pts = pts + rng.uniform(-0.25 * h, 0.25 * h, size=pts.shape)
    pos = pts.astype(np.float32)
    return pos, np.full(len(pos), h ** 3, dtype=np.float32), floor


def press_scene(solver_cls, n_grid: int = 256, grid_lim: float = 1.0, plate_speed: float = 0.1, seed: int = 0,
                **solver_kw):
    """The granular press: `press_heap` of mu(I) grains (mu_s 0.38, delta_mu 0.26,
    I0 0.28, rho 2500, E 1e6, nu 0.3) on a sticky floor inside domain walls, pressed
    by a kinematic plate (half size 0.2 x 0.2 x 2 dx) descending at `plate_speed`
    from just above the highest grain. Runs with sparse blocks and a particle sort
    every 8 ticks. dt is the elastic CFL bound 0.3 dx / c_p. Returns (solver, plate
    handle, plate centre at t = 0, plate half size, dt)."""
    from .materials import granular
    from .solver import GridConfig
    grid = GridConfig(n_grid=n_grid, grid_lim=grid_lim)
    pos, vol, floor = press_heap(n_grid, grid_lim, seed)
    kw = dict(sparse=True, sort_interval=8)
    kw.update(solver_kw)
    s = solver_cls(grid=grid, **kw).load_particles(pos, vol)
    s.set_material(granular(**PRESS_GRANULAR))
    s.add_plane((0, 0, floor), (0, 0, 1), "sticky")
    s.add_domain_walls()
    dx = grid.dx
    center = (0.5 * grid_lim, 0.5 * grid_lim, float(pos[:, 2].max()) + 3 * dx)
    half = (0.2 * grid_lim, 0.2 * grid_lim, 2 * dx)
    plate = s.add_box(center, half, velocity=(0.0, 0.0, -plate_speed))
    E, nu, rho = PRESS_GRANULAR["E"], PRESS_GRANULAR["nu"], PRESS_GRANULAR["density"]
    c_p = float(np.sqrt(E * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho))
    return s, plate, center, half, 0.3 * dx / c_p


# ---- batched dough-squeeze scenes ---------------------------------------------------
def squeeze_scene(solver_cls, n_particles: int, n_grid: int, material, grid_lim: float = 0.3,
                  plate_speed: float = 0.05, seed: int = 0, plate_gap: float = 1.0, floor_cells: float = 3.0,
                  **solver_kw):
    """A cubic block of about `n_particles` (8 per cell, jittered) resting on a sticky
    floor `floor_cells` cells up, squeezed by a kinematic plate descending at
    `plate_speed` whose lower face starts `plate_gap` cells above the block (negative:
    pressed into it). Returns (solver, plate handle)."""
    from .solver import GridConfig
    grid = GridConfig(n_grid=n_grid, grid_lim=grid_lim)
    dx = grid.dx
    h = 0.5 * dx
    side = max(4, int(round((n_particles ** (1.0 / 3.0)))))
    edge = side * h
    floor = floor_cells * dx
    c = 0.5 * grid_lim
    ax = np.arange(side) * h + 0.5 * h
    pts = np.stack(np.meshgrid(ax + c - 0.5 * edge, ax + c - 0.5 * edge, ax + floor, indexing="ij"),
                   axis=-1).reshape(-1, 3)
    pts = pts + np.random.default_rng(seed).uniform(-0.25 * h, 0.25 * h, size=pts.shape)
    s = solver_cls(grid=grid, **solver_kw).load_particles(pts.astype(np.float32), np.full(len(pts), h ** 3, np.float32))
    s.set_material(material)
    s.add_plane((0, 0, floor), (0, 0, 1), "sticky")
    s.add_domain_walls()
    top = floor + edge
    plate = s.add_box((c, c, top + (plate_gap + 1.0) * dx), (0.6 * edge + 2 * dx, 0.6 * edge + 2 * dx, dx),
                      velocity=(0.0, 0.0, -plate_speed))
    return s, plate


def squeeze_batch_specs(n_scenes: int = 64, seed: int = 0):
    """Seeded scene parameters of the batched forward workload: particle counts
    log-uniform in [8k, 120k], grids 48^3..128^3, E log-uniform [1e4, 1e6], nu in
    [0.2, 0.45], yield log-uniform [1e2, 1e4], von Mises or elastic."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_scenes):
        specs.append(dict(
            n_particles=int(np.exp(rng.uniform(np.log(8e3), np.log(120e3)))),
            n_grid=int(rng.choice([48, 64, 80, 96, 112, 128])),
            E=float(np.exp(rng.uniform(np.log(1e4), np.log(1e6)))),
            nu=float(rng.uniform(0.2, 0.45)),
            yield_stress=float(np.exp(rng.uniform(np.log(1e2), np.log(1e4)))),
            vonmises=bool(i % 2 == 0),
            seed=i,
        ))
    return specs


def squeeze_from_spec(solver_cls, spec: dict, **solver_kw):
    from .materials import elastic, vonmises
    mat = (vonmises(E=spec["E"], nu=spec["nu"], yield_stress=spec["yield_stress"], density=1000.0)
           if spec["vonmises"] else elastic(E=spec["E"], nu=spec["nu"], density=1000.0))
    return squeeze_scene(solver_cls, spec["n_particles"], spec["n_grid"], mat, seed=spec["seed"], **solver_kw)


__all__ = ["HONEY", "PRESS_GRANULAR", "PourTrajectory", "block", "dam_break_lattice", "dough", "pour_scene",
           "pour_substeps", "press_heap", "press_scene", "squeeze_batch_specs", "squeeze_from_spec", "squeeze_scene"]
