#!/usr/bin/env python3
"""Particle-substeps/s of the explicit MLS/APIC step on the 340,489-particle pour.

One bench step = one 1/60 s frame = 432 substeps of Solver.step on the reference
pour geometry (default GlassProfile filled to 80 %, 192^3 grid on a 0.7 m domain,
honey eta 10 Pa s, rho 1420, K 9e5, separable floor, domain walls, a tilting
source glass and a receiver). Inputs are seeded synthetic (cup_fill lattice with
seeded jitter); no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's algorithm on the host cores instead:
the CPU restatement in oracle/ (Warp, the reference's runtime, is not installed),
all host threads, a bounded sample of the same frame per step.

Under torchrun (N > 1) every rank runs an independent replica of the scene on its
own GPU (the path has no cross-GPU exchange); value sums all ranks' work over the
slowest rank's time.

Beside the headline the line carries:
- `roofline`: the fused particle pass against the measured HBM copy;
- `e2e`: the same frames through the public API with host inputs and outputs;
- `cpu_baseline`: the oracle on all host cores and on one thread;
- `pour_phases`: the upright and the tilting frames;
- `batched` and `batched_adjoint`: many scenes in one graph, sharded whole
  across ranks;
- `pour_cdf`: the pour with CPIC glasses;
- `flood_vehicle`: rigid-body coupling;
- `press`: the granular press, graded against FP32 and HBM;
- `dam` and `pour_hb`: the 64^3 dam break (362,250 particles, 100 substeps a step)
  and the pour with the Herschel-Bulkley fluid, timed like the headline.
Each can be switched off with its --no-* flag.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "particle-substeps/s on 340k pour"
UNIT = "particle-substeps/s"
# algorithmic bytes per unit (particle-substep): x, v, C, F read + write (192 B) and
# mass + volume read (8 B); grid traffic per active node (56 B) is attributed to the
# grid kernel, not the particle pass this roofline line describes
BYTES_PER_PARTICLE_SUBSTEP = 200.0
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["pour", "pour_hb", "pour_cdf", "dam", "press"], default="pour")
    ap.add_argument("--n-grid", type=int, default=192)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-cdf", action="store_true")
    ap.add_argument("--no-flood", action="store_true")
    ap.add_argument("--no-press", action="store_true")
    ap.add_argument("--no-others", action="store_true", help="skip the dam-break and Herschel-Bulkley pour lines")
    return ap.parse_args()


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(name: str, n_grid: int, solver_cls, **kw):
    """Returns (solver, frame(i) callable, particles, substeps per step, description)."""
    from mpm_engine_gb300 import newtonian
    from mpm_engine_gb300.scenes import dam_break_lattice, pour_scene
    if name in ("pour", "pour_hb", "pour_cdf"):
        mat = None
        if name == "pour_hb":
            mat = newtonian(eta=0.0, density=1400.0, bulk_modulus=9.0e5).with_yield(50.0).with_powerlaw(K=20.0, n=0.6)
        glass = "cdf" if name == "pour_cdf" else "cup"
        s, src, rcv, traj, S, dt = pour_scene(solver_cls, n_grid=n_grid, material=mat, glass=glass, **kw)

        def frame(i, s=s, n=None):
            t = i / 60.0
            c, q, v, w = traj.command(t, 1.0 / 60.0)
            if glass == "cdf":
                s.set_cdf_pose(src, center=c, quat=(q[1], q[2], q[3], q[0]), velocity=v, omega=w)
            else:
                s.set_cup(src, center=c, quat=q, velocity=v, omega=w)
            s.step(dt, S if n is None else n)

        label = {"pour": "honey", "pour_hb": "herschel_bulkley", "pour_cdf": "honey_cdf_glasses"}[name]
        desc = {"workload": f"pour_{label}_{n_grid}^3",
                "particles": s.n_particles, "substeps_per_step": S, "dt": dt, "grid_lim": 0.7}
        return s, frame, s.n_particles, S, desc
    if name == "dam":
        # dam break: 8 particles per cell over [0.05,0.4]x[0.05,0.6]x[0.05,0.95] of the unit cube,
        # Newtonian water (eta 1e-2, rho 1000, K 1e4), six sticky planes 3 dx inside the faces
        from mpm_engine_gb300.solver import GridConfig
        pos, vol = dam_break_lattice(n_grid, 1.0)
        s = solver_cls(grid=GridConfig(n_grid=n_grid, grid_lim=1.0), **kw).load_particles(pos, vol)
        s.set_material(newtonian(eta=1.0e-2, density=1000.0, bulk_modulus=1.0e4), g=[0.0, 0.0, -9.8])
        dx = 1.0 / n_grid
        for axis in range(3):
            for val, nrm in ((3 * dx, 1.0), (1.0 - 3 * dx, -1.0)):
                p, q = [0.0] * 3, [0.0] * 3
                p[axis], q[axis] = val, nrm
                s.add_plane(tuple(p), tuple(q), "sticky")
        s.add_domain_walls()
        S, dt = 100, 1.0e-4

        def frame(i, s=s, n=None):
            s.step(dt, S if n is None else n)

        desc = {"workload": f"dam_break_{n_grid}^3", "particles": s.n_particles, "substeps_per_step": S, "dt": dt,
                "grid_lim": 1.0}
        return s, frame, s.n_particles, S, desc
    if name == "press":
        # the granular press as the main workload: one step = one 20-substep tick
        from mpm_engine_gb300.scenes import press_scene
        s, plate, center, half, dt = press_scene(solver_cls, n_grid=n_grid, **kw)
        S = 20

        def frame(i, s=s, n=None):
            s.step(dt, S if n is None else n)

        desc = {"workload": f"press_mu_i_{n_grid}^3", "particles": s.n_particles, "substeps_per_step": S, "dt": dt,
                "grid_lim": 1.0}
        return s, frame, s.n_particles, S, desc
    raise SystemExit(f"unknown workload {name}")


def batched_measure(n_scenes: int, ticks: int, substeps: int = 100, dt: float = 1.0e-5, device: str = "cuda:0",
                    rank: int = 0, world: int = 1):
    """Batched forward workload: n_scenes seeded dough-squeeze scenes (8k..120k
    particles, 48^3..128^3 grids, per-scene E, nu, yield, von Mises or elastic,
    plate at 0.05 m/s). One scene-tick = `substeps` substeps of one scene. The plain
    path steps the Solvers one after another (the reference's serial rollouts); the
    batched path advances all scenes in one CUDA graph. With several ranks the
    scenes are sharded whole (sharding.partition, balanced by particle count): each
    rank builds and steps only its share, and the rates are every rank's
    scene-ticks over the slowest rank's time."""
    import torch
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.scenes import squeeze_batch_specs, squeeze_from_spec
    from mpm_engine_gb300.sharding import ShardedBatch, sharded_throughput
    specs = squeeze_batch_specs(n_scenes)
    shard = ShardedBatch(lambda i: squeeze_from_spec(Solver, specs[i], device=device)[0],
                         [sp["n_particles"] for sp in specs], rank, world)
    scenes, batch = shard.scenes, shard.batch
    n_local = len(scenes)
    tuned = None
    if batch is not None:                  # the project's autotuner picks the launch shape
        tuned = batch.autotune(dt, substeps, ticks=1)
        tuned = {"choice": dict(zip(("single_launch", "tile_threads", "tile_occ", "grid_ctas_per_sm"),
                                    tuned["tuning"])), "cached": tuned["cached"],
                 "ms_per_tick_by_candidate": tuned["ms_per_tick"]}
    for sc in scenes:                      # warm-up: capture each scene's own graph
        sc.step(dt, substeps)
    shard.step(dt, substeps)               # warm-up: capture the batch graph
    torch.cuda.synchronize()

    def timed(fn):
        t0 = time.perf_counter()
        for _ in range(ticks):
            fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    t_plain = timed(lambda: [sc.step(dt, substeps) for sc in scenes])
    launches0 = batch.launch_count() if batch else 0
    t_batch = timed(lambda: shard.step(dt, substeps))
    launches = (batch.launch_count() if batch else 0) - launches0
    red = "cuda" if world > 1 and torch.distributed.get_backend() == "nccl" else "cpu"
    rate_b, _, _ = sharded_throughput(n_local * ticks, t_batch, device=red)
    rate_p, _, _ = sharded_throughput(n_local * ticks, t_plain, device=red)
    rate_pp, n_part, _ = sharded_throughput(shard.particles() * substeps * ticks, t_batch, device=red)
    n_part /= substeps * ticks
    return {"metric": "batched forward scene-ticks/s", "unit": f"scene-ticks/s ({substeps} substeps each)",
            "value": rate_b, "plain_value": rate_p, "speedup_vs_plain": rate_b / rate_p,
            "scenes": n_scenes, "particles_total": int(n_part), "ticks": ticks, "dt": dt,
            "particle_substeps_per_s": rate_pp, "gpu_launches": launches, "substeps_timed": ticks * substeps,
            "autotuned": tuned,
            "sharding": {"ranks": world, "scenes_on_rank0": n_local} if world > 1 else None}


def workload_measure(name: str, n_grid: int, frames: int = 4, warmup: int = 3, device: str = "cuda:0"):
    """Another configuration timed like the headline (CUDA events per frame, 256 MB
    written between frames to flush L2): ms per step and particle-substeps/s."""
    import torch
    from mpm_engine_gb300 import Solver
    s, frame, n, S, desc = build_workload(name, n_grid, Solver, device=device)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=device)
    for i in range(warmup):
        frame(i)
    torch.cuda.synchronize()
    ms = []
    for k in range(frames):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        frame(warmup + k)
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    per = sum(ms) / len(ms)
    out = {**desc, "ms_per_step": per, "particle_substeps_per_s": n * S / (per / 1e3), "frames": [warmup,
           warmup + frames - 1]}
    del s, frame, flush
    torch.cuda.empty_cache()
    return out


def cdf_pour_measure(n_grid: int = 192, frames: int = 4, warmup: int = 24, device: str = "cuda:0"):
    """The pour with both glasses as CPIC (CDF) sheets, the reference's costly case:
    ms per 1/60 s frame, timed mid-tilt (from t = 0.4 s), where the source glass
    restamps every substep (live ticks)."""
    import torch
    from mpm_engine_gb300 import Solver
    s, frame, n, S, desc = build_workload("pour_cdf", n_grid, Solver, device=device)
    for i in range(warmup):
        frame(i)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for i in range(frames):
        frame(warmup + i)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / frames
    return {"workload": desc["workload"], "particles": n, "substeps_per_frame": S, "ms_per_frame": ms,
            "particle_substeps_per_s": n * S / (ms / 1e3), "frames": frames,
            "cdf_stamps": s.cdf_grids()[2]}


def flood_measure(n_grid: int = 128, frames: int = 3, warmup: int = 2, device: str = "cuda:0"):
    """A flood surge hitting a rigid body, the two-way coupling of warpmpm.vehicle
    (src/warpmpm/vehicle.py:213-310) at its scale: a 1 m domain, a water slab
    (density 1000, eta 1e-3, bulk modulus 4e4) rushing at 1.2 m/s toward a
    0.25 x 0.12 x 0.10 m rigid box (density 400) resting on a slip floor; the floor
    and four side walls are restitution surfaces (e = 0.05). Substeps per 1/60 s
    frame from the acoustic, viscous and advective bounds, as the reference sets
    them. The reference runs such scenes on its split pipeline with a host restitution
    loop every substep; here they stay on the fused, graph-captured tick."""
    import torch
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    lim = 1.0
    dx = lim / n_grid
    h = dx / 2
    wall, floor = 4 * dx, 3 * dx
    rng = np.random.default_rng(0)
    ax = lambda a, b: np.arange(a + 0.5 * h, b, h)  # noqa: E731
    water = np.stack(np.meshgrid(ax(wall, 0.55), ax(wall, lim - wall), ax(floor, floor + 0.12), indexing="ij"), -1)
    water = (water.reshape(-1, 3) + rng.uniform(-0.2 * h, 0.2 * h, (water.size // 3, 3))).astype(np.float32)
    box = np.stack(np.meshgrid(ax(0.62, 0.87), ax(0.44, 0.56), ax(floor, floor + 0.10), indexing="ij"), -1)
    box = box.reshape(-1, 3).astype(np.float32)
    pos = np.concatenate([water, box])
    s = Solver(grid=GridConfig(n_grid=n_grid, grid_lim=lim), device=device).load_particles(
        pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(newtonian(eta=1.0e-3, density=1000.0, bulk_modulus=4.0e4))
    s.set_material_range(len(water), len(pos), "rigid", obj_id=0, density=400.0)
    s.finalize_rigid_bodies()
    s.add_plane((0, 0, floor), (0, 0, 1), "slip", friction=0.3, restitution=0.05)
    for pt, nrm in (((wall, 0, 0), (1, 0, 0)), ((lim - wall, 0, 0), (-1, 0, 0)),
                    ((0, wall, 0), (0, 1, 0)), ((0, lim - wall, 0), (0, -1, 0))):
        s.add_plane(pt, nrm, "slip", friction=0.0, restitution=0.05)
    s.add_domain_walls()
    c = float(np.sqrt(1.1 * 4.0e4 / 1000.0))
    rate = max(c / (0.28 * dx), 6.0 * 1.0e-3 / (1000.0 * dx * dx), 1.2 / (0.5 * dx))
    S = int(np.ceil(rate / 60.0))
    dt = (1.0 / 60.0) / S
    v = np.zeros_like(pos)
    v[: len(water), 0] = 1.2
    s.set_v(v)
    for _ in range(warmup):
        s.step(dt, S)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(frames):
        s.step(dt, S)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / frames
    st = s.rigid_state(0)
    return {"workload": f"flood_vehicle_{n_grid}^3", "particles": len(pos), "rigid_particles": len(box),
            "substeps_per_frame": S, "ms_per_frame": ms, "particle_substeps_per_s": len(pos) * S / (ms / 1e3),
            "frames": frames, "body_com_x": float(st["com"][0]), "body_v_x": float(st["v"][0])}


def adjoint_measure(n_scenes: int = 32, n_particles: int = 50_000, n_grid: int = 48, substeps: int = 400,
                    every: int = 20, dt: float = 1.0e-5, device: str = "cuda:0", seed: int = 0):
    """Batched forward+adjoint workload (the identification loss): n_scenes von Mises
    cubes of about n_particles (8 per cell, jittered) on n_grid^3 grids, squeezed by
    a plate at 0.05 m/s; per scene seeded E log-uniform [1e4, 1e6], nu in
    [0.2, 0.45], yield log-uniform [1e2, 1e4]. Each scene has a seeded target rollout
    (E, nu and the yield 30 %, 5 % and 30 % higher; run once, untimed). One scene =
    a rollout of `substeps` substeps with checkpoints every `every`, the loss
    L = |x - x_target|^2 + |F - F_target|^2 over the final positions and the plate's
    per-segment reaction-force trace, and the reverse pass to v0, E, nu, the yield
    and the plate's velocity. Plain runs the scenes one after another, each keeping
    every substep's state from its forward pass (3 GB a scene) so that its reverse
    pass replays nothing; batched runs all forwards in one CUDA graph per segment and
    the reverse passes, which replay their segments, on one stream per scene."""
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    from mpm_engine_gb300.materials import vonmises
    from mpm_engine_gb300.scenes import squeeze_scene
    rng = np.random.default_rng(seed)
    params = []
    for i in range(n_scenes):
        E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        nu = float(rng.uniform(0.2, 0.45))
        ys = float(np.exp(rng.uniform(np.log(1e2), np.log(1e4))))
        params.append((E, nu, ys))

    def build(scale):
        out, handles = [], []
        for i, (E, nu, ys) in enumerate(params):
            s, h = squeeze_scene(Solver, n_particles, n_grid,
                                 vonmises(E=E * scale[0], nu=nu * scale[1], yield_stress=ys * scale[2],
                                          density=1000.0), seed=i, device=device)
            out.append(s)
            handles.append(h)
        return out, handles

    targets, th = build((1.3, 1.05, 1.3))
    tr = adjoint.BatchRollout(targets, dt, substeps, every, batched=True, plates=th)
    target_out = tr.forward()
    x_t = [o[0].double() for o in target_out]
    F_t = [o[2] for o in target_out]
    del tr, targets
    scenes, handles = build((1.0, 1.0, 1.0))
    starts = [adjoint._snapshot(s) for s in scenes]
    split = {}

    def cotangents(outs):
        return ([2.0 * (o[0].double() - xt) for o, xt in zip(outs, x_t)], [None] * len(outs),
                [2.0 * (o[2] - ft) for o, ft in zip(outs, F_t)])

    keep = [None, None]

    def run(batched, k):
        for s, st in zip(scenes, starts):
            adjoint._restore(s, st)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t_fwd = 0.0
        if batched:
            r = adjoint.BatchRollout(scenes, dt, k, every, batched=True, plates=handles)
            keep[0] = r.keep
            outs = r.forward()
            torch.cuda.synchronize()
            t_fwd = time.perf_counter() - t0
            if k == substeps:
                xb, vb, fb = cotangents(outs)
            else:   # warm-up: any cotangent
                xb, vb, fb = [o[0] for o in outs], [None] * len(outs), [o[2] for o in outs]
            r.backward(xb, vb, fb)
        else:
            for i, s in enumerate(scenes):
                t1 = time.perf_counter()
                r = adjoint.BatchRollout([s], dt, k, every, batched=False, plates=[handles[i]])
                keep[1] = r.keep
                out = r.forward()[0]
                torch.cuda.synchronize()
                t_fwd += time.perf_counter() - t1
                if k == substeps:
                    xb = 2.0 * (out[0].double() - x_t[i])
                    fb = 2.0 * (out[2] - F_t[i])
                else:
                    xb, fb = out[0], out[2]
                r.backward([xb], [None], [fb])
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        split["batched" if batched else "plain"] = {"forward_s": t_fwd, "backward_s": el - t_fwd}
        return el

    run(True, 2 * every)     # warm-up: scratch, graphs
    run(False, 2 * every)
    t_plain = run(False, substeps)
    t_batch = run(True, substeps)
    n_total = sum(s.n_particles for s in scenes)
    return {"metric": "batched forward+adjoint scenes/s", "unit": f"scenes/s ({substeps} substeps each)",
            "value": n_scenes / t_batch, "plain_value": n_scenes / t_plain, "speedup_vs_plain": t_plain / t_batch,
            "scenes": n_scenes, "particles_total": n_total, "grid": f"{n_grid}^3", "substeps": substeps,
            "checkpoint_every": every, "dt": dt,
            "loss": "|x - x_target|^2 + |plate force trace - target trace|^2 (seeded target rollouts)",
            "gradients": ["v0", "mu and lam (so E and nu)", "yield_stress", "plate_velocity"],
            "states": {"batched": "kept from the forward pass" if keep[0] else "segments replayed",
                       "plain": "kept from the forward pass" if keep[1] else "segments replayed"},
            "seconds": split,
            "particle_substeps_per_s": n_total * substeps / t_batch}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def fp32_sgemm_tflops(device: str = "cuda:0", n: int = 8192, reps: int = 5) -> float:
    """FP32 issue ceiling measured on this GPU: cuBLAS SGEMM with TF32 off (CUDA-core
    FMAs), n^3 x 2 FLOP per product, best of `reps` after one warm-up."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, device=device)
        b = torch.randn(n, n, device=device)
        torch.mm(a, b)
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.mm(a, b)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def captured_value(name: str, key: str):
    """A `key: value` line of a committed ncu summary under profiles/, or None."""
    f = REPO / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith(key + ":"):
            return float(line.split(":", 1)[1])
    return None


def press_measure(n_grid: int = 256, ticks: int = 100, substeps: int = 20, device: str = "cuda:0"):
    """The granular press: a seeded random-height heap of mu(I) grains (about 2 M
    particles at 256^3) pressed by a plate at 0.1 m/s, sparse blocks, a particle sort
    every 8 ticks, `ticks` ticks of `substeps` substeps (2000 in all). After every
    tick the plate's stress-integral contact wrench (box_contact_wrench,
    coupling/wrench.py:15-46) is reduced on the device and read back, as the
    reference's press loop records it. Sparse mode runs the split passes, as in the
    reference. The substep is graded against both ceilings. HBM: N x 212 B (x, v, C and
    F read and written, mass, volume, mu, lambda and yield) plus 56 B per active node.
    FP32: N x the FLOPs per particle-substep that ncu counted over the three
    particle passes, against a cuBLAS SGEMM with TF32 off."""
    import torch
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.scenes import press_scene
    s, plate, center, half, dt = press_scene(Solver, n_grid=n_grid, device=device)
    n = s.n_particles
    vz = -0.1
    t = 0.0

    def tick():
        nonlocal t
        s.step(dt, substeps)
        t += dt * substeps
        c = (center[0], center[1], center[2] + vz * t)
        return s.contact_wrench(c, half, layer_cells=2.0, dx=s.grid.dx)

    for _ in range(2):
        tick()
    torch.cuda.synchronize()
    fz = []
    t0 = time.perf_counter()
    for _ in range(ticks):
        fz.append(float(tick()["Fz"]))
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    us_substep = el / (ticks * substeps) * 1e6
    active_nodes = int(s._sim._block_counts[0]) * 64
    bytes_substep = n * 212.0 + active_nodes * 56.0
    hbm_peak, _ = peaks()
    hbm = bytes_substep / (us_substep / 1e6) / 1e9
    flops_p = captured_value("particle_passes_press_mu_i_256.txt", "fp32_flops_per_particle_substep")
    fp32_peak = fp32_sgemm_tflops(device)
    fp32 = None if flops_p is None else n * flops_p / (us_substep / 1e6) / 1e12
    rl = {"hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
                  "bytes_per_substep": bytes_substep, "active_nodes": active_nodes},
          "fp32": {"achieved": fp32, "peak": fp32_peak, "unit": "TFLOP/s",
                   "frac": None if fp32 is None else fp32 / fp32_peak, "flops_per_particle_substep": flops_p,
                   "peak_kind": "measured: cuBLAS SGEMM, TF32 off"}}
    fr = [v["frac"] for v in rl.values() if v["frac"] is not None]
    rl["binding"] = max((k for k in ("hbm", "fp32") if rl[k]["frac"] is not None), key=lambda k: rl[k]["frac"])
    return {"workload": f"press_mu_i_{n_grid}^3", "particles": n, "substeps": ticks * substeps, "dt": dt,
            "us_per_substep": us_substep, "particle_substeps_per_s": n * ticks * substeps / el,
            "plate_Fz_last_N": fz[-1], "roofline": rl, "pipeline": "fused (sparse)", "max_frac": max(fr)}


def captured_traffic(workload: str):
    """DRAM bytes per launch of the fused particle kernel from the committed ncu
    summary of this workload (profiles/k_particles_tiled_<workload>.txt), or None."""
    name = workload.replace("^3", "")
    f = REPO / "profiles" / f"k_particles_tiled_{name}.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


def replica_value(total_ms: float, units_per_step: float, steps: int, world: int, dist=None, device="cpu"):
    """Whole-job throughput of N independent replicas: every rank's units over the
    slowest rank's time (max all-reduce of the timed region). Returns (value, ms)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return world * units_per_step * steps / (total_ms / 1e3), total_ms


def start_state(args):
    """The scene state at the first timed frame of the GPU arm (after `warmup`
    frames), reached on the GPU engine; None without a GPU."""
    import torch
    if not torch.cuda.is_available():
        return None
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.build import build_native
    build_native()
    g, gframe, _, _, _ = build_workload(args.workload, args.n_grid, Solver, device="cuda:0")
    for i in range(args.warmup):
        gframe(i)
    torch.cuda.synchronize()
    st = g.export_state()
    del g, gframe
    torch.cuda.empty_cache()
    return st


def run_reference(args):
    """CPU arm: the oracle restatement of the reference step, all host threads, on
    the frames the GPU arm times. The GPU engine advances the scene through the
    warm-up frames (setup only); from that state the oracle steps the timed frames,
    each step a bounded sample of that frame's substeps under the frame's own
    collider commands."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from oracle.oracle import OracleSolver, build
    build()
    threads = os.cpu_count() or 1
    s, frame, n, S, desc = build_workload(args.workload, args.n_grid, OracleSolver, threads=threads)
    st = start_state(args)
    same = st is not None
    if same:   # the frame callable drives the oracle built from the GPU arm's state
        s = OracleSolver.from_state(st, args.n_grid, desc["grid_lim"], threads=threads)
    # bounded sample per step: calibrate substeps so the whole run stays within minutes
    first = args.warmup if same else 0
    t0 = time.perf_counter()
    frame(first, s=s, n=1)
    per = time.perf_counter() - t0
    m = max(1, min(S, int(args.cpu_seconds / max(per, 1e-6) / max(args.steps + args.warmup, 1))))
    if not same:
        for i in range(args.warmup):
            frame(i, s=s, n=m)
    t0 = time.perf_counter()
    for k in range(args.steps):
        frame(first + k, s=s, n=m)
    el = time.perf_counter() - t0
    value = n * m * args.steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {**desc, "sample_substeps_per_step": m, "l2": "n/a (host CPU)",
                       "frames": [first, first + args.steps - 1],
                       "start_state": "the GPU arm's state after its warm-up frames" if same else "frame 0"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{m} substeps of each of frames {first}..{first + args.steps - 1} of the "
                                       f"{desc['workload']} scene (CPU restatement of the reference step, not Warp)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def s_dt(desc):
    return desc["dt"]


def cpu_baseline(st, desc, seconds: float):
    from oracle.oracle import OracleSolver, build
    build()
    threads = os.cpu_count() or 1
    o = OracleSolver.from_state(st, int(desc["workload"].split("_")[-1].split("^")[0]), desc["grid_lim"],
                                threads=threads)
    t0 = time.perf_counter()
    o.step(desc["dt"], 1)
    per = time.perf_counter() - t0
    m = max(1, int(seconds / max(per, 1e-6)))
    t0 = time.perf_counter()
    o.step(desc["dt"], m)
    el = time.perf_counter() - t0
    n = len(st["x"])
    # one thread as well: Warp's CPU kernels run single-threaded, so this is the
    # closer analogue of the reference's own CPU path (about a quarter of the time)
    o.threads = 1
    t0 = time.perf_counter()
    o.step(desc["dt"], 1)
    per1 = time.perf_counter() - t0
    m1 = max(1, int(0.25 * seconds / max(per1, 1e-6)))
    t0 = time.perf_counter()
    o.step(desc["dt"], m1)
    el1 = time.perf_counter() - t0
    return {"value": n * m / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{m} substeps of the {desc['workload']} frame state after warm-up "
                      f"({n} particles; CPU restatement of the reference step, not Warp)",
            "single_thread": {"value": n * m1 / el1, "cores": 1, "sample": f"{m1} further substeps"}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.build import build_native
    build_native()

    s, frame, n, S, desc = build_workload(args.workload, args.n_grid, Solver, device=f"cuda:{local}")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")   # 256 MB > L2
    for i in range(args.warmup):
        frame(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = s.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record()
        frame(args.warmup + k)
        ev[k][1].record()
    torch.cuda.synchronize()
    launches = s.launch_count() - launches0
    clk = clocks.stop()
    frame_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(frame_ms)
    phases_of_pour = None
    if args.workload.startswith("pour"):
        # the source glass stands upright until t = 0.1 s (frame 6), then tilts
        idx = [args.warmup + k for k in range(args.steps)]
        up = [m for i, m in zip(idx, frame_ms) if i / 60.0 < 0.1]
        tilt = [m for i, m in zip(idx, frame_ms) if i / 60.0 >= 0.1]
        phases_of_pour = {"upright_ms_per_frame": sum(up) / len(up) if up else None,
                          "tilting_ms_per_frame": sum(tilt) / len(tilt) if tilt else None,
                          "frames": [idx[0], idx[-1]]}
    value, total_ms = replica_value(total_ms, n * S, args.steps, world, dist, device=f"cuda:{local}")
    ms_per_step = total_ms / args.steps

    # dominant kernel duration: one frame with per-phase CUDA events (live launches)
    s.profile = True
    s._eng.lib.gbmpm_profile(s._eng.h, None, None, 1)
    frame(args.warmup + args.steps)
    import ctypes as C
    msv = (C.c_double * 6)()
    cnt = (C.c_int64 * 6)()
    s._eng.lib.gbmpm_profile(s._eng.h, msv, cnt, 0)
    s.profile = False
    # The profiled frame brackets every launch with events, so its per-launch times
    # carry launch gaps and lose the programmatic overlap of consecutive passes. The
    # fused pass's in-graph duration is the graph-timed frame apportioned by the
    # profiled frame's shares: ms_per_step x (fused time / all phases) / fused launches.
    live_fused_ms = msv[2] / max(cnt[2], 1)
    grid_ms = msv[3] / max(cnt[3], 1)
    total_prof = sum(msv[i] for i in range(6))
    fused_share = msv[2] / total_prof if total_prof > 0 else 0.0
    fused_ms = ms_per_step * fused_share / cnt[2] if cnt[2] else 0.0
    peak, peak_kind = peaks()
    # split-pipeline workloads (the sparse press) have no fused pass to grade here
    achieved = n * BYTES_PER_PARTICLE_SUBSTEP / (fused_ms / 1e3) / 1e9 if fused_ms > 0 else None
    phases = {s._eng.lib.gbmpm_phase_name(i).decode(): round(msv[i] / max(cnt[i], 1), 5)
              for i in range(6) if cnt[i]}
    traffic = captured_traffic(desc["workload"])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved is not None else None,
                "traffic": traffic, "traffic_unit": "bytes per launch (ncu dram read + write, cold cache)",
                "algorithmic_bytes_per_launch": n * BYTES_PER_PARTICLE_SUBSTEP,
                "kernel": "k_particles_tiled (fused G2P2G)", "kernel_ms": fused_ms,
                "kernel_ms_how": "graph-timed ms_per_step x the fused pass's share of a profiled frame / its "
                                 "launches per frame",
                "fused_share": fused_share, "live_kernel_ms": live_fused_ms,
                "grid_kernel_ms": grid_ms, "peak_kind": peak_kind, "phase_ms_per_launch": phases}

    e2e = None
    if not args.no_e2e:
        # A second instance of the workload, warmed up like the first, so that this
        # host-driven loop steps the same frames as the device-timed region. Each
        # step uploads the positions and velocities the host holds (pinned memory)
        # and reads both back; the state stays the simulation's own.
        s2, frame2, _, _, _ = build_workload(args.workload, args.n_grid, Solver, device=f"cuda:{local}")
        for i in range(args.warmup):
            frame2(i)
        xh = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        vh = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        s2.x_into(xh)
        s2.v_into(vh)
        torch.cuda.synchronize()
        reps = args.steps
        el = 0.0
        for k in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2.set_x(xh)
            s2.set_v(vh)
            frame2(args.warmup + k)
            s2.x_into(xh)
            s2.v_into(vh)
            torch.cuda.synchronize()
            el += time.perf_counter() - t0
        e2e = {"value": world * n * S * reps / el, "unit": UNIT, "h2d_bytes_per_step": 2 * n * 12,
               "d2h_bytes_per_step": 2 * n * 12, "frames": [args.warmup, args.warmup + reps - 1]}
        del s2, frame2
        torch.cuda.empty_cache()

    batched = None
    if not args.no_batched:
        batched = batched_measure(args.batch_scenes, ticks=10, device=f"cuda:{local}", rank=rank, world=world)

    others = None
    if not args.no_others and args.workload == "pour":
        others = {"dam": workload_measure("dam", 64, device=f"cuda:{local}"),
                  "pour_hb": workload_measure("pour_hb", args.n_grid, device=f"cuda:{local}")}

    cdf = None
    if not args.no_cdf and args.workload == "pour":
        cdf = cdf_pour_measure(args.n_grid, device=f"cuda:{local}")

    adj = None
    if not args.no_adjoint:
        adj = adjoint_measure(device=f"cuda:{local}")

    flood = None
    if not args.no_flood and args.workload == "pour":
        flood = flood_measure(device=f"cuda:{local}")

    press = None
    if not args.no_press and args.workload == "pour":
        press = press_measure(device=f"cuda:{local}")

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(s.export_state(), desc, args.cpu_seconds)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {**desc, "l2": "256 MB buffer written between timed steps", "parallelism":
                           "replicas" if world > 1 else "single"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk, "pour_phases": phases_of_pour, "batched": batched, "batched_adjoint": adj,
                "dam": others and others["dam"], "pour_hb": others and others["pour_hb"],
                "pour_cdf": cdf, "flood_vehicle": flood, "press": press}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
