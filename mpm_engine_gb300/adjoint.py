"""Differentiable rollouts: reverse-mode gradients through a Solver's substeps.

The reference has no adjoint; gradient-based identification there is done by
finite differences over serial rollouts. Here `rollout` runs a scene forward on
the engine and returns its final positions and velocities as torch tensors whose
gradients flow, through the engine's adjoint kernels, to the initial velocity
field, Young's modulus, Poisson's ratio, the yield stress and the Newtonian
viscosity. With a kinematic cuboid (`plate`, an add_box handle) the rollout also
returns the cuboid's reaction-force trace, one force per checkpoint segment (what
tool_force reads after each segment, core/solver.py:415-427), and differentiates
the cuboid's trajectory: its velocity, which moves the box and drives the nodes it
covers, is an input like the material parameters.

Memory follows the usual checkpoint-and-recompute scheme: the forward keeps the
state (x, v, C, F_trial, L, yield, and mu, lam, which softening can zero) and the
collider poses every `checkpoint_every` substeps; the backward restores each checkpoint in reverse, replays that segment
one substep at a time (the engine keeps every substep's starting state on the
device) and carries the adjoints back through it (`gbmpm_adjoint_segment`).

Scope: jelly (FCR), von Mises (with or without hardening, with or without
softening), Drucker-Prager sand, mu(I), tabulated mu(I) and mu(I)-Phi(I) granular
flow (its packing state Jp carried as adjoint state), water, Newtonian (Bingham,
Herschel-Bulkley) and tabulated viscous particles; plane, cuboid, domain-wall,
revolved-SDF cup and mesh-SDF colliders; no periodic axis, rpic_damping = 0,
particle order fixed during the rollout (sort_interval = 0). Not covered: CDF
colliders, rigid bodies and particle modifiers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .solver import _torch

_STATE = ("x", "v", "C", "F_trial", "L", "yield_stress", "mu", "lam", "Jp")


def _snapshot(s, particles: bool = True):
    """The scene's clock, collider poses and (with `particles`) particle state."""
    s._pull_colliders()
    cols = []
    for rec in s._cols:
        r = _abi.Collider()
        C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
        cols.append(r)
    return ({k: s._t[k].clone() for k in _STATE} if particles else None), cols, s._time


def _restore(s, snap):
    state, cols, t = snap
    if state is not None:
        for k in _STATE:
            s._t[k].copy_(state[k])
    s._cols = []
    for rec in cols:
        r = _abi.Collider()
        C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
        s._cols.append(r)
    s._cols_dirty = True
    s._time = t
    s._sync_engine()


def _check(s):
    s._require_loaded()
    if s.sort_interval:
        raise ValueError("rollout needs a fixed particle order: set sort_interval = 0")
    if s._cdf:
        raise NotImplementedError("the adjoint does not cover CDF colliders")


STATE_FLOATS = 37   # floats a particle keeps per substep: x 3, v 3, C 9, F_trial 9, L 9, yield, mu, lam, Jp


def state_bytes(n_particles: int, substeps: int) -> int:
    """Device bytes that keeping every substep's state of a rollout takes."""
    return STATE_FLOATS * 4 * int(n_particles) * int(substeps)


def _keep_states(s, substeps, keep):
    """Whether a rollout keeps every substep's state (None: when it takes less than
    half of the free device memory) instead of replaying each segment backwards."""
    if keep is not None:
        return bool(keep)
    torch = _torch()
    free, _ = torch.cuda.mem_get_info(s._t["x"].device)
    return state_bytes(s.n_particles, substeps) < 0.5 * free


def _segment_forward(s, dt, k):
    """Steps one segment on the split schedule, keeping each substep's starting state
    (a device tensor of STATE_FLOATS x n x k floats); the bookkeeping is Solver.step's."""
    torch = _torch()
    if s._tick % max(1, s.guard_interval) == 0:
        s._update_grid_box(dt, k)
    s._tick += 1
    s._pull_colliders()
    s._sync_engine()
    states = torch.empty(STATE_FLOATS * s.n_particles * k, dtype=torch.float32, device=s._t["x"].device)
    t = C.c_double(s._time)
    _abi.check(s._eng.lib.gbmpm_adjoint_forward(s._eng.h, C.byref(t), float(dt), int(k), states.data_ptr(),
                                                s._stream()), "gbmpm_adjoint_forward")
    s._time = t.value
    s._step += k
    return states


def _forward(s, dt, substeps, every, plate=None, keep=False):
    """Runs the rollout, keeping a checkpoint per segment (with `keep`, the segment's
    every substep state instead of its starting particle state); with a plate handle
    also returns the plate's reaction force over each segment ([segments][3] float64)."""
    ckpts, forces = [], []
    done = 0
    while done < substeps:
        k = min(every, substeps - done)
        snap = _snapshot(s, particles=not keep)
        if plate is not None:
            s.reset_tool_force(plate)
        if keep:
            ckpts.append((snap, k, _segment_forward(s, dt, k)))
        else:
            s.step(dt, k)
            ckpts.append((snap, k, None))
        if plate is not None:
            forces.append(s.tool_force(plate, dt * k))
        done += k
    return (ckpts, forces) if plate is not None else ckpts


def _adj_setup(s, xb, vb, plate, kmax):
    """The adjoint arrays of one scene's reverse pass (seeded with the final-state
    adjoints xb, vb) and their ABI record; with a plate also its collider buffers."""
    torch = _torch()
    n = s.n_particles
    dev = s._t["x"].device
    f = dict(device=dev, dtype=torch.float32)
    g = {
        "x": (xb.detach().to(**f).reshape(n, 3).clone() if xb is not None else torch.zeros(n, 3, **f)),
        "v": (vb.detach().to(**f).reshape(n, 3).clone() if vb is not None else torch.zeros(n, 3, **f)),
        "C": torch.zeros(n, 3, 3, **f), "F_trial": torch.zeros(n, 3, 3, **f),
        "yield_stress": torch.zeros(n, **f), "mu": torch.zeros(n, **f), "lam": torch.zeros(n, **f),
        "L": torch.zeros(n, 3, 3, **f), "viscosity": torch.zeros(n, **f), "Jp": torch.zeros(n, **f),
    }
    rec = _abi.AdjGrads(**{k: g[k].data_ptr() for k in g})
    ncol = max(1, len(s._cols))
    col = s._col(plate) if plate is not None else None
    fb = None
    if col is not None:
        g["collider_velocity"] = torch.zeros(ncol, 3, **f)
        rec.collider_velocity = g["collider_velocity"].data_ptr()
        # one buffer for every segment, so the engine's captured segment graph (keyed
        # on the adjoint arrays) is reused; each segment rewrites it in stream order
        fb = torch.zeros(kmax, ncol, 3, **f)
        rec.collider_force = fb.data_ptr()
    return g, rec, fb, col


def _adj_segment(s, dt, rec, snap, k, fb, col, force_bar_j, states=None):
    """Runs one checkpoint segment's reverse substeps (stream order): from its kept
    states, or replaying the segment from its checkpoint first."""
    _restore(s, snap)
    if col is not None:
        # the segment's force is sum_substeps sum_nodes m (v_free - v_box) / (dt k)
        fb.zero_()
        if force_bar_j is not None:
            fb[:k, col, :] = force_bar_j.to(device=fb.device, dtype=fb.dtype) / (dt * k)
    t = C.c_double(s._time)
    if states is not None:
        _abi.check(s._eng.lib.gbmpm_adjoint_reverse(s._eng.h, C.byref(t), float(dt), int(k), states.data_ptr(),
                                                    C.byref(rec), s._stream()), "gbmpm_adjoint_reverse")
    else:
        _abi.check(s._eng.lib.gbmpm_adjoint_segment(s._eng.h, C.byref(t), float(dt), int(k), C.byref(rec),
                                                    s._stream()), "gbmpm_adjoint_segment")


def _adj_finish(g, col):
    if col is not None:
        g["plate_velocity"] = g["collider_velocity"][col].clone()
    return g


def _backward(s, dt, ckpts, xb, vb, plate=None, force_bar=None):
    g, rec, fb, col = _adj_setup(s, xb, vb, plate, max(c[1] for c in ckpts))
    for j in reversed(range(len(ckpts))):
        snap, k, states = ckpts[j]
        _adj_segment(s, dt, rec, snap, k, fb, col, None if force_bar is None else force_bar[j], states)
    return _adj_finish(g, col)


NEWTONIAN = 10   # material id whose per-type viscosity `viscosity` sets


class _Rollout(_torch().autograd.Function):
    @staticmethod
    def forward(ctx, v0, mu, lam, ys0, eta, plate_v, solver, dt, substeps, every, plate, keep):
        torch = _torch()
        s = solver
        s._t["v"].copy_(v0.detach().reshape(-1, 3))
        s._t["mu"].copy_(mu.detach())
        s._t["lam"].copy_(lam.detach())
        s._t["yield_stress"].copy_(ys0.detach())
        s._model.plastic_viscosity[NEWTONIAN] = float(eta)
        s._model_dirty = True
        if plate is not None:
            s.set_box(plate, velocity=tuple(float(c) for c in plate_v.detach().cpu()))
        ctx.solver, ctx.dt, ctx.plate = s, dt, plate
        if plate is not None:
            ctx.ckpts, forces = _forward(s, dt, substeps, every, plate, keep)
            F = torch.tensor(np.array(forces), dtype=torch.float64, device=v0.device)
        else:
            ctx.ckpts = _forward(s, dt, substeps, every, None, keep)
            F = torch.zeros(0, 3, dtype=torch.float64, device=v0.device)
        x, v = s._t["x"].clone(), s._t["v"].clone()
        ctx.final = _snapshot(s)
        return x, v, F

    @staticmethod
    def backward(ctx, xb, vb, Fb):
        s = ctx.solver
        g = _backward(s, ctx.dt, ctx.ckpts, xb, vb, ctx.plate, Fb if ctx.plate is not None else None)
        _restore(s, ctx.final)
        pvb = g.get("plate_velocity")
        return (g["v"], g["mu"], g["lam"], g["yield_stress"], g["viscosity"].sum(), pvb, None, None, None, None,
                None, None)


def mu_lam(E, nu):
    """compute_mu_lam_from_E_nu (mpm_utils.py:583-588) on torch tensors."""
    return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))


def rollout(solver, dt: float, substeps: int, *, v0=None, E=None, nu=None, yield_stress=None, viscosity=None,
            checkpoint_every: int = 20, plate=None, plate_velocity=None, keep_states=None):
    """Advance `solver` by `substeps` substeps of dt and return (x, v) at the end.

    v0 ((N, 3)), E, nu and yield_stress (scalars or (N,) tensors) and viscosity (the
    Newtonian plastic viscosity, a scalar) are the differentiable inputs; any left
    as None keeps the scene's current value and is not differentiated. E and nu set
    mu and lam of every particle through the reference's formula. The solver is
    left at the end state of the rollout.

    With `plate` (an add_box handle) the call returns (x, v, F): F is the plate's
    reaction force over each checkpoint segment ((segments, 3) float64, the
    tool_force of that segment), and `plate_velocity` ((3,), default the plate's
    current velocity) is differentiable: it moves the plate through the rollout and
    drives the grid nodes inside it. Gradients reach it through the positions and
    velocities and through the force trace.

    `keep_states` keeps every substep's state from the forward pass (state_bytes of
    device memory) so that the reverse pass does not replay each segment; None keeps
    them when they take less than half of the free device memory."""
    torch = _torch()
    _check(solver)
    s = solver
    n = s.n_particles
    dev = s._t["x"].device
    f = dict(device=dev, dtype=torch.float32)
    v0 = s._t["v"].clone() if v0 is None else v0.to(**f)
    if E is None and nu is None:
        mu, lam = s._t["mu"].clone(), s._t["lam"].clone()
    else:
        if E is None or nu is None:
            raise ValueError("E and nu are given together")
        E = torch.as_tensor(E, **f) if not torch.is_tensor(E) else E.to(**f)
        nu = torch.as_tensor(nu, **f) if not torch.is_tensor(nu) else nu.to(**f)
        mu, lam = mu_lam(E, nu)
        mu, lam = mu.expand(n), lam.expand(n)
    if yield_stress is None:
        ys = s._t["yield_stress"].clone()
    else:
        ys = (yield_stress if torch.is_tensor(yield_stress) else torch.as_tensor(yield_stress)).to(**f).expand(n)
    if viscosity is None:
        eta = torch.tensor(float(s._model.plastic_viscosity[NEWTONIAN]), **f)
    else:
        eta = (viscosity if torch.is_tensor(viscosity) else torch.as_tensor(viscosity)).to(**f)
    if plate is None:
        pv = torch.zeros(3, **f)
    else:
        rec = s._cols[s._col(plate)]
        if rec.kind != _abi.COLLIDER_BOX:
            raise ValueError("plate must be an add_box handle")
        pv = (torch.tensor(list(rec.velocity), **f) if plate_velocity is None else
              (plate_velocity if torch.is_tensor(plate_velocity) else torch.as_tensor(plate_velocity)).to(**f))
    keep = _keep_states(s, substeps, keep_states)
    x, v, F = _Rollout.apply(v0, mu, lam, ys, eta, pv, s, float(dt), int(substeps), int(checkpoint_every), plate,
                             keep)
    return (x, v) if plate is None else (x, v, F)


class BatchRollout:
    """Forward and reverse passes of many independent scenes (the batched
    identification workload). Each scene is a loaded Solver whose current state
    and parameters define its rollout. With `batched` the forward advances all
    scenes in one CUDA graph per segment (BatchSolver) and the reverse pass runs
    each scene's segments on its own stream; otherwise scenes run one after
    another, as serial rollouts would. `plates` (one add_box handle or None per
    scene) adds each plate's reaction-force trace to the outputs, one force per
    checkpoint segment, and its adjoint to the reverse pass. `keep_states` keeps
    every substep's state from the forward pass (as in `rollout`), so that the
    reverse pass does not replay the segments; the batched forward then runs each
    scene's segments on its own stream. None keeps them for scenes run one after
    another (when they fit in half of the free device memory) and replays in a batch."""

    def __init__(self, solvers, dt: float, substeps: int, checkpoint_every: int = 20, batched: bool = True,
                 plates=None, keep_states=None):
        torch = _torch()
        from .solver import BatchSolver
        self.solvers = list(solvers)
        for s in self.solvers:
            _check(s)
        self.plates = list(plates) if plates is not None else [None] * len(self.solvers)
        if len(self.plates) != len(self.solvers):
            raise ValueError("one plate handle (or None) per scene")
        self.dt, self.substeps, self.every = float(dt), int(substeps), int(checkpoint_every)
        self.batched = batched
        if keep_states is None:
            # One after another, a scene's reverse pass waits for each segment's replay,
            # so kept states pay (the identification workload: 1.67 -> 0.87 s for 32
            # scenes' reverse passes). In a batch the replays run beside other scenes'
            # reverse kernels and cost nothing measurable, while the forward that keeps
            # states runs each scene on its own split-schedule launches instead of the
            # batched graph (0.29 -> 0.36 s): batches replay.
            free, _ = torch.cuda.mem_get_info(self.solvers[0]._t["x"].device)
            keep_states = (not batched) and \
                sum(state_bytes(s.n_particles, self.substeps) for s in self.solvers) < 0.5 * free
        self.keep = bool(keep_states)
        self.batch = BatchSolver(self.solvers) if batched and not self.keep else None
        self.streams = [torch.cuda.Stream(device=s._t["x"].device) for s in self.solvers] if batched else None
        self.ckpts = None

    def forward(self):
        """Runs every rollout; returns [(x, v)] at the end, or [(x, v, F)] with the
        force trace F ((segments, 3) float64) of the scenes that have a plate."""
        torch = _torch()
        forces = [[] for _ in self.solvers]
        if not self.batched:
            self.ckpts = []
            for i, s in enumerate(self.solvers):
                r = _forward(s, self.dt, self.substeps, self.every, self.plates[i], self.keep)
                if self.plates[i] is not None:
                    r, forces[i] = r
                self.ckpts.append(r)
        elif self.keep:   # each scene's segment on its own stream, the states kept
            self.ckpts = [[] for _ in self.solvers]
            done = 0
            while done < self.substeps:
                k = min(self.every, self.substeps - done)
                for i, s in enumerate(self.solvers):
                    snap = _snapshot(s, particles=False)
                    with torch.cuda.stream(self.streams[i]):
                        if self.plates[i] is not None:
                            s.reset_tool_force(self.plates[i])
                        self.ckpts[i].append((snap, k, _segment_forward(s, self.dt, k)))
                for i, s in enumerate(self.solvers):
                    if self.plates[i] is not None:
                        with torch.cuda.stream(self.streams[i]):
                            forces[i].append(s.tool_force(self.plates[i], self.dt * k))
                done += k
            torch.cuda.synchronize()
        else:
            self.ckpts = [[] for _ in self.solvers]
            done = 0
            while done < self.substeps:
                k = min(self.every, self.substeps - done)
                for i, s in enumerate(self.solvers):
                    self.ckpts[i].append((_snapshot(s), k, None))
                    if self.plates[i] is not None:
                        s.reset_tool_force(self.plates[i])
                self.batch.step(self.dt, k)
                for i, s in enumerate(self.solvers):
                    if self.plates[i] is not None:
                        forces[i].append(s.tool_force(self.plates[i], self.dt * k))
                done += k
        self.final = [_snapshot(s) for s in self.solvers]
        out = []
        for i, s in enumerate(self.solvers):
            xv = (s._t["x"].clone(), s._t["v"].clone())
            if self.plates[i] is not None:
                xv = xv + (torch.tensor(np.array(forces[i]), dtype=torch.float64, device=s._t["x"].device),)
            out.append(xv)
        return out

    def backward(self, xbs, vbs, force_bars=None):
        """Adjoints of the rollouts' starting states and parameters for the given
        adjoints of their final (x, v) and of their force traces: [{'v', 'x', 'C',
        'F_trial', 'L', 'yield_stress', 'mu', 'lam', 'viscosity'}, plus
        'plate_velocity' where a scene has a plate]. Leaves every solver at its
        rollout's end state."""
        torch = _torch()
        if self.ckpts is None:
            raise RuntimeError("forward must run first")
        fbars = list(force_bars) if force_bars is not None else [None] * len(self.solvers)
        if not self.batched:
            out = [_backward(s, self.dt, ck, xb, vb, pl, fbar)
                   for s, ck, xb, vb, pl, fbar in zip(self.solvers, self.ckpts, xbs, vbs, self.plates, fbars)]
        else:
            torch.cuda.synchronize()
            setups = [_adj_setup(s, xb, vb, pl, max(c[1] for c in ck))
                      for s, ck, xb, vb, pl in zip(self.solvers, self.ckpts, xbs, vbs, self.plates)]
            torch.cuda.synchronize()
            nseg = len(self.ckpts[0])
            for j in reversed(range(nseg)):
                for i, s in enumerate(self.solvers):
                    snap, k, states = self.ckpts[i][j]
                    g, rec, fb, col = setups[i]
                    with torch.cuda.stream(self.streams[i]):
                        _adj_segment(s, self.dt, rec, snap, k, fb, col, None if fbars[i] is None else fbars[i][j],
                                     states)
            torch.cuda.synchronize()
            out = [_adj_finish(g, col) for g, rec, fb, col in setups]
        for s, snap in zip(self.solvers, self.final):
            _restore(s, snap)
        return out


__all__ = ["BatchRollout", "mu_lam", "rollout", "state_bytes"]
