"""The engine's adjoint against central finite differences of the float64 oracle.

The float32 forward cannot resolve a finite difference at h = 1e-3 relative: over
a few substeps the parameters move the loss by about 1e-6 of its size, the same
order as the rounding of 4,500 float32 positions, so float32 differences scatter by
percents. The oracle built with its arithmetic in float64 (oracle/, precision=64)
steps the same scene from the same starting state with the rounding taken out.
Central differences of it at h = 1e-3 relative have a truncation error of order
h^2 and no visible noise, so they measure the adjoint itself.

Bound: the adjoint's gradient (float32 kernels along the float32 trajectory, the
loss summed in float64) within 1e-3 relative of the float64 differences, for
dL/dE, dL/dnu, dL/dyield, dL/dviscosity and a unit direction of dL/dv0.

Where the rollout crosses a kink of the map (a particle switching between elastic
and plastic response, a node entering a collider's contact band, a granular
particle reaching the cone's apex), a central difference over +-h averages the
slopes on both sides for every particle whose switch lies within the step, an
error of order h. In float64 the step can shrink without rounding noise, so when
h = 1e-3 misses the bound the difference is repeated at h = 1e-4 and 1e-5 and the
closest one counts; the test prints every step's error. Measured on the GB300:
von Mises dL/dyield misses by 3.4e-3 at h = 1e-3, 4.8e-4 at 1e-4 and 3.9e-6 at
1e-5, the cup's dL/dE converges to 6e-6 and sand's dL/dnu to 1e-5: the adjoint is
the exact derivative and the excess at 1e-3 is the step's own bias.
"""
import numpy as np
import pytest

from test_gpu_adjoint import K, N, NG, Case, _loss_np

pytestmark = pytest.mark.gpu

H = 1.0e-3
TOL = 1.0e-3


def fd64(c, which, rel=H, direction=None, k=K):
    """Central difference of the loss of a k-substep rollout of the float64 oracle
    from the case's starting state: parameters perturbed by +-rel relative (v0 by
    +-rel along a unit direction), mu and lambda formed from E and nu in float64."""
    from oracle.oracle import OracleSolver
    base = {"E": c.E, "nu": c.nu, "ys": c.ys, "eta": c.eta}

    def at(sg):
        p = dict(base)
        if which != "v0":
            p[which] = p[which] * (1.0 + sg * rel)
        o = OracleSolver.from_state(c.state, NG, 0.4, precision=64, threads=8)
        E, nu = float(p["E"]), float(p["nu"])
        o.a["mu"][:] = E / (2.0 * (1.0 + nu))
        o.a["lam"][:] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
        o.a["yield_stress"][:] = p["ys"]
        o.model.plastic_viscosity[10] = p["eta"]
        eta_used = float(o.model.plastic_viscosity[10])   # the model record holds float32
        if which == "v0":
            o.a["v"][:] = o.a["v"] + sg * rel * direction
        o.step(c.dt, k)
        return _loss_np(o.a["x"], o.a["v"]), eta_used
    (lp, ep), (lm, em) = at(1.0), at(-1.0)
    if which == "v0":
        h = rel
    elif which == "eta":
        h = 0.5 * (ep - em)
    else:
        h = rel * base[which]
    return (lp - lm) / (2.0 * h)


STEPS = (H, 1.0e-4, 1.0e-5)


def check(c, params, tol=TOL, seed=7):
    """Adjoint against float64 central differences at h = 1e-3; a parameter that
    misses the bound there is retried at h = 1e-4 and 1e-5 (kink bias is of order
    h) and its best step counts. Prints the error at every step tried."""
    import torch
    g = c.grads()
    d = torch.randn(c.v0.shape, generator=torch.Generator().manual_seed(seed)).double()
    d = (d / d.norm()).numpy()
    ad = {p: g[p] for p in params}
    ad["v0"] = float((g["v0"].double().cpu().numpy() * d).sum())
    errs, table = {}, {}
    for p in ad:
        table[p] = []
        for h in STEPS:
            fd = fd64(c, p, rel=h, direction=d if p == "v0" else None)
            e = abs(ad[p] - fd) / abs(fd)
            table[p].append(f"h={h:g}: {e:.2e}")
            errs[p] = e if h == STEPS[0] else min(errs[p], e)
            if errs[p] <= tol:
                break
    print(c.key, c.kw, table)
    bad = {k: e for k, e in errs.items() if not e <= tol}
    assert not bad, f"{c.key} {c.kw}: relative gradient errors {bad} exceed {tol} at every step: {table}"


@pytest.mark.parametrize("key,kw,params", [
    ("jelly", {}, ("E", "nu")),
    ("jelly", {"floor": "separate", "plate": True}, ("E", "nu")),
    ("metal", {}, ("E", "nu", "ys")),
    ("metal_hardening", {"plate": True}, ("E", "nu", "ys")),
    ("jelly", {"cup": True}, ("E", "nu")),
    ("jelly", {"sphere": True}, ("E", "nu")),
])
def test_elastic_and_von_mises_gradients_match_float64_differences(cuda, key, kw, params):
    check(Case(key, **kw), params)


@pytest.mark.parametrize("key,kw,params", [
    ("sand", {"prestrain": True}, ("E", "nu")),
    ("plasticine", {"plate": True}, ("E", "nu", "ys")),
    ("mu_i", {"prestrain": True}, ("E", "nu")),
    ("mu_i_table", {"prestrain": True}, ("E", "nu")),
])
def test_granular_and_softening_gradients_match_float64_differences(cuda, key, kw, params):
    """The granular laws start pre-compressed and sheared (F0 = 0.97 I plus shear),
    where every particle is in compression and flowing. On blobs that start at rest
    in F, which straddle the tension apex (tr(log sigma) = 0, F sent to U V^T), the
    v0 derivative keeps a residual that does not shrink with h (5e-4 for sand,
    1.1e-3 for mu(I)): the reverse pass at the apex is a known limitation."""
    check(Case(key, **kw), params)


@pytest.mark.parametrize("key,kw,params", [
    ("newtonian_soft", {"free": True}, ("eta",)),
    ("bingham_yield", {"free": True}, ("ys",)),
    ("tabulated_soft", {"free": True}, ()),
])
def test_fluid_gradients_match_float64_differences(cuda, key, kw, params):
    check(Case(key, **kw), params)


def test_mu_i_phi_gradients_match_float64_differences(cuda):
    check(Case("mu_i_phi", free=True, pre=0, prestrain=True), ("E", "nu"))


IDENT_FLOOR_CELLS = 3.3   # floor plane 0.3 cells above a node row
IDENT_PLATE_GAP = -0.37   # plate face 0.37 cells into the block, between node rows


def identification_errors(floor_cells=IDENT_FLOOR_CELLS, plate_gap=IDENT_PLATE_GAP, steps=STEPS, tol=TOL,
                          ys0=100.0, reference="f64", linearized=True):
    """One scene of the batched identification workload at its full length: a von
    Mises cube of about 50k particles on a 48^3 grid, resting on a sticky floor and
    squeezed by a plate pressed into its top at 0.05 m/s, 400 substeps of 1e-5 s with
    checkpoints every 20. The loss is the squared distance of the final positions to
    a seeded target rollout (the same scene with E, nu and the yield stress 30 %, 5 %
    and 30 % higher), plus the squared distance of the plate's reaction-force trace
    (one force per 20-substep segment) to the target's, plus a seeded projection of
    the final velocities. Returns the adjoint's dL/dE, dL/dnu, dL/dyield, dL/d(plate
    velocity, z) and a unit direction of dL/dv0, each parameter's relative error
    against central differences of the float64 oracle (h = 1e-3 relative, retried at
    the smaller steps while above `tol`, the best counting) and the table of every
    step's error. reference="f32" takes the differences of the engine's own float32
    rollout instead of the float64 oracle's; linearized=False differences the loss
    itself instead of its linearisation at the engine's trajectory."""
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    from mpm_engine_gb300.materials import vonmises
    from mpm_engine_gb300.scenes import squeeze_scene
    from oracle.oracle import OracleSolver
    E0, nu0, dt, K5, every = 1.0e5, 0.3, 1.0e-5, 400, 20

    def scene(E, nu, ys):
        s, _ = squeeze_scene(Solver, 50_000, 48, vonmises(E=E, nu=nu, yield_stress=ys, density=1000.0),
                             seed=3, plate_gap=plate_gap, floor_cells=floor_cells)
        return s

    nseg = K5 // every
    tgt = scene(1.3 * E0, 1.05 * nu0, 1.3 * ys0)
    ht = _plate_handle(tgt)
    F_t = []
    for _ in range(nseg):
        tgt.reset_tool_force(ht)
        tgt.step(dt, every)
        F_t.append(tgt.tool_force(ht, dt * every))
    F_t = np.array(F_t)
    x_t = tgt._t["x"].double().clone()
    s = scene(E0, nu0, ys0)
    hp = _plate_handle(s)
    vel0 = np.array(s._cols[s._col(hp)].velocity[:], np.float64)
    n = s.n_particles
    st = s.export_state()
    b = torch.from_numpy(np.random.default_rng(8).standard_normal((n, 3))).to(x_t.device)
    dev = x_t.device
    F_tt = torch.from_numpy(F_t).to(dev)
    t = lambda x: torch.tensor(x, device=dev, dtype=torch.float32, requires_grad=True)  # noqa: E731
    snap = adjoint._snapshot(s)
    v0 = s._t["v"].clone().requires_grad_(True)
    E, nu, ys, pv = t(E0), t(nu0), t(ys0), t(vel0.tolist())
    x, v, F = adjoint.rollout(s, dt, K5, v0=v0, E=E, nu=nu, yield_stress=ys, checkpoint_every=every, plate=hp,
                              plate_velocity=pv)
    L = ((x.double() - x_t) ** 2).sum() + ((F - F_tt) ** 2).sum() + (v.double() * b).sum()
    L.backward()
    d = np.random.default_rng(12).standard_normal((n, 3))
    d /= np.linalg.norm(d)
    g = {"E": float(E.grad), "nu": float(nu.grad), "ys": float(ys.grad), "plate_vz": float(pv.grad[2]),
         "v0": float((v0.grad.double().cpu().numpy() * d).sum())}
    xt = x_t.cpu().numpy()
    bn = b.cpu().numpy()
    # the loss linearised at the engine's trajectory: the same cotangents the adjoint
    # starts from, 2 (x - x_target) and 2 (F - F_target), as fixed weights
    wx = 2.0 * (x.detach().double() - x_t).cpu().numpy()
    wF = 2.0 * (F.detach().double() - F_tt).cpu().numpy()

    def value(xo, Fo, vo):
        xo, Fo, vo = (np.asarray(a, np.float64) for a in (xo, Fo, vo))
        if linearized:
            return float((wx * xo).sum() + (wF * Fo).sum() + (bn * vo).sum())
        return float(((xo - xt) ** 2).sum() + ((Fo - F_t) ** 2).sum() + (vo * bn).sum())

    def loss32(E_, nu_, ys_, dv=None, vel=vel0):
        adjoint._restore(s, snap)
        f = dict(device=dev, dtype=torch.float32)
        v_init = snap[0]["v"].clone() if dv is None else (snap[0]["v"].double() + torch.from_numpy(dv).to(dev)).float()
        pvel = torch.tensor(vel, **f)
        with torch.no_grad():
            x_, v_, F_ = adjoint.rollout(s, dt, K5, v0=v_init, E=torch.tensor(E_, **f), nu=torch.tensor(nu_, **f),
                                         yield_stress=torch.tensor(ys_, **f), checkpoint_every=every, plate=hp,
                                         plate_velocity=pvel)
        return value(x_.cpu().numpy(), F_.cpu().numpy(), v_.cpu().numpy()), float(pvel[2])

    def loss64(E_, nu_, ys_, dv=None, vel=vel0):
        if reference == "f32":
            return loss32(E_, nu_, ys_, dv, vel)
        o = OracleSolver.from_state(st, 48, 0.3, precision=64, threads=16)
        o.a["mu"][:] = E_ / (2.0 * (1.0 + nu_))
        o.a["lam"][:] = E_ * nu_ / ((1.0 + nu_) * (1.0 - 2.0 * nu_))
        o.a["yield_stress"][:] = ys_
        o.set_box(hp, velocity=tuple(vel))
        if dv is not None:
            o.a["v"][:] = o.a["v"] + dv
        Fs = []
        for _ in range(nseg):
            o.reset_wrench(hp)
            o.step(dt, every)
            Fs.append(o.wrench_of(hp, dt * every)["force"])
        return value(o.a["x"], np.array(Fs), o.a["v"]), float(o.cols[o.handles[hp]].velocity[2])

    def fd(p, h):
        if p == "E":
            return (loss64(E0 * (1 + h), nu0, ys0)[0] - loss64(E0 * (1 - h), nu0, ys0)[0]) / (2 * h * E0)
        if p == "nu":
            return (loss64(E0, nu0 * (1 + h), ys0)[0] - loss64(E0, nu0 * (1 - h), ys0)[0]) / (2 * h * nu0)
        if p == "ys":
            return (loss64(E0, nu0, ys0 * (1 + h))[0] - loss64(E0, nu0, ys0 * (1 - h))[0]) / (2 * h * ys0)
        if p == "plate_vz":
            e = np.array([0.0, 0.0, h * abs(vel0[2])])
            (lp, vp), (lm, vm) = loss64(E0, nu0, ys0, vel=vel0 + e), loss64(E0, nu0, ys0, vel=vel0 - e)
            return (lp - lm) / (vp - vm)
        return (loss64(E0, nu0, ys0, h * d)[0] - loss64(E0, nu0, ys0, -h * d)[0]) / (2 * h)

    errs, table = {}, {}
    for p in g:
        table[p] = []
        for h in steps:
            f = fd(p, h)
            assert f != 0.0, f"{p} does not move the loss"
            e = abs(g[p] - f) / abs(f)
            table[p].append(f"h={h:g}: {g[p]:.6e} vs {f:.6e} ({e:.2e})")
            errs[p] = min(errs.get(p, e), e)
            if errs[p] <= tol:
                break
    return g, errs, table


IDENT_YIELD = 300.0   # Pa: inside the batched workloads' 1e2..1e4 range; the cube yields under the plate's edge


def test_identification_scene_full_length(cuda):
    """The identification scene at full length (`identification_errors`, yield stress
    300 Pa): dL/dE, dL/dnu, dL/dyield, dL/d(plate velocity) and a v0 direction, each
    within 1e-3 of the float64 differences of the loss linearised at the engine's
    trajectory.

    Why linearised: the loss's cotangent 2 (x - x_target) is the difference of two
    rollouts that agree to about 1e-4 m, while each float32 position carries about
    1e-7 m of accumulated rounding. The float64 oracle's own trajectory therefore
    sees a cotangent that differs from the engine's by about 1 %, and a difference
    of the loss itself measures the derivative at that other cotangent (measured:
    1.3e-2 for E at yield 100 Pa). Fixing the cotangents at the engine's trajectory
    leaves the derivative of the rollout, which is what the adjoint computes.

    Why off node rows: the floor and the plate's faces sit between node rows. A face
    exactly on a node row makes that row's contact test a tie. The float32 engine and
    the float64 oracle then round the node's distance to the face to opposite signs
    (at 48^3 the float32 distance of the floor row is 0, not in contact, and the
    float64 one -4.7e-10, in contact), so the two step different maps."""
    g, errs, table = identification_errors(ys0=IDENT_YIELD)
    print("identification scene, 400 substeps:", table)
    bad = {k: e for k, e in errs.items() if not e <= TOL}
    assert not bad, f"identification scene: relative gradient errors {bad} exceed {TOL}: {table}"


def _plate_handle(s):
    """The handle of the scene's add_box plate."""
    from mpm_engine_gb300 import _abi
    for h, i in enumerate(s._handles):
        if i is not None and s._cols[i].kind == _abi.COLLIDER_BOX:
            return h
    raise AssertionError("no plate")


@pytest.mark.parametrize("key", ["jelly", "metal_hardening"])
def test_plate_trajectory_and_force_trace_gradients(cuda, key):
    """Collider trajectories: a blob pressed by a descending plate (a kinematic
    cuboid) over K substeps in segments of 2. The loss adds a seeded projection of
    the plate's reaction-force trace (one force per segment, as tool_force reads
    it) to the particle terms; its gradient with respect to the plate's velocity,
    E and nu is checked against central differences of the float64 oracle."""
    import torch
    from mpm_engine_gb300 import adjoint
    from oracle.oracle import OracleSolver
    from test_gpu_adjoint import EVERY, _weights
    c = Case(key, plate=True)
    s = c.s
    h = _plate_handle(s)
    nseg = (K + EVERY - 1) // EVERY
    wf = torch.from_numpy(np.random.default_rng(21).standard_normal((nseg, 3))).to(c.dev)
    vel0 = np.array(s._cols[s._col(h)].velocity[:], np.float64)
    dev = c.dev
    t = lambda x: torch.tensor(x, device=dev, dtype=torch.float32, requires_grad=True)  # noqa: E731
    adjoint._restore(s, c.snap)
    pv, E, nu = t(vel0.tolist()), t(c.E), t(c.nu)
    x, v, F = adjoint.rollout(s, c.dt, K, E=E, nu=nu, checkpoint_every=EVERY, plate=h, plate_velocity=pv)
    assert F.shape == (nseg, 3) and float(F.abs().max()) > 0.0
    L = (x.double() * c.a).sum() + (v.double() * c.b).sum() + (F * wf).sum()
    L.backward()
    g = {"E": float(E.grad), "nu": float(nu.grad)}
    g.update({f"plate_v{d}": float(pv.grad[d]) for d in range(3)})
    a, b = _weights()
    wfn = wf.cpu().numpy()
    hh = {"E": H * c.E, "nu": H * c.nu, "plate_v": H * max(1.0, float(np.abs(vel0).max()))}

    def loss64(E_, nu_, vel):
        o = OracleSolver.from_state(c.state, NG, 0.4, precision=64, threads=8)
        o.a["mu"][:] = E_ / (2.0 * (1.0 + nu_))
        o.a["lam"][:] = E_ * nu_ / ((1.0 + nu_) * (1.0 - 2.0 * nu_))
        o.set_box(h, velocity=tuple(vel))
        vel_used = np.array(o.cols[o.handles[h]].velocity[:], np.float64)   # the record holds float32
        Fs = []
        left = K
        while left > 0:
            k = min(EVERY, left)
            o.reset_wrench(h)
            o.step(c.dt, k)
            Fs.append(o.wrench_of(h, c.dt * k)["force"])
            left -= k
        val = float((o.a["x"] * a).sum() + (o.a["v"] * b).sum() + (np.array(Fs) * wfn).sum())
        return val, vel_used

    fd = {"E": (loss64(c.E + hh["E"], c.nu, vel0)[0] - loss64(c.E - hh["E"], c.nu, vel0)[0]) / (2 * hh["E"]),
          "nu": (loss64(c.E, c.nu + hh["nu"], vel0)[0] - loss64(c.E, c.nu - hh["nu"], vel0)[0]) / (2 * hh["nu"])}
    for d in range(3):
        e = np.zeros(3)
        e[d] = hh["plate_v"]
        (lp, vp), (lm, vm) = loss64(c.E, c.nu, vel0 + e), loss64(c.E, c.nu, vel0 - e)
        fd[f"plate_v{d}"] = (lp - lm) / (vp[d] - vm[d])
    errs = {k: abs(g[k] - fd[k]) / max(abs(fd[k]), 1e-12) for k in fd}
    print(key, "plate:", {k: (g[k], fd[k], f"{errs[k]:.2e}") for k in fd})
    bad = {k: e for k, e in errs.items() if not e <= TOL}
    assert not bad, f"{key} with plate: relative gradient errors {bad} exceed {TOL}"
