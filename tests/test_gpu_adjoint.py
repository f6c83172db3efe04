"""Reverse-mode gradients of rollouts (adjoint.rollout) against central finite
differences of the forward, on the GPU engine and on the CPU oracle.

Scenes: a jelly or von Mises blob thrown, spinning, into a sticky or separable
floor inside domain walls, some with a descending cuboid plate, pre-rolled 20
substeps into contact. The gradient is that of a 4-substep rollout from that
state (checkpoints every 2 substeps) of L = sum(a * x_K) + sum(b * v_K), summed in
float64. Over a few substeps the fp32 forward is smooth enough in the parameters
for central differences at 1e-2 relative to resolve the derivative to well under
1 %; over long impact rollouts rounding is amplified by the dynamics and finite
differences scatter by about 10 %, so long horizons are checked for consistency
(checkpoint interval) instead.
"""
import numpy as np
import pytest

from scenes_lib import MATERIALS, NAME_PARAMS, blob, make, spin_velocity

pytestmark = pytest.mark.gpu

DT, PRE, K, EVERY = 1.0e-4, 20, 4, 2
N, NG = 1500, 32

# a Bingham fluid gentle enough for dt = 1e-4 on this grid (its apparent viscosity
# tops out at eta + tau_y / 0.02 = 102 Pa s, inside the explicit viscous limit)
MATS = dict(MATERIALS, bingham_soft=lambda: __import__("mpm_engine_gb300").newtonian(
    eta=2.0, density=1000.0, bulk_modulus=2.0e5).with_yield(2.0))
# fluids for a free, straining blob: a soft equation of state keeps pressure rounding
# (K (J^-1.1 - 1) near J = 1) below the viscous and yield stresses under test; the
# Bingham one is yield-dominated (eta_app up to 500 Pa s, explicit limit 5e-5 s)
MATS["newtonian_soft"] = lambda: __import__("mpm_engine_gb300").newtonian(
    eta=2.0, density=1000.0, bulk_modulus=2.0e4)
MATS["bingham_yield"] = lambda: __import__("mpm_engine_gb300").newtonian(
    eta=0.2, density=1000.0, bulk_modulus=2.0e4).with_yield(10.0)
DT_OF = {"bingham_yield": 4.0e-5, "mu_i_phi": 2.0e-5}
# the remaining laws: Drucker-Prager sand, von Mises with softening, mu(I) and its
# tabulated form (by engine name and parameters), and a tabulated viscous fluid
MATS["sand"] = ("sand", NAME_PARAMS["sand"])
MATS["plasticine"] = ("plasticine", NAME_PARAMS["plasticine"])
MATS["mu_i_table"] = ("tabulated_mu_i", dict(E=1.0e5, nu=0.3, density=2500.0, eta_table=[0.38, 0.45, 0.55, 0.64],
                                             eta_table_smin=-4.0, eta_table_smax=0.0, grain_diameter=1.0e-3,
                                             grain_density=2650.0))
MATS["tabulated_soft"] = lambda: __import__("mpm_engine_gb300").tabulated_viscous(
    [8.0, 4.0, 2.0, 1.0, 0.5], smin=-1.0, smax=2.0, density=1000.0, bulk_modulus=2.0e4)


def _set_material(s, key):
    m = MATS[key]
    if isinstance(m, tuple):
        s.set_material(m[0], g=[0.0, 0.0, -9.8], **m[1])
    else:
        s.set_material(m(), g=[0.0, 0.0, -9.8])


def _mat_params(key):
    """(E, nu, yield) of a test material."""
    m = MATS[key]
    if isinstance(m, tuple):
        kw = m[1]
        return float(kw.get("E", 1e5)), float(kw.get("nu", 0.3)), float(kw.get("yield_stress", 0.0))
    m = m()
    return float(m.E), float(m.nu), float(m.yield_stress)


PRESTRAIN_F0 = np.array([[0.97, 0.10, 0.0], [0.0, 0.97, 0.0], [0.0, 0.0, 0.97]], np.float32)


def _scene(cls, key, floor="sticky", plate=False, cup=False, sphere=False, drop=0.0, free=False, pre=PRE,
           prestrain=False):
    from mpm_engine_gb300.geometry import analytic_sdf
    from scenes_lib import SMALL_CUP
    pts, vol = blob(n=N, lo=0.12, size=0.08)
    pts[:, 2] -= drop
    s = make(cls, NG, 0.4).load_particles(pts, vol)
    _set_material(s, key)
    dx = 0.4 / NG
    if free:      # no contact within the rollout: a straining flow loads the stress
        pass
    elif cup:     # the blob lands on the cup's floor and presses its walls
        s.add_cup(SMALL_CUP, (0.16, 0.16, 0.155), friction=0.3)
    elif sphere:  # the blob lands on a mesh-SDF sphere
        s.add_sdf_collider(analytic_sdf("sphere", radius=0.03), center=(0.16, 0.16, 0.095), friction=0.3)
    else:
        s.add_plane((0, 0, 0.121), (0, 0, 1), floor, friction=0.0 if floor == "sticky" else 0.3)
    s.add_domain_walls()
    if plate:
        s.add_box((0.16, 0.16, 0.20 + dx), (0.06, 0.06, dx), velocity=(0.0, 0.0, -0.5))
    vel = spin_velocity(pts, lin=(0.3, 0.2, -1.0), omega=(0.0, 2.0, 5.0))
    if free:      # plus shear and extension, 4/s
        A = np.array([[2.0, 2.0, 0.0], [2.0, -2.0, 1.0], [0.0, 1.0, 0.0]], np.float32)
        vel = vel + (pts - pts.mean(axis=0)) @ A.T
    s.set_v(vel.astype(np.float32))
    if prestrain:   # compressed and sheared: every granular particle under pressure and flowing
        import torch
        for k in ("F", "F_trial"):
            s._t[k].copy_(torch.from_numpy(np.tile(PRESTRAIN_F0, (s.n_particles, 1, 1))))
    if pre:
        s.step(DT_OF.get(key, DT), pre)
    return s


def _weights():
    rng = np.random.default_rng(3)
    return rng.standard_normal((N, 3)), rng.standard_normal((N, 3))


def _loss_np(x, v):
    a, b = _weights()
    return float((np.asarray(x, np.float64) * a).sum() + (np.asarray(v, np.float64) * b).sum())


class Case:
    def __init__(self, key, **kw):
        import torch
        from mpm_engine_gb300 import Solver, adjoint
        self.key, self.kw = key, kw
        self.dt = DT_OF.get(key, DT)
        self.s = _scene(Solver, key, **kw)
        self.snap = adjoint._snapshot(self.s)
        self.state = self.s.export_state()
        self.E, self.nu, self.ys = _mat_params(key)
        self.eta = float(self.s._model.plastic_viscosity[10])
        self.v0 = self.s._t["v"].clone()
        dev = self.v0.device
        self.dev = dev
        self.a, self.b = (torch.from_numpy(w).to(dev) for w in _weights())

    def rollout(self, v0, E, nu, ys, eta=None, grad=False):
        import torch
        from mpm_engine_gb300 import adjoint
        adjoint._restore(self.s, self.snap)
        eta = self.eta if eta is None else eta
        x, v = adjoint.rollout(self.s, self.dt, K, v0=v0, E=E, nu=nu, yield_stress=ys, viscosity=eta,
                               checkpoint_every=EVERY)
        L = (x.double() * self.a).sum() + (v.double() * self.b).sum()
        if grad:
            L.backward()
        return float(L.detach())

    def grads(self):
        import torch
        t = lambda x: torch.tensor(x, device=self.dev, requires_grad=True)  # noqa: E731
        v0 = self.v0.clone().requires_grad_(True)
        E, nu, ys, eta = t(self.E), t(self.nu), t(self.ys), t(self.eta)
        self.rollout(v0, E, nu, ys, eta, grad=True)
        return {"v0": v0.grad, "E": float(E.grad), "nu": float(nu.grad), "ys": float(ys.grad),
                "eta": float(eta.grad)}

    def fd_gpu(self, which, rel=1e-2, direction=None):
        base = {"v0": self.v0, "E": self.E, "nu": self.nu, "ys": self.ys, "eta": self.eta}

        def at(sg):
            p = dict(base)
            if which == "v0":
                p["v0"] = self.v0 + sg * rel * direction
            else:
                p[which] = p[which] * (1.0 + sg * rel)
            return self.rollout(p["v0"], p["E"], p["nu"], p["ys"], p["eta"])
        h = rel if which == "v0" else rel * base[which]
        return (at(1.0) - at(-1.0)) / (2.0 * h)

    def fd_oracle(self, O, which, rel=1e-2, direction=None):
        from mpm_engine_gb300.host import mu_lam_from_E_nu_f32
        base = {"E": self.E, "nu": self.nu, "ys": self.ys, "eta": self.eta}

        def at(sg):
            p = dict(base)
            if which != "v0":
                p[which] = p[which] * (1.0 + sg * rel)
            o = O.from_state(self.state, NG, 0.4)
            mu, lam = mu_lam_from_E_nu_f32(np.full(N, p["E"], np.float32), np.full(N, p["nu"], np.float32))
            o.a["mu"][:] = mu
            o.a["lam"][:] = lam
            o.a["yield_stress"][:] = np.float32(p["ys"])
            o.model.plastic_viscosity[10] = np.float32(p["eta"])
            if which == "v0":
                o.a["v"][:] = (o.a["v"].astype(np.float64) + sg * rel * direction).astype(np.float32)
            o.step(self.dt, K)
            return _loss_np(o.a["x"], o.a["v"])
        h = rel if which == "v0" else rel * base[which]
        return (at(1.0) - at(-1.0)) / (2.0 * h)


def _close(ad, fd, tol, what):
    assert abs(ad - fd) <= tol * abs(fd), f"{what}: adjoint {ad:.6g} vs finite difference {fd:.6g}"


CASES = [("jelly", {}), ("jelly", {"floor": "separate", "plate": True}), ("metal", {}),
         ("metal_hardening", {"plate": True})]


@pytest.mark.parametrize("key,kw", CASES)
def test_gradients_match_gpu_finite_differences(cuda, key, kw):
    import torch
    c = Case(key, **kw)
    g = c.grads()
    for p in ("E", "nu") + (("ys",) if key.startswith("metal") else ()):
        _close(g[p], c.fd_gpu(p), 0.02, f"{key} d/d{p}")
    d = torch.randn(c.v0.shape, generator=torch.Generator().manual_seed(7)).to(c.dev)
    d = d / d.norm()
    # a unit direction over all N x 3 components moves each by ~0.015 per unit step;
    # a step of 0.1 m/s keeps the response linear and well above atomic-order noise
    _close(float((g["v0"] * d).sum()), c.fd_gpu("v0", rel=1e-1, direction=d), 0.02, f"{key} d/dv0")


@pytest.mark.parametrize("key,kw", [CASES[0], CASES[3]])
def test_gradients_match_oracle_finite_differences(cuda, oracle_lib, key, kw):
    c = Case(key, **kw)
    g = c.grads()
    for p in ("E", "nu") + (("ys",) if key.startswith("metal") else ()):
        _close(g[p], c.fd_oracle(oracle_lib.OracleSolver, p), 0.02, f"{key} d/d{p} (oracle)")
    d = np.random.default_rng(11).standard_normal((N, 3))
    d /= np.linalg.norm(d)
    gv = g["v0"].double().cpu().numpy()
    _close(float((gv * d).sum()), c.fd_oracle(oracle_lib.OracleSolver, "v0", rel=1e-1, direction=d), 0.02,
           f"{key} d/dv0 (oracle)")


@pytest.mark.parametrize("key,kw,params,tol", [
    ("jelly", {"cup": True}, ("E", "nu"), 0.02),
    ("jelly", {"sphere": True}, ("E", "nu"), 0.02),
    ("newtonian_soft", {"free": True}, ("eta",), 0.03),
    ("bingham_yield", {"free": True}, ("ys",), 0.05),
])
def test_fluid_cup_and_sdf_gradients_match_finite_differences(cuda, oracle_lib, key, kw, params, tol):
    """The revolved-SDF cup and mesh-SDF colliders with a jelly blob landing on them,
    and the Newtonian family (viscosity, Bingham yield) in a free straining flow.
    A fluid landing in a cup is chaotic at fp32 level (stiff pressure and contact
    branches scatter its finite differences by 10-20 % from run to run), so the
    fluid laws are checked without contact; their parameters move the loss by about
    1e-5 per percent, near the GPU's atomic-order noise, so they are checked against
    deterministic oracle differences. Their fp32 differences spread by about 2 %
    (Newtonian viscosity) and 3-6 % (Bingham yield) across step sizes, which sets
    those bounds; the viscosity of the yield-dominated fluid is too weak an input
    (eta << tau_y / strain rate) to resolve and is left to the Newtonian case."""
    import torch
    c = Case(key, **kw)
    g = c.grads()
    for p in params:
        fd = c.fd_oracle(oracle_lib.OracleSolver, p, rel=3e-2) if p in ("eta", "ys") else c.fd_gpu(p)
        _close(g[p], fd, tol, f"{key} d/d{p}")
    d = torch.randn(c.v0.shape, generator=torch.Generator().manual_seed(5)).to(c.dev)
    d = d / d.norm()
    fd = c.fd_oracle(oracle_lib.OracleSolver, "v0", rel=1e-2, direction=d.double().cpu().numpy())
    _close(float((g["v0"] * d).sum()), fd, tol, f"{key} d/dv0")


@pytest.mark.parametrize("key,kw,params,tol", [
    ("sand", {}, ("E", "nu"), 0.03),
    ("plasticine", {"plate": True}, ("E", "nu", "ys"), 0.03),
    ("mu_i", {}, ("E", "nu"), 0.05),
    ("mu_i_table", {}, ("E", "nu"), 0.05),
    ("tabulated_soft", {"free": True}, (), 0.03),
])
def test_granular_softening_and_tabulated_gradients(cuda, oracle_lib, key, kw, params, tol):
    """Drucker-Prager sand and mu(I) (closed-form and tabulated) landing on a sticky
    floor, softening von Mises pressed by a plate, and a tabulated viscous fluid in a
    free straining flow, against deterministic oracle differences. The mu(I) laws
    switch branch where a particle's volumetric strain changes sign (tension resets
    F to its rotation), which makes their differences the noisiest, hence 5 %.
    Branches at the start of the rollout (from the pre-rolled F_trial): sand 28 %
    elastic, 37 % apex, 35 % on the cone; plasticine 61 % yielding; mu(I) 39 %
    tension, 61 % flowing."""
    import torch
    c = Case(key, **kw)
    g = c.grads()
    for p in params:
        _close(g[p], c.fd_oracle(oracle_lib.OracleSolver, p), tol, f"{key} d/d{p}")
    d = torch.randn(c.v0.shape, generator=torch.Generator().manual_seed(9)).to(c.dev)
    d = d / d.norm()
    fd = c.fd_oracle(oracle_lib.OracleSolver, "v0", rel=1e-2, direction=d.double().cpu().numpy())
    _close(float((g["v0"] * d).sum()), fd, tol, f"{key} d/dv0")


def test_mu_i_phi_gradients_match_oracle(cuda, oracle_lib):
    """mu(I)-Phi(I), whose packing state Jp joins the adjoint state, on a free blob
    held in compression and shear (F0 = 0.97 I plus shear): the compaction pressure
    is positive and the material flows at every particle. Where that pressure
    reaches zero Jp jumps to its critical-state value, a discontinuity no finite
    difference follows, so the rollout (4 substeps of 2e-5 s) ends before the free
    surface relaxes."""
    import torch
    c = Case("mu_i_phi", free=True, pre=0, prestrain=True)
    g = c.grads()
    for p in ("E", "nu"):
        _close(g[p], c.fd_oracle(oracle_lib.OracleSolver, p), 0.03, f"mu_i_phi d/d{p}")
    d = torch.randn(c.v0.shape, generator=torch.Generator().manual_seed(4)).to(c.dev)
    d = d / d.norm()
    fd = c.fd_oracle(oracle_lib.OracleSolver, "v0", rel=1e-2, direction=d.double().cpu().numpy())
    _close(float((g["v0"] * d).sum()), fd, 0.03, "mu_i_phi d/dv0")


def test_long_rollout_checkpoint_interval_does_not_change_gradients(cuda):
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    out = []
    for every in (5, 40):
        s = _scene(Solver, "metal_hardening", plate=True)
        v0 = s._t["v"].clone().requires_grad_(True)
        E = torch.tensor(1.0e5, device=v0.device, requires_grad=True)
        x, v = adjoint.rollout(s, DT, 40, v0=v0, E=E, nu=0.3, checkpoint_every=every)
        a, b = (torch.from_numpy(w).to(v0.device) for w in _weights())
        ((x.double() * a).sum() + (v.double() * b).sum()).backward()
        out.append((v0.grad.cpu().numpy(), float(E.grad)))
    assert np.abs(out[0][0] - out[1][0]).max() <= 2e-3 * np.abs(out[1][0]).max()
    assert abs(out[0][1] - out[1][1]) <= 2e-3 * abs(out[1][1])


def test_unsupported_scenes_are_refused(cuda):
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    pts, vol = blob(n=500)
    s = make(Solver, 32, 0.4).load_particles(pts, vol)
    s.set_material(MATERIALS["mu_i"]())
    s.add_impulse_on_particles((0.0, 0.0, 1.0e-3), DT)      # particle modifiers are outside the adjoint
    with pytest.raises(NotImplementedError):
        x, v = adjoint.rollout(s, DT, 4, v0=torch.zeros(len(pts), 3, device="cuda", requires_grad=True))
        x.sum().backward()


@pytest.mark.parametrize("keep", [True, False])
def test_batch_rollout_with_plates_matches_scenes_run_one_by_one(cuda, keep):
    """BatchRollout with plate force traces: batched (all forwards in one CUDA graph
    per segment, each scene's reverse pass on its own stream; with kept states each
    scene's forward on its own stream too) against the same scenes rolled out and
    reversed one after another. Force traces within 1e-5 and every
    gradient (v0, mu, lam, yield, plate velocity) within 1e-3 relative: the two
    differ only in float atomic order, which can move a particle across the yield
    surface in one run and not the other."""
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    from mpm_engine_gb300.materials import vonmises
    from mpm_engine_gb300.scenes import squeeze_scene
    specs = [(1.0e5, 0.3, 300.0), (3.0e4, 0.25, 1.0e3), (2.0e5, 0.4, 150.0)]
    res = {}
    for batched in (True, False):
        built = [squeeze_scene(Solver, 8000, 32, vonmises(E=E, nu=nu, yield_stress=ys, density=1000.0), seed=i,
                               plate_gap=-0.37, floor_cells=3.3) for i, (E, nu, ys) in enumerate(specs)]
        scenes, plates = [b[0] for b in built], [b[1] for b in built]
        r = adjoint.BatchRollout(scenes, 1.0e-5, 40, 10, batched=batched, plates=plates, keep_states=keep)
        outs = r.forward()
        rng = np.random.default_rng(4)
        xb = [torch.from_numpy(rng.standard_normal((s.n_particles, 3))).to(o[0].device) for s, o in zip(scenes, outs)]
        fb = [torch.from_numpy(rng.standard_normal(tuple(o[2].shape))).to(o[0].device) for o in outs]
        res[batched] = (outs, r.backward(xb, [None] * len(scenes), fb))
    (ob, gb), (op, gp) = res[True], res[False]
    for i in range(len(specs)):
        Fb, Fp = ob[i][2].cpu().numpy(), op[i][2].cpu().numpy()
        assert Fp.shape == (4, 3) and np.abs(Fp).max() > 0.0
        assert np.abs(Fb - Fp).max() <= 1e-5 * np.abs(Fp).max(), (i, Fb, Fp)
        for k in ("v", "mu", "lam", "yield_stress", "plate_velocity"):
            a = gb[i][k].double().cpu().numpy()
            b = gp[i][k].double().cpu().numpy()
            if k in ("mu", "lam", "yield_stress"):
                a, b = np.array([a.sum()]), np.array([b.sum()])
            assert np.abs(a - b).max() <= 1e-3 * np.abs(b).max() + 1e-30, (i, k, np.abs(a - b).max(), np.abs(b).max())


@pytest.mark.parametrize("key", ["jelly", "metal_hardening"])
def test_kept_states_and_replayed_segments_give_the_same_gradients(cuda, key):
    """rollout(keep_states=True) keeps every substep's state from the forward pass;
    keep_states=False replays each segment from its checkpoint in the reverse pass.
    Both linearise along the split schedule's trajectory and differ only in float
    atomic order: gradients within 1e-4 relative (1e-3 for the von Mises scene,
    whose yield kinks rounding may move)."""
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    out = {}
    for keep in (True, False):
        s = _scene(Solver, key, plate=True)
        v0 = s._t["v"].clone().requires_grad_(True)
        E = torch.tensor(_mat_params(key)[0], device=v0.device, requires_grad=True)
        x, v = adjoint.rollout(s, DT, 12, v0=v0, E=E, nu=0.3, checkpoint_every=5, keep_states=keep)
        a, b = (torch.from_numpy(w).to(v0.device) for w in _weights())
        ((x.double() * a).sum() + (v.double() * b).sum()).backward()
        out[keep] = (v0.grad.double().cpu().numpy(), float(E.grad))
    tol = 1e-4 if key == "jelly" else 1e-3
    (gk, Ek), (gr, Er) = out[True], out[False]
    assert np.abs(gk - gr).max() <= tol * np.abs(gr).max(), (np.abs(gk - gr).max(), np.abs(gr).max())
    assert abs(Ek - Er) <= tol * abs(Er), (Ek, Er)
