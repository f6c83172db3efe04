"""Reverse-mode gradients of rollouts (adjoint.rollout) against central finite
differences of the forward, on the GPU engine and on the CPU oracle.

Scenes: a jelly or von Mises blob thrown, spinning, onto a sticky or separable
floor inside domain walls, some with a descending cuboid plate. Loss:
L = sum(a * x_K) + sum(b * v_K) with seeded weights. Finite differences use
central steps of 5e-3 relative for E, nu and yield and 1e-3 m/s along a seeded
unit direction for v0; the forward runs in fp32 with float atomics, so the
comparison allows 5 % relative error.
"""
import numpy as np
import pytest

from scenes_lib import MATERIALS, blob, make, spin_velocity

pytestmark = pytest.mark.gpu

DT, K, EVERY = 1.0e-4, 30, 10


def _scene(cls, key, floor="sticky", plate=False, n=1500, n_grid=32):
    pts, vol = blob(n=n, lo=0.12, size=0.08)
    s = make(cls, n_grid, 0.4).load_particles(pts, vol)
    s.set_material(MATERIALS[key](), g=[0.0, 0.0, -9.8])
    dx = 0.4 / n_grid
    s.add_plane((0, 0, 0.11), (0, 0, 1), floor, friction=0.0 if floor == "sticky" else 0.3)
    s.add_domain_walls()
    if plate:
        s.add_box((0.16, 0.16, 0.21 + 2 * dx), (0.06, 0.06, dx), velocity=(0.0, 0.0, -0.5))
    return s, pts


def _loss_weights(n, seed=3):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, 3)).astype(np.float32), rng.standard_normal((n, 3)).astype(np.float32)


def _run(Solver, key, v0, E, nu, ys, **kw):
    import torch
    from mpm_engine_gb300 import adjoint
    s, pts = _scene(Solver, key, **kw)
    a, b = _loss_weights(len(pts))
    x, v = adjoint.rollout(s, DT, K, v0=v0, E=E, nu=nu, yield_stress=ys, checkpoint_every=EVERY)
    dev = x.device
    return float((x * torch.from_numpy(a).to(dev)).sum() + (v * torch.from_numpy(b).to(dev)).sum())


def _grads(key, **kw):
    import torch
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300 import adjoint
    s, pts = _scene(Solver, key, **kw)
    dev = s._t["x"].device
    v0 = torch.from_numpy(spin_velocity(pts, lin=(0.3, 0.2, -1.0), omega=(0.0, 2.0, 5.0))).to(dev).requires_grad_(True)
    mat = MATERIALS[key]()
    E = torch.tensor(float(mat.E), device=dev, requires_grad=True)
    nu = torch.tensor(float(mat.nu), device=dev, requires_grad=True)
    ys = torch.tensor(float(mat.yield_stress), device=dev, requires_grad=True)
    a, b = _loss_weights(len(pts))
    x, v = adjoint.rollout(s, DT, K, v0=v0, E=E, nu=nu, yield_stress=ys, checkpoint_every=EVERY)
    L = (x * torch.from_numpy(a).to(dev)).sum() + (v * torch.from_numpy(b).to(dev)).sum()
    L.backward()
    return v0.detach(), E.detach(), nu.detach(), ys.detach(), v0.grad, E.grad, nu.grad, ys.grad


def _fd(key, v0, E, nu, ys, which, h, direction=None, **kw):
    from mpm_engine_gb300 import Solver

    def at(sign):
        args = dict(v0=v0, E=E, nu=nu, ys=ys)
        if which == "v0":
            args["v0"] = v0 + sign * h * direction
        else:
            args[which] = args[which] + sign * h
        return _run(Solver, key, **args, **kw)
    return (at(1.0) - at(-1.0)) / (2.0 * h)


def _close(ad, fd, tol=0.05):
    assert abs(ad - fd) <= tol * max(abs(fd), 1e-12), f"adjoint {ad:.6g} vs finite difference {fd:.6g}"


@pytest.mark.parametrize("key,kw", [("jelly", {}), ("jelly", {"floor": "separate", "plate": True}),
                                    ("metal", {}), ("metal_hardening", {"plate": True})])
def test_gradients_match_finite_differences(cuda, key, kw):
    import torch
    v0, E, nu, ys, gv, gE, gnu, gys = _grads(key, **kw)
    _close(float(gE), _fd(key, v0, E, nu, ys, "E", 5e-3 * float(E), **kw))
    _close(float(gnu), _fd(key, v0, E, nu, ys, "nu", 5e-3 * float(nu), **kw))
    if key.startswith("metal"):
        _close(float(gys), _fd(key, v0, E, nu, ys, "ys", 5e-3 * float(ys), **kw))
    d = torch.randn(v0.shape, generator=torch.Generator().manual_seed(7)).to(v0.device)
    d = d / d.norm()
    _close(float((gv * d).sum()), _fd(key, v0, E, nu, ys, "v0", 1e-3, direction=d, **kw))


def test_checkpoint_interval_does_not_change_gradients(cuda):
    global EVERY
    out = []
    for every in (5, 30):
        EVERY = every
        out.append(_grads("metal", plate=True))
    EVERY = 10
    for ga, gb in zip(out[0][4:], out[1][4:]):
        ga, gb = ga.cpu().numpy(), gb.cpu().numpy()
        assert np.abs(ga - gb).max() <= 1e-3 * np.abs(gb).max() + 1e-12


def test_gradient_matches_oracle_finite_difference(cuda, oracle_lib):
    """dL/dE from the GPU adjoint against central differences of the CPU oracle."""
    from mpm_engine_gb300 import Solver
    v0, E, nu, ys, gv, gE, gnu, gys = _grads("jelly")
    O = oracle_lib.OracleSolver
    a, b = _loss_weights(1500)

    def loss(Ev):
        s, _ = _scene(Solver, "jelly")
        s.set_v(v0.cpu().numpy())
        st = s.export_state()
        o = O.from_state(st, 32, 0.4)
        from mpm_engine_gb300.host import mu_lam_from_E_nu_f32
        mu, lam = mu_lam_from_E_nu_f32(np.full(1500, Ev, np.float32), np.full(1500, float(nu), np.float32))
        o.a["mu"][:] = mu
        o.a["lam"][:] = lam
        o.step(DT, K)
        return float((o.a["x"] * a).sum() + (o.a["v"] * b).sum())
    h = 5e-3 * float(E)
    fd = (loss(float(E) + h) - loss(float(E) - h)) / (2 * h)
    _close(float(gE), fd)


def test_unsupported_scenes_are_refused(cuda):
    import torch
    from mpm_engine_gb300 import Solver, adjoint
    s, pts = _scene(Solver, "newtonian")
    with pytest.raises(NotImplementedError):
        x, v = adjoint.rollout(s, DT, 4, v0=torch.zeros(len(pts), 3, device="cuda", requires_grad=True))
        x.sum().backward()
