"""Deterministic ticks (Solver(deterministic=True)) against the oracle, bit for bit.

The deterministic passes round every operation once, in the order of the fp32
statement of the reference's kernels, and sum the P2G deposits of each node in
particle order (sorted records, no float atomics). The oracle run on one thread
deposits in particle order too. So the two must agree exactly, not within a
tolerance: x, v, C, F and the stress, compared with np.array_equal after every
check point, for every material law. Both sides evaluate logarithms, exponentials
and powers in double by the same written-out method (no libm) and round them once,
and run the SVD in double in the same order.

The reference's own precedent for bitwise checks is fused == split on one device
(tests/test_fused_pipeline.py:59-75).
"""
import numpy as np
import pytest

from scenes_lib import EXTRA_MATERIALS, MATERIALS, NAME_PARAMS, make, spin_velocity

pytestmark = pytest.mark.gpu

NG, LIM = 32, 0.4
DX = LIM / NG


GRANULAR = ("sand", "mu_i", "mu_i_phi", "tabulated_mu_i")
PRESTRAIN_F0 = np.array([[0.97, 0.10, 0.0], [0.0, 0.97, 0.0], [0.0, 0.0, 0.97]], np.float32)


def scene(cls, key, fused=True, n=3000, seed=5, **kw):
    """A thrown, spinning blob whose lower part starts inside the floor's contact
    band (a separable floor with friction, 0.3 cells off its node row), inside
    domain walls, under a descending plate that reaches the blob's top. Granular
    blobs start compressed and sheared (F0 = 0.97 I plus shear), so that their return
    maps flow from the first substep."""
    rng = np.random.default_rng(seed)
    pts = (rng.random((n, 3)) * np.array([0.09, 0.09, 0.06]) + np.array([0.15, 0.15, 3.1 * DX])).astype(np.float32)
    vol = np.full(n, 1.0e-7, np.float32)
    s = make(cls, NG, LIM, fused=fused, **kw).load_particles(pts, vol)
    vel = spin_velocity(pts, lin=(0.3, 0.1, -0.6), omega=(0.0, 2.0, 4.0))
    if cls.__name__ == "OracleSolver":
        s.a["v"][:] = vel
    else:
        s.set_v(vel)
    mat = MATERIALS[key] if key in MATERIALS else EXTRA_MATERIALS[key]
    if isinstance(mat, tuple):
        s.set_material(mat[0], **mat[1])
    elif isinstance(mat, str):
        s.set_material(mat, **NAME_PARAMS[mat])
    else:
        s.set_material(mat())
    if key in GRANULAR:
        F0 = np.tile(PRESTRAIN_F0, (n, 1, 1))
        if cls.__name__ == "OracleSolver":
            s.a["F"][:] = F0.reshape(s.a["F"].shape)
            s.a["F_trial"][:] = F0.reshape(s.a["F_trial"].shape)
        else:
            import torch
            for f in ("F", "F_trial"):
                s._t[f].copy_(torch.from_numpy(F0))
    s.add_plane((0, 0, 3.3 * DX), (0, 0, 1), "separate", friction=0.3)
    s.add_domain_walls()
    s.add_box((0.196, 0.196, 3.1 * DX + 0.06 + 0.3 * DX + 0.01), (0.07, 0.07, 0.01), velocity=(0.0, 0.0, -1.5))
    return s


def fields(side):
    if hasattr(side, "a"):
        a = side.a
        return {"x": a["x"], "v": a["v"], "C": a["C"], "F": a["F"], "stress": a["stress"]}
    t = side._t
    return {k: t[k].detach().cpu().numpy() for k in ("x", "v", "C", "F", "stress")}


def assert_bitwise(s, o, what):
    g, r = fields(s), fields(o)
    bad = {}
    for k in g:
        a = np.asarray(g[k], np.float32).reshape(len(r["x"]), -1)
        b = np.asarray(r[k], np.float32).reshape(len(r["x"]), -1)
        if not np.array_equal(a.view(np.uint32), b.view(np.uint32)):
            diff = np.abs(a.astype(np.float64) - b.astype(np.float64)).max(axis=1)
            bad[k] = {"particles": int((a.view(np.uint32) != b.view(np.uint32)).any(axis=1).sum()),
                      "max_abs": float(diff.max()), "first": int(np.argmax(diff > 0) if diff.max() > 0 else -1)}
    assert not bad, f"{what}: not bitwise equal: {bad}"


ALL = ["newtonian", "herschel_bulkley", "bingham", "water", "tabulated", "jelly", "metal", "metal_hardening",
       "plasticine", "sand", "mu_i", "tabulated_mu_i", "mu_i_phi"]


@pytest.mark.parametrize("key,fused", [(k, True) for k in ALL] +
                         [("newtonian", False), ("jelly", False), ("metal_hardening", False), ("mu_i", False)])
def test_deterministic_ticks_equal_oracle_bitwise(cuda, oracle_lib, key, fused):
    from mpm_engine_gb300 import Solver
    s = scene(Solver, key, fused=fused, deterministic=True)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), NG, LIM, fused=fused, threads=1)
    dt = 1.0e-4
    k = 0
    for n in (1, 4, 15, 30):
        s.step(dt, n)
        o.step(dt, n)
        k += n
        assert_bitwise(s, o, f"{key} ({'fused' if fused else 'split'}) after {k} substeps")


def test_deterministic_ticks_repeat_bitwise_and_match_the_fast_path(cuda):
    """Two deterministic runs from one state, one through a captured CUDA graph and
    one launched live, give the same bits; the tiled path from the same state stays
    within the parity contract (k x 1e-5) of them."""
    from mpm_engine_gb300 import Solver
    from test_gpu_parity import assert_close

    a = scene(Solver, "jelly", deterministic=True)   # the scenes are built identically
    b = scene(Solver, "jelly", deterministic=True)
    b._sim.use_cuda_graph = False
    c = scene(Solver, "jelly")
    for side in (a, b, c):
        side.step(1.0e-4, 10)
    fa, fb = fields(a), fields(b)
    for k in fa:
        assert np.array_equal(np.asarray(fa[k]).view(np.uint32), np.asarray(fb[k]).view(np.uint32)), k

    class _View:   # the deterministic run, read as the parity helpers read the oracle
        def __init__(self, f):
            self.a = f
            self.dx = DX
    view = _View({"x": a.x(), "v": a.v(), "C": a.C(), "F": a.F()})
    assert_close(c, view, 10 * 1e-5, "tiled path against the deterministic passes after 10 substeps")


@pytest.mark.parametrize("fused", [True, False])
def test_deterministic_ticks_with_particle_modifiers_equal_oracle_bitwise(cuda, oracle_lib, fused):
    """An impulse (active three substeps), a held velocity translation and a rotating
    cylinder on the jelly blob. The rotation's acos, sin and cos are evaluated in
    double by the written-out method both sides share, so the ticks stay bit for
    bit equal to the oracle, which runs the reference's split pipeline."""
    from mpm_engine_gb300 import Solver
    dt = 1.0e-4
    s = scene(Solver, "jelly", fused=fused, deterministic=True)
    s.add_impulse_on_particles((0.0, 0.0, 5.0e-4), dt, point=(0.17, 0.17, 0.06), size=(0.02, 0.02, 0.02), num_dt=3,
                               start_time=2 * dt)
    s.enforce_particle_velocity_translation((0.22, 0.22, 0.07), (0.015, 0.015, 0.015), (0.0, 0.3, 0.0), 0.0, 1.0)
    s.enforce_particle_velocity_rotation((0.19, 0.19, 0.06), (0.3, 0.2, 1.0), (0.02, 0.025), 4.0, 0.1, 5 * dt, 1.0)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), NG, LIM, fused=fused, threads=1)
    k = 0
    for n in (1, 4, 15):
        s.step(dt, n)
        o.step(dt, n)
        k += n
        assert_bitwise(s, o, f"modifiers ({'fused' if fused else 'split'}) after {k} substeps")
    assert abs(float(s.v()[:, 1].mean())) > 1e-3     # the translation drags the blob


def test_deterministic_ticks_reject_cdf_colliders(cuda):
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.geometry import sheet_cdf
    s = scene(Solver, "jelly", deterministic=True)
    s.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.2))
    with pytest.raises(NotImplementedError, match="deterministic"):
        s.step(1.0e-4, 1)


@pytest.mark.parametrize("key", ["newtonian", "jelly"])
def test_deterministic_ticks_wrap_the_periodic_axis_bitwise(cuda, oracle_lib, key):
    """A periodic-x domain: a blob straddling the x seam and moving across it, on a
    sticky floor. Stencils wrap in x and positions wrap at the domain length; both
    sides stay bit for bit equal."""
    from mpm_engine_gb300 import Solver
    rng = np.random.default_rng(9)
    n = 2000
    pts = (rng.random((n, 3)) * np.array([0.08, 0.08, 0.05]) + np.array([LIM - 0.04, 0.15, 3.4 * DX]))
    pts[:, 0] = np.mod(pts[:, 0], LIM)
    pts = pts.astype(np.float32)
    s = make(Solver, NG, LIM, periodic_x=True, deterministic=True).load_particles(pts, np.full(n, 1.0e-7, np.float32))
    s.set_v(np.tile(np.array([[0.8, 0.1, -0.2]], np.float32), (n, 1)))
    mat = MATERIALS[key]
    s.set_material(mat())
    s.add_plane((0, 0, 3.3 * DX), (0, 0, 1), "sticky")
    o = oracle_lib.OracleSolver.from_state(s.export_state(), NG, LIM, threads=1)
    k = 0
    for m in (1, 9, 40):
        s.step(1.0e-4, m)
        o.step(1.0e-4, m)
        k += m
        assert_bitwise(s, o, f"{key} periodic after {k} substeps")
    assert float(np.asarray(o.a["x"])[:, 0].min()) >= 0.0
