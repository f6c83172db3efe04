"""CUDA engine (through the C ABI) against the CPU oracle on identical inputs.

Tolerances (the engine's parity contract): x, v, C and F within 1e-5 relative per
substep (a comparison after k substeps allows k x 1e-5) and 1e-3 after 1000 substeps; collider wrenches within 1e-4 relative;
particle mass unchanged. "Relative" is max|gpu - oracle| / (max|oracle| + floor)
per field, with the floors below standing for the field's natural scale. The two
sides differ only in fp32 rounding order (float atomics, FMA contraction, the
fp32 SVD).

The blob scenes are thrown with a translating, spinning velocity field
(scenes_lib.spin_velocity) so that "relative" is measured against a physical
velocity scale: a solid at rest has velocities of order g dt, far below the
velocity change that one fp32 ulp of F - R or log(sigma) in its elastic stress
induces, and a ratio against that would measure rounding, not agreement.
"""
import numpy as np
import pytest

from scenes_lib import MATERIALS, blob_scene, dam_break, free_blob

pytestmark = pytest.mark.gpu

FLOOR = {"x": 1e-6, "v": 1e-6, "F": 1e-6}


def rel_err(a, b, floor):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / (np.abs(b).max() + floor))


def c_floor(o):
    """C = 4/dx sum_i w_i v_i (x_i - x_p)/dx is a cancelling sum of terms of size
    4 |v| / dx; its rounding error scales with that term size, not with |C|."""
    return 4.0 / o.dx * float(np.abs(o.a["v"]).max()) + 1e-12


def fields_gpu(s):
    return {"x": s.x(), "v": s.v(), "C": s.C(), "F": s.F()}


def fields_oracle(o):
    return {"x": o.a["x"], "v": o.a["v"], "C": o.a["C"], "F": o.a["F"]}


def worst(s, o, key):
    """Where field `key` differs most: particle index, |difference|, and that
    particle's position and oracle velocity (for failure messages)."""
    g, r = fields_gpu(s)[key], fields_oracle(o)[key]
    n = len(r)
    d = np.abs(np.asarray(g, np.float64).reshape(n, -1) - np.asarray(r, np.float64).reshape(n, -1)).max(axis=1)
    p = int(np.argmax(d))
    above = int((d > 0.5 * d[p]).sum())
    return {"particle": p, "diff": float(d[p]), "x": o.a["x"][p].tolist(), "v": o.a["v"][p].tolist(),
            "particles_above_half_max": above}


def assert_close(s, o, tol, what=""):
    g, r = fields_gpu(s), fields_oracle(o)
    floors = dict(FLOOR, C=c_floor(o))
    errs = {k: rel_err(g[k], r[k], floors[k]) for k in g}
    bad = {k: e for k, e in errs.items() if not e <= tol}
    if bad:
        where = {k: worst(s, o, k) for k in bad}
        raise AssertionError(f"{what}: relative errors {errs} exceed {tol}; worst particles {where}")
    return errs


def assert_close_most(s, o, tol, max_frac, what=""):
    """Per particle: the largest relative error over x, v, C and F (against each
    field's scale as in assert_close) must be within tol for all but max_frac of the
    particles."""
    g, r = fields_gpu(s), fields_oracle(o)
    floors = dict(FLOOR, C=c_floor(o))
    n = len(r["x"])
    worst = np.zeros(n)
    for k in g:
        a = np.asarray(g[k], np.float64).reshape(n, -1)
        b = np.asarray(r[k], np.float64).reshape(n, -1)
        worst = np.maximum(worst, np.abs(a - b).max(axis=1) / (np.abs(b).max() + floors[k]))
    frac = float((worst > tol).mean())
    assert frac <= max_frac, f"{what}: {frac:.2%} of particles beyond {tol} (max {worst.max():.3g})"
    return frac


# The mu(I)-Phi law is discontinuous where the compaction pressure reaches zero: at
# p_c = 0 the particle is stress-free and keeps Jp, at p_c = 0+ it yields with an
# unbounded inertial number and Jp jumps to J_cs (mpm_utils.py:433-522). A blob under
# pressure relaxes through that point at its free surface, and fp32 rounding (float
# atomic order) decides the branch of the particles that sit on it; their neighbours
# follow through the grid. That material is compared strictly per substep, and after
# the 12-substep tick on all but 2 % of its particles.
DISCONTINUOUS = {"mu_i_phi"}


def pair(cuda, oracle_lib, builder, *args, fused=True, **kw):
    from mpm_engine_gb300 import Solver
    if builder is blob_scene:
        kw.setdefault("v0", True)
    s, h = builder(Solver, *args, fused=fused, **kw)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim, fused=fused)
    return s, o, h


# explicit-stability step per material on the 48^3 / 0.4 m blob: the yield-stress
# fluids carry eta_app up to tau_y / 0.02 (the strain-rate regularization), so their
# viscous limit rho dx^2 / (6 eta) is a few microseconds
DT = {"bingham": 1.0e-6, "herschel_bulkley": 5.0e-6}


# The granular return maps branch on the sign of tr(log sigma) and on
# tau > mu p (mpm_utils.py:274-300, 543-580). A freely flying blob sits at
# tr(log sigma) = 0, where fp32 rounding picks the branch on either side, so
# these scenes start pre-compressed and sheared, clearly inside one branch.
PRESTRAIN = {"mu_i", "mu_i_phi", "sand"}


def prestrain(s):
    F0 = np.array([[0.97, 0.10, 0.0], [0.0, 0.97, 0.0], [0.0, 0.0, 0.97]], np.float32)
    for key in ("F", "F_trial"):
        s._t[key].copy_(__import__("torch").from_numpy(np.tile(F0, (s.n_particles, 1, 1))))


@pytest.mark.parametrize("key", sorted(MATERIALS))
def test_per_substep_parity_all_materials(cuda, oracle_lib, key):
    from mpm_engine_gb300 import Solver
    s, _ = blob_scene(Solver, key, v0=True)
    if key in PRESTRAIN:
        prestrain(s)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    dt = DT.get(key, 2.0e-4)
    for i in range(4):
        s.step(dt, 1)
        o.step(dt, 1)
        assert_close(s, o, 1e-5, f"{key} substep {i}")
    s.step(dt, 8)
    o.step(dt, 8)
    # the per-substep bound composes: 12 substeps may accumulate 12 x 1e-5
    if key in DISCONTINUOUS:
        assert_close_most(s, o, 12 * 1e-5, 0.02, f"{key} after a fused 8-substep tick")
    else:
        assert_close(s, o, 12 * 1e-5, f"{key} after a fused 8-substep tick")
    np.testing.assert_array_equal(s._t["mass"].cpu().numpy(), o.a["mass"])


@pytest.mark.parametrize("key", ["newtonian", "metal", "mu_i"])
def test_parity_direct_kernel_path(cuda, oracle_lib, key):
    """The unsorted one-thread-per-particle path (no working-set reorder)."""
    from mpm_engine_gb300 import Solver
    s, _ = blob_scene(Solver, key, v0=True)
    if key in PRESTRAIN:
        prestrain(s)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    s._sim.reorder = False
    for t in range(3):
        s.step(2.0e-4, 4)
        o.step(2.0e-4, 4)
        assert_close(s, o, 4 * (t + 1) * 1e-5, f"{key} direct path")


def test_parity_split_pipeline(cuda, oracle_lib):
    s, o, _ = pair(cuda, oracle_lib, blob_scene, "metal", fused=False)
    for t in range(3):
        s.step(2.0e-4, 4)
        o.step(2.0e-4, 4)
        assert_close(s, o, 4 * (t + 1) * 1e-5, "split")


def test_cup_wrench_parity(cuda, oracle_lib):
    s, o, h = pair(cuda, oracle_lib, blob_scene, "newtonian", cup=True)
    dt, n = 2.0e-4, 6
    for _ in range(5):
        s.reset_cup_wrench(h)
        o.reset_wrench(h)
        s.step(dt, n)
        o.step(dt, n)
        assert_close(s, o, 1e-5, "cup scene")
        wg, wo = s.cup_wrench(h, dt * n), o.wrench_of(h, dt * n)
        for k in ("force", "torque"):
            assert rel_err(wg[k], wo[k], 1e-9) < 1e-4, (k, wg[k], wo[k])


def test_box_tool_force_parity(cuda, oracle_lib):
    s, o, h = pair(cuda, oracle_lib, blob_scene, "jelly", box=True)
    dt, n = 2.0e-4, 5
    for _ in range(6):
        s.reset_tool_force(h)
        o.reset_wrench(h)
        s.step(dt, n)
        o.step(dt, n)
        fg, fo = s.tool_force(h, dt * n), o.wrench_of(h, dt * n)["force"]
        assert rel_err(fg, fo, 1e-9) < 1e-4, (fg, fo)
    assert_close(s, o, 1e-5, "box scene")


def test_long_horizon_1000_substeps(cuda, oracle_lib):
    from mpm_engine_gb300 import Solver
    s, o = None, None
    s, _ = blob_scene(Solver, "newtonian", v0=True)
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    for _ in range(10):
        s.step(1.0e-4, 100)
        o.step(1.0e-4, 100)
    errs = assert_close(s, o, 1e-3, "1000 substeps")
    print("1000-substep relative errors", errs)


def test_dam_break_momentum_and_mass(cuda, oracle_lib):
    from mpm_engine_gb300 import Solver
    s = dam_break(Solver, n_grid=32, hi=(0.4, 0.6, 0.85))
    o = oracle_lib.OracleSolver.from_state(s.export_state(), 32, 1.0)
    m = s._t["mass"].cpu().numpy().astype(np.float64)
    for _ in range(5):
        s.step(1.0e-4, 20)
        o.step(1.0e-4, 20)
    assert_close(s, o, 1e-4, "dam break 100 substeps")
    pg = (m[:, None] * s.v()).sum(0)
    po = (m[:, None] * o.a["v"].astype(np.float64)).sum(0)
    assert np.abs(pg - po).max() <= 1e-5 * np.abs(po).max() + 1e-12
    np.testing.assert_array_equal(s._t["mass"].cpu().numpy(), o.a["mass"])


def test_reordered_tiles_equal_direct_path(cuda):
    from mpm_engine_gb300 import Solver
    outs = []
    for reorder in (True, False):
        s, h = blob_scene(Solver, "newtonian", cup=True, n=6000)
        s._sim.reorder = reorder
        for _ in range(4):
            s.step(2.0e-4, 8)
        outs.append((s.x(), s.v(), s.cup_wrench(h, 1.0)["force"]))
    np.testing.assert_allclose(outs[0][0], outs[1][0], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(outs[0][1], outs[1][1], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(outs[0][2], outs[1][2], rtol=1e-4)


def test_graph_replay_equals_live_launches(cuda):
    from mpm_engine_gb300 import Solver
    outs = []
    for graph in (True, False):
        s, _ = blob_scene(Solver, "newtonian")
        s._sim.use_cuda_graph = graph
        for _ in range(3):
            s.step(2.0e-4, 8)
        outs.append(s.x())
    np.testing.assert_allclose(outs[0], outs[1], rtol=1e-5, atol=1e-7)


def test_free_fall_gates_on_gpu(cuda):
    """tests/test_engine.py:51-73 on the engine."""
    from mpm_engine_gb300 import Solver
    s = free_blob(Solver)
    dt, n = 2.0e-5, 100
    s.step(dt, n)
    expect = -9.81 * dt * n
    assert abs(float(s.v()[:, 2].mean()) - expect) < 0.05 * abs(expect)
    s.step(dt, 105)
    assert abs(float(np.abs(np.linalg.det(s.F())).mean()) - 1.0) < 5e-3


def test_sort_bit_exact_against_oracle(cuda, oracle_lib):
    from mpm_engine_gb300 import Solver
    s, _ = blob_scene(Solver, "newtonian", n=5000)
    s.step(2.0e-4, 10)
    x0 = s.x().copy()
    vol0 = s._vol0.copy()
    fields = {k: s._t[k].cpu().numpy().copy() for k in ("v", "F", "C", "mass", "material")}
    moved_ref, perm_ref, _ = oracle_lib.sort_perm(x0, s.grid.dx, s.grid.n_grid)
    assert moved_ref
    assert s._sort_particles()
    perm = s._t["perm"].cpu().numpy()[: s.n_particles]
    np.testing.assert_array_equal(perm, perm_ref)
    np.testing.assert_array_equal(s.x(), x0[perm_ref])
    np.testing.assert_array_equal(s._vol0, vol0[perm_ref])
    for k, a in fields.items():
        np.testing.assert_array_equal(s._t[k].cpu().numpy(), a[perm_ref])
    assert not s._sort_particles()  # already ordered: skipped


def test_active_block_counts_match_oracle(cuda, oracle_lib):
    """rebuild_active_blocks (mpm_solver_warp.py:989-1026): the sparse solver rebuilds
    from the positions at the start of each tick; counts = {current, union with previous}."""
    from mpm_engine_gb300 import Solver
    s, _ = blob_scene(Solver, "newtonian", sparse=True)
    xs = []
    for _ in range(3):
        xs.append(s.x().copy())
        s.step(2.0e-4, 5)
    inv_dx = float(s._model.inv_dx)
    prev, _ = oracle_lib.blocks(xs[-1], inv_dx, s.grid.n_grid)
    s._rebuild_active_blocks()
    _, counts = oracle_lib.blocks(s.x(), inv_dx, s.grid.n_grid, prev)
    assert s._sim._block_counts == (int(counts[0]), int(counts[1]))
    assert 0.0 < s._sim.active_block_fraction() < 1.0


def test_R_and_cov_exports_match_oracle(cuda, oracle_lib):
    from mpm_engine_gb300 import Solver
    from scenes_lib import MATERIALS, blob
    pts, vol = blob(n=1500)
    cov = np.tile(np.array([1e-6, 0, 0, 1e-6, 0, 1e-6], np.float32), (len(pts), 1))
    s = Solver(grid=__import__("mpm_engine_gb300").GridConfig(48, 0.4)).load_particles(pts, vol, cov=cov,
                                                                                     cov_mode="from_F")
    s.set_material(MATERIALS["jelly"]())
    s.add_plane((0, 0, 0.025), (0, 0, 1), "sticky")
    s.step(2.0e-4, 20)
    Ft = s._t["F_trial"].cpu().numpy().reshape(-1, 9)
    R_ref = np.zeros_like(Ft)
    oracle_lib.load().gbmpm_oracle_R(Ft.ctypes.data, len(Ft), R_ref.ctypes.data)
    np.testing.assert_allclose(s.R(), np.transpose(R_ref.reshape(-1, 3, 3), (0, 2, 1)), atol=2e-5)
    c_ref = np.zeros((len(Ft), 6), np.float32)
    oracle_lib.load().gbmpm_oracle_cov(Ft.ctypes.data, cov.ctypes.data, len(Ft), c_ref.ctypes.data)
    np.testing.assert_allclose(s.cov(), c_ref, rtol=1e-5, atol=1e-12)


def _cov_field(n, seed=2):
    """Symmetric positive-definite covariances, 6-packed (xx, xy, xz, yy, yz, zz)."""
    rng = np.random.default_rng(seed)
    A = rng.normal(0.0, 1.0e-3, (n, 3, 3)).astype(np.float64)
    S = A @ np.transpose(A, (0, 2, 1)) + 1.0e-7 * np.eye(3)
    return S[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]].astype(np.float32)


@pytest.mark.parametrize("key", ["jelly", "newtonian", "metal"])
def test_cov_step_parity(cuda, oracle_lib, key):
    """load_particles(cov=..., cov_mode="step") (core/solver.py:148-156): the
    covariance advects every substep, cov += dt (L cov + cov L^T) (update_cov,
    mpm_utils.py:613-633), beside x, v, C and F. Per substep within 1e-5 relative,
    the covariance against its own scale."""
    from mpm_engine_gb300 import Solver
    cov = _cov_field(2000)
    s, _ = blob_scene(Solver, key, v0=True, cov=cov, cov_mode="step")
    assert s._update_cov
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    assert o.model.update_cov_with_F == 1
    c0 = s.cov().copy()
    for i in range(4):
        s.step(2.0e-4, 1)
        o.step(2.0e-4, 1)
        assert_close(s, o, 1e-5, f"{key} with covariance, substep {i}")
        assert rel_err(s.cov(), o.a["cov"], 1e-12) <= 1e-5, f"{key} covariance, substep {i}"
    s.step(2.0e-4, 8)
    o.step(2.0e-4, 8)
    assert_close(s, o, 12e-5, f"{key} with covariance after a fused 8-substep tick")
    assert rel_err(s.cov(), o.a["cov"], 1e-12) <= 12e-5
    assert np.abs(s.cov() - c0).max() > 1e-3 * np.abs(c0).max()   # the covariance did advect


def test_tabulated_mu_i_forward_parity(cuda, oracle_lib):
    """Tabulated mu(I) (id 13; mpm_utils.py:327-407): the mu(I) return map with the
    friction coefficient interpolated from a table over log10 I, pre-strained so every
    grain is under pressure and flowing. Per substep within 1e-5 relative, and the
    composed bound after a fused 8-substep tick."""
    from mpm_engine_gb300 import Solver
    s, _ = blob_scene(Solver, "tabulated_mu_i", v0=True)
    prestrain(s)
    assert int(s._t["material"][0]) == 13
    o = oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
    for i in range(4):
        s.step(2.0e-4, 1)
        o.step(2.0e-4, 1)
        assert_close(s, o, 1e-5, f"tabulated mu(I) substep {i}")
    s.step(2.0e-4, 8)
    o.step(2.0e-4, 8)
    assert_close(s, o, 12e-5, "tabulated mu(I) after a fused 8-substep tick")


@pytest.mark.parametrize("key", ["newtonian", "jelly", "metal"])
def test_p2g_conserves_mass_and_momentum(cuda, key):
    """The P2G deposit of a thrown, spinning blob in mid-flight: the grid's summed
    mass equals the particles' summed mass within 1e-6 relative, and its summed
    momentum the particles' momentum within 1e-6 of sum m |v| (the quadratic weights
    sum to one; the APIC term sum_i w_i (x_i - x_p) and the stress term sum_i grad w_i
    vanish). Sums in float64 on both sides."""
    import ctypes as C
    from mpm_engine_gb300 import Solver, _abi
    s, _ = blob_scene(Solver, key, v0=True)
    s.step(2.0e-4, 6)
    out = (C.c_double * 4)()
    _abi.check(s._eng.lib.gbmpm_debug_deposit_sums(s._eng.h, 2.0e-4, out, s._stream()), "deposit sums")
    m = s._t["mass"].double().cpu().numpy()
    v = s.v().astype(np.float64)
    m_sum = float(m.sum())
    p_sum = (m[:, None] * v).sum(0)
    assert abs(out[0] - m_sum) <= 1e-6 * m_sum, (out[0], m_sum)
    scale = float((m * np.linalg.norm(v, axis=1)).sum())
    assert np.abs(np.array(out[1:]) - p_sum).max() <= 1e-6 * scale, (list(out[1:]), p_sum)
    # the hook leaves the grid as a tick leaves it: the next steps still match a
    # scene that never called it
    s2, _ = blob_scene(Solver, key, v0=True)
    s2.step(2.0e-4, 6)
    s.step(2.0e-4, 4)
    s2.step(2.0e-4, 4)
    np.testing.assert_allclose(s.x(), s2.x(), rtol=0, atol=1e-6)
