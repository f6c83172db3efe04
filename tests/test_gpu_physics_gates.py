"""Physics gates of the reference suite, restated on the CUDA engine.

The reference pins its step through physics-level gates rather than golden arrays.
These tests pose the same scenes and apply the same acceptance bounds:

- a block on a frictional incline (tests/test_analytic_benchmarks.py:43-93);
- a water column on a box scale (:98-151);
- a free-free elastic bar's longitudinal period (:156-201);
- a tabulated viscosity table against the parametric Herschel-Bulkley kernel
  (tests/test_tabulated_material.py:20-68);
- sparse active blocks against the dense path (tests/test_sparse_blocks.py:20-73);
- periodic-x transfers: a block crossing the wrap, and a mu(I) chute developing
  the Bagnold profile (tests/test_periodic_chute.py:20-98);
- a settled column's base pressure (tests/test_engine.py:109-131);
- von Mises hardening evolving the yield stress
  (tests/test_material_review_fixes.py:16-60).

The reference runs them on Warp's deterministic CPU backend. Here they run on the
GPU, so the one bitwise comparison (sparse against dense) becomes a rounding
bound.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAV = 9.81


def _fill(x0, x1, y0, y1, z0, z1, h):
    ax = [np.arange(a + h / 2, b, h) for a, b in ((x0, x1), (y0, y1), (z0, z1))]
    return np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)


def _grid(n=32, lim=0.4):
    from mpm_engine_gb300 import GridConfig
    return GridConfig(n_grid=n, grid_lim=lim)


# ---- incline: a = g (sin th - mu cos th), and mu > tan th holds ---------------------
THETA = np.deg2rad(30.0)


def _incline(mu):
    """Horizontal floor under gravity tilted by theta: the plane carries the normal
    load m g cos th and the drive m g sin th of a 30-degree incline."""
    from mpm_engine_gb300 import Solver, elastic
    g = _grid()
    h = g.dx / 2
    z0 = 3 * g.dx
    pos = _fill(0.10, 0.18, 0.16, 0.24, z0, z0 + 0.04, h)
    s = Solver(grid=g).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(elastic(E=1.0e6, nu=0.3, density=1000.0), g=[GRAV * np.sin(THETA), 0.0, -GRAV * np.cos(THETA)])
    s.add_plane((0, 0, z0), (0, 0, 1), "separate", friction=mu)
    return s


def test_incline_block_slides_at_the_coulomb_rate(cuda):
    mu, dt, sub = 0.3, 2e-4, 10
    s = _incline(mu)
    for _ in range(20):                      # past the contact transient
        s.step(dt, sub)
    v1 = float(s.v()[:, 0].mean())
    n = 50
    for _ in range(n):
        s.step(dt, sub)
    a = (float(s.v()[:, 0].mean()) - v1) / (n * dt * sub)
    a_true = GRAV * (np.sin(THETA) - mu * np.cos(THETA))
    assert abs(a - a_true) / a_true < 0.15, (a, a_true)


def test_incline_block_holds_when_mu_exceeds_tan_theta(cuda):
    s = _incline(0.8)
    for _ in range(70):
        s.step(2e-4, 10)
    assert abs(float(s.v()[:, 0].mean())) < 0.02


# ---- water column on a box scale: the grid reaction equals rho V g --------------------
def test_water_column_weighs_its_weight_on_a_scale(cuda):
    """A column in a frictionless shaft (four slip walls) settles on a static box;
    averaged over 60 ticks the box's reaction reads -rho V g within 8 %."""
    from mpm_engine_gb300 import Solver, newtonian
    g = _grid()
    h = g.dx / 2
    z0 = 4 * g.dx
    rho = 1000.0
    pos = _fill(0.14, 0.26, 0.14, 0.26, z0, z0 + 0.12, h)
    s = Solver(grid=g).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(newtonian(eta=0.5, density=rho, bulk_modulus=5.0e4), g=[0.0, 0.0, -GRAV])
    scale = s.add_box(center=(0.2, 0.2, z0 - 0.045), half_size=(0.12, 0.12, 0.045))
    for pt, nrm in (((0.14, 0, 0), (1, 0, 0)), ((0.26, 0, 0), (-1, 0, 0)),
                    ((0, 0.14, 0), (0, 1, 0)), ((0, 0.26, 0), (0, -1, 0))):
        s.add_plane(pt, nrm, "slip")
    weight = float(len(pos) * h ** 3 * rho * GRAV)
    for _ in range(100):                     # undamped: pressure waves equilibrate
        s.step(2e-4, 10)
    s._sim.mpm_model.grid_v_damping_scale = 0.999
    for _ in range(50):
        s.step(2e-4, 10)
    n = 60
    s.reset_tool_force(scale)
    for _ in range(n):
        s.step(2e-4, 10)
    fz = float(s.tool_force(scale, n * 2e-3)[2])
    assert fz < 0.0
    assert abs(-fz - weight) / weight < 0.08, (fz, weight)


# ---- free-free bar: T = 2 L / sqrt(E / rho) ------------------------------------------
def test_free_free_bar_period(cuda):
    """A free bar (nu = 0, no gravity, no boundary) excited with an antisymmetric
    axial velocity oscillates at T = 2 L / c. The period is read from the zero
    crossings of the two halves' mean velocity difference, within 3 %."""
    from mpm_engine_gb300 import Solver, elastic
    g = _grid(48)
    h = g.dx / 2
    E, rho, L, x0 = 1.0e6, 1000.0, 0.2, 0.1
    pos = _fill(x0, x0 + L, 0.17, 0.22, 0.17, 0.22, h)
    s = Solver(grid=g).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(elastic(E=E, nu=0.0, density=rho), g=[0.0, 0.0, 0.0])
    xc = x0 + L / 2
    v = np.zeros_like(pos)
    v[:, 0] = 0.1 * (pos[:, 0] - xc) / (L / 2)
    s.set_v(v)
    T = 2.0 * L / np.sqrt(E / rho)
    dt, sub = 5e-5, 10
    right = pos[:, 0] > xc
    ts, dv = [], []
    for tick in range(int(3.2 * T / (dt * sub))):
        s.step(dt, sub)
        vx = s.v()[:, 0]
        ts.append((tick + 1) * dt * sub)
        dv.append(float(vx[right].mean() - vx[~right].mean()))
    ts, dv = np.asarray(ts), np.asarray(dv)
    c = np.where(np.diff(np.sign(dv)) != 0)[0]
    assert len(c) >= 3
    tc = ts[c] - dv[c] * (ts[c + 1] - ts[c]) / (dv[c + 1] - dv[c])
    T_meas = 2.0 * float(np.mean(np.diff(tc)))
    assert abs(T_meas - T) / T < 0.03, (T_meas, T)


# ---- tabulated viscosity against the parametric Herschel-Bulkley kernel -------------
HB = dict(eta=10.0, tau_y=40.0, pk=60.0, pn=0.4)
EPS = 0.05


def _eta_hb(gd):
    gg = np.sqrt(gd ** 2 + EPS ** 2)
    return HB["eta"] + HB["tau_y"] / gg + HB["pk"] * gg ** (HB["pn"] - 1.0)


def _shear(material, frames=6, dt=1.0e-4, sub=10):
    """A dough block on a sticky floor sheared by a box held at its top face and
    driven at 0.1 m/s; returns the box's reaction over the last frame and v."""
    from mpm_engine_gb300 import Solver
    g = _grid()
    dx, h = g.dx, g.dx / 2
    cx = cy = 0.2
    floor = 3 * dx
    geom = (0.10, 0.04, 0.045)
    pos = _fill(cx - geom[0] / 2, cx + geom[0] / 2, cy - geom[1] / 2, cy + geom[1] / 2, floor, floor + geom[2], h)
    pos += np.random.default_rng(0).uniform(-0.2 * h, 0.2 * h, pos.shape).astype(np.float32)
    s = Solver(grid=g).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(material)
    s.add_plane((0, 0, floor), (0, 0, 1), "sticky")
    top = floor + geom[2]
    tool = s.add_box((cx, cy, top), (0.45 * g.grid_lim, 0.5 * geom[1] + 0.012, 0.6 * dx), velocity=(0.1, 0.0, 0.0))
    F = np.zeros(3)
    for _ in range(frames):
        s.set_box(tool, center=(cx, cy, top), velocity=(0.1, 0.0, 0.0))
        s.reset_tool_force(tool)
        s.step(dt, sub)
        F = np.asarray(s.tool_force(tool, dt * sub), float)
    return F, s.v()


def test_tabulated_viscosity_matches_parametric_kernel(cuda):
    from mpm_engine_gb300 import newtonian, tabulated_viscous
    par = newtonian(eta=HB["eta"], density=1000.0, bulk_modulus=9.0e5).with_yield(HB["tau_y"]) \
        .with_powerlaw(K=HB["pk"], n=HB["pn"])
    tab = tabulated_viscous(_eta_hb(10.0 ** np.linspace(-1.0, 2.0, 128)), smin=-1.0, smax=2.0, density=1000.0,
                            bulk_modulus=9.0e5)
    Fp, vp = _shear(par)
    Ft, vt = _shear(tab)
    assert np.linalg.norm(Ft - Fp) / max(np.linalg.norm(Fp), 1e-12) < 5e-3
    assert np.linalg.norm(vt - vp) / max(np.linalg.norm(vp), 1e-12) < 5e-3
    # not vacuous: a constant table gives a materially different reaction
    Fc, _ = _shear(tabulated_viscous(np.full(128, HB["eta"]), smin=-1.0, smax=2.0, density=1000.0,
                                     bulk_modulus=9.0e5))
    assert np.linalg.norm(Fc - Fp) / np.linalg.norm(Fp) > 0.05


# ---- sparse active blocks against the dense path ------------------------------------
def test_sparse_matches_dense_two_blobs(cuda):
    """Two blobs at opposite ends of the domain: the sparse run (split passes over
    rebuilt active blocks, as the reference's sparse mode) and the dense run (the
    fused tick) agree to the float-atomic rounding of 60 substeps, and the active
    set hugs the material."""
    from mpm_engine_gb300 import Solver, newtonian

    def make(sparse):
        g = _grid(64)
        h = g.dx / 2
        pts = np.concatenate([_fill(cx - 0.02, cx + 0.02, 0.18, 0.22, 0.06, 0.10, h) for cx in (0.08, 0.32)])
        s = Solver(grid=g, sparse=sparse).load_particles(pts, np.full(len(pts), h ** 3, np.float32))
        s.set_material(newtonian(eta=5.0, density=1000.0, bulk_modulus=5.0e5))
        s.add_plane((0, 0, 3 * g.dx), (0, 0, 1), "slip", friction=0.2)
        return s

    sa, sb = make(True), make(False)
    for _ in range(20):
        sa.step(2.0e-4, substeps=3)
        sb.step(2.0e-4, substeps=3)
    np.testing.assert_allclose(sa.x(), sb.x(), rtol=0, atol=60 * 1e-5 * 0.4)
    assert 0.0 < sa._sim.active_block_fraction() < 0.15


# ---- periodic-x transfers -------------------------------------------------------------
@pytest.mark.parametrize("fused", [False, True])
def test_block_crosses_the_periodic_wrap_coherently(cuda, fused):
    """A stress-free elastic block translating at 1 m/s crosses x = L and comes out
    rigid: extents within 2 h of the loaded ones, velocity still uniform."""
    from mpm_engine_gb300 import Solver, elastic
    g = _grid()
    h = g.dx / 2
    pos = _fill(0.30, 0.38, 0.18, 0.22, 0.18, 0.22, h)
    s = Solver(grid=g, periodic_x=True, fused=fused).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(elastic(E=1.0e5, nu=0.3, density=1000.0), g=[0.0, 0.0, 0.0])
    v = np.zeros_like(pos)
    v[:, 0] = 1.0
    s.set_v(v)
    for _ in range(200):                     # 0.4 m: one domain length
        s.step(2e-4, 10)
    x, vf = s.x(), s.v()
    assert np.isfinite(x).all()
    xw = x[:, 0].astype(np.float64)
    xs = np.sort(xw)
    if xs[-1] - xs[0] > 0.2:                 # straddles the wrap: unwrap the low side
        gap = int(np.argmax(np.diff(xs)))
        xw[xw < 0.5 * (xs[gap] + xs[gap + 1])] += g.grid_lim
    span0 = np.array([0.08, 0.04, 0.04]) - h
    span = np.array([np.ptp(xw), np.ptp(x[:, 1]), np.ptp(x[:, 2])])
    assert np.all(np.abs(span - span0) < 2 * h), (span, span0)
    assert abs(float(vf[:, 0].mean()) - 1.0) < 1e-3
    assert float(vf[:, 0].std()) < 1e-3


def test_mu_i_chute_develops_the_bagnold_profile(cuda):
    """A mu(I) layer under gravity tilted to tan th = 0.5 (inside mu_s = 0.38 ..
    mu_s + dmu = 0.64) over a sticky base, periodic in x: it flows, its acceleration
    decays, and its velocity profile correlates with h^1.5 - (h - z)^1.5 above 0.99."""
    from mpm_engine_gb300 import Solver, granular
    g = _grid()
    dx = g.dx
    theta = np.arctan(0.5)
    z0, layer, hp = 3 * dx, 0.125, dx / 2
    pos = _fill(0.0, g.grid_lim, 0.14, 0.26, z0, z0 + layer, hp)
    s = Solver(grid=g, periodic_x=True).load_particles(pos, np.full(len(pos), hp ** 3, np.float32))
    s.set_material(granular(mu_s=0.38, delta_mu=0.26, I0=0.3, density=1590.0, grain_diameter=5.0e-3,
                            grain_density=2650.0, E=1.0e6, nu=0.3),
                   g=[GRAV * np.sin(theta), 0.0, -GRAV * np.cos(theta)])
    s.add_plane((0, 0, z0), (0, 0, 1), "sticky")
    s.add_plane((0, 0.14, 0), (0, 1, 0), "slip")
    s.add_plane((0, 0.26, 0), (0, -1, 0), "slip")
    prev, accel = 0.0, []
    for tick in range(900):
        s.step(1.2e-4, 10)
        if (tick + 1) % 300 == 0:
            v95 = float(np.quantile(s.v()[:, 0], 0.95))
            accel.append(v95 - prev)
            prev = v95
    assert prev > 0.5, prev
    assert accel[-1] < accel[0], accel
    x, v = s.x(), s.v()
    zr = x[:, 2] - z0
    zb = np.linspace(0.5 * dx, layer - 0.5 * dx, 9)
    zc = 0.5 * (zb[1:] + zb[:-1])
    prof = np.array([v[(zr >= zb[i]) & (zr < zb[i + 1]), 0].mean() for i in range(8)])
    he = float(np.quantile(zr, 0.99))
    bag = he ** 1.5 - (he - np.minimum(zc, he)) ** 1.5
    assert float(np.corrcoef(prof, bag)[0, 1]) > 0.99


# ---- a settled column carries hydrostatic-order pressure at its base -------------------
def test_static_column_pressure_grows_with_depth(cuda):
    """A dough block settling on a sticky floor (tests/test_engine.py:109-131): the
    lowest third carries more compressive pressure -tr(sigma)/3 than the top third,
    and within an order of magnitude of rho g h."""
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.scenes import block, dough
    g = _grid(48)
    pos, vol, floor = block(g, size=(0.08, 0.08, 0.12), ppc=2)
    s = Solver(grid=g).load_particles(pos, vol)
    s.set_material(dough())
    s.add_plane((0, 0, floor), (0, 0, 1), "sticky")
    s.step(2.0e-5, 2000)
    x, c = s.x(), s.cauchy()
    p = -(c[:, 0, 0] + c[:, 1, 1] + c[:, 2, 2]) / 3.0
    z = x[:, 2]
    lo, hi = z < np.quantile(z, 0.33), z > np.quantile(z, 0.67)
    assert p[lo].mean() > p[hi].mean() and p[lo].mean() > 0.0
    p_hydro = 1000.0 * GRAV * float(z.max() - z.min())
    assert 0.1 * p_hydro < p[lo].mean() < 10.0 * p_hydro, (p[lo].mean(), p_hydro)


# ---- von Mises hardening evolves the yield stress --------------------------------------
def _squeeze_yield(xi):
    """A von Mises block crushed 12 mm by a plate (tests/test_material_review_fixes.py
    :16-49); returns the per-particle yield stress after sustained plastic flow."""
    from mpm_engine_gb300 import Solver, vonmises
    g = _grid()
    h = g.dx / 2
    pos = _fill(0.16, 0.24, 0.16, 0.24, 0.16, 0.24, h)
    s = Solver(grid=g).load_particles(pos, np.full(len(pos), h ** 3, np.float32))
    s.set_material(vonmises(E=5.0e5, nu=0.3, yield_stress=2.0e3, hardening_xi=xi), g=[0.0, 0.0, 0.0])
    s.add_plane((0, 0, 0.16), (0, 0, 1), "sticky")
    s.add_box(center=(0.2, 0.2, 0.30), half_size=(0.1, 0.1, 0.06), velocity=(0.0, 0.0, -0.2))
    for _ in range(30):
        s.step(2e-4, 10)
    return s._sim.mpm_model.yield_stress.numpy()


def test_von_mises_hardening_evolves_the_yield(cuda):
    assert float(_squeeze_yield(0.0).max()) == pytest.approx(2.0e3)
    assert float(_squeeze_yield(5.0e4).max()) > 2.1e3
