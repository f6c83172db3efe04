"""Python driver of the CPU oracle (mpm_oracle.cpp) - test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker and as the timed CPU restatement. The product
(mpm_engine_gb300) never imports it.

`OracleSolver` mirrors the host side of warpmpm's Solver on numpy arrays (the
parameter and collider conventions come from mpm_engine_gb300.host) and steps
through gbmpm_oracle_tick. `OracleSolver.from_state` replays a scene exported
from the GPU Solver, so both run the same inputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

from mpm_engine_gb300 import _abi, host  # noqa: E402
from mpm_engine_gb300.glass import quat_to_mat  # noqa: E402
from mpm_engine_gb300.materials import material_id  # noqa: E402

LIB = HERE / "_build" / "libmpm_oracle.so"
# the same source with the arithmetic in float64: a rounding-free forward for
# finite-difference checks of the engine's adjoint (never a parity checker)
LIB64 = HERE / "_build" / "libmpm_oracle64.so"
SRC = HERE / "mpm_oracle.cpp"
_libs: dict = {}


def build(force: bool = False) -> Path:
    """g++ recipe: fp contraction off so every product and sum rounds as written.
    Builds the float32 oracle and its float64 twin (-DORACLE_REAL=double) in parallel."""
    LIB.parent.mkdir(parents=True, exist_ok=True)
    deps = [SRC, REPO / "include" / "gbmpm.h"]
    procs = []
    for out, real in ((LIB, "float"), (LIB64, "double")):
        if out.exists() and not force and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
            continue
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", f"-DORACLE_REAL={real}", "-I", str(REPO / "include"), "-o", str(out), str(SRC)]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    for pr in procs:
        out, _ = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + out)
    return LIB


def load(precision: int = 32):
    """The oracle library: float32 (the parity checker) or its float64 twin."""
    if precision in _libs:
        return _libs[precision]
    path = LIB64 if precision == 64 else LIB
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    P = C.POINTER
    lib.gbmpm_oracle_tick.restype = C.c_int
    lib.gbmpm_oracle_tick.argtypes = [P(_abi.Particles), P(_abi.Model), P(_abi.Collider), C.c_int32, C.c_void_p,
                                      P(C.c_double), C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                      C.c_void_p]
    lib.gbmpm_oracle_cdf_new.restype = C.c_void_p
    lib.gbmpm_oracle_cdf_new.argtypes = [C.c_int32]
    lib.gbmpm_oracle_cdf_free.argtypes = [C.c_void_p]
    lib.gbmpm_oracle_cdf_stamp_count.restype = C.c_int32
    lib.gbmpm_oracle_cdf_stamp_count.argtypes = [C.c_void_p]
    lib.gbmpm_oracle_cdf_set.argtypes = [C.c_void_p, P(_abi.Cdf), C.c_int32, C.c_double]
    lib.gbmpm_oracle_cdf_get.argtypes = [C.c_void_p, P(_abi.Cdf), C.c_int32]
    lib.gbmpm_oracle_cdf_grids.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gbmpm_oracle_svd3.argtypes = [C.c_void_p] * 4
    lib.gbmpm_oracle_glass_sdf.restype = C.c_float
    lib.gbmpm_oracle_glass_sdf.argtypes = [P(_abi.Collider), C.c_void_p]
    lib.gbmpm_oracle_integrate_pose.argtypes = [P(_abi.Collider), C.c_double, C.c_double]
    lib.gbmpm_oracle_sort_perm.restype = C.c_int32
    lib.gbmpm_oracle_sort_perm.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_void_p]
    lib.gbmpm_oracle_blocks.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_int32, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
    lib.gbmpm_oracle_R.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    lib.gbmpm_oracle_cov.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    lib.gbmpm_oracle_last_error.restype = C.c_char_p
    lib.gbmpm_oracle_abi_layout.argtypes = [C.c_void_p]
    lib.gbmpm_oracle_set_rigid.argtypes = [P(_abi.RigidBody), C.c_int32, P(_abi.RigidSurface), C.c_int32]
    lib.gbmpm_oracle_get_rigid.argtypes = [P(_abi.RigidBody), C.c_int32]
    lib.gbmpm_oracle_set_modifiers.argtypes = [P(_abi.Modifier), C.c_int32]
    lib.gbmpm_oracle_trig.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]
    lib.gbmpm_oracle_trig.restype = None
    _libs[precision] = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


def _copy(cls, rec):
    r = cls()
    C.memmove(C.byref(r), C.byref(rec), C.sizeof(cls))
    return r


def abi_layout() -> list[int]:
    out = np.zeros(10, np.int64)
    load().gbmpm_oracle_abi_layout(_p(out))
    return [int(v) for v in out]


def trig(x: np.ndarray, kind: str) -> np.ndarray:
    """The oracle's own double sin, cos or acos (the rotation modifier's functions)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    load().gbmpm_oracle_trig(_p(x), x.size, {"sin": 0, "cos": 1, "acos": 2}[kind], _p(out))
    return out


def svd3(F: np.ndarray):
    lib = load()
    F = np.ascontiguousarray(F, dtype=np.float32).reshape(3, 3)
    U = np.zeros((3, 3), np.float32)
    V = np.zeros((3, 3), np.float32)
    s = np.zeros(3, np.float32)
    lib.gbmpm_oracle_svd3(_p(F), _p(U), _p(s), _p(V))
    return U, s, V


def sort_perm(x: np.ndarray, dx: float, n_grid: int):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    keys = np.zeros(len(x), np.int64)
    perm = np.arange(len(x), dtype=np.int32)
    moved = lib.gbmpm_oracle_sort_perm(_p(x), len(x), float(dx), int(n_grid), _p(keys), _p(perm))
    return bool(moved), perm, keys


def blocks(x: np.ndarray, inv_dx: float, n_grid: int, prev: np.ndarray | None = None):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    bd = (n_grid + 3) // 4
    cur = np.zeros(bd ** 3, np.int32)
    counts = np.zeros(2, np.int32)
    lib.gbmpm_oracle_blocks(_p(x), len(x), float(inv_dx), int(n_grid),
                            None if prev is None else _p(np.ascontiguousarray(prev, np.int32)), _p(cur), _p(counts))
    return cur, counts


_KEYS = ("x", "v", "C", "F", "F_trial", "L", "stress", "mass", "vol", "density", "Jp", "mu", "lam", "yield_stress",
         "material", "selection", "cov", "init_cov", "cdf_tag", "rigid_id", "x_ref", "mod_mask")


def box_contact_wrench(x, cauchy, vol, box_center, box_half, layer_cells=None, dx=None, compressive_only=True):
    """Stress-integral reaction on a box (coupling/wrench.py:15-46), restated in numpy."""
    cx, cy, cz = box_center
    hx, hy, hz = box_half
    h = float(np.mean(vol) ** (1.0 / 3.0))
    T = (layer_cells * dx) if (layer_cells and dx) else 3.0 * h
    bottom = cz - hz
    under = (np.abs(x[:, 0] - cx) < hx) & (np.abs(x[:, 1] - cy) < hy)
    contact = under & (x[:, 2] > bottom - T) & (x[:, 2] < bottom + 0.5 * T)
    if compressive_only:
        contact &= cauchy[:, 2, 2] < 0.0
    if contact.sum() < 3:
        return {"force": np.zeros(3), "torque": np.zeros(3), "n_contact": 0, "Fz": 0.0}
    f_per = -cauchy[contact][:, :, 2] * (vol[contact, None] / T)
    force = f_per.sum(0)
    r = x[contact] - np.array(box_center)
    torque = np.cross(r, f_per).sum(0)
    return {"force": force, "torque": torque, "n_contact": int(contact.sum()), "Fz": float(force[2])}


_FLOAT_KEYS = ("x", "v", "C", "F", "F_trial", "L", "stress", "mass", "vol", "density", "Jp", "mu", "lam",
               "yield_stress", "cov", "init_cov", "x_ref")


class OracleSolver:
    """numpy twin of mpm_engine_gb300.Solver's host side, stepping the C++ oracle.
    precision=64 steps the float64 build: particle arrays, grid and accumulators in
    float64 (a finite-difference reference without rounding noise)."""

    def __init__(self, n_grid: int = 64, grid_lim: float = 0.4, fused: bool = True, threads: int = 1,
                 periodic_x: bool = False, grid=None, precision: int = 32, **_ignored):
        if grid is not None:
            n_grid, grid_lim = grid.n_grid, grid.grid_lim
        if precision not in (32, 64):
            raise ValueError("precision is 32 or 64")
        self.precision = precision
        self.fdt = np.float64 if precision == 64 else np.float32
        self.n_grid, self.grid_lim = int(n_grid), float(grid_lim)
        self.dx = self.grid_lim / self.n_grid
        self.fused = fused
        self.threads = threads
        self.a: dict = {}
        self.model = host.default_model(self.n_grid, self.grid_lim)
        self.model.periodic_x = 1 if periodic_x else 0
        self.eta_table = np.zeros(2, np.float32)
        self.model.eta_table = _p(self.eta_table)
        self.cols: list = []
        self.handles: list = []
        self.sdf_arrays: list = []
        self.time = 0.0
        self.mat_current = 0
        self.wrench = np.zeros((0, 6), self.fdt)
        self.cdf_lanes: list = []
        self.cdf_arrays: list = []
        self.cdf_state = None
        self.cdf_wrench_acc = np.zeros((4, 6), self.fdt)
        self.rigid_bodies: list = []
        self.rigid_surfaces: list = []
        self.modifiers: list = []

    def __del__(self):
        if getattr(self, "cdf_state", None):
            load(self.precision).gbmpm_oracle_cdf_free(self.cdf_state)
            self.cdf_state = None

    # ----------------------------------------------------------------- setup
    def load_particles(self, pos, vol, cov=None, cov_mode="step"):
        n = len(pos)
        fdt = self.fdt
        eye = np.tile(np.eye(3, dtype=fdt), (n, 1, 1))
        z = lambda *s: np.zeros(s, fdt)  # noqa: E731
        self.a = {"x": np.ascontiguousarray(pos, np.float32).astype(fdt).reshape(n, 3).copy(), "v": z(n, 3),
                  "C": z(n, 3, 3), "F": eye.copy(), "F_trial": eye.copy(), "L": z(n, 3, 3), "stress": z(n, 3, 3),
                  "mass": z(n), "vol": np.asarray(vol, np.float32).astype(fdt).copy(), "density": z(n), "Jp": z(n),
                  "mu": z(n), "lam": z(n), "yield_stress": z(n), "material": np.zeros(n, np.int32),
                  "selection": np.zeros(n, np.int32), "cov": None, "init_cov": None,
                  "cdf_tag": np.zeros(n, np.int32), "rigid_id": np.zeros(n, np.int32), "x_ref": z(n, 3),
                  "mod_mask": np.zeros(n, np.int32)}
        if cov is not None:
            c6 = np.ascontiguousarray(cov, np.float32).astype(fdt).reshape(n, 6)
            self.a["init_cov"] = c6.copy()
            self.a["cov"] = c6.copy() if cov_mode == "step" else np.zeros_like(c6)
            self.model.update_cov_with_F = 1 if cov_mode == "step" else 0
        return self

    def _apply(self, kw, lo=None, hi=None):
        a, m = self.a, self.model
        ranged = lo is not None
        sl = slice(lo, hi) if ranged else slice(None)
        if "material" in kw:
            mid = material_id(kw["material"])
            a["material"][sl] = mid
            if ranged:
                m.material_mask |= 1 << mid
            else:
                self.mat_current = mid
                m.material_mask = 1 << mid
            mat = mid
        else:
            mat = self.mat_current
        host.apply_type_params(m, mat, kw)
        if "yield_stress" in kw:
            a["yield_stress"][sl] = np.float32(kw["yield_stress"])
        if "eta_table" in kw:
            self.eta_table = np.asarray(kw["eta_table"], np.float32).reshape(-1).copy()
            m.eta_table = _p(self.eta_table)
            m.eta_table_n = len(self.eta_table)
        if "eta_table_smin" in kw:
            m.eta_table_smin = host.f32(kw["eta_table_smin"])
        if "eta_table_smax" in kw:
            m.eta_table_smax = host.f32(kw["eta_table_smax"])
        if "g" in kw and not ranged:
            m.gravity[:] = tuple(host.f32(g) for g in kw["g"])
        if "obj_id" in kw:
            a["rigid_id"][sl] = int(kw["obj_id"])
        if "density" in kw:
            a["density"][sl] = np.float32(kw["density"])
            a["mass"][sl] = a["density"][sl] * a["vol"][sl]
        if "E" in kw or "nu" in kw:
            if ranged:
                E, nu = float(m.E[mat]), float(m.nu[mat])
                a["mu"][sl] = E / (2.0 * (1.0 + nu))
                a["lam"][sl] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
            else:
                self._mu_lam()
        if "rpic_damping" in kw:
            m.rpic_damping = host.f32(kw["rpic_damping"])
        if "grid_v_damping_scale" in kw:
            m.grid_v_damping_scale = host.f32(kw["grid_v_damping_scale"])

    def _mu_lam(self):
        idx = self.a["material"]
        mu, lam = host.mu_lam_from_E_nu_f32(np.array(self.model.E[:], np.float32)[idx],
                                            np.array(self.model.nu[:], np.float32)[idx])
        self.a["mu"][:] = mu
        self.a["lam"][:] = lam

    def set_material(self, material, **overrides):
        name, params = material.resolve() if hasattr(material, "resolve") else (str(material), {})
        self._apply({"material": name, "g": [0.0, 0.0, -9.81], **params, **overrides})
        self._mu_lam()
        return self

    def set_material_range(self, start, end, material, **overrides):
        name, params = material.resolve() if hasattr(material, "resolve") else (str(material), {})
        self._apply({"material": name, **params, **overrides}, lo=int(start), hi=int(end))
        return self

    def _add(self, rec, slots=1):
        self.cols.append(rec)
        first = len(self.handles)
        self.handles.append(len(self.cols) - 1)
        self.handles.extend([None] * (slots - 1))
        self.wrench = np.zeros((len(self.cols), 6), self.fdt)
        return first

    def add_plane(self, point, normal, surface="sticky", friction=0.0, restitution=0.0):
        self._add(host.plane_collider(point, normal, surface, friction))
        if restitution != 0.0:
            self.rigid_surfaces.append(host.rigid_surface(point, normal, friction, restitution))
        return self

    def finalize_rigid_bodies(self):
        self.rigid_bodies, x_ref = host.rigid_bodies(self.a["x"], self.a["mass"], self.a["material"],
                                                     self.a["rigid_id"])
        self.a["x_ref"][:] = x_ref
        return self

    def set_rigid_body_velocity(self, body_id, v_cm=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0)):
        self.rigid_bodies[body_id].v_cm[:] = tuple(float(c) for c in v_cm)
        self.rigid_bodies[body_id].omega[:] = tuple(float(c) for c in omega)
        return self

    def _add_modifier(self, rec, mask):
        self.a["mod_mask"] |= (mask.astype(np.int32) << len(self.modifiers))
        self.modifiers.append(rec)

    def add_impulse_on_particles(self, force, dt, point=(1, 1, 1), size=(1, 1, 1), num_dt=1, start_time=0.0):
        self._add_modifier(host.impulse_modifier(force, dt, num_dt, start_time), host.box_mask(self.a["x"], point, size))
        return self

    def enforce_particle_velocity_translation(self, point, size, velocity, start_time, end_time):
        self._add_modifier(host.translation_modifier(velocity, start_time, end_time),
                           host.box_mask(self.a["x"], point, size))
        return self

    def enforce_particle_velocity_rotation(self, point, normal, half_height_and_radius, rotation_scale,
                                           translation_scale, start_time, end_time):
        rec = host.rotation_modifier(point, normal, rotation_scale, translation_scale, start_time, end_time)
        self._add_modifier(rec, host.cylinder_mask(self.a["x"], point, rec.normal[:], half_height_and_radius[0],
                                                   half_height_and_radius[1]))
        return self

    def add_box(self, center, half_size, velocity=(0.0, 0.0, 0.0), start_time=0.0, end_time=1.0e9):
        return self._add(host.box_collider(center, half_size, velocity, start_time, end_time))

    def add_cup(self, profile, center, quat=(1.0, 0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0),
                friction=0.05, sticky_cells=1.5, contact_cells=0.5, start_time=0.0, end_time=1.0e9):
        sticky = min(sticky_cells * self.dx, 0.45 * profile.wall_thickness)
        return self._add(host.cup_collider(center, quat_to_mat(quat), velocity, omega, profile.outer_radius,
                                           profile.inner_radius, profile.half_height, profile.inner_floor_z,
                                           profile.fillet_radius, friction, sticky, contact_cells * self.dx,
                                           start_time, end_time))

    def set_cup(self, handle, center=None, quat=None, velocity=None, omega=None):
        c = self.cols[self.handles[handle]]
        if center is not None:
            host._vec(c.point, center)
        if quat is not None:
            host.set_rotation(c, quat_to_mat(quat))
        if velocity is not None:
            host._vec(c.velocity, velocity)
        if omega is not None:
            host._vec(c.omega, omega)
        return self

    def set_box(self, handle, center=None, velocity=None):
        c = self.cols[self.handles[handle]]
        if center is not None:
            host._vec(c.point, center)
        if velocity is not None:
            host._vec(c.velocity, velocity)
        return self

    def add_domain_walls(self, start_time=0.0, end_time=1.0e9):
        self._add(host.walls_collider(start_time, end_time), slots=6)
        return self

    def add_sdf_collider(self, sdf, center, quat=(0.0, 0.0, 0.0, 1.0), velocity=(0.0, 0.0, 0.0),
                         omega=(0.0, 0.0, 0.0), band=None, surface="separable", friction=0.4, start_time=0.0,
                         end_time=1.0e9):
        val = np.ascontiguousarray(sdf.values, np.float32)
        grad = np.ascontiguousarray(sdf.grads, np.float32)
        self.sdf_arrays += [val, grad]
        band = float(self.model.dx) if band is None else band
        return self._add(host.sdf_collider(_p(val), _p(grad), val.shape[0], sdf.origin, sdf.cell, center, quat,
                                           velocity, omega, band, host.SDF_SURFACES[surface], friction,
                                           start_time, end_time))

    def _push_cdf(self):
        lib = load(self.precision)
        if self.cdf_state is None:
            self.cdf_state = lib.gbmpm_oracle_cdf_new(self.n_grid)
        arr = (_abi.Cdf * max(1, len(self.cdf_lanes)))(*self.cdf_lanes)
        rc = lib.gbmpm_oracle_cdf_set(self.cdf_state, arr, len(self.cdf_lanes), float(self.time))
        if rc != 0:
            raise ValueError(lib.gbmpm_oracle_last_error().decode())

    def _pull_cdf(self):
        if self.cdf_state is None or not self.cdf_lanes:
            return
        arr = (_abi.Cdf * len(self.cdf_lanes))()
        load(self.precision).gbmpm_oracle_cdf_get(self.cdf_state, arr, len(self.cdf_lanes))
        self.cdf_lanes = [arr[i] for i in range(len(self.cdf_lanes))]

    def add_cdf_collider(self, cdf, center, quat=(0.0, 0.0, 0.0, 1.0), velocity=(0.0, 0.0, 0.0),
                         omega=(0.0, 0.0, 0.0), band=None, surface="separable", friction=0.4, start_time=0.0,
                         end_time=1.0e9):
        if len(self.cdf_lanes) >= _abi.MAX_CDF:
            raise ValueError("at most 4 CDF colliders per scene")
        band = host.cdf_band(cdf.band, self.dx, band)
        vals = np.ascontiguousarray(cdf.values, np.float32)
        valid = np.ascontiguousarray(cdf.valid, np.float32)
        self.cdf_arrays += [vals, valid]
        self._pull_cdf()
        self.cdf_lanes.append(host.cdf_lane(_p(vals), _p(valid), vals.shape[0], cdf.origin, cdf.cell, center, quat,
                                            velocity, omega, band, host.SDF_SURFACES[surface], friction,
                                            start_time, end_time))
        self._push_cdf()
        return len(self.cdf_lanes) - 1

    def set_cdf_pose(self, handle, center=None, quat=None, velocity=None, omega=None):
        self._pull_cdf()
        c = self.cdf_lanes[handle]
        if center is not None:
            host._vec(c.center, center)
        if quat is not None:
            host._vec(c.quat, quat)
        if velocity is not None:
            host._vec(c.velocity, velocity)
        if omega is not None:
            host._vec(c.omega, omega)
        self._push_cdf()
        return self

    def reset_cdf_wrench(self):
        self.cdf_wrench_acc[:] = 0.0
        return self

    def cdf_grids(self):
        """(tag, distance) node grids of the last stamp and the number of stamps so far."""
        ng = self.n_grid
        tag = np.zeros((ng, ng, ng), np.int32)
        d = np.zeros((ng, ng, ng), self.fdt)
        if self.cdf_state is None:
            return tag, d, 0
        lib = load(self.precision)
        lib.gbmpm_oracle_cdf_grids(self.cdf_state, _p(tag), _p(d))
        return tag, d, int(lib.gbmpm_oracle_cdf_stamp_count(self.cdf_state))

    def cdf_wrench(self, handle, dt):
        w = self.cdf_wrench_acc[handle].astype(float)
        return {"force": w[:3] / dt, "torque": w[3:] / dt}

    def wrench_of(self, handle, dt):
        w = self.wrench[self.handles[handle]].astype(float)
        return {"force": w[:3] / dt, "torque": w[3:] / dt}

    def reset_wrench(self, handle):
        self.wrench[self.handles[handle]] = 0.0

    # ------------------------------------------------------------ from GPU
    @classmethod
    def from_state(cls, st: dict, n_grid: int, grid_lim: float, fused: bool = True, threads: int = 1,
                   precision: int = 32):
        o = cls(n_grid, grid_lim, fused=fused, threads=threads, precision=precision)
        o.a = {k: (None if st.get(k) is None else np.ascontiguousarray(st[k]).copy()) for k in _KEYS}
        for k in _FLOAT_KEYS:
            if o.a.get(k) is not None:
                o.a[k] = np.ascontiguousarray(o.a[k], o.fdt)
        C.memmove(C.byref(o.model), C.byref(st["model"]), C.sizeof(_abi.Model))
        o.eta_table = np.ascontiguousarray(st["eta_table"], np.float32).copy()
        o.model.eta_table = _p(o.eta_table)
        for rec in st["colliders"]:
            r = _abi.Collider()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
            if r.kind == _abi.COLLIDER_SDF:
                val = np.ascontiguousarray(st["sdf_host"][rec.sdf_val], np.float32)
                grad = np.ascontiguousarray(st["sdf_host"][rec.sdf_grad], np.float32)
                o.sdf_arrays += [val, grad]
                r.sdf_val, r.sdf_grad = _p(val), _p(grad)
            o.cols.append(r)
        o.handles = list(st.get("handles", range(len(o.cols))))
        o.wrench = np.zeros((len(o.cols), 6), o.fdt)
        o.time = float(st["time"])
        n = len(o.a["x"])
        for k, shape, dt in (("cdf_tag", (n,), np.int32), ("rigid_id", (n,), np.int32), ("x_ref", (n, 3), o.fdt),
                             ("mod_mask", (n,), np.int32)):
            if o.a.get(k) is None:
                o.a[k] = np.zeros(shape, dt)
        o.rigid_bodies = [_copy(_abi.RigidBody, r) for r in st.get("rigid_bodies", [])]
        o.rigid_surfaces = [_copy(_abi.RigidSurface, r) for r in st.get("rigid_surfaces", [])]
        o.modifiers = [_copy(_abi.Modifier, r) for r in st.get("modifiers", [])]
        for rec in st.get("cdf_lanes", []):
            r = _abi.Cdf()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Cdf))
            vals = np.ascontiguousarray(st["cdf_host"][rec.values], np.float32)
            valid = np.ascontiguousarray(st["cdf_host"][rec.valid], np.float32)
            o.cdf_arrays += [vals, valid]
            r.values, r.valid = _p(vals), _p(valid)
            o.cdf_lanes.append(r)
        if o.cdf_lanes:
            o._push_cdf()
        return o

    # ------------------------------------------------------------------ step
    def _particles(self):
        p = _abi.Particles()
        p.n = len(self.a["x"])
        for k in _KEYS:
            setattr(p, k, _p(self.a[k]))
        return p

    def step(self, dt, substeps=1):
        """One control tick; scenes with rigid bodies or particle modifiers run the
        split pipeline, as the reference's Solver.step does."""
        lib = load(self.precision)
        p = self._particles()
        nb, ns, nm = len(self.rigid_bodies), len(self.rigid_surfaces), len(self.modifiers)
        bodies = (_abi.RigidBody * max(1, nb))(*self.rigid_bodies)
        lib.gbmpm_oracle_set_rigid(bodies, nb, (_abi.RigidSurface * max(1, ns))(*self.rigid_surfaces), ns)
        lib.gbmpm_oracle_set_modifiers((_abi.Modifier * max(1, nm))(*self.modifiers), nm)
        arr = (_abi.Collider * max(1, len(self.cols)))(*self.cols)
        t = C.c_double(self.time)
        rc = lib.gbmpm_oracle_tick(C.byref(p), C.byref(self.model), arr, len(self.cols), _p(self.wrench),
                                   C.byref(t), float(dt), int(substeps), 1 if self.fused else 0, int(self.threads),
                                   self.cdf_state if self.cdf_lanes else None, _p(self.cdf_wrench_acc))
        lib.gbmpm_oracle_get_rigid(bodies, nb)
        self.rigid_bodies = [_copy(_abi.RigidBody, bodies[i]) for i in range(nb)]
        if rc != 0:
            raise RuntimeError(f"oracle tick failed ({rc}): {lib.gbmpm_oracle_last_error().decode()}")
        self.cols = [arr[i] for i in range(len(self.cols))]
        self.time = t.value
        return self

    def rigid_state(self, body: int = 0) -> dict:
        r = self.rigid_bodies[body]
        return {"com": np.array(r.x_cm[:], np.float32), "v": np.array(r.v_cm[:], np.float32),
                "omega": np.array(r.omega[:], np.float32), "R": np.array(r.R[:], np.float32).reshape(3, 3)}

    def x(self):
        return self.a["x"]

    def v(self):
        return self.a["v"]

    def F(self):
        return self.a["F"]

    @property
    def n_particles(self):
        return len(self.a["x"])
