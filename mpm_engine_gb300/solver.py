"""Drop-in replacement of warpmpm's typed `Solver` (src/warpmpm/core/solver.py:47-642).

Same constructor fields, method names, argument meaning, return values and
exceptions. Particle and grid state are PyTorch CUDA tensors owned by the
solver; the substep runs in libgbmpm.so (hand-written sm_103a kernels) through
the C ABI of include/gbmpm.h, given the tensors' device pointers. There is no
Warp, no Triton and no CPU path: a solver whose device is not CUDA, or whose
native library is missing, raises.
"""
from __future__ import annotations

import ctypes as C
import os
import warnings
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _abi, host
from .glass import quat_to_mat
from .materials import material_id

_COV6_IDX = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))
_DEVICE_ANNOUNCED = False


def _torch():
    import torch
    return torch


def _cov_to_six(cov: np.ndarray) -> np.ndarray:
    """(N, 6) upper-triangle or (N, 3, 3) symmetric -> (N, 6) float32 xx, xy, xz, yy, yz, zz."""
    cov = np.asarray(cov)
    if cov.ndim == 2 and cov.shape[1] == 6:
        return np.ascontiguousarray(cov, dtype=np.float32)
    if cov.ndim == 3 and cov.shape[1:] == (3, 3):
        return np.ascontiguousarray(np.stack([cov[:, i, j] for i, j in _COV6_IDX], axis=1), dtype=np.float32)
    raise ValueError(f"cov must be (N, 6) or (N, 3, 3), got shape {cov.shape}")


@dataclass
class GridConfig:
    n_grid: int = 64
    grid_lim: float = 0.4  # cubic domain edge, metres

    @property
    def dx(self) -> float:
        return self.grid_lim / self.n_grid


class _Engine:
    """Owner of one native engine handle."""

    def __init__(self):
        self.lib = _abi.load()
        h = C.c_void_p()
        _abi.check(self.lib.gbmpm_engine_create(C.byref(h)), "gbmpm_engine_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gbmpm_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """Minimal stand-in for the wp.array handles tests reach through `_sim`."""

    def __init__(self, t):
        self._t = t

    def numpy(self):
        return self._t.detach().cpu().numpy()

    @property
    def ptr(self) -> int:
        return self._t.data_ptr()

    @property
    def shape(self):
        return tuple(self._t.shape)

    def zero_(self):
        self._t.zero_()


class _HostArray:
    """A host array behind Warp's `.numpy()` accessor."""

    def __init__(self, a):
        self._a = a

    def numpy(self):
        return self._a


class _StateView:
    def __init__(self, s: Solver):
        self._s = s

    def __getattr__(self, name):
        t = self._s._t
        key = name[len("particle_"):] if name.startswith("particle_") else None
        if key in t:
            return _DeviceArray(t[key])
        if name in ("grid_cdf_tag", "grid_cdf_d"):   # the CPIC node grids (mpm_solver_warp.py:94-183)
            tag, d, _ = self._s.cdf_grids()
            return _HostArray(tag if name == "grid_cdf_tag" else d)
        raise AttributeError(name)


class _ModelView:
    def __init__(self, s: Solver):
        self._s = s

    @property
    def mu(self):
        return _DeviceArray(self._s._t["mu"])

    @property
    def lam(self):
        return _DeviceArray(self._s._t["lam"])

    @property
    def yield_stress(self):
        return _DeviceArray(self._s._t["yield_stress"])

    def _get(self, name):
        return getattr(self._s._model, name)

    def _set(self, name, value):
        setattr(self._s._model, name, value)
        self._s._model_dirty = True

    grid_v_damping_scale = property(lambda self: self._get("grid_v_damping_scale"),
                                    lambda self, v: self._set("grid_v_damping_scale", host.f32(v)))
    rpic_damping = property(lambda self: self._get("rpic_damping"),
                            lambda self, v: self._set("rpic_damping", host.f32(v)))
    periodic_x = property(lambda self: self._get("periodic_x"), lambda self, v: self._set("periodic_x", int(v)))
    n_grid = property(lambda self: self._get("n_grid"))
    dx = property(lambda self: self._get("dx"))
    inv_dx = property(lambda self: self._get("inv_dx"))

    @property
    def cdf_mask_off(self) -> int:
        """1: every particle scans its stencil for CPIC tags (no block-mask early-out)."""
        return 1 if self._s._cdf_mask_off else 0

    @cdf_mask_off.setter
    def cdf_mask_off(self, v):
        s = self._s
        s._cdf_mask_off = bool(v)
        if s._eng is not None:
            _abi.check(s._eng.lib.gbmpm_cdf_mask_off(s._eng.h, 1 if v else 0), "gbmpm_cdf_mask_off")


class _SimShim:
    """The parts of MPM_Simulator_WARP that tests and scripts touch through
    `Solver._sim` (mpm_solver_warp.py), mapped onto this engine."""

    def __init__(self, s: Solver):
        self._s = s
        self.mpm_state = _StateView(s)
        self.mpm_model = _ModelView(s)
        self.use_cuda_graph = os.environ.get("WARPMPM_NO_CUDA_GRAPH", "") != "1" and \
            os.environ.get("GBMPM_NO_CUDA_GRAPH", "") != "1"
        self.restrict_bc = True
        self.restrict_grid = True
        # run each tick on a block-sorted working copy with shared-memory grid tiles
        self.reorder = os.environ.get("GBMPM_NO_REORDER", "") != "1"
        self.pre_p2g_operations = []
        self.particle_velocity_modifiers = []
        self.n_rigid_bodies = 0
        self.profile = False
        self.time_profile: dict = {}
        self._block_counts = None

    @property
    def n_particles(self) -> int:
        return self._s._n

    @property
    def _graph_A(self):
        """Non-None once the engine holds a captured tick graph."""
        s = self._s
        return "tick graph" if s._eng is not None and s._eng.lib.gbmpm_graph_state(s._eng.h) > 0 else None

    @property
    def collider_aabbs(self):
        """One callable per collider record, in order, giving the grid node box
        ((lo), (dims)) the collider can reach, or None when it lies outside the grid
        (the restricted-launch boxes of mpm_solver_warp.py:1283-1336). The engine
        applies colliders over the active blocks only, so the boxes are informational."""
        return [lambda rec=rec: self._s._collider_box(rec) for rec in self._s._cols]

    def _stamp_cdf(self, dt=None, device=None):
        """Stamp every CDF lane now (mpm_solver_warp.py:3040-3098)."""
        s = self._s
        s._sync_engine()
        _abi.check(s._eng.lib.gbmpm_cdf_restamp(s._eng.h, float(s._time), s._stream()), "gbmpm_cdf_restamp")

    @property
    def _cdf_force_stamp(self):
        return self._s._cdf_force

    @_cdf_force_stamp.setter
    def _cdf_force_stamp(self, on):
        s = self._s
        s._cdf_force = bool(on)
        _abi.check(s._eng.lib.gbmpm_cdf_force_stamp(s._eng.h, 1 if on else 0), "gbmpm_cdf_force_stamp")

    @property
    def _cdf_stamp_count(self):
        return self._s.cdf_grids()[2]

    # rigid-body arrays of MPM_Simulator_WARP (mpm_solver_warp.py:495-504), read from the engine
    def _rigid_field(self, name, shape):
        s = self._s
        recs = s._rigid_bodies() if s._n_bodies else []
        return _HostArray(np.array([np.array(getattr(r, name)[:], np.float32).reshape(shape) for r in recs],
                                   np.float32).reshape((len(recs),) + shape))

    @property
    def rigid_mass(self):
        recs = self._s._rigid_bodies() if self._s._n_bodies else []
        return _HostArray(np.array([r.mass for r in recs], np.float32))

    @property
    def rigid_x_cm(self):
        return self._rigid_field("x_cm", (3,))

    @property
    def rigid_v_cm(self):
        return self._rigid_field("v_cm", (3,))

    @property
    def rigid_omega(self):
        return self._rigid_field("omega", (3,))

    @property
    def rigid_orientation(self):
        return self._rigid_field("R", (3, 3))

    def finalize_rigid_bodies(self, device=None):
        self._s.finalize_rigid_bodies()

    def set_rigid_body_velocity(self, body_id, v_cm=(0, 0, 0), omega=(0, 0, 0), device=None):
        self._s.set_rigid_body_velocity(body_id, v_cm, omega)

    def add_impulse_on_particles(self, force, dt, point=(1, 1, 1), size=(1, 1, 1), num_dt=1, start_time=0.0,
                                 device=None):
        self._s.add_impulse_on_particles(force, dt, point, size, num_dt, start_time)

    def enforce_particle_velocity_translation(self, point, size, velocity, start_time, end_time, device=None):
        self._s.enforce_particle_velocity_translation(point, size, velocity, start_time, end_time)

    def enforce_particle_velocity_rotation(self, point, normal, half_height_and_radius, rotation_scale,
                                           translation_scale, start_time, end_time, device=None):
        self._s.enforce_particle_velocity_rotation(point, normal, half_height_and_radius, rotation_scale,
                                                   translation_scale, start_time, end_time)

    @property
    def time(self) -> float:
        return self._s._time

    def rebuild_active_blocks(self, device=None):
        self._s._rebuild_active_blocks()

    def active_block_fraction(self) -> float:
        if self._block_counts is None:
            return 1.0
        bd = (self._s.grid.n_grid + 3) // 4
        return self._block_counts[0] / float(bd ** 3)

    def _import(self, key, tensor, shape):
        torch = _torch()
        src = tensor.detach().reshape(shape).to(device=self._s._t[key].device, dtype=self._s._t[key].dtype)
        self._s._t[key].copy_(src)
        torch.cuda.synchronize()

    def import_particle_x_from_torch(self, t, clone=True, device=None):
        if t is not None:
            self._import("x", t, (-1, 3))

    def import_particle_v_from_torch(self, t, clone=True, device=None):
        if t is not None:
            self._import("v", t, (-1, 3))

    def import_particle_F_from_torch(self, t, clone=True, device=None):
        if t is not None:
            self._import("F", t, (-1, 3, 3))

    def import_particle_C_from_torch(self, t, clone=True, device=None):
        if t is not None:
            self._import("C", t, (-1, 3, 3))

    def export_particle_x_to_torch(self):
        return self._s._t["x"]

    def export_particle_v_to_torch(self):
        return self._s._t["v"]

    def export_particle_F_to_torch(self):
        return self._s._t["F"].reshape(-1, 9)

    def export_particle_stress_to_torch(self):
        return self._s._t["stress"].reshape(-1, 9)


@dataclass
class Solver:
    """One scene on one GPU. Field meanings follow warpmpm.Solver."""

    grid: GridConfig = field(default_factory=GridConfig)
    device: str = "auto"
    guard_interval: int = 1
    sparse: bool = False
    fused: bool = True
    sort_interval: int = 0
    profile: bool = False
    inversion_policy: str = "warn"
    periodic_x: bool = False
    # deterministic passes: every operation rounded once and P2G summed per node in
    # particle order, so runs repeat bit for bit (every material law but the rigid
    # bodies', and the particle modifiers; slower than the fast path)
    deterministic: bool = False
    _sim: Any = field(default=None, init=False, repr=False)
    _step: int = field(default=0, init=False, repr=False)
    _tick: int = field(default=0, init=False, repr=False)
    _vol0: Any = field(default=None, init=False, repr=False)

    def __post_init__(self) -> None:
        if self.inversion_policy not in {"warn", "raise", "nan"}:
            raise ValueError("inversion_policy must be 'warn', 'raise', or 'nan'")
        self._eng = None
        self._t: dict = {}
        self._n = 0
        self._time = 0.0
        self._model = None
        self._model_dirty = True
        self._cols: list = []          # engine collider records (engine copy is authoritative)
        self._handles: list = []       # reference handle -> engine collider index (None: extra wall slots)
        self._cols_dirty = True
        self._keep: list = []          # tensors referenced by collider records
        self._mat_current = 0
        self._sdf_guard: dict = {}
        self._cdf: list = []           # CPIC lane records (engine copy is authoritative)
        self._cdf_guard: dict = {}
        self._cdf_keep: list = []      # device copies of the lanes' fields
        self._rigid_surfaces: list = []
        self._n_bodies = 0
        self._mods: list = []          # particle modifier records, in registration order
        self._cdf_force = False
        self._cdf_mask_off = False
        self._update_cov = False

    # ------------------------------------------------------------------ setup
    def _resolve_device(self) -> None:
        torch = _torch()
        if self.device == "auto":
            self.device = "cuda:0" if torch.cuda.is_available() else "cpu"
            global _DEVICE_ANNOUNCED
            if not _DEVICE_ANNOUNCED:
                _DEVICE_ANNOUNCED = True
                print(f"mpm_engine_gb300: device auto -> {self.device}")
        if not str(self.device).startswith("cuda"):
            raise RuntimeError(f"mpm_engine_gb300 runs on CUDA devices only (device={self.device!r}); "
                               f"there is no CPU path")
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA is not available: mpm_engine_gb300 has no CPU path")

    def load_particles(self, pos: np.ndarray, vol: np.ndarray, cov: np.ndarray | None = None,
                       cov_mode: str = "step") -> Solver:
        """Load positions (N,3) and volumes (N,); optional per-particle covariance (N,6)
        or (N,3,3), advected each substep ("step") or rebuilt from F at export ("from_F")."""
        torch = _torch()
        self._resolve_device()
        _abi.load()
        dev = torch.device(self.device)
        torch.cuda.set_device(dev)
        pos = np.asarray(pos)
        n = len(pos)
        self._n = n
        self._vol0 = np.asarray(vol).astype(np.float32).copy()
        cov6 = None
        if cov is not None:
            if cov_mode not in ("step", "from_F"):
                raise ValueError(f"cov_mode must be 'step' or 'from_F', got {cov_mode!r}")
            cov6 = _cov_to_six(cov)
            if cov6.shape[0] != n:
                raise ValueError(f"cov has {cov6.shape[0]} rows, expected {n}")
        f = dict(device=dev, dtype=torch.float32)
        eye = torch.eye(3, **f).expand(n, 3, 3).contiguous()
        t = {
            "x": torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float32)).to(dev),
            "v": torch.zeros(n, 3, **f), "C": torch.zeros(n, 3, 3, **f), "F": eye.clone(),
            "F_trial": eye.clone(), "L": torch.zeros(n, 3, 3, **f), "stress": torch.zeros(n, 3, 3, **f),
            "R": torch.zeros(n, 3, 3, **f),
            "vol": torch.from_numpy(self._vol0.copy()).to(dev), "mass": torch.zeros(n, **f),
            "density": torch.zeros(n, **f), "Jp": torch.zeros(n, **f), "mu": torch.zeros(n, **f),
            "lam": torch.zeros(n, **f), "yield_stress": torch.zeros(n, **f),
            "material": torch.zeros(n, device=dev, dtype=torch.int32),
            "selection": torch.zeros(n, device=dev, dtype=torch.int32),
            "cdf_tag": torch.zeros(n, device=dev, dtype=torch.int32),
            "rigid_id": torch.zeros(n, device=dev, dtype=torch.int32), "x_ref": torch.zeros(n, 3, **f),
            "mod_mask": torch.zeros(n, device=dev, dtype=torch.int32),
            "init_cov": None, "cov": None,
        }
        if cov6 is not None:
            t["init_cov"] = torch.from_numpy(cov6).to(dev)
            t["cov"] = t["init_cov"].clone() if cov_mode == "step" else torch.zeros_like(t["init_cov"])
        ng = int(self.grid.n_grid)
        t["grid_mv"] = torch.zeros(ng * ng * ng, 4, **f)
        t["grid_v"] = torch.zeros(ng * ng * ng, 4, **f)
        t["perm"] = torch.zeros(max(n, 1), device=dev, dtype=torch.int32)
        t["eta_table"] = torch.zeros(2, **f)
        self._t = t
        self._update_cov = cov6 is not None and cov_mode == "step"
        self._model = host.default_model(ng, self.grid.grid_lim)
        self._model.periodic_x = 1 if self.periodic_x else 0
        self._model.update_cov_with_F = 1 if self._update_cov else 0
        self._model.eta_table = t["eta_table"].data_ptr()
        self._eng = _Engine()
        self._bind()
        if self._cdf_force:
            _abi.check(self._eng.lib.gbmpm_cdf_force_stamp(self._eng.h, 1), "gbmpm_cdf_force_stamp")
        if self._cdf_mask_off:
            _abi.check(self._eng.lib.gbmpm_cdf_mask_off(self._eng.h, 1), "gbmpm_cdf_mask_off")
        self._model_dirty = True
        self._sim = _SimShim(self)
        return self

    def _ptr(self, key) -> int | None:
        tt = self._t.get(key)
        return None if tt is None else tt.data_ptr()

    def _bind(self) -> None:
        p = _abi.Particles()
        p.n = self._n
        for k in ("x", "v", "C", "F", "F_trial", "L", "stress", "mass", "vol", "density", "Jp", "mu", "lam",
                  "yield_stress", "material", "selection", "cov", "init_cov", "cdf_tag", "rigid_id", "x_ref",
                  "mod_mask"):
            setattr(p, k, self._ptr(k))
        g = _abi.Grid()
        g.n_grid = int(self.grid.n_grid)
        g.mv = self._ptr("grid_mv")
        g.v = self._ptr("grid_v")
        lib = self._eng.lib
        _abi.check(lib.gbmpm_bind(self._eng.h, C.byref(p), C.byref(g)), "gbmpm_bind")

    def _stream(self) -> int:
        return _torch().cuda.current_stream().cuda_stream

    def _require_loaded(self) -> None:
        if self._eng is None:
            raise RuntimeError("load_particles must be called first")

    # -------------------------------------------------------------- materials
    def _apply_params(self, kw: dict, lo: int | None = None, hi: int | None = None) -> None:
        """set_parameters_dict (whole scene) or set_parameters_for_particles ([lo, hi))."""
        torch = _torch()
        t, m = self._t, self._model
        ranged = lo is not None
        sl = slice(lo, hi) if ranged else slice(None)
        if "material" in kw:
            mid = material_id(kw["material"])
            t["material"][sl] = mid
            if ranged:
                m.material_mask |= 1 << mid
            else:
                self._mat_current = mid
                m.material_mask = 1 << mid
            mat = mid
        else:
            mat = self._mat_current
        host.apply_type_params(m, mat, kw)
        if "yield_stress" in kw:
            t["yield_stress"][sl] = float(kw["yield_stress"])
        if "eta_table" in kw:
            tab = np.asarray(kw["eta_table"], dtype=np.float32).reshape(-1)
            t["eta_table"] = torch.from_numpy(tab.copy()).to(t["x"].device)
            m.eta_table = t["eta_table"].data_ptr()
            m.eta_table_n = int(tab.shape[0])
        if "eta_table_smin" in kw:
            m.eta_table_smin = host.f32(kw["eta_table_smin"])
        if "eta_table_smax" in kw:
            m.eta_table_smax = host.f32(kw["eta_table_smax"])
        if "g" in kw and not ranged:
            g = kw["g"]
            m.gravity[:] = (host.f32(g[0]), host.f32(g[1]), host.f32(g[2]))
        if "density" in kw:
            t["density"][sl] = float(kw["density"])
            t["mass"][sl] = t["density"][sl] * t["vol"][sl]
        if "E" in kw or "nu" in kw:
            if ranged:
                # the range path computes in float64 from the fp32 table values (:1774-1783)
                E_val, nu_val = float(m.E[mat]), float(m.nu[mat])
                t["mu"][sl] = E_val / (2.0 * (1.0 + nu_val))
                t["lam"][sl] = E_val * nu_val / ((1.0 + nu_val) * (1.0 - 2.0 * nu_val))
            else:
                self._finalize_mu_lam()
        if "rpic_damping" in kw:
            m.rpic_damping = host.f32(kw["rpic_damping"])
        if "grid_v_damping_scale" in kw:
            m.grid_v_damping_scale = host.f32(kw["grid_v_damping_scale"])
        if "obj_id" in kw:   # rigid body of material-8 particles (mpm_solver_warp.py:1755-1758)
            t["rigid_id"][sl] = int(kw["obj_id"])
        if "additional_material_params" in kw:
            raise NotImplementedError("regional additional_material_params are not supported")
        self._model_dirty = True

    def _finalize_mu_lam(self) -> None:
        torch = _torch()
        t, m = self._t, self._model
        dev = t["x"].device
        E = torch.tensor(list(m.E), device=dev, dtype=torch.float32)
        nu = torch.tensor(list(m.nu), device=dev, dtype=torch.float32)
        idx = t["material"].long()
        Ep, nup = E[idx], nu[idx]
        t["mu"].copy_(Ep / (2.0 * (1.0 + nup)))
        t["lam"].copy_(Ep * nup / ((1.0 + nup) * (1.0 - 2.0 * nup)))

    def set_material(self, material, **overrides: float) -> Solver:
        """A Material (or material name) applied to every particle; gravity defaults
        to (0, 0, -9.81) unless overridden."""
        self._require_loaded()
        if hasattr(material, "resolve"):
            name, params = material.resolve()
        else:
            name, params = str(material), {}
        params = {**params, **overrides}
        self._apply_params({"material": name, "g": [0.0, 0.0, -9.81], **params})
        self._finalize_mu_lam()
        return self

    def set_material_range(self, start: int, end: int, material, **overrides) -> Solver:
        """Material for particles [start, end); per-type parameters are shared by id."""
        self._require_loaded()
        if hasattr(material, "resolve"):
            name, params = material.resolve()
        else:
            name, params = str(material), {}
        if name in ("tabulated_viscous", "tabulated_mu_i"):
            raise NotImplementedError("tabulated materials are global-only (one eta table on the model); "
                                      "use set_material")
        self._apply_params({"material": name, **params, **overrides}, lo=int(start), hi=int(end))
        return self

    # ------------------------------------------------------------- rigid bodies
    def finalize_rigid_bodies(self) -> Solver:
        """Each rigid body's mass, centre of mass and body-frame inverse inertia from
        the particles assigned material "rigid" and their obj_id, and every rigid
        particle's body-frame position (finalize_rigid_bodies, mpm_solver_warp.py:
        834-879). Bodies start at rest with identity orientation. Call after every
        set_material_range and before the first step."""
        self._require_loaded()
        torch = _torch()
        t = self._t
        recs, x_ref = host.rigid_bodies(t["x"].cpu().numpy(), t["mass"].cpu().numpy(), t["material"].cpu().numpy(),
                                        t["rigid_id"].cpu().numpy())
        if not recs:
            return self
        t["x_ref"].copy_(torch.from_numpy(x_ref))
        self._n_bodies = len(recs)
        self._sim.n_rigid_bodies = len(recs)
        self._push_rigid((_abi.RigidBody * len(recs))(*recs))
        return self

    def _collider_box(self, rec):
        """Grid node box a collider record can reach, or None outside the grid."""
        ng, dx = int(self.grid.n_grid), float(self.grid.dx)
        c = np.array(rec.point[:], np.float64)
        if rec.kind == _abi.COLLIDER_SDF:
            ext = host.sdf_r_max(np.array(rec.sdf_origin[:]), float(rec.sdf_cell), int(rec.sdf_res)) + float(rec.band)
        elif rec.kind == _abi.COLLIDER_CUP:
            ext = float(rec.outer_radius) + float(rec.half_height) + float(rec.contact_band)
        elif rec.kind == _abi.COLLIDER_BOX:
            ext = np.abs(np.array(rec.size[:], np.float64))
        else:
            return (0, 0, 0), (ng, ng, ng)
        lo = np.maximum(np.floor((c - ext) / dx).astype(int) - 2, 0)
        hi = np.minimum(np.ceil((c + ext) / dx).astype(int) + 3, ng)
        if np.any(hi <= lo):
            return None
        return tuple(int(v) for v in lo), tuple(int(v) for v in hi - lo)

    def _surface_records(self):
        arr = (_abi.RigidSurface * max(1, len(self._rigid_surfaces)))()
        for i, rec in enumerate(self._rigid_surfaces):
            arr[i] = rec
        return arr

    def _push_rigid(self, bodies=None) -> None:
        if self._n_bodies == 0:
            return
        if bodies is None:
            bodies = self._rigid_bodies()
        _abi.check(self._eng.lib.gbmpm_set_rigid(self._eng.h, bodies, self._n_bodies, self._surface_records(),
                                                 len(self._rigid_surfaces)), "gbmpm_set_rigid")

    def _rigid_bodies(self):
        arr = (_abi.RigidBody * self._n_bodies)()
        _abi.check(self._eng.lib.gbmpm_get_rigid(self._eng.h, arr, self._n_bodies, self._stream()), "gbmpm_get_rigid")
        return arr

    def rigid_state(self, body: int = 0) -> dict:
        """State of one rigid body: com (3,), v (3,), omega (3,), R (3, 3)
        (core/solver.py:200-210)."""
        if not 0 <= body < self._n_bodies:
            raise IndexError(f"no rigid body {body}")
        r = self._rigid_bodies()[body]
        return {"com": np.array(r.x_cm[:], np.float32), "v": np.array(r.v_cm[:], np.float32),
                "omega": np.array(r.omega[:], np.float32), "R": np.array(r.R[:], np.float32).reshape(3, 3)}

    def set_rigid_body_velocity(self, body_id: int, v_cm=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0)) -> Solver:
        """Linear and angular velocity of one rigid body (mpm_solver_warp.py:881-885)."""
        bodies = self._rigid_bodies()
        bodies[body_id].v_cm[:] = tuple(float(c) for c in v_cm)
        bodies[body_id].omega[:] = tuple(float(c) for c in omega)
        self._push_rigid(bodies)
        return self

    # ------------------------------------------------------- particle modifiers
    def _add_modifier(self, rec, mask) -> None:
        if len(self._mods) >= _abi.MAX_MODIFIERS:
            raise ValueError(f"at most {_abi.MAX_MODIFIERS} particle modifiers")
        bit = len(self._mods)
        self._t["mod_mask"] |= (mask.to(_torch().int32) << bit)
        self._mods.append(rec)
        arr = (_abi.Modifier * len(self._mods))(*self._mods)
        _abi.check(self._eng.lib.gbmpm_set_modifiers(self._eng.h, arr, len(self._mods)), "gbmpm_set_modifiers")

    def _mask(self, mask_np):
        return _torch().from_numpy(mask_np).to(self._t["x"].device)

    def add_impulse_on_particles(self, force, dt, point=(1, 1, 1), size=(1, 1, 1), num_dt: int = 1,
                                 start_time: float = 0.0) -> Solver:
        """For num_dt substeps from start_time, v += force / m * dt on the particles
        within the box |x - point| < size, chosen now (mpm_solver_warp.py:2385-2427)."""
        self._require_loaded()
        rec = host.impulse_modifier(force, dt, num_dt, start_time)
        self._add_modifier(rec, self._mask(host.box_mask(self.x(), point, size)))
        self._sim.pre_p2g_operations.append(rec)
        return self

    def enforce_particle_velocity_translation(self, point, size, velocity, start_time, end_time) -> Solver:
        """Between start_time and end_time, v = velocity on the particles within the box
        |x - point| < size, chosen now (mpm_solver_warp.py:2431-2469)."""
        self._require_loaded()
        rec = host.translation_modifier(velocity, start_time, end_time)
        self._add_modifier(rec, self._mask(host.box_mask(self.x(), point, size)))
        self._sim.particle_velocity_modifiers.append(rec)
        return self

    def enforce_particle_velocity_rotation(self, point, normal, half_height_and_radius, rotation_scale,
                                           translation_scale, start_time, end_time) -> Solver:
        """Between start_time and end_time, the particles within the cylinder about the
        axis through `point` along `normal` (half height, radius), chosen now, turn at
        rotation_scale about the axis and move at translation_scale along it
        (mpm_solver_warp.py:2475-2539)."""
        self._require_loaded()
        rec = host.rotation_modifier(point, normal, rotation_scale, translation_scale, start_time, end_time)
        mask = host.cylinder_mask(self.x(), point, rec.normal[:], half_height_and_radius[0], half_height_and_radius[1])
        self._add_modifier(rec, self._mask(mask))
        self._sim.particle_velocity_modifiers.append(rec)
        return self

    # -------------------------------------------------------------- colliders
    def _add_collider(self, rec, slots: int = 1) -> int:
        idx = len(self._cols)
        self._cols.append(rec)
        first = len(self._handles)
        self._handles.append(idx)
        for _ in range(slots - 1):
            self._handles.append(None)
        self._cols_dirty = True
        return first

    def _pull_colliders(self) -> None:
        """Bring the engine's integrated poses into the host records."""
        if self._cols_dirty or not self._cols:
            return
        arr = (_abi.Collider * len(self._cols))()
        _abi.check(self._eng.lib.gbmpm_get_colliders(self._eng.h, arr, len(self._cols)), "gbmpm_get_colliders")
        self._cols = [arr[i] for i in range(len(self._cols))]

    def _push_colliders(self) -> None:
        if not self._cols_dirty:
            return
        arr = (_abi.Collider * max(1, len(self._cols)))(*self._cols)
        _abi.check(self._eng.lib.gbmpm_set_colliders(self._eng.h, arr, len(self._cols)), "gbmpm_set_colliders")
        self._cols_dirty = False

    def _col(self, handle: int):
        if handle < 0 or handle >= len(self._handles) or self._handles[handle] is None:
            raise IndexError(f"no collider with handle {handle}")
        self._pull_colliders()
        return self._handles[handle]

    def add_plane(self, point, normal, surface: str = "sticky", friction: float = 0.0,
                  restitution: float = 0.0) -> Solver:
        """Half-space boundary behind `point` along `normal` (sticky / slip / separable)."""
        self._require_loaded()
        rec = host.plane_collider(point, normal, surface, friction)
        if restitution != 0.0:
            if not (0.0 < restitution <= 1.0):
                raise ValueError("restitution must be between 0 (exclusive) and 1 (inclusive).")
            if len(self._rigid_surfaces) >= _abi.MAX_RIGID_SURFACES:
                raise ValueError(f"at most {_abi.MAX_RIGID_SURFACES} rigid contact surfaces")
            self._rigid_surfaces.append(host.rigid_surface(point, normal, friction, restitution))
            self._push_rigid()
        self._pull_colliders()
        self._add_collider(rec)
        return self

    def add_box(self, center, half_size, velocity=(0.0, 0.0, 0.0), start_time: float = 0.0,
                end_time: float = 1.0e9) -> int:
        """Kinematic axis-aligned box imposing its velocity on covered nodes; returns a handle."""
        self._require_loaded()
        self._pull_colliders()
        return self._add_collider(host.box_collider(center, half_size, velocity, start_time, end_time))

    def set_box(self, handle: int, center=None, velocity=None) -> Solver:
        """Start-of-tick centre and per-tick velocity (the box sweeps center -> center + dt*v)."""
        i = self._col(handle)
        c = self._cols[i]
        if center is not None:
            host._vec(c.point, center)
        if velocity is not None:
            host._vec(c.velocity, velocity)
        self._cols_dirty = True
        return self

    def add_cup(self, profile, center, quat=(1.0, 0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0),
                omega=(0.0, 0.0, 0.0), friction: float = 0.05, sticky_cells: float = 1.5,
                contact_cells: float = 0.5, start_time: float = 0.0, end_time: float = 1.0e9) -> int:
        """Kinematic open-top glass (analytic revolved SDF, quat w x y z); returns a handle."""
        self._require_loaded()
        sticky_depth = min(sticky_cells * self.grid.dx, 0.45 * profile.wall_thickness)
        rec = host.cup_collider(center, quat_to_mat(quat), velocity, omega, profile.outer_radius,
                                profile.inner_radius, profile.half_height, profile.inner_floor_z,
                                profile.fillet_radius, friction, sticky_depth, contact_cells * self.grid.dx,
                                start_time, end_time)
        self._pull_colliders()
        return self._add_collider(rec)

    def set_cup(self, handle: int, center=None, quat=None, velocity=None, omega=None) -> Solver:
        i = self._col(handle)
        c = self._cols[i]
        if center is not None:
            host._vec(c.point, center)
        if quat is not None:
            host.set_rotation(c, quat_to_mat(quat))
        if velocity is not None:
            host._vec(c.velocity, velocity)
        if omega is not None:
            host._vec(c.omega, omega)
        self._cols_dirty = True
        return self

    def _wrench(self, handle: int) -> np.ndarray:
        i = self._col(handle)
        self._push_colliders()
        out = (C.c_double * 6)()
        _abi.check(self._eng.lib.gbmpm_wrench(self._eng.h, i, out, self._stream()), "gbmpm_wrench")
        return np.array(out[:], dtype=float)

    def _reset_wrench(self, handle: int) -> None:
        i = self._col(handle)
        self._push_colliders()
        _abi.check(self._eng.lib.gbmpm_reset_wrench(self._eng.h, i, self._stream()), "gbmpm_reset_wrench")

    def reset_cup_wrench(self, handle: int) -> Solver:
        self._reset_wrench(handle)
        return self

    def cup_wrench(self, handle: int, dt: float) -> dict:
        """Accumulated reaction impulse / dt: {'force': (3,), 'torque': (3,)} (torque about the cup centre)."""
        w = self._wrench(handle)
        return {"force": w[:3] / dt, "torque": w[3:] / dt}

    def add_domain_walls(self, start_time: float = 0.0, end_time: float = 1.0e9) -> Solver:
        """Zero outward velocity in a three-cell band at each domain face."""
        self._require_loaded()
        self._pull_colliders()
        self._add_collider(host.walls_collider(start_time, end_time), slots=6)
        return self

    def add_sdf_collider(self, sdf, center, quat=(0.0, 0.0, 0.0, 1.0), velocity=(0.0, 0.0, 0.0),
                         omega=(0.0, 0.0, 0.0), band=None, surface: str = "separable", friction: float = 0.4,
                         start_time: float = 0.0, end_time: float = 1.0e9) -> int:
        """Moving signed-distance-field collider (geometry.SDFData, quat x y z w); returns a handle."""
        self._require_loaded()
        torch = _torch()
        res = int(np.asarray(sdf.values).shape[0])
        if band is None:
            band = float(self._model.dx)
        surface_id = host.SDF_SURFACES[surface]
        bmin = host.sdf_boundary_min(sdf.values)
        if band >= bmin:
            raise ValueError(
                f"SDF collider contact band ({band * 1e3:.1f} mm) reaches or exceeds the SDF "
                f"grid margin ({bmin * 1e3:.1f} mm): near-surface space outside the "
                f"stored grid would get no collision. Rebuild the SDF with more margin_cells "
                f"or reduce band.")
        dev = self._t["x"].device
        val = torch.from_numpy(np.ascontiguousarray(sdf.values, dtype=np.float32)).to(dev)
        grad = torch.from_numpy(np.ascontiguousarray(sdf.grads, dtype=np.float32)).to(dev)
        self._keep += [val, grad]
        rec = host.sdf_collider(val.data_ptr(), grad.data_ptr(), res, sdf.origin, sdf.cell, center, quat,
                                velocity, omega, band, surface_id, friction, start_time, end_time)
        self._pull_colliders()
        h = self._add_collider(rec)
        self._sdf_guard[h] = {"r_max": host.sdf_r_max(sdf.origin, sdf.cell, res), "band": float(band),
                              "warned": False}
        return h

    def set_sdf_pose(self, handle: int, center=None, quat=None, velocity=None, omega=None) -> Solver:
        i = self._col(handle)
        c = self._cols[i]
        guard = self._sdf_guard.get(handle)
        if guard is not None and not guard["warned"]:
            jump = 0.0
            if center is not None:
                jump += float(np.linalg.norm(np.array([float(center[k]) - c.point[k] for k in range(3)])))
            if quat is not None:
                dot = abs(sum(float(quat[k]) * c.quat[k] for k in range(4)))
                jump += 2.0 * float(np.arccos(min(1.0, dot))) * guard["r_max"]
            if jump > guard["band"]:
                guard["warned"] = True
                warnings.warn(
                    f"set_sdf_pose jumped the collider surface by up to {jump * 1e3:.2f} mm in one tick, more "
                    f"than the contact band ({guard['band'] * 1e3:.2f} mm): material inside the swept region "
                    f"can be tunnelled through. Drive the pose in smaller per-tick steps (or via "
                    f"velocity/omega).", RuntimeWarning, stacklevel=2)
        if center is not None:
            host._vec(c.point, center)
        if quat is not None:
            host._vec(c.quat, quat)
        if velocity is not None:
            host._vec(c.velocity, velocity)
        if omega is not None:
            host._vec(c.omega, omega)
        self._cols_dirty = True
        return self

    def reset_sdf_force(self, handle: int) -> Solver:
        self._reset_wrench(handle)
        return self

    def sdf_wrench(self, handle: int, dt: float) -> dict:
        w = self._wrench(handle)
        return {"force": w[:3] / dt, "torque": w[3:] / dt}

    def add_cdf_collider(self, cdf, center, quat=(0.0, 0.0, 0.0, 1.0), velocity=(0.0, 0.0, 0.0),
                         omega=(0.0, 0.0, 0.0), band=None, surface: str = "separable", friction: float = 0.4,
                         start_time: float = 0.0, end_time: float = 1.0e9) -> int:
        """An OPEN oriented surface (geometry.CDFData) as a CPIC thin-boundary collider
        (core/solver.py:363-386, mpm_solver_warp.py:2819-2881): particle-node transfers
        across the surface are severed. Returns a lane handle, a separate space from the
        grid-BC colliders; at most 4 lanes per scene."""
        if self.periodic_x:
            raise NotImplementedError("CDF colliders do not wrap the periodic x axis")
        self._require_loaded()
        torch = _torch()
        lane = len(self._cdf)
        if lane >= _abi.MAX_CDF:
            raise ValueError(f"at most {_abi.MAX_CDF} CDF colliders per scene")
        band = host.cdf_band(cdf.band, float(self._model.dx), band)
        surface_id = host.SDF_SURFACES[surface]
        res = int(np.asarray(cdf.values).shape[0])
        dev = self._t["x"].device
        val = torch.from_numpy(np.ascontiguousarray(cdf.values, dtype=np.float32)).to(dev)
        valid = torch.from_numpy(np.ascontiguousarray(cdf.valid, dtype=np.float32)).to(dev)
        self._cdf_keep += [val, valid]
        rec = host.cdf_lane(val.data_ptr(), valid.data_ptr(), res, cdf.origin, cdf.cell, center, quat, velocity,
                            omega, band, surface_id, friction, start_time, end_time)
        self._cdf_guard[lane] = {"r_max": host.sdf_r_max(cdf.origin, cdf.cell, res), "band": float(band),
                                 "warned": False}
        self._sync_engine()
        self._pull_cdf()
        self._cdf.append(rec)
        self._push_cdf()
        return lane

    def _pull_cdf(self) -> None:
        n = len(self._cdf)
        if n == 0:
            return
        arr = (_abi.Cdf * n)()
        _abi.check(self._eng.lib.gbmpm_get_cdf(self._eng.h, arr, n), "gbmpm_get_cdf")
        self._cdf = [arr[i] for i in range(n)]

    def _push_cdf(self) -> None:
        n = len(self._cdf)
        arr = (_abi.Cdf * max(1, n))(*self._cdf)
        _abi.check(self._eng.lib.gbmpm_set_cdf(self._eng.h, arr, n), "gbmpm_set_cdf")

    def set_cdf_pose(self, handle: int, center=None, quat=None, velocity=None, omega=None) -> Solver:
        """Start-of-tick pose of a CDF collider (mpm_solver_warp.py:2945-2996); ticks
        integrate centre and quaternion per substep from velocity and omega. Warns once
        when a jump sweeps the surface farther than the band."""
        if not 0 <= handle < len(self._cdf):
            raise IndexError(f"no CDF collider with handle {handle}")
        self._pull_cdf()
        c = self._cdf[handle]
        guard = self._cdf_guard.get(handle)
        if guard is not None and not guard["warned"]:
            jump = 0.0
            if center is not None:
                jump += float(np.linalg.norm(np.array([float(center[k]) - c.center[k] for k in range(3)])))
            if quat is not None:
                dot = abs(sum(float(quat[k]) * c.quat[k] for k in range(4)))
                jump += 2.0 * float(np.arccos(min(1.0, dot))) * guard["r_max"]
            if jump > guard["band"]:
                guard["warned"] = True
                warnings.warn(
                    f"set_cdf_pose jumped the surface by up to {jump * 1e3:.2f} mm in one tick, more than the "
                    f"band ({guard['band'] * 1e3:.2f} mm): material in the swept region can end up on the wrong "
                    f"side. Drive the pose in smaller per-tick steps.", RuntimeWarning, stacklevel=2)
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

    def reset_cdf_wrench(self) -> Solver:
        """Zero the CDF reaction accumulators of every lane."""
        if self._cdf:
            _abi.check(self._eng.lib.gbmpm_reset_cdf_wrench(self._eng.h, self._stream()), "gbmpm_reset_cdf_wrench")
        return self

    def contact_wrench(self, box_center, box_half, layer_cells: float | None = None, dx: float | None = None,
                       compressive_only: bool = True) -> dict:
        """Stress-integral reaction on a box end-effector, computed on the device
        (box_contact_wrench, coupling/wrench.py:15-46, over x, cauchy() and vol()):
        {'force', 'torque', 'n_contact', 'Fz'}. Only 9 numbers cross to the host."""
        self._require_loaded()
        policy = {"warn": 0, "nan": 1, "raise": 2}[self.inversion_policy]
        layer = float(layer_cells) * float(dx) if (layer_cells and dx) else 0.0
        c = (C.c_double * 3)(*[float(v) for v in box_center])
        h = (C.c_double * 3)(*[float(v) for v in box_half])
        out = (C.c_double * 9)()
        rc = self._eng.lib.gbmpm_contact_wrench(self._eng.h, c, h, layer, 1 if compressive_only else 0, policy, out,
                                                self._stream())
        if rc == _abi.ERR_STATE and policy == 2:
            raise RuntimeError(self._eng.lib.gbmpm_last_error().decode())
        _abi.check(rc, "gbmpm_contact_wrench")
        if out[8] > 0 and policy == 0 and not getattr(self, "_warned_inverted", False):
            self._warned_inverted = True
            warnings.warn(f"{int(out[8])} particles have non-finite or non-positive det(F); current volume and "
                          f"Cauchy stress are undefined for an inverted configuration; using |det(F)| for "
                          f"compatibility. Set inversion_policy='raise' to reject or 'nan' to mark these particles.",
                          RuntimeWarning, stacklevel=2)
        n_contact = int(out[6])
        if n_contact < 3:
            return {"force": np.zeros(3), "torque": np.zeros(3), "n_contact": 0, "Fz": 0.0}
        force = np.array(out[0:3], dtype=float)
        return {"force": force, "torque": np.array(out[3:6], dtype=float), "n_contact": n_contact,
                "Fz": float(force[2])}

    def cdf_grids(self):
        """(tag, distance) node grids of the last CPIC stamp as host arrays, and the
        number of stamps so far."""
        torch = _torch()
        ng = int(self.grid.n_grid)
        dev = self._t["x"].device
        stamps = C.c_int64(0)
        if not self._cdf:
            return np.zeros((ng, ng, ng), np.int32), np.zeros((ng, ng, ng), np.float32), 0
        tag = torch.empty(ng, ng, ng, device=dev, dtype=torch.int32)
        d = torch.empty(ng, ng, ng, device=dev, dtype=torch.float32)
        _abi.check(self._eng.lib.gbmpm_cdf_grids(self._eng.h, tag.data_ptr(), d.data_ptr(), C.byref(stamps),
                                                 self._stream()), "gbmpm_cdf_grids")
        return tag.cpu().numpy(), d.cpu().numpy(), int(stamps.value)

    def _cdf_tunnel_check(self, dt: float) -> None:
        """Warn once per lane whose surface sweeps more than its band per substep
        (mpm_solver_warp.py:3119-3137)."""
        for lane, c in enumerate(self._cdf):
            guard = self._cdf_guard[lane]
            if guard["warned"] or not (c.start_time <= self._time < c.end_time):
                continue
            v = [c.velocity[k] for k in range(3)]
            w = np.array([c.omega[k] for k in range(3)], dtype=float)
            if v[0] == 0.0 and v[1] == 0.0 and v[2] == 0.0 and not w.any():
                continue
            speed = float(np.hypot(np.hypot(v[0], v[1]), v[2])) + float(np.linalg.norm(w)) * guard["r_max"]
            if speed * dt > guard["band"]:
                guard["warned"] = True
                warnings.warn(
                    f"CDF collider surface sweeps {speed * dt * 1e3:.2f} mm per substep, more than the band "
                    f"({guard['band'] * 1e3:.2f} mm): material can end up on the wrong side. Reduce dt or the "
                    f"pose rate, or rebuild with a larger band.", RuntimeWarning, stacklevel=3)

    def cdf_wrench(self, handle: int, dt: float) -> dict:
        """Reaction the material exerts on a CDF collider, summed from the blocked P2G
        deposits since the last reset (core/solver.py:401-413): {'force', 'torque'}."""
        out = (C.c_double * 6)()
        _abi.check(self._eng.lib.gbmpm_cdf_wrench(self._eng.h, int(handle), out, self._stream()),
                   "gbmpm_cdf_wrench")
        w = np.array(out[:], dtype=float)
        return {"force": w[:3] / dt, "torque": w[3:] / dt}

    def reset_tool_force(self, handle: int) -> Solver:
        self._reset_wrench(handle)
        return self

    def tool_force(self, handle: int, dt: float) -> np.ndarray:
        """Box reaction force: accumulated sum of m (v_free - v_box) / dt."""
        return self._wrench(handle)[:3] / dt

    # ------------------------------------------------------------------- step
    def _sync_engine(self) -> None:
        lib, h = self._eng.lib, self._eng.h
        if self._model_dirty:
            self._model.update_cov_with_F = 1 if self._update_cov else 0
            _abi.check(lib.gbmpm_set_model(h, C.byref(self._model)), "gbmpm_set_model")
            self._model_dirty = False
        self._push_colliders()

    def _sdf_tunnel_check(self, dt: float) -> None:
        for handle, guard in self._sdf_guard.items():
            if guard["warned"]:
                continue
            c = self._cols[self._handles[handle]]
            speed = float(np.hypot(np.hypot(c.velocity[0], c.velocity[1]), c.velocity[2])) + \
                float(np.linalg.norm([c.omega[0], c.omega[1], c.omega[2]])) * guard["r_max"]
            live = c.start_time <= self._time < c.end_time
            if live and speed * dt > guard["band"]:
                guard["warned"] = True
                warnings.warn(
                    f"SDF collider surface sweeps {speed * dt * 1e3:.2f} mm per substep, more than the contact "
                    f"band ({guard['band'] * 1e3:.2f} mm): fast material can tunnel through. Reduce dt, "
                    f"velocity/omega, or raise band (and the SDF margin).", RuntimeWarning, stacklevel=3)

    def _tick_flags(self) -> int:
        # Sparse ticks stay on the fused schedule. The reference drops to the split one
        # in sparse mode (core/solver.py:441-444) because its active-block lists are
        # rebuilt per phase; here every particle pass marks the blocks it deposits into
        # and the grid pass visits exactly those, on either schedule, and the two
        # schedules compute the same substep (fused == split in the oracle, bit for bit).
        flags = 0
        if self.fused:
            flags |= _abi.TICK_FUSED
        if self.profile:
            flags |= _abi.TICK_PROFILE
        elif self._sim.use_cuda_graph:
            flags |= _abi.TICK_GRAPH
        if self._sim.reorder:
            flags |= _abi.TICK_REORDER
        if self.deterministic:
            flags |= _abi.TICK_DETERMINISTIC
        return flags

    def step(self, dt: float, substeps: int = 1) -> Solver:
        """Advance `substeps` substeps of size dt (one control tick)."""
        self._require_loaded()
        if self._tick % max(1, self.guard_interval) == 0:
            self._update_grid_box(dt, substeps)
        if self.sort_interval and self._tick % self.sort_interval == 0:
            self._sort_particles()
        if self.sparse:
            self._rebuild_active_blocks()
        self._sim.profile = self.profile
        self._tick += 1
        self._pull_colliders()
        if self._sdf_guard:
            self._sdf_tunnel_check(dt)
        if self._cdf:
            self._pull_cdf()
            self._cdf_tunnel_check(dt)
        self._sync_engine()
        flags = self._tick_flags()
        t = C.c_double(self._time)
        _abi.check(self._eng.lib.gbmpm_tick(self._eng.h, C.byref(t), float(dt), int(substeps), flags,
                                            self._stream()), "gbmpm_tick")
        if flags & _abi.TICK_GRAPH and self._eng.lib.gbmpm_graph_state(self._eng.h) < 0:
            # the capture failed and the engine ran this tick live; like the reference,
            # stay on live launches (mpm_solver_warp.py:1118-1125)
            self._sim.use_cuda_graph = False
        self._time = t.value
        self._step += substeps
        return self

    def _rebuild_active_blocks(self) -> None:
        self._sync_engine()
        counts = (C.c_int32 * 2)()
        _abi.check(self._eng.lib.gbmpm_rebuild_active_blocks(self._eng.h, counts, self._stream()),
                   "gbmpm_rebuild_active_blocks")
        self._sim._block_counts = (int(counts[0]), int(counts[1]))

    def _sort_particles(self) -> bool:
        """Stable block-key sort (4^3 blocks of the stencil base, float64 keys); skipped
        when already ordered. Returns True when particles were permuted."""
        self._require_loaded()
        flag = C.c_int32(0)
        perm = self._t["perm"]
        _abi.check(self._eng.lib.gbmpm_sort_particles(self._eng.h, float(self.grid.dx), C.byref(flag),
                                                      perm.data_ptr(), self._stream()), "gbmpm_sort_particles")
        if not flag.value:
            return False
        p = perm[: self._n].cpu().numpy().astype(np.int64)
        self._vol0 = self._vol0[p]
        return True

    def autotune(self, dt: float, substeps: int, ticks: int = 2, use_cache: bool = True) -> dict:
        """Picks the fastest launch shape of this scene's passes
        (mpm_engine_gb300.autotune); the scene's state is restored after the search."""
        from .autotune import tune_solver
        self._require_loaded()
        return tune_solver(self, dt, substeps, ticks=ticks, use_cache=use_cache)

    def profile_report(self) -> str:
        """Per-phase device time collected while profile=True (CUDA events, live launches)."""
        if self._eng is None:
            return "profile_report: no samples (set solver.profile = True and step)"
        ms = (C.c_double * _abi.NUM_PHASES)()
        cnt = (C.c_int64 * _abi.NUM_PHASES)()
        _abi.check(self._eng.lib.gbmpm_profile(self._eng.h, ms, cnt, 0), "gbmpm_profile")
        rows = [(self._eng.lib.gbmpm_phase_name(i).decode(), ms[i] / 1000.0, cnt[i])
                for i in range(_abi.NUM_PHASES) if cnt[i]]
        if not rows:
            return "profile_report: no samples (set solver.profile = True and step)"
        timed = sum(r[1] for r in rows)
        rows.sort(key=lambda r: -r[1])
        lines = [f"substep profile over {self._step} substeps (timed device work {timed:.1f}s; "
                 f"live launches + per-phase sync):"]
        for name, tot, n in rows:
            lines.append(f"  {name:<28s} {tot:7.1f}s  {tot / max(n, 1) * 1000:8.3f} ms/substep"
                         f"  {tot / timed * 100:5.1f}%")
        return "\n".join(lines)

    def _update_grid_box(self, dt: float, substeps: int) -> None:
        """Edge guard once per control tick (core/solver.py:485-518), reduced on the device."""
        out = (C.c_float * 7)()
        st = C.c_uint32(0)
        _abi.check(self._eng.lib.gbmpm_guard(self._eng.h, out, C.byref(st), self._stream()), "gbmpm_guard")
        self._check_guard(list(out), int(st.value))

    def _check_guard(self, out, status: int) -> None:
        if status & _abi.FLAG_STENCIL_OOB:
            raise RuntimeError("a particle's P2G stencil left the grid during the previous tick; the kernels "
                               "skipped it. Enlarge grid_lim or add a bounding box / wall collider.")
        dx, lim = self.grid.dx, self.grid.grid_lim
        lo = np.array(out[0:3], dtype=np.float32)
        hi = np.array(out[3:6], dtype=np.float32)
        if self.periodic_x:
            gmin, gmax = float(lo[1:].min()), float(hi[1:].max())
        else:
            gmin, gmax = float(lo.min()), float(hi.max())
        if gmin < 1.5 * dx or gmax > lim - 2.5 * dx:
            raise RuntimeError(host.grid_guard_message(gmin, gmax, lim, dx))

    # ---------------------------------------------------------------- imports
    def _import_rows(self, key: str, data) -> None:
        torch = _torch()
        if isinstance(data, torch.Tensor):
            # a (pinned) host or device tensor: stream-ordered copy into the existing buffer
            self._t[key].copy_(data.reshape(-1, 3), non_blocking=True)
            return
        self._t[key].copy_(torch.from_numpy(np.ascontiguousarray(data, dtype=np.float32)).reshape(-1, 3))
        torch.cuda.synchronize()

    def set_x(self, pos) -> Solver:
        """Copy positions into the existing device buffer (pointers stay stable)."""
        self._import_rows("x", pos)
        return self

    def set_v(self, vel) -> Solver:
        self._import_rows("v", vel)
        return self

    def x_into(self, out) -> None:
        """Stream-ordered copy of the positions into a caller (pinned host) tensor."""
        out.copy_(self._t["x"], non_blocking=True)

    def v_into(self, out) -> None:
        """Stream-ordered copy of the velocities into a caller (pinned host) tensor."""
        out.copy_(self._t["v"], non_blocking=True)

    # ---------------------------------------------------------------- exports
    def x(self) -> np.ndarray:
        return self._t["x"].cpu().numpy()

    def v(self) -> np.ndarray:
        return self._t["v"].cpu().numpy()

    def F(self) -> np.ndarray:
        return self._t["F"].cpu().numpy().reshape(-1, 3, 3)

    def stress(self) -> np.ndarray:
        return self._t["stress"].cpu().numpy().reshape(-1, 3, 3)

    def L(self) -> np.ndarray:
        """Velocity gradient L_ij = dv_i/dx_j from the most recent gather."""
        return self._t["L"].cpu().numpy().reshape(-1, 3, 3)

    def C(self) -> np.ndarray:
        return self._t["C"].cpu().numpy().reshape(-1, 3, 3)

    def inverted_count(self) -> int:
        J = np.linalg.det(self.F())
        return int(np.count_nonzero(~np.isfinite(J) | (J <= 0.0)))

    def _checked_jacobian(self) -> np.ndarray:
        if self.inversion_policy not in {"warn", "raise", "nan"}:
            raise ValueError("inversion_policy must be 'warn', 'raise', or 'nan'")
        J = np.linalg.det(self.F())
        bad = ~np.isfinite(J) | (J <= 0.0)
        n = int(np.count_nonzero(bad))
        if not n:
            return J
        message = (f"{n} particles have non-finite or non-positive det(F); current volume "
                   "and Cauchy stress are undefined for an inverted configuration")
        if self.inversion_policy == "raise":
            raise RuntimeError(message)
        if self.inversion_policy == "warn":
            if not getattr(self, "_warned_inverted", False):
                self._warned_inverted = True
                warnings.warn(f"{message}; using |det(F)| for compatibility. Set inversion_policy='raise' to "
                              "reject or 'nan' to mark these particles.", RuntimeWarning, stacklevel=3)
            out = np.abs(J)
            out[~np.isfinite(out)] = np.nan
            return out
        J = J.copy()
        J[bad] = np.nan
        return J

    def _device_exports(self, cauchy: bool, vol: bool):
        """Cauchy stress and current volume computed on the device under the
        inversion policy; raises or warns as _checked_jacobian does."""
        if self.inversion_policy not in {"warn", "raise", "nan"}:
            raise ValueError("inversion_policy must be 'warn', 'raise', or 'nan'")
        torch = _torch()
        n = self._n
        dev = self._t["x"].device
        c = torch.empty(n, 3, 3, device=dev, dtype=torch.float32) if cauchy else None
        v = torch.empty(n, device=dev, dtype=torch.float32) if vol else None
        bad = C.c_int32(0)
        policy = {"warn": 0, "nan": 1, "raise": 2}[self.inversion_policy]
        _abi.check(self._eng.lib.gbmpm_compute_cauchy(self._eng.h, None if c is None else c.data_ptr(),
                                                      None if v is None else v.data_ptr(), None, policy,
                                                      C.byref(bad), self._stream()), "gbmpm_compute_cauchy")
        if bad.value:
            message = (f"{bad.value} particles have non-finite or non-positive det(F); current volume "
                       "and Cauchy stress are undefined for an inverted configuration")
            if self.inversion_policy == "raise":
                raise RuntimeError(message)
            if self.inversion_policy == "warn" and not getattr(self, "_warned_inverted", False):
                self._warned_inverted = True
                warnings.warn(f"{message}; using |det(F)| for compatibility. Set inversion_policy='raise' to "
                              "reject or 'nan' to mark these particles.", RuntimeWarning, stacklevel=3)
        return c, v

    def vol_torch(self):
        """Current volume vol0 * det(F) as a device tensor (inversion policy applied)."""
        return self._device_exports(False, True)[1]

    def cauchy_torch(self):
        """Cauchy stress = Kirchhoff / det(F) as a device tensor (inversion policy applied)."""
        return self._device_exports(True, False)[0]

    def vol(self) -> np.ndarray:
        return self.vol_torch().cpu().numpy()

    def cauchy(self) -> np.ndarray:
        """Cauchy stress = Kirchhoff / det(F) under the inversion policy."""
        return self.cauchy_torch().cpu().numpy()

    def _cov_tensor(self):
        if self._t.get("cov") is None:
            raise ValueError("no covariance was loaded (load_particles(cov=...))")
        if not self._update_cov:
            _abi.check(self._eng.lib.gbmpm_compute_cov(self._eng.h, self._t["cov"].data_ptr(), self._stream()),
                       "gbmpm_compute_cov")
        return self._t["cov"]

    def cov(self) -> np.ndarray:
        return self._cov_tensor().cpu().numpy().reshape(-1, 6)

    def _R_tensor(self):
        _abi.check(self._eng.lib.gbmpm_compute_R(self._eng.h, self._t["R"].data_ptr(), self._stream()),
                   "gbmpm_compute_R")
        return self._t["R"]

    def R(self) -> np.ndarray:
        """Polar rotation R of F (the kernel stores R^T; this returns R)."""
        return np.transpose(self._R_tensor().cpu().numpy().reshape(-1, 3, 3), (0, 2, 1))

    def x_torch(self):
        return self._t["x"]

    def v_torch(self):
        return self._t["v"]

    def F_torch(self):
        return self._t["F"].reshape(-1, 3, 3)

    def cov_torch(self):
        return self._cov_tensor().reshape(-1, 6)

    def R_torch(self):
        return self._R_tensor().reshape(-1, 3, 3).transpose(1, 2)

    @property
    def n_particles(self) -> int:
        return 0 if self._eng is None else self._n

    @property
    def time(self) -> float:
        return self._time

    def launch_count(self) -> int:
        return 0 if self._eng is None else int(self._eng.lib.gbmpm_launch_count(self._eng.h))

    # ------------------------------------------------------------ test access
    # per-particle arrays a checkpoint carries: everything the step reads or writes
    _CHECKPOINT_FIELDS = ("x", "v", "C", "F", "F_trial", "L", "stress", "mass", "vol", "density", "Jp", "mu", "lam",
                          "yield_stress", "material", "selection", "cov", "init_cov", "cdf_tag", "rigid_id", "x_ref",
                          "mod_mask")

    def state_dict(self) -> dict:
        """Checkpoint of the simulation. It holds device copies of every per-particle
        array, the clock and tick counters, the collider poses and the rigid bodies'
        states. The reference has no full-state checkpoint; its pour script caches
        x and v only (examples/pour_franka.py:367-387)."""
        self._require_loaded()
        self._pull_colliders()
        cols = []
        for rec in self._cols:
            r = _abi.Collider()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
            cols.append(r)
        bodies = []
        if self._n_bodies:
            arr = self._rigid_bodies()
            for i in range(self._n_bodies):
                b = _abi.RigidBody()
                C.memmove(C.byref(b), C.byref(arr[i]), C.sizeof(_abi.RigidBody))
                bodies.append(b)
        return {"particles": {k: t.detach().clone() for k, t in self._t.items()
                              if k in self._CHECKPOINT_FIELDS and t is not None},
                "vol0": None if self._vol0 is None else np.array(self._vol0, copy=True),
                "time": self._time, "step": self._step, "tick": self._tick, "colliders": cols,
                "rigid_bodies": bodies, "n_particles": self._n, "n_grid": self.grid.n_grid}

    def load_state_dict(self, state: dict) -> Solver:
        """Restores a `state_dict` of this scene (same particles, grid and colliders).
        The arrays are copied in place, so buffer addresses and captured tick graphs
        stay valid; the working copy, the grid and the active blocks are rebuilt by
        the next tick from these arrays. Scenes with CDF lanes are refused: their
        per-particle scan cache and stamp history are not part of the checkpoint."""
        self._require_loaded()
        if state.get("n_particles") != self._n or state.get("n_grid") != self.grid.n_grid:
            raise ValueError("state_dict is of another scene (particle count or grid differs)")
        if self._cdf:
            raise NotImplementedError("load_state_dict does not restore CDF (CPIC) lane state")
        if len(state["colliders"]) != len(self._cols) or len(state["rigid_bodies"]) != self._n_bodies:
            raise ValueError("state_dict has another collider or rigid-body set")
        for k, t in state["particles"].items():
            if self._t.get(k) is None:
                raise ValueError(f"state_dict carries '{k}', which this scene does not allocate")
            self._t[k].copy_(t)
        self._cols = []
        for rec in state["colliders"]:
            r = _abi.Collider()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
            self._cols.append(r)
        self._cols_dirty = True
        if self._n_bodies:
            arr = (_abi.RigidBody * self._n_bodies)(*state["rigid_bodies"])
            self._push_rigid(arr)
        if state.get("vol0") is not None:
            self._vol0 = np.array(state["vol0"], copy=True)
        self._time, self._step, self._tick = state["time"], state["step"], state["tick"]
        self._sync_engine()
        return self

    def export_state(self) -> dict:
        """Host copies of the engine inputs (particles, model, colliders, clock) used to
        replay the same scene elsewhere."""
        self._pull_colliders()
        out = {k: (None if v is None else v.detach().cpu().numpy().copy())
               for k, v in self._t.items() if k in ("x", "v", "C", "F", "F_trial", "L", "stress", "mass", "vol",
                                                    "density", "Jp", "mu", "lam", "yield_stress", "material",
                                                    "selection", "cov", "init_cov", "cdf_tag", "rigid_id", "x_ref",
                                                    "mod_mask")}
        model = _abi.Model()
        C.memmove(C.byref(model), C.byref(self._model), C.sizeof(_abi.Model))
        out["model"] = model
        out["eta_table"] = self._t["eta_table"].cpu().numpy().copy()
        cols = []
        for rec in self._cols:
            r = _abi.Collider()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Collider))
            cols.append(r)
        out["colliders"] = cols
        out["handles"] = list(self._handles)
        out["sdf_host"] = {t.data_ptr(): t.cpu().numpy().copy() for t in self._keep}
        self._pull_cdf()
        lanes = []
        for rec in self._cdf:
            r = _abi.Cdf()
            C.memmove(C.byref(r), C.byref(rec), C.sizeof(_abi.Cdf))
            lanes.append(r)
        out["cdf_lanes"] = lanes
        out["cdf_host"] = {t.data_ptr(): t.cpu().numpy().copy() for t in self._cdf_keep}
        out["rigid_bodies"] = list(self._rigid_bodies()) if self._n_bodies else []
        out["rigid_surfaces"] = list(self._surface_records())[:len(self._rigid_surfaces)]
        out["modifiers"] = list(self._mods)
        out["time"] = self._time
        return out


class BatchSolver:
    """Many independent scenes advanced together on one GPU.

    Each scene is a loaded `Solver` (its own particles, grid, materials and
    colliders). `step` runs every scene's edge guard with one synchronization and
    then advances all scenes in one CUDA graph whose branches are the scenes'
    ticks, so scenes that each fill only part of the GPU run concurrently. The
    reference has no counterpart: its planners step one Solver at a time
    (experiments/shape_planning.py:107). Per-scene block sorting, sparse mode and
    profiling are not available inside a batch.
    """

    def __init__(self, solvers):
        self.solvers = list(solvers)
        if not self.solvers:
            raise ValueError("BatchSolver needs at least one Solver")
        for s in self.solvers:
            s._require_loaded()
            if s.sort_interval or s.sparse or s.profile or s.deterministic:
                raise ValueError("sort_interval, sparse, profile and deterministic are per-Solver features; "
                                 "not in a batch")
        if len({s.fused for s in self.solvers}) != 1:
            raise ValueError("all scenes of a batch must share the fused setting")
        self.lib = _abi.load()
        n = len(self.solvers)
        hs = (C.c_void_p * n)(*[s._eng.h.value for s in self.solvers])
        b = C.c_void_p()
        _abi.check(self.lib.gbmpm_batch_create(hs, n, C.byref(b)), "gbmpm_batch_create")
        self.h = b
        self.use_graph = True

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gbmpm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.solvers)

    def step(self, dt: float, substeps: int = 1) -> BatchSolver:
        n = len(self.solvers)
        stream = self.solvers[0]._stream()
        if any(s._tick % max(1, s.guard_interval) == 0 for s in self.solvers):
            out = (C.c_float * (7 * n))()
            st = (C.c_uint32 * n)()
            _abi.check(self.lib.gbmpm_batch_guard(self.h, out, st, stream), "gbmpm_batch_guard")
            for i, s in enumerate(self.solvers):
                if s._tick % max(1, s.guard_interval) == 0:
                    s._check_guard(list(out[7 * i:7 * i + 7]), int(st[i]))
        for s in self.solvers:
            s._pull_colliders()
            if s._sdf_guard:
                s._sdf_tunnel_check(dt)
            s._sync_engine()
        flags = self.solvers[0]._tick_flags()
        if not self.use_graph:
            flags &= ~_abi.TICK_GRAPH
        times = (C.c_double * n)(*[s._time for s in self.solvers])
        _abi.check(self.lib.gbmpm_batch_tick(self.h, times, float(dt), int(substeps), flags, stream),
                   "gbmpm_batch_tick")
        if flags & _abi.TICK_GRAPH and self.lib.gbmpm_batch_graph_state(self.h) < 0:
            self.use_graph = False   # the capture failed; the engine ran this tick live
        for i, s in enumerate(self.solvers):
            s._time = times[i]
            s._step += substeps
            s._tick += 1
        return self

    def launch_count(self) -> int:
        return int(self.lib.gbmpm_batch_launch_count(self.h))

    def autotune(self, dt: float, substeps: int, ticks: int = 2, use_cache: bool = True) -> dict:
        """Picks the fastest launch shape for these scenes (mpm_engine_gb300.autotune):
        every candidate is timed on the scenes' own state, which is restored after."""
        from .autotune import tune_batch
        return tune_batch(self, dt, substeps, ticks=ticks, use_cache=use_cache)

    @property
    def tuning(self) -> dict:
        """The launch shape in use: single-launch schedule, particles per CTA,
        resident CTAs per SM, grid CTAs per SM."""
        from .autotune import batch_tuning
        return batch_tuning(self)

    def set_tuning(self, single_launch: bool = True, tile_threads: int = 128, tile_occ: int = 3,
                   grid_ctas_per_sm: int = 2) -> BatchSolver:
        from .autotune import set_batch_tuning
        set_batch_tuning(self, (int(single_launch), tile_threads, tile_occ, grid_ctas_per_sm))
        return self
