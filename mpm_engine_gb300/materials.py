"""Physics-named material descriptions and their mapping to engine material ids.

Same public surface as warpmpm.materials (src/warpmpm/materials/__init__.py:27-166):
a frozen `Material` composed with `with_*` modifiers and factories `newtonian`,
`granular`, `elastic`, `vonmises`, `tabulated_viscous`. `resolve()` returns the
engine material name and the parameter dict that `Solver.set_material` applies;
the mapping (names, keys, defaults, validation messages) follows the reference
so scripts written against it run unchanged.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass
from typing import Any

# material ids are pinned by the reference (kernels/mpm_solver_warp.py:14-19)
MATERIAL_IDS = {
    "jelly": 0, "metal": 1, "sand": 2, "plasticine": 5, "fluid": 6, "stationary": 7,
    "rigid": 8, "mu_i_sand": 9, "newtonian": 10, "mu_i_phi": 11, "tabulated_viscous": 12,
    "tabulated_mu_i": 13,
}


def material_id(name) -> int:
    if isinstance(name, int):
        return name
    if name not in MATERIAL_IDS:
        raise TypeError(f"Undefined material type: {name}")
    return MATERIAL_IDS[name]


@dataclass(frozen=True)
class Material:
    base: str
    E: float = 1.0e5
    nu: float = 0.3
    density: float = 1000.0
    bulk_modulus: float = 9.0e5
    viscosity: float = 0.0
    yield_stress: float = 0.0
    powerlaw_K: float = 0.0
    powerlaw_n: float = 1.0
    hardening_xi: float = 0.0
    mu_s: float = 0.0
    delta_mu: float = 0.0
    I0: float = 0.3
    grain_diameter: float = 1.0e-3
    grain_density: float = 2650.0
    dilatant: bool = False
    phi_init: float = 0.6
    phi_chi: float = 0.2
    eta_table: Any = None
    eta_smin: float = -1.0
    eta_smax: float = 2.0

    # composition: each returns a new frozen Material
    def with_viscosity(self, eta: float) -> Material:
        return dataclasses.replace(self, viscosity=eta)

    def with_yield(self, tau_y: float) -> Material:
        return dataclasses.replace(self, yield_stress=tau_y)

    def with_powerlaw(self, K: float, n: float) -> Material:
        return dataclasses.replace(self, powerlaw_K=K, powerlaw_n=n)

    def with_friction(self, mu_s: float, delta_mu: float = 0.0, I0: float = 0.3) -> Material:
        return dataclasses.replace(self, mu_s=mu_s, delta_mu=delta_mu, I0=I0)

    def with_dilatancy(self, phi_init: float = 0.6, chi: float = 0.2) -> Material:
        return dataclasses.replace(self, dilatant=True, phi_init=phi_init, phi_chi=chi)

    def with_density(self, rho: float) -> Material:
        return dataclasses.replace(self, density=rho)

    def resolve(self) -> tuple[str, dict[str, float]]:
        """Engine material name and parameters. Herschel-Bulkley K and n travel in
        the per-type `hardening` / `softening` slots of the newtonian law."""
        b = self.base
        if b == "newtonian":
            return "newtonian", {
                "E": self.E, "nu": self.nu, "density": self.density, "bulk_modulus": self.bulk_modulus,
                "plastic_viscosity": self.viscosity, "yield_stress": self.yield_stress,
                "hardening": self.powerlaw_K, "softening": self.powerlaw_n,
            }
        if b == "granular":
            out = {"E": self.E, "nu": self.nu, "density": self.density, "mu_s": self.mu_s,
                   "delta_mu": self.delta_mu, "I0": self.I0, "grain_diameter": self.grain_diameter,
                   "grain_density": self.grain_density}
            if self.dilatant:
                out["phi_init"] = self.phi_init
                out["phi_chi"] = self.phi_chi
                return "mu_i_phi", out
            return "mu_i_sand", out
        if b == "elastic":
            return "jelly", {"E": self.E, "nu": self.nu, "density": self.density}
        if b == "vonmises":
            # the yield update is gated on the hardening flag, so the flag follows xi
            return "metal", {"E": self.E, "nu": self.nu, "density": self.density,
                             "yield_stress": self.yield_stress, "xi": self.hardening_xi,
                             "hardening": 0.0 if self.hardening_xi == 0.0 else 1.0}
        if b == "tabulated":
            if self.eta_table is None:
                raise ValueError("tabulated material needs eta_table")
            tab = [float(t) for t in self.eta_table]
            if len(tab) < 2:
                raise ValueError("eta_table needs at least 2 samples")
            if any(not math.isfinite(t) for t in tab):
                raise ValueError("eta_table contains non-finite values")
            if min(tab) < 0.0:
                raise ValueError("eta_table viscosities must be nonnegative")
            ok = math.isfinite(self.eta_smin) and math.isfinite(self.eta_smax) and self.eta_smax > self.eta_smin
            if not ok:
                raise ValueError("tabulated material needs smax > smin (finite)")
            return "tabulated_viscous", {"E": self.E, "nu": self.nu, "density": self.density,
                                         "bulk_modulus": self.bulk_modulus, "eta_table": tab,
                                         "eta_table_smin": self.eta_smin, "eta_table_smax": self.eta_smax}
        raise ValueError(f"unknown material base {b!r}")


def newtonian(eta: float = 0.0, density: float = 1000.0, bulk_modulus: float = 9.0e5,
              E: float = 1.0e5, nu: float = 0.3) -> Material:
    """Weakly compressible generalized-Newtonian fluid; `.with_yield` gives Bingham,
    `.with_powerlaw` Herschel-Bulkley."""
    return Material(base="newtonian", viscosity=eta, density=density, bulk_modulus=bulk_modulus, E=E, nu=nu)


def granular(mu_s: float, delta_mu: float = 0.0, I0: float = 0.3, density: float = 1590.0,
             grain_diameter: float = 1.0e-3, grain_density: float = 2650.0,
             E: float = 1.0e6, nu: float = 0.3) -> Material:
    """Local mu(I) granular rheology; `.with_dilatancy` gives mu(I)-Phi(I)."""
    return Material(base="granular", mu_s=mu_s, delta_mu=delta_mu, I0=I0, density=density,
                    grain_diameter=grain_diameter, grain_density=grain_density, E=E, nu=nu)


def elastic(E: float = 1.0e5, nu: float = 0.3, density: float = 1000.0) -> Material:
    """Fixed-corotated hyperelastic solid."""
    return Material(base="elastic", E=E, nu=nu, density=density)


def vonmises(E: float = 5.0e5, nu: float = 0.3, yield_stress: float = 2.0e3,
             hardening_xi: float = 0.0, density: float = 1000.0) -> Material:
    """von Mises (J2) elasto-plastic solid with optional isotropic hardening."""
    return Material(base="vonmises", E=E, nu=nu, yield_stress=yield_stress,
                    hardening_xi=hardening_xi, density=density)


def tabulated_viscous(eta_table, smin: float = -1.0, smax: float = 2.0,
                      density: float = 1000.0, bulk_modulus: float = 9.0e5) -> Material:
    """Fluid whose apparent viscosity eta_app(gd) is a table on log10(gd) in [smin, smax]."""
    return Material(base="tabulated", eta_table=eta_table, eta_smin=smin, eta_smax=smax,
                    density=density, bulk_modulus=bulk_modulus)


__all__ = ["MATERIAL_IDS", "Material", "elastic", "granular", "material_id", "newtonian",
           "tabulated_viscous", "vonmises"]
