"""GB300-native MLS/APIC material-point engine, a drop-in for warpmpm's Solver.

    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    s = Solver(grid=GridConfig(n_grid=64, grid_lim=0.4)).load_particles(pos, vol)
    s.set_material(newtonian(eta=10.0)).add_plane((0, 0, 0.02), (0, 0, 1), "sticky")
    s.step(1e-4, 100)

The substep runs in libgbmpm.so (hand-written sm_103a CUDA kernels) through the
C ABI in include/gbmpm.h; build it with mpm_engine_gb300.build.build_native().
"""
from __future__ import annotations

from .geometry import SDFData, analytic_sdf, load_sdf, save_sdf
from .glass import GlassProfile, cup_fill, glass_sdf_local, quat_from_axis_angle, quat_mul, quat_to_mat
from .materials import Material, elastic, granular, newtonian, tabulated_viscous, vonmises
from .scenes import block, dam_break_lattice, dough
from .solver import BatchSolver, GridConfig, Solver

__version__ = "0.1.0"
__all__ = [
    "BatchSolver", "GlassProfile", "GridConfig", "Material", "SDFData", "Solver", "__version__", "analytic_sdf", "block",
    "cup_fill", "dam_break_lattice", "dough", "elastic", "glass_sdf_local", "granular", "load_sdf", "newtonian",
    "quat_from_axis_angle", "quat_mul", "quat_to_mat", "save_sdf", "tabulated_viscous", "vonmises",
]
