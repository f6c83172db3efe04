"""Launch-shape autotuner for single scenes and batches.

The reference has nothing to tune: Warp picks one launch per kernel. Here the
particle pass comes in several compiled shapes (particles per CTA, resident CTAs
per SM, the SVD laws compiled in or out) and the grid pass can be spread over more
or fewer CTAs per SM, and which is fastest depends on the scene mix: particle
counts, grid sizes and materials. `tune_batch` and `tune_solver` time every
candidate on the caller's own scenes (a few ticks each, from a checkpoint that is
restored afterwards, so the simulation state is unchanged) and keep the fastest.
Choices are cached per bucket of (scene count, total particles, grid sizes,
material class, substeps per tick) in memory and in a JSON file
($GBMPM_AUTOTUNE_CACHE, default ~/.cache/mpm_engine_gb300/autotune.json), so later
runs with the same kind of workload skip the search.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from pathlib import Path

from . import _abi

# (single_launch, tile_threads, tile_occ, grid_ctas)
BATCH_CANDIDATES = [(1, 128, 3, 2), (1, 128, 2, 2), (1, 64, 3, 2), (1, 64, 2, 2), (1, 256, 3, 2), (1, 256, 2, 2),
                    (1, 128, 3, 4), (1, 128, 3, 1), (0, 128, 3, 2)]
# (tile_occ, grid_ctas)
SOLVER_CANDIDATES = [(3, 2), (2, 2), (4, 2), (3, 1), (3, 4)]

_memory: dict = {}


def cache_path() -> Path:
    p = os.environ.get("GBMPM_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "mpm_engine_gb300" / "autotune.json"


def _load_cache() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, value) -> None:
    _memory[key] = value
    data = _load_cache()
    data[key] = value
    try:
        path = cache_path()
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(path)
    except OSError:
        pass   # an unwritable cache only costs a search next time


def _lookup(key: str):
    if key in _memory:
        return _memory[key]
    return _load_cache().get(key)


def _material_class(solver) -> str:
    fluid = (1 << 6) | (1 << 7) | (1 << 8) | (1 << 10) | (1 << 12)
    return "solids" if int(solver._model.material_mask) & ~fluid else "fluids"


def _bucket(n: int) -> int:
    return int(round(math.log2(max(1, n)) * 2))   # half-octave buckets


def batch_key(solvers, substeps: int) -> str:
    grids = sorted({int(s.grid.n_grid) for s in solvers})
    mats = sorted({_material_class(s) for s in solvers})
    total = sum(s.n_particles for s in solvers)
    return (f"batch|scenes={len(solvers)}|particles~{_bucket(total)}|grids={grids[0]}-{grids[-1]}|"
            f"{'+'.join(mats)}|substeps={substeps}")


def solver_key(solver, substeps: int) -> str:
    return (f"solver|particles~{_bucket(solver.n_particles)}|grid={int(solver.grid.n_grid)}|"
            f"{_material_class(solver)}|substeps={substeps}")


def _time_ticks(step, ticks: int) -> float:
    import torch
    step()                                  # capture the graph of this shape
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(ticks):
        step()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / ticks


def set_batch_tuning(batch, tuning) -> None:
    single, th, occ, gc = (int(v) for v in tuning)
    _abi.check(batch.lib.gbmpm_batch_set_tuning(batch.h, single, th, occ, gc), "gbmpm_batch_set_tuning")


def batch_tuning(batch) -> dict:
    out = (C.c_int32 * 5)()
    _abi.check(batch.lib.gbmpm_batch_get_tuning(batch.h, out), "gbmpm_batch_get_tuning")
    return {"single_launch": bool(out[0]), "tile_threads": int(out[1]), "tile_occ": int(out[2]),
            "grid_ctas_per_sm": int(out[3]), "last_graph_single_launch": bool(out[4])}


def tune_batch(batch, dt: float, substeps: int, ticks: int = 2, candidates=None, use_cache: bool = True) -> dict:
    """Times each candidate launch shape on `batch` (a BatchSolver) for `ticks`
    ticks of `substeps` substeps after one warm-up tick, restores every scene to
    its state before the search, and keeps the fastest. Returns
    {"tuning": ..., "ms_per_tick": {candidate: ms}, "cached": bool, "key": ...}."""
    key = batch_key(batch.solvers, substeps)
    if use_cache:
        hit = _lookup(key)
        if hit is not None:
            set_batch_tuning(batch, hit["tuning"])
            return {**hit, "cached": True, "key": key}
    cands = list(candidates or BATCH_CANDIDATES)
    start = [s.state_dict() for s in batch.solvers]
    times = {}
    for cand in cands:
        set_batch_tuning(batch, cand)
        for s, st in zip(batch.solvers, start):
            s.load_state_dict(st)
        times[cand] = _time_ticks(lambda: batch.step(dt, substeps), ticks)
    for s, st in zip(batch.solvers, start):
        s.load_state_dict(st)
    best = min(times, key=times.get)
    set_batch_tuning(batch, best)
    rec = {"tuning": list(best), "ms_per_tick": {",".join(map(str, c)): t for c, t in times.items()}}
    _store(key, rec)
    return {**rec, "cached": False, "key": key}


def set_solver_tuning(solver, tuning) -> None:
    occ, gc = (int(v) for v in tuning)
    _abi.check(solver._eng.lib.gbmpm_set_tuning(solver._eng.h, occ, gc), "gbmpm_set_tuning")


def set_solver_resort(solver, substeps: int) -> None:
    """Substeps between re-sorts of the solver's working copy inside a tick: 0 sorts
    once per tick, _abi.RESORT_AUTO (the default) every max(50, S / 3) substeps of a
    tick of S >= 100 in a scene of 150,000 particles or more. Long ticks keep the
    scatter's runs of one cell long this way."""
    _abi.check(solver._eng.lib.gbmpm_set_resort(solver._eng.h, int(substeps)), "gbmpm_set_resort")


def solver_resort(solver) -> int:
    return int(solver._eng.lib.gbmpm_get_resort(solver._eng.h))


def solver_tuning(solver) -> dict:
    out = (C.c_int32 * 2)()
    _abi.check(solver._eng.lib.gbmpm_get_tuning(solver._eng.h, out), "gbmpm_get_tuning")
    return {"tile_occ": int(out[0]), "grid_ctas_per_sm": int(out[1])}


def tune_solver(solver, dt: float, substeps: int, ticks: int = 2, candidates=None, use_cache: bool = True) -> dict:
    """As tune_batch for one Solver: the tiled particle kernel's occupancy variant
    and the grid pass's CTAs per SM. Scenes with SVD-based laws skip occupancy 4."""
    key = solver_key(solver, substeps)
    if use_cache:
        hit = _lookup(key)
        if hit is not None:
            set_solver_tuning(solver, hit["tuning"])
            return {**hit, "cached": True, "key": key}
    cands = list(candidates or SOLVER_CANDIDATES)
    if _material_class(solver) == "solids":
        cands = [c for c in cands if c[0] <= 3]
    start = solver.state_dict()
    times = {}
    for cand in cands:
        set_solver_tuning(solver, cand)
        solver.load_state_dict(start)
        times[cand] = _time_ticks(lambda: solver.step(dt, substeps), ticks)
    solver.load_state_dict(start)
    best = min(times, key=times.get)
    set_solver_tuning(solver, best)
    rec = {"tuning": list(best), "ms_per_tick": {",".join(map(str, c)): t for c, t in times.items()}}
    _store(key, rec)
    return {**rec, "cached": False, "key": key}


__all__ = ["batch_key", "batch_tuning", "cache_path", "set_batch_tuning", "set_solver_resort", "set_solver_tuning",
           "solver_key", "solver_resort", "solver_tuning", "tune_batch", "tune_solver"]
