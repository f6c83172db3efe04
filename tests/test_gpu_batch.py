"""Batched scenes: a BatchSolver advances independent scenes in one CUDA graph with
one branch per scene. Each scene must evolve as it does when stepped alone, and
match the oracle."""
import numpy as np
import pytest

from scenes_lib import blob_scene

pytestmark = pytest.mark.gpu


def _scenes(Solver):
    out = []
    for key, n, ng in (("newtonian", 1500, 32), ("jelly", 3000, 48), ("metal", 800, 40), ("mu_i", 2200, 48)):
        s, _ = blob_scene(Solver, key, n_grid=ng, n=n, v0=True)
        out.append(s)
    return out


def test_batch_equals_scenes_stepped_alone(cuda):
    from mpm_engine_gb300 import BatchSolver, Solver
    alone = _scenes(Solver)
    batched = _scenes(Solver)
    b = BatchSolver(batched)
    for _ in range(3):
        for s in alone:
            s.step(2.0e-4, 6)
        b.step(2.0e-4, 6)
    # two GPU runs of one scene differ only in float atomic order: 18 substeps
    # of at most 1e-5 relative each, measured against the field's largest value
    for a, s in zip(alone, batched):
        for got, want in ((s.x(), a.x()), (s.v(), a.v())):
            assert np.abs(got - want).max() <= 18e-5 * np.abs(want).max()
        assert s.time == pytest.approx(a.time)


def test_batch_scene_matches_oracle(cuda, oracle_lib):
    from mpm_engine_gb300 import BatchSolver, Solver
    from test_gpu_parity import assert_close
    scenes = _scenes(Solver)
    oracles = [oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim)
               for s in scenes[:2]]
    b = BatchSolver(scenes)
    for _ in range(2):
        b.step(2.0e-4, 5)
        for o in oracles:
            o.step(2.0e-4, 5)
    for s, o in zip(scenes[:2], oracles):
        assert_close(s, o, 1e-5, "batched scene")


def test_batch_serial_path_and_guard(cuda):
    from mpm_engine_gb300 import BatchSolver, Solver
    scenes = _scenes(Solver)
    b = BatchSolver(scenes)
    b.use_graph = False
    b.step(2.0e-4, 4)
    assert all(np.isfinite(s.x()).all() for s in scenes)
    x = scenes[1].x()
    x[0] = (0.001, 0.2, 0.2)
    scenes[1].set_x(x)
    with pytest.raises(RuntimeError, match="out of bounds"):
        b.step(2.0e-4, 1)


def test_batch_squeeze_workload_runs(cuda):
    from mpm_engine_gb300 import BatchSolver, Solver
    from mpm_engine_gb300.scenes import squeeze_batch_specs, squeeze_from_spec
    specs = squeeze_batch_specs(6, seed=1)
    for sp in specs:
        sp["n_particles"] = min(sp["n_particles"], 20000)
    scenes = [squeeze_from_spec(Solver, sp)[0] for sp in specs]
    b = BatchSolver(scenes)
    for _ in range(2):
        b.step(1.0e-5, 50)
    for s in scenes:
        assert np.isfinite(s.x()).all()


def test_batch_capture_failure_falls_back_to_live_launches(cuda):
    """As for one scene: the test hook discards the batch's capture as failed, the
    batch keeps stepping live (scene after scene), and the scenes advance as a
    graph batch of the same scenes does, to rounding."""
    from mpm_engine_gb300 import BatchSolver, Solver
    a, b = _scenes(Solver), _scenes(Solver)
    ba, bb = BatchSolver(a), BatchSolver(b)
    ba.lib.gbmpm_batch_debug_fail_next_capture(ba.h)
    for _ in range(4):
        ba.step(2.0e-4, 4)
        bb.step(2.0e-4, 4)
    assert ba.use_graph is False and ba.lib.gbmpm_batch_graph_state(ba.h) == -1
    assert bb.lib.gbmpm_batch_graph_state(bb.h) == 1
    for sa, sb in zip(a, b):
        np.testing.assert_allclose(sa.x(), sb.x(), rtol=1e-5, atol=1e-6)


SHAPES = [(1, 64, 2, 2), (1, 64, 3, 2), (1, 128, 2, 2), (1, 128, 3, 1), (1, 256, 2, 4), (1, 256, 3, 2)]


@pytest.mark.parametrize("tuning", SHAPES)
def test_single_launch_shapes_match_oracle(cuda, oracle_lib, tuning):
    """The single-launch schedule: every particle pass and every grid pass is one
    launch over all four scenes (different grids, particle counts and laws), each CTA
    finding its scene and tile in the batch's tables. Every compiled launch shape
    (particles per CTA, resident CTAs per SM, grid CTAs per SM) keeps every scene
    within the parity bound of the oracle (1e-5 per substep, composed)."""
    from mpm_engine_gb300 import BatchSolver, Solver
    from test_gpu_parity import assert_close
    scenes = _scenes(Solver)
    oracles = [oracle_lib.OracleSolver.from_state(s.export_state(), s.grid.n_grid, s.grid.grid_lim) for s in scenes]
    b = BatchSolver(scenes).set_tuning(*tuning)
    for _ in range(2):
        b.step(2.0e-4, 5)
        for o in oracles:
            o.step(2.0e-4, 5)
    tun = b.tuning
    assert tun["last_graph_single_launch"] and tun["tile_threads"] == tuning[1]
    for s, o in zip(scenes, oracles):
        assert_close(s, o, 10 * 1e-5, f"single-launch batch {tuning}")


def test_single_launch_equals_branch_schedule_and_counts_launches(cuda):
    """The same scenes under the single-launch schedule and under one graph branch
    per scene agree to float-atomic rounding; the single-launch tick issues two
    launches per substep for all scenes instead of two per scene."""
    from mpm_engine_gb300 import BatchSolver, Solver
    a, c = _scenes(Solver), _scenes(Solver)
    ba = BatchSolver(a).set_tuning(single_launch=True)
    bc = BatchSolver(c).set_tuning(single_launch=False)
    for _ in range(3):
        ba.step(2.0e-4, 6)
        bc.step(2.0e-4, 6)
    assert ba.tuning["last_graph_single_launch"] and not bc.tuning["last_graph_single_launch"]
    for sa, sc in zip(a, c):
        assert np.abs(sa.x() - sc.x()).max() <= 18e-5 * np.abs(sc.x()).max()
        assert np.abs(sa.v() - sc.v()).max() <= 18e-5 * np.abs(sc.v()).max()
    n0, m0 = ba.launch_count(), bc.launch_count()
    ba.step(2.0e-4, 6)
    bc.step(2.0e-4, 6)
    single, branch = ba.launch_count() - n0, bc.launch_count() - m0
    # both sort and scatter each scene's working set; the substeps' 2 x 6 passes and
    # the closing G2P are issued once instead of once per scene
    assert branch - single == (len(a) - 1) * (2 * 6 + 1), (single, branch)


def test_batch_with_modifiers_takes_the_branch_schedule(cuda):
    """A scene with particle modifiers adds launches between the passes, so the batch
    falls back to one branch per scene and still advances every scene as it would
    alone."""
    from mpm_engine_gb300 import BatchSolver, Solver
    alone, batched = _scenes(Solver), _scenes(Solver)
    for group in (alone, batched):
        group[0].add_impulse_on_particles((0.0, 0.0, 1.0e-4), 2.0e-4, point=(0.1, 0.1, 0.1), size=(0.2, 0.2, 0.2))
    b = BatchSolver(batched)
    for _ in range(2):
        for s in alone:
            s.step(2.0e-4, 5)
        b.step(2.0e-4, 5)
    assert not b.tuning["last_graph_single_launch"]
    for a, s in zip(alone, batched):
        assert np.abs(s.x() - a.x()).max() <= 10e-5 * np.abs(a.x()).max()


def test_autotune_keeps_state_picks_a_candidate_and_caches(cuda, tmp_path, monkeypatch):
    """The autotuner times each candidate launch shape on the batch's own scenes,
    restores the scenes to their state before the search, keeps the fastest and
    caches it: a second batch of the same kind reads the choice from the cache."""
    from mpm_engine_gb300 import BatchSolver, Solver, autotune
    monkeypatch.setenv("GBMPM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_memory", {})
    scenes, ref = _scenes(Solver), _scenes(Solver)
    x0 = [s.x().copy() for s in scenes]
    b = BatchSolver(scenes)
    cands = [(1, 128, 3, 2), (1, 64, 2, 2), (0, 128, 3, 2)]
    res = autotune.tune_batch(b, 2.0e-4, 5, ticks=1, candidates=cands)
    assert not res["cached"] and tuple(res["tuning"]) in cands and len(res["ms_per_tick"]) == 3
    for s, x in zip(scenes, x0):
        np.testing.assert_array_equal(s.x(), x)
    t = b.tuning
    assert (int(t["single_launch"]), t["tile_threads"], t["tile_occ"], t["grid_ctas_per_sm"]) == tuple(res["tuning"])
    # the tuned batch steps as an untuned one does, to rounding
    rb = BatchSolver(ref)
    b.step(2.0e-4, 5)
    rb.step(2.0e-4, 5)
    for s, r in zip(scenes, ref):
        assert np.abs(s.x() - r.x()).max() <= 5e-5 * np.abs(r.x()).max()
    assert (tmp_path / "tune.json").exists()
    monkeypatch.setattr(autotune, "_memory", {})
    again = autotune.tune_batch(BatchSolver(_scenes(Solver)), 2.0e-4, 5, ticks=1, candidates=cands)
    assert again["cached"] and again["tuning"] == res["tuning"]


def test_solver_autotune(cuda, tmp_path, monkeypatch):
    from mpm_engine_gb300 import Solver, autotune
    monkeypatch.setenv("GBMPM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_memory", {})
    s = _scenes(Solver)[0]
    x0 = s.x().copy()
    res = s.autotune(2.0e-4, 5, ticks=1)
    assert tuple(res["tuning"]) in autotune.SOLVER_CANDIDATES
    np.testing.assert_array_equal(s.x(), x0)
    assert autotune.solver_tuning(s)["tile_occ"] == res["tuning"][0]
