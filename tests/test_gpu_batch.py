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
