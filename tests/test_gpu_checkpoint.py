"""Checkpoint and resume: Solver.state_dict / load_state_dict.

Stepping from a restored state must repeat the run that followed the checkpoint.
Two GPU runs agree to float-atomic rounding, not bit for bit. Buffers keep their
addresses, so the captured tick graph stays in use. Checkpoints of another scene
and CPIC scenes are refused."""
import numpy as np
import pytest

from scenes_lib import blob_scene, rigid_scene
from test_gpu_parity import rel_err

pytestmark = pytest.mark.gpu


def test_rewind_repeats_the_run(cuda):
    """A thrown von Mises blob in a moving cup, sorted every 3 ticks: checkpoint after
    6 ticks, run 4 more, rewind, run the same 4 again."""
    from mpm_engine_gb300 import Solver
    s, h = blob_scene(Solver, "metal", cup=True, v0=True, sort_interval=3)
    dt, sub = 2.0e-4, 5
    for _ in range(6):
        s.step(dt, sub)
    sd = s.state_dict()
    ptr = s.x_torch().data_ptr()
    first = []
    for _ in range(4):
        s.step(dt, sub)
        first.append((s.x().copy(), s.v().copy(), s.F().copy()))
    s.load_state_dict(sd)
    assert s._tick == 6 and s.x_torch().data_ptr() == ptr
    np.testing.assert_array_equal(s.x(), sd["particles"]["x"].cpu().numpy())
    # the tick-6 sort permuted the particles and their initial volumes; both are back
    np.testing.assert_array_equal(s._t["vol"].cpu().numpy(), s._vol0)
    for t in range(4):
        s.step(dt, sub)
        x, v, F = first[t]
        k = sub * (t + 1)
        assert rel_err(s.x(), x, 1e-6) < k * 1e-5
        assert rel_err(s.v(), v, 1e-6) < k * 1e-5
        assert rel_err(s.F(), F, 1e-6) < k * 1e-5
    assert s._sim._graph_A is not None


def test_rigid_body_state_is_restored(cuda):
    from mpm_engine_gb300 import Solver
    s, _ = rigid_scene(Solver, water=True)
    dt, sub = 1.0e-4, 10
    for _ in range(3):
        s.step(dt, sub)
    sd = s.state_dict()
    for _ in range(3):
        s.step(dt, sub)
    a = s.rigid_state(0)
    s.load_state_dict(sd)
    for _ in range(3):
        s.step(dt, sub)
    b = s.rigid_state(0)
    for key in ("com", "v", "R"):
        np.testing.assert_allclose(b[key], a[key], rtol=1e-4, atol=1e-6)


def test_checkpoint_of_another_scene_and_cdf_scenes_are_refused(cuda):
    from mpm_engine_gb300 import Solver
    from mpm_engine_gb300.geometry import sheet_cdf
    from scenes_lib import cdf_solver, cdf_water
    a, _ = blob_scene(Solver, "jelly", n=2000)
    b, _ = blob_scene(Solver, "jelly", n=1500)
    with pytest.raises(ValueError, match="another scene"):
        b.load_state_dict(a.state_dict())
    c = cdf_solver(Solver, cdf_water(0.14, 0.26, 0.14, 0.26, 0.21, 0.25))
    c.add_cdf_collider(sheet_cdf("z"), center=(0.2, 0.2, 0.20))
    with pytest.raises(NotImplementedError, match="CDF"):
        c.load_state_dict(c.state_dict())
