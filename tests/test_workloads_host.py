"""The seeded synthetic workloads the benchmark measures (no GPU needed): sizes and
bounds of the dam-break lattice and the granular press heap, and that they are
reproducible from their seeds."""
import numpy as np

from mpm_engine_gb300.scenes import PRESS_GRANULAR, dam_break_lattice, press_heap


def test_dam_break_lattice_is_362250_particles_at_64():
    pos, vol = dam_break_lattice(64, 1.0)
    assert len(pos) == 362250
    h = 0.5 / 64
    assert np.all(vol == np.float32(h ** 3))
    lo, hi = np.array([0.05, 0.05, 0.05]), np.array([0.4, 0.6, 0.95])
    assert np.all(pos >= lo - 0.25 * h) and np.all(pos <= hi + 0.25 * h)


def test_press_heap_size_bounds_and_seed():
    pos, vol, floor = press_heap(256, 1.0, seed=0)
    assert len(pos) == 1978257                     # about 2 M grains at 8 per cell
    dx = 1.0 / 256
    h = dx / 2
    assert floor == 3 * dx
    assert np.all(vol == np.float32(h ** 3))
    assert pos[:, :2].min() > 0.25 - h and pos[:, :2].max() < 0.75 + h
    assert pos[:, 2].min() > floor - 0.25 * h
    assert pos[:, 2].max() < floor + 1.0 * (0.06 + 0.025) + h
    again, _, _ = press_heap(256, 1.0, seed=0)
    np.testing.assert_array_equal(pos, again)
    other, _, _ = press_heap(256, 1.0, seed=1)
    assert len(other) != len(pos) or not np.array_equal(other, pos)
    # the heap's height varies across the footprint: the plate meets the peaks first
    cols = np.round((pos[:, :2] - 0.25) / h).astype(np.int64)
    top = np.zeros((int(cols[:, 0].max()) + 1, int(cols[:, 1].max()) + 1))
    np.maximum.at(top, (cols[:, 0], cols[:, 1]), pos[:, 2])
    assert top.max() - top.min() > 0.02


def test_press_material_is_the_survey_granular():
    assert PRESS_GRANULAR == dict(mu_s=0.38, delta_mu=0.26, I0=0.28, density=2500.0, E=1.0e6, nu=0.3)
