"""The in-place block sort on the CUDA engine (tests/test_particle_sort.py:16-103,
restated). The permutation is an exact multiset of particle rows, and per-particle
material parameters stay attached to their particles. Buffers keep their
addresses. Trajectories with a sort every 2 ticks match unsorted ones up to P2G
summation order, on the fused tick. The permutation itself is checked bit for bit
against the oracle in test_gpu_parity.py and at full size in test_gpu_fullsize.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(sort_interval=0, n=3000, seed=1):
    """Two separated blobs, scrambled, so block keys are far from sorted at load."""
    from mpm_engine_gb300 import GridConfig, Solver, newtonian
    grid = GridConfig(n_grid=48, grid_lim=0.4)
    rng = np.random.default_rng(seed)
    a = rng.random((n // 2, 3), dtype=np.float32) * 0.08 + 0.12
    b = rng.random((n - n // 2, 3), dtype=np.float32) * 0.08 + np.array([0.24, 0.24, 0.12], np.float32)
    pts = np.concatenate([a, b])[rng.permutation(n)].astype(np.float32)
    s = Solver(grid=grid, sort_interval=sort_interval).load_particles(pts, np.full(n, 1.0e-7, np.float32))
    s.set_material(newtonian(eta=2.0, density=1000.0, bulk_modulus=2.0e5))
    s.add_plane((0, 0, 3 * grid.dx), (0, 0, 1), "separate", friction=0.3)
    s.add_domain_walls()
    return s


def _rows(s):
    return np.concatenate([s.x(), s.v(), s.F().reshape(s.n_particles, -1)], axis=1)


def test_sort_is_an_exact_multiset_and_runs_once(cuda):
    s = _scene()
    before = _rows(s)
    assert s._sort_particles() is True
    after = _rows(s)
    np.testing.assert_array_equal(before[np.lexsort(before.T)], after[np.lexsort(after.T)])
    assert s._sort_particles() is False


def test_sort_keeps_material_parameters_attached(cuda):
    import torch
    s = _scene(n=600)
    n = s.n_particles
    m = s._sim.mpm_model
    for name, lo, hi in (("mu", 10.0, 20.0), ("lam", 30.0, 50.0), ("yield_stress", 60.0, 90.0)):
        s._t[name].copy_(torch.from_numpy(np.linspace(lo, hi, n, dtype=np.float32)))
    cols = lambda: np.column_stack([s.x(), m.mu.numpy(), m.lam.numpy(), m.yield_stress.numpy()])  # noqa: E731
    before = cols()
    ptrs = (m.mu.ptr, m.lam.ptr, m.yield_stress.ptr)
    assert s._sort_particles() is True
    after = cols()
    np.testing.assert_array_equal(before[np.lexsort(before[:, :3].T)], after[np.lexsort(after[:, :3].T)])
    assert (m.mu.ptr, m.lam.ptr, m.yield_stress.ptr) == ptrs


def test_sorted_run_keeps_pointers_and_matches_unsorted(cuda):
    ref, srt = _scene(sort_interval=0), _scene(sort_interval=2)
    st = srt._sim.mpm_state
    ptrs = (st.particle_x.ptr, st.particle_F.ptr)
    for _ in range(8):
        ref.step(2.0e-4, 6)
        srt.step(2.0e-4, 6)
    assert (st.particle_x.ptr, st.particle_F.ptr) == ptrs, "the sort replaced a buffer"
    xr, xs = ref.x(), srt.x()
    assert np.isfinite(xs).all()
    np.testing.assert_allclose(xs.sum(0), xr.sum(0), rtol=1e-5)
    np.testing.assert_allclose(srt.v().sum(0), ref.v().sum(0), rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(xs[np.lexsort(xs.T)], xr[np.lexsort(xr.T)], rtol=1e-4, atol=1e-6)
