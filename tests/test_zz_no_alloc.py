"""gbmpm_guard_noalloc: the edge-guard reduction for callers that cannot allocate.

Some callers of this engine cannot call cudaMalloc: a process whose device memory
is entirely owned by another allocator, or a control loop that must not take
cudaMalloc's implicit device synchronization between ticks. This entry point
computes the same guard numbers as gbmpm_guard with its scratch in a static
device array instead of engine-allocated memory. The test calls both through the
C ABI on the same particles, twice in a row (the second time on moved particles),
and requires identical results: a min/max reduction has no rounding, so the
tolerance is exact equality.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _guard_engine(lib, torch, x, v):
    """gbmpm_guard through an engine bound to the same device arrays."""
    from mpm_engine_gb300 import _abi
    n = x.shape[0]
    dev = x.device
    keep = {k: torch.zeros(n, 9, device=dev) for k in ("C", "F", "Ft", "L", "S")}
    keep.update({k: torch.zeros(n, device=dev) for k in ("m", "vol", "Jp", "mu", "lam", "ys")})
    keep["mat"] = torch.zeros(n, dtype=torch.int32, device=dev)
    keep["mv"] = torch.zeros(16 ** 3, 4, device=dev)
    keep["gv"] = torch.zeros(16 ** 3, 4, device=dev)
    p = _abi.Particles(n=n, x=x.data_ptr(), v=v.data_ptr(), C=keep["C"].data_ptr(), F=keep["F"].data_ptr(),
                       F_trial=keep["Ft"].data_ptr(), L=keep["L"].data_ptr(), stress=keep["S"].data_ptr(),
                       mass=keep["m"].data_ptr(), vol=keep["vol"].data_ptr(), Jp=keep["Jp"].data_ptr(),
                       mu=keep["mu"].data_ptr(), lam=keep["lam"].data_ptr(), yield_stress=keep["ys"].data_ptr(),
                       material=keep["mat"].data_ptr())
    g = _abi.Grid(n_grid=16, mv=keep["mv"].data_ptr(), v=keep["gv"].data_ptr())
    eng = C.c_void_p()
    _abi.check(lib.gbmpm_engine_create(C.byref(eng)))
    _abi.check(lib.gbmpm_bind(eng, C.byref(p), C.byref(g)))
    out = (C.c_float * 7)()
    st = C.c_uint32(0)
    _abi.check(lib.gbmpm_guard(eng, out, C.byref(st), None))
    lib.gbmpm_engine_destroy(eng)
    return np.array(out[:], np.float32), int(st.value & _abi.FLAG_NONFINITE != 0)


def _guard_noalloc(lib, x, v):
    from mpm_engine_gb300 import _abi
    out = (C.c_float * 7)()
    bad = C.c_int32(-1)
    _abi.check(lib.gbmpm_guard_noalloc(x.data_ptr(), v.data_ptr(), x.shape[0], out, C.byref(bad), None))
    return np.array(out[:], np.float32), int(bad.value)


def test_noalloc_guard_matches_engine_guard_twice(cuda):
    torch = cuda
    from mpm_engine_gb300 import _abi
    lib = _abi.load()
    rng = np.random.default_rng(5)
    n = 300_001  # several partial blocks plus a ragged tail
    x = torch.from_numpy(rng.uniform(0.02, 0.38, size=(n, 3)).astype(np.float32)).cuda()
    v = torch.from_numpy(rng.normal(0.0, 0.5, size=(n, 3)).astype(np.float32)).cuda()
    for call in range(2):
        got, bad = _guard_noalloc(lib, x, v)
        want, want_bad = _guard_engine(lib, torch, x, v)
        np.testing.assert_array_equal(got, want)
        assert bad == want_bad == 0
        np.testing.assert_allclose(got[:3], x.min(0).values.cpu().numpy())
        np.testing.assert_allclose(got[3:6], x.max(0).values.cpu().numpy())
        x[n // 2, 1] = 0.001 * (call + 1)     # moved particles: the second call must not return stale results
        v[7, 2] = 9.0 + call
    x[3, 0] = float("nan")
    got, bad = _guard_noalloc(lib, x, v)
    assert bad == 1


def test_noalloc_guard_rejects_oversize(cuda):
    from mpm_engine_gb300 import _abi
    lib = _abi.load()
    out = (C.c_float * 7)()
    rc = lib.gbmpm_guard_noalloc(None, None, 4194305, out, None, None)
    assert rc == _abi.ERR_ARG
    assert b"4194304" in lib.gbmpm_last_error()


def test_noalloc_guard_empty_and_full_size(cuda):
    """n = 0 (only the final fold runs, over no partials) and n at the limit (every
    partial slot of the static array in use)."""
    torch = cuda
    from mpm_engine_gb300 import _abi
    lib = _abi.load()
    out = (C.c_float * 7)()
    bad = C.c_int32(-1)
    _abi.check(lib.gbmpm_guard_noalloc(None, None, 0, out, C.byref(bad), None))
    got = np.array(out[:], np.float32)
    assert np.all(got[:3] == np.inf) and np.all(got[3:6] == -np.inf)
    assert got[6] == 0.0 and bad.value == 0
    n = 4_194_304
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.rand(n, 3, device="cuda", generator=g) * 0.3 + 0.05
    v = torch.randn(n, 3, device="cuda", generator=g)
    x[n - 1] = torch.tensor([0.01, 0.39, 0.02], device="cuda")   # extremes in the last slice
    v[n - 1, 1] = -7.5
    for _ in range(2):
        got, bad = _guard_noalloc(lib, x, v)
        want, want_bad = _guard_engine(lib, torch, x, v)
        np.testing.assert_array_equal(got, want)
        assert bad == want_bad == 0
        assert got[6] == 7.5
