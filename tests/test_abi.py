"""The C-ABI boundary without a GPU: the library builds, loads, exports every entry
point include/gbmpm.h declares, and the ctypes records match the C layout."""
import ctypes as C
import re
from pathlib import Path

import pytest

from mpm_engine_gb300 import _abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "gbmpm.h"


def header_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(gbmpm_\w+)\s*\(", text, re.M)))


def test_header_and_ctypes_declare_the_same_entry_points():
    assert header_symbols() == sorted(_abi.declared_symbols())


def test_library_exports_every_declared_symbol(native_built):
    lib = C.CDLL(str(native_built))
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_ctypes_records_match_c_layout(oracle_lib):
    want = oracle_lib.abi_layout()
    got = [C.sizeof(_abi.Particles), C.sizeof(_abi.Grid), C.sizeof(_abi.Model), C.sizeof(_abi.Collider),
           _abi.Model.eta_table.offset, _abi.Model.eta_table_smax.offset, _abi.Collider.sdf_val.offset,
           _abi.Collider.rot64.offset, _abi.Particles.init_cov.offset, _abi.Model.material_mask.offset]
    assert got == want


def test_error_mapping_without_gpu(native_built):
    lib = _abi.load()
    # every entry point rejects a NULL engine with GBMPM_ERR_ARG, no CUDA call made
    assert lib.gbmpm_bind(None, None, None) == _abi.ERR_ARG
    assert lib.gbmpm_tick(None, None, 1e-4, 1, 0, None) == _abi.ERR_ARG
    with pytest.raises(ValueError):
        _abi.check(_abi.ERR_ARG, "x")
    with pytest.raises(NotImplementedError):
        _abi.check(_abi.ERR_UNSUPPORTED, "x")
    with pytest.raises(RuntimeError):
        _abi.check(_abi.ERR_CUDA, "x")


def test_solver_refuses_cpu_device():
    import numpy as np
    from mpm_engine_gb300 import Solver
    s = Solver(device="cpu")
    with pytest.raises(RuntimeError, match="CUDA"):
        s.load_particles(np.zeros((4, 3), np.float32), np.ones(4, np.float32))
