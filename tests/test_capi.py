"""The C ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import rank_structured_cholesky_gb300 as rs

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rschol_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rschol_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(rs.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(rs.EXPORTED) == names


def test_context_without_device_fails_loudly():
    ctx = rs.Context()
    prob = rs.diffusion(2, 6)
    try:
        rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals)
    except rs.RscholError as e:
        assert e.status in (7, 4)   # no device / CUDA error, never a silent CPU path
    else:
        import pytest
        pytest.skip("a CUDA device is present")


def test_default_params_match_reference_driver():
    p = rs.default_params()
    assert (p.max_dense_block, p.max_diag_block, p.explicit_threshold) == (200, 400, 4000)
    assert (p.oversampling, p.power_iters, p.seed) == (5, 1, 152)
    assert abs(p.rank_constant - 0.4) < 1e-15 and abs(p.diag_rank_constant - 0.5) < 1e-15
    assert p.max_factor_attempts == 10 and abs(p.rank_alpha - 1.25) < 1e-15


def test_bad_input_is_rejected():
    ctx = rs.Context()
    lib = rs.load_library()
    import numpy as np
    cp = np.array([0, 1, 2], np.int32)
    ri = np.array([0, 5], np.int32)   # row index out of range
    v = np.ones(2)
    h = ctypes.c_void_p()
    st = lib.rschol_factor_create(ctx.h, 2, rs._ip(cp), rs._ip(ri), rs._dp(v), None, ctypes.byref(h))
    assert st in (1, 7)
