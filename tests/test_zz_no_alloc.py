"""The allocation-free preconditioner apply against the allocating one.

rschol_precond_apply_device_noalloc runs the same single-vector kernels on
the same factor as rschol_precond_apply_device called with one right-hand
side; only the permuted work vector differs (a static device array instead
of a buffer allocated on first use).  Two calls in a row, both precisions,
two right-hand sides per no-alloc call.  The device's free memory is the
same before and after the first no-alloc call of a fresh context: the
static array's address is looked up when the context is created, so the
call itself loads and allocates nothing.
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs

pytestmark = pytest.mark.gpu

TOL = 1e-12   # relative, per right-hand side


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_noalloc_apply_matches_device_apply(precision):
    torch = pytest.importorskip("torch")
    lib = rs.load_library()
    prob = rs.diffusion(3, 16, sigma=1.0, seed=1, nrhs=2)
    ctx = rs.Context(max_dense_block=30, max_diag_block=60, nd_leaf=16, precision=precision)
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    n = prob.n
    assert n <= 2097152
    b = torch.tensor(np.stack(prob.rhs), dtype=torch.float64, device="cuda")
    x_warm = torch.zeros_like(b)
    x_first = torch.zeros_like(b)
    torch.cuda.synchronize()
    # the single-vector kernels are loaded by one allocating apply first
    assert lib.rschol_precond_apply_device(G.h, b[0].data_ptr(), x_warm[0].data_ptr(), 1) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert lib.rschol_precond_apply_device_noalloc(G.h, b.data_ptr(), x_first.data_ptr(), 2) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    for _ in range(2):
        x_ref = torch.zeros_like(b)
        x_na = torch.full_like(b, float("nan"))
        torch.cuda.synchronize()   # the library works on its own stream
        for k in range(2):   # one right-hand side per call: the same single-vector kernels
            assert lib.rschol_precond_apply_device(G.h, b[k].data_ptr(), x_ref[k].data_ptr(), 1) == 0
        assert lib.rschol_precond_apply_device_noalloc(G.h, b.data_ptr(), x_na.data_ptr(), 2) == 0
        ref, got = x_ref.cpu().numpy(), x_na.cpu().numpy()
        assert np.all(np.isfinite(got))
        for k in range(2):
            assert np.linalg.norm(got[k] - ref[k]) <= TOL * np.linalg.norm(ref[k])
        # and it is the preconditioner: compare with the host entry point
        host = G.apply(prob.rhs[0])
        assert np.linalg.norm(got[0] - host) <= TOL * np.linalg.norm(host)
