"""Bounded waits give up cleanly (no fault, no hang) and the context survives.

The fused Cholesky's work items wait, bounded, on tile counters written by
other thread blocks.  RSCHOL_WAIT_LIMIT sets the number of polls before such
a wait gives up; the test switch RSCHOL_TEST_DROP_CHOL_ITEM=1 plans one
POTRF item out of the schedule, so the TRSM items that need it wait on a
counter that nothing sets.  The factorisation must return RSCHOL_E_TIMEOUT,
and the same context must then factor and solve the system normally.
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs

pytestmark = pytest.mark.gpu

PARAMS = dict(max_dense_block=30, max_diag_block=60, nd_leaf=16)


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_unmet_dependency_times_out_and_context_recovers(precision, monkeypatch):
    prob = rs.diffusion(3, 16, sigma=1.0, seed=1)
    ctx = rs.Context(**PARAMS, precision=precision)
    monkeypatch.setenv("RSCHOL_WAIT_LIMIT", "256")
    monkeypatch.setenv("RSCHOL_TEST_DROP_CHOL_ITEM", "1")
    with pytest.raises(rs.RscholError) as e:
        rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    assert e.value.status == 6, str(e.value)   # RSCHOL_E_TIMEOUT
    assert "bounded wait" in ctx.last_error()
    monkeypatch.delenv("RSCHOL_TEST_DROP_CHOL_ITEM")
    monkeypatch.delenv("RSCHOL_WAIT_LIMIT")
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    x, info = G.pcg(prob.rhs[0], 1e-8, 500)
    assert info["true_residual"] <= 1e-8
    A = prob.scipy()
    assert np.linalg.norm(prob.rhs[0] - A @ x) / np.linalg.norm(prob.rhs[0]) <= 1e-8
