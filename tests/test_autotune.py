"""The batched apply's autotuner picks tile shapes only, never arithmetic.

rschol_factor_autotune times candidate shapes for each width class (k rounded
up to a power of two); the candidates differ in which thread forms which
(row, column) sum, not in the order of any sum.  So the tuned factor must
give bitwise the same batched applies as one that keeps the fixed shapes, at
every width.
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs

pytestmark = pytest.mark.gpu

PARAMS = dict(max_dense_block=30, max_diag_block=60, nd_leaf=16)


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_autotuned_shapes_give_identical_results(precision):
    prob = rs.diffusion(3, 14, sigma=1.0, seed=21)
    rng = np.random.default_rng(3)
    factors = {}
    for mode in ("1", "0"):
        factors[mode] = rs.GpuFactor(rs.Context(precision=precision, **PARAMS), prob.colptr, prob.rowind, prob.vals,
                                     prob.xyz)
    factors["1"].autotune(64)
    for k in (2, 3, 8, 16, 40):
        B = rng.standard_normal((k, prob.n))
        x_tuned = factors["1"].apply(B)
        x_fixed = factors["0"].apply(B)
        assert np.all(np.isfinite(x_tuned))
        assert np.array_equal(x_tuned, x_fixed), k
    tuning = factors["1"].describe()["batch_tuning"]
    assert {int(row[0]) for row in tuning} >= {2, 4, 8, 16, 64}
    assert all(row[5] > 0 for row in tuning)                 # every class was timed
    assert all(row[5] == 0 for row in factors["0"].describe()["batch_tuning"])


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_schedule_tuner_leaves_a_working_factor(precision):
    """rschol_factor_tune_schedule times the factor's candidate schedules (tensor-core
    threshold, fused or per-panel blocked Cholesky), keeps the fastest and leaves the
    factor refactored with it: PCG still reaches 1e-8 in the same iteration count +-1."""
    prob = rs.diffusion(3, 16, sigma=1.0, seed=3)
    G = rs.GpuFactor(rs.Context(precision=precision, **PARAMS), prob.colptr, prob.rowind, prob.vals, prob.xyz)
    _, i0 = G.pcg(prob.rhs[0], 1e-8, 500)
    sch = G.tune_schedule(2)
    assert sch["tuned_ms"] > 0 and isinstance(sch["fused"], bool)
    assert sch["tc_min_k"] in ((128, 256, -1) if precision == rs.MIXED else (-1, 128))
    _, i1 = G.pcg(prob.rhs[0], 1e-8, 500)
    assert i1["true_residual"] <= 1e-8 and abs(i1["iterations"] - i0["iterations"]) <= 1
