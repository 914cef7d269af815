"""The CPU oracle (FP64 restatement of the reference path) on small cases.

Pins: exactness without compression, convergence with compression, the
committed oracle fixtures (tests/golden/oracle_*.npz, see make_golden.py),
the identity-basis fallback and the indefinite-diagonal retry policy.
"""
import os

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def make(case):
    from tests.golden import make_golden
    return make_golden.make_problem(make_golden.CASES[case]["problem"]), make_golden.CASES[case]["params"]


@pytest.mark.parametrize("prob", [("d2", 24), ("d3", 10), ("el", 4)])
def test_uncompressed_factor_is_exact(prob):
    kind, size = prob
    p = rs.diffusion(2, size, sigma=1.0) if kind == "d2" else (
        rs.diffusion(3, size, sigma=1.0, seed=1) if kind == "d3" else rs.elasticity(size))
    F = po.OracleFactor(p.colptr, p.rowind, p.vals, p.xyz, dict(max_dense_block=100000, nd_leaf=16))
    assert F.factor() == 0
    assert all(not F.node_info(j)["compressed"] for j in range(F.num_nodes()))
    x, it, rec, true = F.pcg(p.rhs[0], 1e-12, 50)
    assert it == 1 and true < 1e-12
    A = p.scipy()
    np.testing.assert_allclose(A @ F.apply(p.rhs[0]), p.rhs[0], rtol=0, atol=1e-10 * np.abs(p.rhs[0]).max())


@pytest.mark.parametrize("case", ["2d48", "3d16", "3d20h", "el5"])
def test_oracle_matches_golden(case):
    prob, params = make(case)
    g = np.load(os.path.join(GOLDEN, "oracle_%s.npz" % case))
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert F.factor() == 0
    assert np.array_equal(F.perm(), g["perm"])
    x, it, rec, true = F.pcg(prob.rhs[0], 1e-8, 2000)
    assert abs(it - int(g["iterations"])) <= 1
    assert true <= 1e-8
    np.testing.assert_allclose(F.apply(prob.rhs[0]), g["apply"], rtol=1e-9, atol=1e-12)
    for j in g["compressed_nodes"]:
        l11 = F.node_l11(int(j))
        probe = np.random.default_rng(1000 + int(j)).standard_normal(l11.shape[1])
        ref = g["l11p_%d" % j]
        assert np.linalg.norm(l11 @ probe - ref) <= 1e-9 * np.linalg.norm(ref)
        if "l21p_%d" % j in g:
            ref = g["l21p_%d" % j]
            assert np.linalg.norm(F.node_l21(int(j)) @ probe - ref) <= 1e-8 * max(np.linalg.norm(ref), 1e-300)


def test_compressed_factor_is_spd_preconditioner():
    prob, params = make("3d16")
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert F.factor() == 0
    rng = np.random.default_rng(5)
    y, z = rng.standard_normal((2, prob.n))
    # M^{-1} = L^{-T} L^{-1} is symmetric positive definite
    assert abs(y @ F.apply(z) - z @ F.apply(y)) <= 1e-10 * abs(y @ F.apply(z))
    assert y @ F.apply(y) > 0


def test_identity_basis_fallback_is_exact():
    # every compressed separator has at most 16 columns, so each rank equals
    # its column count and the basis is the identity: the factor is exact
    prob = rs.diffusion(2, 20, sigma=1.0)
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz,
                        dict(max_dense_block=4, max_diag_block=64, nd_leaf=4))
    assert F.factor() == 0
    comp = [j for j in range(F.num_nodes()) if F.node_info(j)["compressed"]]
    info = [F.node_info(j) for j in comp]
    assert comp and all(i["m"] == 0 or i["rank"] == i["c1"] - i["c0"] + 1 for i in info)
    x, it, rec, true = F.pcg(prob.rhs[0], 1e-10, 50)
    assert it <= 2 and true < 1e-10


def test_recursive_hodlr_diagonal_runs():
    prob, params = make("3d20h")
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert F.factor() == 0
    hn = [F.node_info(j)["hodlr_nodes"] for j in range(F.num_nodes())]
    assert max(hn) >= 7    # at least one diagonal with >= 4 leaves
    x, it, rec, true = F.pcg(prob.rhs[0], 1e-8, 500)
    assert true <= 1e-8


@pytest.mark.parametrize("compressed", [False, True])
def test_oracle_retry_policy(compressed):
    """Indefinite diagonal of a compressed node: 10 attempts with a growing
    diagonal rank constant; of an uncompressed node: no retry (the
    reference aborts there)."""
    from tests.test_gpu_parity import indefinite_case
    prob, params, vals, node = indefinite_case(compressed)
    O = po.OracleFactor(prob.colptr, prob.rowind, vals, prob.xyz, params)
    assert O.factor() == node + 1
    t = O.times()
    assert t["attempts"] == (10 if compressed else 1)
    if compressed:
        assert abs(t["diag_rank_constant"] - 0.5 * 1.25 ** 10) < 1e-9


@pytest.mark.parametrize("shape,prm", [
    ((2, 40, 37, None), dict(max_dense_block=100, max_diag_block=12, nd_leaf=32)),
    ((2, 40, 37, None), dict(max_dense_block=8, max_diag_block=12, nd_leaf=32)),
    ((3, 12, 11, 10), dict(max_dense_block=400, max_diag_block=16, nd_leaf=48)),
    ((3, 12, 11, 10), dict(max_dense_block=24, max_diag_block=16, nd_leaf=48)),
])
def test_hierarchical_diagonal_on_uncompressed_supernodes(shape, prm):
    """Uncompressed supernodes wider than max_diag_block get a HODLR diagonal,
    factored by the same block-list walk as a compressed supernode's over
    their explicit Schur complement, with their stored rows solved by the
    expanded L11 (the reference factors every diagonal through its
    DiagonalBlock).  Every block explicit and every rank full: the factor is
    exact (one PCG iteration); at the default ranks the PCG converges."""
    d, nx, ny, nz = shape
    p = rs.diffusion(d, nx, ny, nz, sigma=1.0, seed=3)
    exact = po.OracleFactor(p.colptr, p.rowind, p.vals, p.xyz, dict(prm, rank_constant=1e3, diag_rank_constant=1e3))
    assert exact.factor() == 0
    infos = [exact.node_info(j) for j in range(exact.num_nodes())]
    assert sum(1 for i in infos if not i["compressed"] and i["hodlr_nodes"] > 1) > 0
    _, it, _, true = exact.pcg(p.rhs[0], 1e-8, 100)
    assert it == 1 and true < 1e-12, (it, true)
    F = po.OracleFactor(p.colptr, p.rowind, p.vals, p.xyz, prm)
    assert F.factor() == 0
    _, it, _, true = F.pcg(p.rhs[0], 1e-8, 100)
    assert it <= 20 and true <= 1e-8, (it, true)
