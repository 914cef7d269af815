"""GPU parity: the CUDA factor / preconditioner / PCG against the CPU oracle.

Tolerances (FP64 path), relative Frobenius / 2-norm error against the oracle:
  * EXACT_TOL = 1e-11 for blocks no compression touches (interior factor
    panels of supernodes whose interior block has no compressed ancestor
    contribution, i.e. everything below the first compressed separator);
  * COMPRESSED_TOL = 1e-5 for everything a randomized compression feeds
    (L11 of HODLR diagonals, V U^T, and every block assembled from them).
    The sketch Y = (L21^T L21) L21^T G has numerical rank below r; the basis
    columns beyond that rank are fixed by rounding in any QR (LAPACK's
    included), so V U^T = L21 U U^T agrees only up to the neglected singular
    values of L21 (the CPU oracle run once with OpenBLAS and once with plain
    loops differs by 3.1e-6 on the 2d48 case);
  * APPLY_TOL = 1e-7 for one preconditioner application.
PCG reaches ||r||/||b|| <= 1e-8 in the oracle's iteration count +-1.  Mixed
precision (FP32 factor, FP64 PCG) must reach the same 1e-8 residual in the
FP64 oracle's iteration count +-1; its error against the FP64 oracle is
asserted below 1e-3.  Every supernode's blocks are compared.
"""
import os

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

EXACT_TOL = 1e-11
COMPRESSED_TOL = 1e-5
APPLY_TOL = 1e-7


def make(case):
    from tests.golden import make_golden
    return make_golden.make_problem(make_golden.CASES[case]["problem"]), make_golden.CASES[case]["params"]


def gpu_factor(prob, params, **extra):
    ctx = rs.Context(**params, **extra)
    return rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def oracles():
    cache = {}

    def get(case):
        if case not in cache:
            prob, params = make(case)
            F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
            assert F.factor() == 0
            cache[case] = (prob, params, F)
        return cache[case]
    return get


@pytest.mark.parametrize("case", ["2d48", "3d16", "3d20h", "el5"])
def test_factor_blocks_match_oracle(case, oracles):
    prob, params, O = oracles(case)
    G = gpu_factor(prob, params)
    assert G.num_nodes() == O.num_nodes()
    for j in range(G.num_nodes()):
        gi, oi = G.node_info(j), O.node_info(j)
        assert (gi["c0"], gi["c1"], gi["compressed"]) == (oi["c0"], oi["c1"], oi["compressed"])
        tol = COMPRESSED_TOL if gi["compressed"] else EXACT_TOL
        assert rel(G.node_l11(j), O.node_l11(j)) < tol, ("l11", j, gi)
        l21o = O.node_l21(j)
        if l21o.size:
            assert rel(G.node_l21(j), l21o) < tol, ("l21", j, gi)


@pytest.mark.parametrize("case", ["2d48", "3d16", "3d20h", "el5"])
def test_pcg_matches_oracle(case, oracles):
    prob, params, O = oracles(case)
    G = gpu_factor(prob, params)
    b = prob.rhs[0]
    x, info = G.pcg(b, 1e-8, 2000)
    _, it, _, true = O.pcg(b, 1e-8, 2000)
    assert abs(info["iterations"] - it) <= 1, (info, it)
    assert info["true_residual"] <= 1e-8
    A = prob.scipy()
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1e-8
    assert rel(G.apply(b), O.apply(b)) < APPLY_TOL


@pytest.mark.parametrize("case", ["2d48", "3d16", "3d20h", "el5"])
def test_matches_golden_fixture(case):
    prob, params = make(case)
    g = np.load(os.path.join(GOLDEN, "oracle_%s.npz" % case))
    G = gpu_factor(prob, params)
    assert np.array_equal(G.perm(), g["perm"])
    assert rel(G.apply(prob.rhs[0]), g["apply"]) < APPLY_TOL
    for j in g["compressed_nodes"]:
        l11 = G.node_l11(int(j))
        probe = np.random.default_rng(1000 + int(j)).standard_normal(l11.shape[1])
        assert rel(l11 @ probe, g["l11p_%d" % j]) < COMPRESSED_TOL
        if "l21p_%d" % j in g:
            assert rel(G.node_l21(int(j)) @ probe, g["l21p_%d" % j]) < COMPRESSED_TOL
    x, info = G.pcg(prob.rhs[0], 1e-8, 2000)
    assert abs(info["iterations"] - int(g["iterations"])) <= 1


@pytest.mark.parametrize("case", ["3d16", "el5"])
def test_mixed_precision_reaches_fp64_accuracy(case, oracles):
    prob, params, O = oracles(case)
    G = gpu_factor(prob, params, precision=rs.MIXED)
    x, info = G.pcg(prob.rhs[0], 1e-8, 2000)
    assert info["true_residual"] <= 1e-8
    _, it, _, _ = O.pcg(prob.rhs[0], 1e-8, 2000)
    assert abs(info["iterations"] - it) <= 1, (info, it)
    # error of the FP32 factor against the FP64 oracle, stated as a bound
    assert rel(G.apply(prob.rhs[0]), O.apply(prob.rhs[0])) < 1e-3


def test_results_are_bitwise_reproducible():
    prob, params = make("3d20h")
    a = gpu_factor(prob, params)
    b = gpu_factor(prob, params)
    ya, yb = a.apply(prob.rhs[0]), b.apply(prob.rhs[0])
    assert np.array_equal(ya, yb)
    xa, ia = a.pcg(prob.rhs[0], 1e-8, 500)
    xb, ib = b.pcg(prob.rhs[0], 1e-8, 500)
    assert np.array_equal(xa, xb) and ia["iterations"] == ib["iterations"]


def test_refactor_same_pattern_matches_fresh_factor():
    prob, params = make("3d16")
    G = gpu_factor(prob, params)
    scaled = prob.vals * 2.5
    G.refactor(scaled)
    ctx = rs.Context(**params)
    F = rs.GpuFactor(ctx, prob.colptr, prob.rowind, scaled, prob.xyz)
    assert rel(G.apply(prob.rhs[0]), F.apply(prob.rhs[0])) < 1e-12
    x, info = G.pcg(prob.rhs[0], 1e-8, 500)
    assert info["true_residual"] <= 1e-8


def indefinite_case(compressed):
    """A 2D Poisson matrix with one negative diagonal entry placed in an
    uncompressed (compressed=False) or a compressed supernode, found with the
    oracle's symbolic plan (the same host code as the library's)."""
    prob = rs.diffusion(2, 12, sigma=0.0)
    params = dict(max_dense_block=8, max_diag_block=32)
    O = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert O.factor() == 0
    perm = O.perm()
    node = next(j for j in range(O.num_nodes()) if bool(O.node_info(j)["compressed"]) == compressed)
    row = int(perm[O.node_info(node)["c0"]])
    vals = prob.vals.copy()
    for p in range(prob.colptr[row], prob.colptr[row + 1]):
        if prob.rowind[p] == row:
            vals[p] = -4.0
    return prob, params, vals, node


@pytest.mark.parametrize("compressed", [False, True])
def test_indefinite_matrix_reports_status(compressed):
    """The reference's retry policy: an indefinite diagonal of a compressed
    supernode is retried (10 attempts, then RSCHOL_E_NOT_PD_AFTER_RETRY); a
    non-positive pivot of an uncompressed one is where the reference aborts
    (RSCHOL_E_NOT_PD at once).  The oracle reports the same node."""
    prob, params, vals, node = indefinite_case(compressed)
    ctx = rs.Context(**params)
    with pytest.raises(rs.RscholError) as e:
        rs.GpuFactor(ctx, prob.colptr, prob.rowind, vals, prob.xyz)
    assert e.value.status == (2 if compressed else 9), str(e.value)
    assert ("supernode %d" % node) in ctx.last_error()
    O = po.OracleFactor(prob.colptr, prob.rowind, vals, prob.xyz, params)
    assert O.factor() == node + 1
    assert O.times()["attempts"] == (10 if compressed else 1)


def test_pcg_pysolve_drop_in():
    prob = rs.diffusion(2, 40, sigma=1.0, seed=4)
    A = prob.scipy()
    x = rs.solve(A, prob.rhs[0])
    assert np.linalg.norm(prob.rhs[0] - A @ x) / np.linalg.norm(prob.rhs[0]) <= 1e-6


def test_multiple_rhs_share_the_factor():
    # batched PCG (all right-hand sides in lockstep, one factor pass per apply)
    # against the single-vector solve of each column
    prob = rs.diffusion(3, 12, sigma=1.0, seed=3, nrhs=3)
    G = gpu_factor(prob, dict(max_dense_block=24, max_diag_block=48, nd_leaf=16))
    X, infos = G.pcg(prob.rhs, 1e-8, 500)
    A = prob.scipy()
    for k in range(3):
        assert np.linalg.norm(prob.rhs[k] - A @ X[k]) / np.linalg.norm(prob.rhs[k]) <= 1e-8
        x1, i1 = G.pcg(prob.rhs[k], 1e-8, 500)
        assert abs(infos[k]["iterations"] - i1["iterations"]) <= 1
        assert infos[k]["true_residual"] <= 1e-8
        assert rel(X[k], x1) < 1e-7


@pytest.mark.parametrize("precision,tol", [(rs.FP64, 1e-11), (rs.MIXED, 2e-5)])
@pytest.mark.parametrize("case", ["3d20h", "el5"])
def test_batched_apply_matches_single(case, precision, tol):
    # the batched apply (interior launches widened to k columns, compressed
    # levels as GEMMs) is the same operator as the single-vector apply; only
    # summation order differs
    prob, params = make(case)
    G = gpu_factor(prob, params, precision=precision)
    rng = np.random.default_rng(7)
    B = rng.standard_normal((5, prob.n))
    Y = G.apply(B)
    for k in range(5):
        assert rel(Y[k], G.apply(B[k])) < tol, (k, rel(Y[k], G.apply(B[k])))


def test_batched_pcg_many_columns_and_groups():
    # 70 right-hand sides: one group of 64 and one of 6, each column to 1e-8
    prob = rs.diffusion(2, 48, sigma=1.0, seed=5, nrhs=1)
    params = dict(max_dense_block=8, max_diag_block=16, nd_leaf=8)
    G = gpu_factor(prob, params, precision=rs.MIXED)
    rng = np.random.default_rng(11)
    B = rng.standard_normal((70, prob.n))
    X, infos = G.pcg(B, 1e-8, 500)
    A = prob.scipy()
    _, i1 = G.pcg(B[0], 1e-8, 500)
    for k in range(70):
        assert np.linalg.norm(B[k] - A @ X[k]) / np.linalg.norm(B[k]) <= 1e-8
    assert abs(infos[0]["iterations"] - i1["iterations"]) <= 1


@pytest.mark.parametrize("precision,tol", [(rs.FP64, APPLY_TOL), (rs.MIXED, 1e-3)])
def test_fused_and_per_panel_factor_paths_agree(precision, tol, oracles, monkeypatch):
    """The fused level launches (default) and the per-panel POTRF / TRSM / GEMM
    steps (RSCHOL_FUSED_CHOL=0) block the same factorisation differently; both
    must match the oracle's preconditioner, and each other, within the apply
    tolerance of their precision."""
    prob, params, O = oracles("3d16")
    b = prob.rhs[0]
    y_fused = gpu_factor(prob, params, precision=precision).apply(b)
    monkeypatch.setenv("RSCHOL_FUSED_CHOL", "0")
    y_panel = gpu_factor(prob, params, precision=precision).apply(b)
    y_ref = O.apply(b)
    assert rel(y_fused, y_ref) < tol and rel(y_panel, y_ref) < tol
    assert rel(y_fused, y_panel) < tol


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_graph_pcg_matches_host_loop(precision, monkeypatch):
    """The PCG solve captured as one CUDA graph (a conditional WHILE node
    decides on the device whether another iteration follows) runs the same
    kernels in the same order as the host-driven loop (RSCHOL_PCG_GRAPH=0):
    bitwise the same iterates and counts, for any eps / maxit, replayed across
    calls and with applies in between."""
    prob, params = make("3d20h")
    b = prob.rhs[0]
    monkeypatch.setenv("RSCHOL_PCG_GRAPH", "0")
    H = gpu_factor(prob, params, precision=precision)
    monkeypatch.delenv("RSCHOL_PCG_GRAPH")
    G = gpu_factor(prob, params, precision=precision)
    for eps, maxit in [(1e-8, 500), (1e-4, 500), (1e-12, 3), (1e-8, 0), (1e-8, 500)]:
        xh, ih = H.pcg(b, eps, maxit)
        xg, ig = G.pcg(b, eps, maxit)
        assert ih["iterations"] == ig["iterations"], (eps, maxit, ih, ig)
        assert np.array_equal(xh, xg)
        assert ih["true_residual"] == ig["true_residual"]
        assert np.array_equal(H.apply(b), G.apply(b))
