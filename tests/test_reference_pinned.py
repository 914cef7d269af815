"""Pins against the reference's own code (CPU).

The fixtures under tests/golden/ref_*.json were written by
tests/golden/make_golden.py with tools compiled from the reference's sources
(oracle/_ref/, built by rank_structured_cholesky_gb300/_build.py):

* ref_septree.json -- src/rschol/datastructure/SeparatorTree.h/.cpp, the
  separator sub-ordering and diagonal-block leaves of
  NestedDissection::ReorderNestedSeparators: the library's restatement
  (rschol_separator_tree) must give the identical point order and leaves.
* ref_pcg.json -- PCG_SOLVER::solvePCG (src/rschol/linearalgebra/
  PCG_SOLVER.cpp:226-363) run with the CPU oracle's factor as its
  preconditioner: the oracle's own PCG restatement must stop after the same
  number of iterations at the same residual.

Where the reference sources are present the same checks also run live
against the tools, and the C++ adapter is compiled against the reference's
real headers.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po
from tests.golden import make_golden as mg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)["cases"]


def ours_septree(pts, leaf):
    pts = np.ascontiguousarray(pts, np.float64)
    n = len(pts)
    order = np.zeros(n, np.int32)
    first = np.zeros(n + 1, np.int32)
    nl = rs.load_library().rschol_separator_tree(n, pts.ctypes.data, leaf, order.ctypes.data, first.ctypes.data)
    return order, first[:nl + 1]


@pytest.mark.parametrize("case", [c[0] for c in mg.SEPTREE_CASES])
def test_separator_tree_matches_reference_fixture(case):
    fx = load("ref_septree.json")[case]
    pts = mg.septree_points(fx["kind"], fx["size"], fx["seed"])
    order, first = ours_septree(pts, fx["leaf"])
    assert len(order) == fx["npts"]
    assert first.tolist() == fx["leaf_first"]
    assert mg.order_hash(order) == fx["order_sha256"]


SMALL = ["2d48", "3d16", "3d20h", "el5", "c1", "c3r", "c2s"]


def case_spec(name):
    spec = mg.CASES.get(name) or mg.WORKLOAD_CASES[name]
    return mg.make_problem(spec["problem"]), spec["params"]


@pytest.mark.parametrize("case", SMALL)
def test_oracle_pcg_matches_reference_pcg(case):
    fx = load("ref_pcg.json")[case]
    prob, params = case_spec(case)
    assert prob.n == fx["n"]
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert F.factor() == 0
    x, it, _, true = F.pcg(prob.rhs[0], 1e-8, 2000)
    assert it == fx["iterations"]
    assert abs(true - fx["true_residual"]) <= 1e-6 * fx["true_residual"] + 1e-15
    assert abs(np.linalg.norm(x) - fx["x_norm"]) <= 1e-9 * fx["x_norm"]


def _reference_tools():
    from rank_structured_cholesky_gb300 import _build
    if _build.reference_dir() is None:
        pytest.skip("reference sources not present")
    _build.build_reference_tools()
    from oracle import pyref
    return pyref


@pytest.mark.parametrize("case", ["3d20h", "el5", "c3r"])
def test_live_reference_pcg_is_the_oracle_pcg(case):
    """Same preconditioner, same recurrences: the reference's PCG loop and the
    oracle's give the same iterates (bitwise here, with the same BLAS)."""
    pyref = _reference_tools()
    prob, params = case_spec(case)
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    assert F.factor() == 0
    xr, itr, resr = pyref.pcg(prob.colptr, prob.rowind, prob.vals, prob.rhs[0], F.apply, 1e-8, 2000)
    xo, ito, _, tro = F.pcg(prob.rhs[0], 1e-8, 2000)
    assert itr == ito
    assert np.linalg.norm(xr - xo) <= 1e-13 * np.linalg.norm(xr)


def test_live_reference_separator_tree_random_sets():
    pyref = _reference_tools()
    rng = np.random.default_rng(99)
    for k in range(6):
        n = int(rng.integers(50, 2000))
        pts = rng.random((n, 3)) * rng.integers(1, 50, 3)
        if k % 2:
            pts = np.round(pts)
        leaf = int(rng.integers(8, 300))
        o1, f1 = ours_septree(pts, leaf)
        o2, f2 = pyref.septree(pts, leaf)
        assert np.array_equal(o1, o2) and np.array_equal(f1, f2), (k, n, leaf)


def test_adapter_compiles_against_reference_headers():
    """include/rschol_gpu_preconditioner.hpp against the reference's own
    PRECONDITIONER.h / SPARSE_MATRIX.h / VECTOR.h / TYPES.h (Boost names from
    oracle/ref_shim/)."""
    from rank_structured_cholesky_gb300 import _build
    root = _build.reference_dir()
    if root is None:
        pytest.skip("reference sources not present")
    src = ('#include "rschol_gpu_preconditioner.hpp"\n'
           'static PRECONDITIONER *make() { return new GpuFactorPreconditioner(); }\n'
           'int main() { PRECONDITIONER *p = make(); p->init(); delete p; return 0; }\n')
    subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-x", "c++", "-", "-I", _build.REF_SHIM,
                    "-I", os.path.join(root, "src"), "-I", os.path.join(ROOT, "include")],
                   input=src, text=True, check=True)
