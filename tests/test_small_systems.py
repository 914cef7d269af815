"""Small and odd-sized systems on the GPU against the CPU oracle.

Orders 1 and 2, a diagonal matrix (every supernode without off-diagonal
rows), a disconnected matrix (two grids, no positions: the graph dissection
splits them apart), odd grid shapes below and just above the dissection leaf
size, and small compressing cases whose ranks reach min(rows, cols) (the
identity-basis fallback, FactorManager.cpp:9598-9606).  For each: the
supernode partition is the oracle's, one FP64 application is within
APPLY_TOL of the oracle's, the FP64 PCG stops within one iteration of the
oracle's count at ||r||/||b|| <= 1e-8, and the mixed-precision PCG reaches
the same residual in that count +-1.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-7
COMPRESSING = dict(max_dense_block=8, max_diag_block=48, nd_leaf=8, explicit_threshold=20)


def from_scipy(A):
    A = sp.csc_matrix(A)
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)


def case(name):
    rng = np.random.default_rng(7)
    if name == "order1":
        return from_scipy(np.array([[4.0]])), None, {}
    if name == "order2":
        return from_scipy(np.array([[4.0, 1.0], [1.0, 3.0]])), None, {}
    if name == "diagonal37":
        return from_scipy(sp.diags(rng.uniform(0.5, 4.0, 37))), None, {}
    if name == "two grids":
        g = rs.diffusion(2, 30, sigma=1.0, seed=2).scipy()
        return from_scipy(sp.block_diag([g, 2.0 * g])), None, {}
    shapes = {"2d 5x7": (2, 5, 7, None, {}), "3d 3x3x5": (3, 3, 3, 5, {}), "2d 9x11": (2, 9, 11, None, {}),
              "3d 5x5x5 compressing": (3, 5, 5, 5, COMPRESSING),
              "3d 7x6x5 compressing": (3, 7, 6, 5, COMPRESSING),
              "2d 31x29 compressing": (2, 31, 29, None, dict(COMPRESSING, nd_leaf=16))}
    d, nx, ny, nz, prm = shapes[name]
    p = rs.diffusion(d, nx, ny, nz, sigma=1.0, seed=3)
    return (p.colptr, p.rowind, p.vals), p.xyz, prm


CASES = ["order1", "order2", "diagonal37", "two grids", "2d 5x7", "3d 3x3x5", "2d 9x11",
         "3d 5x5x5 compressing", "3d 7x6x5 compressing", "2d 31x29 compressing"]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", CASES)
def test_small_system_matches_oracle(name):
    (colptr, rowind, vals), xyz, prm = case(name)
    n = len(colptr) - 1
    b = np.random.default_rng(11).standard_normal(n)
    O = po.OracleFactor(colptr, rowind, vals, xyz, prm)
    assert O.factor() == 0
    _, it, _, _ = O.pcg(b, 1e-8, 500)
    G = rs.GpuFactor(rs.Context(**prm), colptr, rowind, vals, xyz)
    assert G.num_nodes() == O.num_nodes()
    for j in range(G.num_nodes()):
        gi, oi = G.node_info(j), O.node_info(j)
        assert (gi["c0"], gi["c1"], gi["compressed"]) == (oi["c0"], oi["c1"], oi["compressed"])
    assert rel(G.apply(b), O.apply(b)) < APPLY_TOL
    x, info = G.pcg(b, 1e-8, 500)
    assert abs(info["iterations"] - it) <= 1, (info, it)
    A = sp.csc_matrix((vals, rowind, colptr), shape=(n, n))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1e-8
    M = rs.GpuFactor(rs.Context(precision=rs.MIXED, **prm), colptr, rowind, vals, xyz)
    xm, im = M.pcg(b, 1e-8, 500)
    assert im["true_residual"] <= 1e-8
    assert abs(im["iterations"] - it) <= 1, (im, it)
