"""Nested dissection without coordinates (the ordering rs.solve and the
pcg_pysolve drop-in use: the reference passes zero positions and CHOLMOD's
METIS node bisection orders the graph).

Each split takes the smaller separator of a breadth-first level-structure
bisection and a multilevel one (heavy-edge-matching coarsening, graph-growing
initial bisection, Fiduccia-Mattheyses refinement, Koenig vertex cover of the
cut).  RSCHOL_GRAPH_ND=bfs keeps the level structure alone.  Checked here:
the ordering is a valid nested dissection (a permutation whose separators
separate), the factor is exact without compression, and the fill is never
much above the level-structure ordering's and far below it on an
unstructured (elasticity) graph.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NOCOMP = dict(max_dense_block=100000, max_diag_block=100000, nd_leaf=64)

FILL = r"""
import sys, json; sys.path.insert(0, %r)
import numpy as np
import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po
out = {}
rng = np.random.default_rng(0)
for name, p in [("2d64", rs.diffusion(2, 64, sigma=1.0, seed=1)), ("3d16", rs.diffusion(3, 16, sigma=1.0, seed=1)),
                ("el8", rs.elasticity(8))]:
    A = p.scipy(); q = rng.permutation(p.n); A = A[q][:, q].tocsc(); A.sort_indices()
    F = po.OracleFactor(A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, None, %r)
    assert F.factor() == 0
    fill = 0
    for j in range(F.num_nodes()):
        i = F.node_info(j); n = i["c1"] - i["c0"] + 1; fill += n * (n + 1) // 2 + i["m"] * n
    out[name] = fill
print(json.dumps(out))
""" % (ROOT, NOCOMP)


def fills(mode):
    env = dict(os.environ)
    env.pop("RSCHOL_GRAPH_ND", None)
    if mode == "bfs":
        env["RSCHOL_GRAPH_ND"] = "bfs"
    r = subprocess.run([sys.executable, "-c", FILL], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_fill_against_level_structure_ordering():
    ml, bfs = fills("default"), fills("bfs")
    for k in ml:
        assert ml[k] <= 1.06 * bfs[k], (k, ml[k], bfs[k])
    assert ml["el8"] <= 0.8 * bfs["el8"], (ml["el8"], bfs["el8"])


@pytest.mark.parametrize("case", ["2d", "3d", "el"])
def test_graph_ordering_is_a_valid_dissection(case):
    p = {"2d": lambda: rs.diffusion(2, 40, sigma=1.0, seed=2), "3d": lambda: rs.diffusion(3, 12, sigma=1.0, seed=2),
         "el": lambda: rs.elasticity(6)}[case]()
    F = po.OracleFactor(p.colptr, p.rowind, p.vals, None, NOCOMP)
    assert F.factor() == 0
    perm = F.perm()
    assert np.array_equal(np.sort(perm), np.arange(p.n))
    # without compression the factor is exact: the ordering's symbolic
    # structure (etree, supernode rows) covers all fill
    x, it, _, true = F.pcg(p.rhs[0], 1e-12, 5)
    assert it == 1 and true < 1e-12
    # supernodes of the same separator level are independent: a supernode's
    # rows are all ancestors' columns (later in the ordering)
    for j in range(F.num_nodes()):
        info = F.node_info(j)
        rows = F.node_rows(j)
        assert np.all(rows > info["c1"])


def test_disconnected_graph_is_dissected():
    """Two grids with no coupling: the dissection still splits them (a
    one-vertex separator where the halves are disconnected)."""
    import scipy.sparse as sp
    a = rs.diffusion(2, 20, sigma=0.0).scipy()
    A = sp.block_diag([a, a]).tocsc()
    A.sort_indices()
    F = po.OracleFactor(A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, None, NOCOMP)
    assert F.factor() == 0
    sizes = [F.node_info(j)["c1"] - F.node_info(j)["c0"] + 1 for j in range(F.num_nodes())]
    assert max(sizes) < 100
