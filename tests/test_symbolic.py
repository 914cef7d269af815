"""Known-answer tests of the host ordering / symbolic restatement.

* rank policy: FactorManager::blockRank / diagonalBlockRank (FactorManager.cpp:7283-7338)
* SeparatorTree kd split (src/rschol/datastructure/SeparatorTree.cpp)
* cs_etree / cs_counts with the identity postorder (NestedDissection.cpp:409-429)
* BuildRelaxedSupernodes (NestedDissection.cpp:1266-1735), hand-worked cases
* row structure of every supernode against brute-force symbolic elimination
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs


@pytest.mark.parametrize("m,n,c,cap,expected", [
    (2048, 2048, 0.4, 0, 104),
    (100, 100, 0.4, 0, 18),
    (16, 5000, 0.4, 0, 16),
    (10, 1000, 0.4, 0, 10),
    (4096, 4096, 0.4, 0, 158),
    (2048, 2048, 0.5, 0, 129),
    (4096, 4096, 0.4, 32, 32),
])
def test_rank_table(m, n, c, cap, expected):
    assert rs.load_library().rschol_block_rank(m, n, c, 5, cap) == expected


def sep_tree(pts, max_leaf):
    pts = np.ascontiguousarray(pts, np.float64)
    npts = len(pts)
    order = np.zeros(npts, np.int32)
    first = np.zeros(npts + 1, np.int32)
    nl = rs.load_library().rschol_separator_tree(npts, pts.ctypes.data, max_leaf, order.ctypes.data,
                                                  first.ctypes.data)
    return order, first[:nl + 1]


def test_separator_tree_line():
    xs = np.array([5, 2, 7, 0, 3, 6, 1, 4], float)
    pts = np.stack([xs, np.zeros(8), np.zeros(8)], 1)
    order, first = sep_tree(pts, 2)
    assert xs[order].tolist() == sorted(xs.tolist())
    assert first.tolist() == [0, 2, 4, 6, 8]


def test_separator_tree_full_tree_hack():
    # 5 points, leaves <= 2: the left half (2 points) is forced to split once
    # more so both subtrees have the same height (power-of-two leaf count).
    pts = np.stack([np.arange(5.0), np.zeros(5), np.zeros(5)], 1)
    order, first = sep_tree(pts, 2)
    assert order.tolist() == [0, 1, 2, 3, 4]
    assert first.tolist() == [0, 1, 2, 3, 5]


def test_separator_tree_grid_longest_axis():
    pts = np.array([[x, y, 0.0] for y in range(2) for x in range(4)])
    order, first = sep_tree(pts, 2)
    assert len(first) == 5
    leaf_x = [sorted(set(pts[order[first[k]:first[k + 1]], 0].tolist())) for k in range(4)]
    assert leaf_x == [[0.0], [1.0], [2.0], [3.0]]


def brute_force_L(n, rows_of):
    L = np.zeros((n, n), bool)
    for j in range(n):
        L[j, j] = True
        for i in rows_of[j]:
            if i > j:
                L[i, j] = True
    for k in range(n):
        nz = np.nonzero(L[k + 1:, k])[0] + k + 1
        for a in nz:
            L[a, nz[nz <= a]] = True
    return L


def etree_counts(n, upper_cols):
    colptr = np.zeros(n + 1, np.int32)
    rowind = []
    for j in range(n):
        rs_ = sorted(i for i in upper_cols[j] if i < j)
        rowind += rs_
        colptr[j + 1] = len(rowind)
    rowind = np.array(rowind, np.int32)
    parent = np.zeros(n, np.int32)
    counts = np.zeros(n, np.int32)
    rs.load_library().rschol_etree_counts(n, colptr.ctypes.data, rowind.ctypes.data, parent.ctypes.data,
                                          counts.ctypes.data)
    return parent, counts


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_etree_and_counts_against_elimination(seed):
    rng = np.random.default_rng(seed)
    n = 40
    adj = [set() for _ in range(n)]
    for _ in range(70):
        a, b = rng.integers(0, n, 2)
        if a != b:
            adj[a].add(int(b))
            adj[b].add(int(a))
    L = brute_force_L(n, [[i for i in adj[j]] for j in range(n)])
    parent = [int(np.nonzero(L[j + 1:, j])[0][0] + j + 1) if L[j + 1:, j].any() else -1 for j in range(n)]
    # postorder the etree so the identity postorder is a valid one
    kids = [[] for _ in range(n)]
    for j in range(n):
        if parent[j] >= 0:
            kids[parent[j]].append(j)
    post = []

    def visit(v):
        for c in kids[v]:
            visit(c)
        post.append(v)
    for r in range(n):
        if parent[r] < 0:
            visit(r)
    inv = np.empty(n, int)
    inv[post] = np.arange(n)
    adj2 = [set(int(inv[i]) for i in adj[post[k]]) for k in range(n)]
    L2 = brute_force_L(n, [list(adj2[j]) for j in range(n)])
    par, cnt = etree_counts(n, adj2)
    exp_par = [int(np.nonzero(L2[j + 1:, j])[0][0] + j + 1) if L2[j + 1:, j].any() else -1 for j in range(n)]
    assert par.tolist() == exp_par
    assert cnt.tolist() == L2.sum(0).tolist()


def relaxed(n, parent, counts, comps, max_block):
    comps = np.array(comps, np.int32)   # rows: size, children, first, parent
    sf = np.zeros(n + 1, np.int32)
    cf = np.zeros(n + 1, np.int32)
    # keep every array alive for the duration of the call
    arrs = [np.ascontiguousarray(a, np.int32) for a in (parent, counts, comps[:, 0], comps[:, 1], comps[:, 2],
                                                        comps[:, 3])]
    ns = rs.load_library().rschol_relaxed_supernodes(
        n, arrs[0].ctypes.data, arrs[1].ctypes.data, len(comps), arrs[2].ctypes.data, arrs[3].ctypes.data,
        arrs[4].ctypes.data, arrs[5].ctypes.data, max_block, sf.ctypes.data, cf.ctypes.data)
    return sf[:ns + 1].tolist(), cf[:ns].tolist()


def test_relaxed_supernodes_chain_merges():
    # tridiagonal 6x6: every column is its own fundamental supernode; the
    # relaxed amalgamation (nrelax 4/16/48, zrelax .8/.1/.05) merges them all.
    parent = [1, 2, 3, 4, 5, -1]
    counts = [2, 2, 2, 2, 2, 1]
    sf, cf = relaxed(6, parent, counts, [[6, 0, 0, -1]], 200)
    assert sf == [0, 6] and cf == [0]


def test_relaxed_supernodes_keep_compressed_separator():
    parent = [1, 2, 3, 4, 5, -1]
    counts = [2, 2, 2, 2, 2, 1]
    sf, cf = relaxed(6, parent, counts, [[4, 0, 0, 1], [2, 1, 4, -1]], 1)
    assert sf == [0, 4, 6] and cf == [0, 1]


def test_supernode_rows_match_brute_force_fill():
    from oracle import pyoracle as po
    prob = rs.diffusion(2, 14, sigma=1.0, seed=0)
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz,
                        dict(max_dense_block=6, max_diag_block=40, nd_leaf=8))
    perm = F.perm()
    iperm = np.empty_like(perm)
    iperm[perm] = np.arange(len(perm))
    n = prob.n
    rows_of = [[] for _ in range(n)]
    for j in range(n):
        for p in range(prob.colptr[j], prob.colptr[j + 1]):
            a, b = iperm[prob.rowind[p]], iperm[j]
            if a > b:
                rows_of[b].append(int(a))
    L = brute_force_L(n, rows_of)
    covered = 0
    for k in range(F.num_nodes()):
        inf = F.node_info(k)
        c0, c1 = inf["c0"], inf["c1"]
        expect = sorted(set(np.nonzero(L[c1 + 1:, c0:c1 + 1].any(1))[0] + c1 + 1))
        assert F.node_rows(k).tolist() == expect
        covered += c1 - c0 + 1
    assert covered == n



def test_structure_check_names_unsupported_hierarchical_diagonal():
    """rschol_check_structure (host ordering + symbolic, no device): a relaxed
    uncompressed supernode wider than max_diag_block would need a HODLR
    diagonal, which the device factorisation does not build -- reported as
    RSCHOL_E_UNSUPPORTED with the width it needs; the default parameters take
    the same matrix; an invalid pattern is RSCHOL_E_BAD_INPUT."""
    p = rs.diffusion(2, 9, 7, sigma=1.0, seed=3)
    st, why = rs.check_structure(p.colptr, p.rowind, p.xyz, max_dense_block=4, max_diag_block=8, nd_leaf=4)
    assert rs.STATUS_NAMES[st] == "RSCHOL_E_UNSUPPORTED"
    assert "more than max_diag_block = 8" in why and "raise max_diag_block to at least" in why, why
    assert rs.check_structure(p.colptr, p.rowind, p.xyz) == (rs.RSCHOL_OK, "")
    bad = p.colptr.copy()
    bad[0] = 1
    st, why = rs.check_structure(bad, p.rowind, p.xyz)
    assert rs.STATUS_NAMES[st] == "RSCHOL_E_BAD_INPUT" and "colptr" in why
