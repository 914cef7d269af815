"""Generates the committed golden fixtures under tests/golden/.

* mt_kat.json   -- draws of the reference's own MERSENNETWISTER class
                   (src/rschol/util/MERSENNETWISTER.h), produced by the tool
                   oracle/_ref/mt_ref_kat that rank_structured_cholesky_gb300/
                   _build.py compiles from the reference header where it lies.
* oracle_*.npz  -- outputs of the CPU oracle (oracle/oracle.cpp) on small
                   seeded problems: PCG iterations, residuals, the solution,
                   one preconditioner application and the factor blocks of
                   the compressed supernodes.
* ref_septree.json -- the reference's own SeparatorTree (oracle/_ref/
                   ref_septree_kat, built from src/rschol/datastructure/
                   SeparatorTree.h/.cpp) on seeded point sets: a hash of the
                   point order and the leaf boundaries.
* ref_pcg.json  -- the reference's own PCG_SOLVER::solvePCG (oracle/_ref/
                   libref_pcg.so) run with the CPU oracle's factor as its
                   preconditioner: iterations and final residual per case.

Run:  python tests/golden/make_golden.py   (needs the reference sources for
mt_kat.json, ref_septree.json and ref_pcg.json; the oracle fixtures only
need the built oracle)
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    "2d48": dict(problem=("diffusion", 2, 48, 1.0, 0), params=dict(max_dense_block=8, max_diag_block=16, nd_leaf=8)),
    "3d16": dict(problem=("diffusion", 3, 16, 1.0, 1), params=dict(max_dense_block=30, max_diag_block=60, nd_leaf=16)),
    "3d20h": dict(problem=("diffusion", 3, 20, 1.0, 1),
                  params=dict(max_dense_block=30, max_diag_block=60, explicit_threshold=250, nd_leaf=16)),
    "el5": dict(problem=("elasticity", 5, 0.0, 0.0, 2), params=dict(max_dense_block=40, max_diag_block=80, nd_leaf=16)),
}

# The configurations the benchmark workloads are quoted on, at sizes the
# oracle factors in seconds (checked by the reference-PCG fixtures and the
# GPU parity tests):
#  c1   -- 2D 5-point Poisson 128 x 128 (seed 0), ND leaves <= 64, ranks
#          capped at 32 with oversampling 10; separators above 16 columns
#          compressed and HODLR leaves of <= 32 so that compression reaches
#          every level (the reference default of 200 compresses nothing on
#          this grid);
#  c3r  -- 3D Q1 elasticity on a 20^3 element mesh (the 48^3 workload
#          reduced), E = 1, nu = 0.3, seed 2, ranks capped at 64;
#  c2s  -- 3D variable-coefficient diffusion 32^3 (sigma 1, seed 1), the
#          reference's default parameters;
#  c2   -- the same at 64^3 (N = 262,144), the benchmark workload itself.
WORKLOAD_CASES = {
    "c1": dict(problem=("diffusion", 2, 128, 0.0, 0),
               params=dict(nd_leaf=64, max_dense_block=16, max_diag_block=32, rank_cap=32, oversampling=10)),
    "c3r": dict(problem=("elasticity", 20, 0.0, 0.0, 2), params=dict(nd_leaf=64, rank_cap=64)),
    "c2s": dict(problem=("diffusion", 3, 32, 1.0, 1), params=dict()),
    "c2": dict(problem=("diffusion", 3, 64, 1.0, 1), params=dict()),
}

# Seeded point sets for the separator-tree known answers: (name, kind, size,
# leaf bound, seed).  "plane" / "slab" are grid separators as nested
# dissection produces them, "line" a 1D separator, "cloud" random points,
# "ties" points on a coarse lattice (many equal coordinates).
SEPTREE_CASES = [
    ("plane64", "plane", 64, 400, 0), ("slab64", "slab", 64, 400, 1), ("line1000", "line", 1000, 64, 2),
    ("cloud3000", "cloud", 3000, 100, 3), ("ties500", "ties", 500, 16, 4), ("plane127", "plane", 127, 400, 5),
    ("rect37x53", "rect", 53, 60, 6), ("plane48", "plane", 48, 250, 7),
]


def septree_points(kind, size, seed):
    rng = np.random.default_rng(seed)
    if kind == "plane":
        pts = np.array([[x, y, 5.0] for y in range(size) for x in range(size)], float)
    elif kind == "slab":
        pts = np.array([[x, 32.0, z] for z in range(size) for x in range(size)], float)
    elif kind == "line":
        pts = np.array([[x, 0.0, 0.0] for x in range(size)], float)
    elif kind == "cloud":
        pts = rng.random((size, 3))
    elif kind == "ties":
        pts = rng.integers(0, 5, (size, 3)).astype(float)
    else:   # rect: a 37-row grid of `size` columns
        pts = np.array([[x, y, 0.0] for y in range(37) for x in range(size)], float)
    return pts[rng.permutation(len(pts))]


def make_problem(spec):
    import rank_structured_cholesky_gb300 as rs
    kind = spec[0]
    if kind == "diffusion":
        _, dim, nx, sigma, seed = spec
        return rs.diffusion(dim, nx, sigma=sigma, seed=seed)
    _, ne, _, _, seed = spec
    return rs.elasticity(ne, seed=seed)


def probe_vector(j, n):
    return np.random.default_rng(1000 + j).standard_normal(n)


def mt_fixture():
    from rank_structured_cholesky_gb300 import _build
    exe = _build.build_reference_tools()
    if exe is None:
        print("reference sources not present; mt_kat.json left as is")
        return
    out = {}
    for seed in (152, 0, 1, 2, 3):
        lines = subprocess.run([exe, str(seed), "1500"], stdout=subprocess.PIPE, text=True, check=True).stdout.split()
        out[str(seed)] = {"randInt": [int(v) for v in lines[:1500]], "randNorm": [float(v) for v in lines[1500:]]}
    with open(os.path.join(HERE, "mt_kat.json"), "w") as f:
        json.dump({"source": "reference MERSENNETWISTER.h via oracle/_ref/mt_ref_kat", "count": 1500,
                   "seeds": out}, f)


def oracle_fixtures():
    from oracle import pyoracle as po
    for name, case in CASES.items():
        prob = make_problem(case["problem"])
        F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, case["params"])
        assert F.factor() == 0
        x, it, rec, tr = F.pcg(prob.rhs[0], 1e-8, 2000)
        y = F.apply(prob.rhs[0])
        comp = [j for j in range(F.num_nodes()) if F.node_info(j)["compressed"]]
        blobs = {"iterations": it, "residual": rec, "true_residual": tr, "x": x, "apply": y,
                 "perm": F.perm(), "compressed_nodes": np.array(comp, np.int32)}
        for j in comp:
            # random projections keep the fixtures small: L11 p and L21 p
            l11 = F.node_l11(j)
            probe = probe_vector(j, l11.shape[1])
            blobs["l11p_%d" % j] = l11 @ probe
            l21 = F.node_l21(j)
            if l21.size:
                blobs["l21p_%d" % j] = l21 @ probe
        np.savez_compressed(os.path.join(HERE, "oracle_%s.npz" % name), **blobs)
        print(name, "n=%d" % prob.n, "iterations", it, "residual %.3e" % tr, "compressed", len(comp))


def order_hash(order):
    return hashlib.sha256(np.ascontiguousarray(order, np.int32).tobytes()).hexdigest()


def ref_fixtures():
    """ref_septree.json and ref_pcg.json from the tools built out of the
    reference's own sources."""
    from rank_structured_cholesky_gb300 import _build
    if _build.build_reference_tools() is None:
        print("reference sources not present; ref_*.json left as is")
        return
    from oracle import pyoracle as po
    from oracle import pyref
    trees = {}
    for name, kind, size, leaf, seed in SEPTREE_CASES:
        order, first = pyref.septree(septree_points(kind, size, seed), leaf)
        trees[name] = {"kind": kind, "size": size, "leaf": leaf, "seed": seed, "npts": int(len(order)),
                       "order_sha256": order_hash(order), "leaf_first": first.tolist()}
    with open(os.path.join(HERE, "ref_septree.json"), "w") as f:
        json.dump({"source": "reference SeparatorTree.h/.cpp via oracle/_ref/ref_septree_kat", "cases": trees}, f,
                  indent=1)
    runs = {}
    for name, case in list(CASES.items()) + list(WORKLOAD_CASES.items()):
        prob = make_problem(case["problem"])
        F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, case["params"])
        assert F.factor() == 0
        x, it, res = pyref.pcg(prob.colptr, prob.rowind, prob.vals, prob.rhs[0], F.apply, 1e-8, 2000)
        runs[name] = {"n": prob.n, "params": case["params"], "iterations": it, "true_residual": res,
                      "x_norm": float(np.linalg.norm(x))}
        print(name, "n=%d" % prob.n, "reference PCG iterations", it, "residual %.3e" % res)
    with open(os.path.join(HERE, "ref_pcg.json"), "w") as f:
        json.dump({"source": "reference PCG_SOLVER::solvePCG via oracle/_ref/libref_pcg.so, preconditioned by "
                             "the CPU oracle's factor; eps 1e-8, x0 = 0, rhs[0] of each case", "cases": runs}, f,
                  indent=1)


if __name__ == "__main__":
    from rank_structured_cholesky_gb300 import _build
    _build.build_library()
    _build.build_oracle()
    which = sys.argv[1:] or ["mt", "oracle", "ref"]
    if "mt" in which:
        mt_fixture()
    if "oracle" in which:
        oracle_fixtures()
    if "ref" in which:
        ref_fixtures()
