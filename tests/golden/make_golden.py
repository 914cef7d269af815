"""Generates the committed golden fixtures under tests/golden/.

* mt_kat.json   -- draws of the reference's own MERSENNETWISTER class
                   (src/rschol/util/MERSENNETWISTER.h), produced by the tool
                   oracle/_ref/mt_ref_kat that rank_structured_cholesky_gb300/
                   _build.py compiles from the reference header where it lies.
* oracle_*.npz  -- outputs of the CPU oracle (oracle/oracle.cpp) on small
                   seeded problems: PCG iterations, residuals, the solution,
                   one preconditioner application and the factor blocks of
                   the compressed supernodes.

Run:  python tests/golden/make_golden.py   (needs the reference sources for
mt_kat.json; the oracle fixtures only need the built oracle)
"""
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


if __name__ == "__main__":
    from rank_structured_cholesky_gb300 import _build
    _build.build_library()
    _build.build_oracle()
    mt_fixture()
    oracle_fixtures()
