"""Continuous batching on one factor (rschol_session_*).

Columns join a session's block at iteration boundaries and leave when they
meet their stopping test.  Each column follows the reference recurrences of
PCG_SOLVER::solvePCG (src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363), so
a request gives the same iterates alone and in a mix, and the same answer as
the batched rschol_pcg path up to the solve tolerance.
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs

pytestmark = pytest.mark.gpu

PARAMS = dict(max_dense_block=30, max_diag_block=60, nd_leaf=16)
EPS = 1e-10
MIX_TOL = 1e-12     # relative, alone vs in a mix (the same recurrences per column)
PCG_TOL = 1e-5      # relative, session vs rschol_pcg (both stop at ||r|| / ||b|| <= 1e-10)


def _run(ses, schedule, max_steps=5000):
    """schedule: {step index: [(tag, B)]}; returns {tag: (status, x, info)}."""
    out, i = {}, 0
    pending = sum(len(v) for v in schedule.values())
    while len(out) < pending:
        for tag, B in schedule.get(i, []):
            ses.add(tag, B, eps=EPS)
        out.update(ses.step())
        i += 1
        assert i < max_steps
    return out


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
@pytest.mark.parametrize("problem", ["3d", "el"])
def test_requests_join_and_leave(precision, problem):
    prob = rs.diffusion(3, 12, sigma=1.0, seed=4) if problem == "3d" else rs.elasticity(5, seed=6)
    G = rs.GpuFactor(rs.Context(precision=precision, **PARAMS), prob.colptr, prob.rowind, prob.vals, prob.xyz)
    rng = np.random.default_rng(8)
    reqs = {t: rng.standard_normal((int(rng.integers(1, 6)), prob.n)) for t in range(1, 9)}
    # staggered arrivals, up to 12 columns at a time: some wait in the queue
    schedule = {0: [(1, reqs[1]), (2, reqs[2])], 2: [(3, reqs[3])], 3: [(4, reqs[4]), (5, reqs[5])],
                7: [(6, reqs[6])], 8: [(7, reqs[7]), (8, reqs[8])]}
    mix = _run(rs.Session(G, max_columns=12), schedule)
    worst_mix = worst_pcg = 0.0
    for t, B in reqs.items():
        st, x, info = mix[t]
        assert st == 0
        alone = _run(rs.Session(G, max_columns=12), {0: [(t, B)]})[t]
        x_pcg, info_pcg = G.pcg(np.vstack([B, B[:1]]), eps=EPS)   # >= 2 columns: the batched path
        for j in range(B.shape[0]):
            assert info[j]["iterations"] == alone[2][j]["iterations"]
            worst_mix = max(worst_mix, np.linalg.norm(x[j] - alone[1][j]) / np.linalg.norm(alone[1][j]))
            assert abs(info[j]["iterations"] - info_pcg[j]["iterations"]) <= 1
            worst_pcg = max(worst_pcg, np.linalg.norm(x[j] - x_pcg[j]) / np.linalg.norm(x_pcg[j]))
            assert info[j]["true_residual"] <= 10 * EPS
    print("session: worst alone-vs-mix %.3e, worst vs rschol_pcg %.3e" % (worst_mix, worst_pcg))
    assert worst_mix <= MIX_TOL
    assert worst_pcg <= PCG_TOL


def test_more_columns_than_the_block():
    prob = rs.diffusion(2, 48, sigma=1.0, seed=9)
    G = rs.GpuFactor(rs.Context(precision=rs.MIXED, **PARAMS), prob.colptr, prob.rowind, prob.vals, prob.xyz)
    ses = rs.Session(G, max_columns=8)
    assert ses.columns == 8
    rng = np.random.default_rng(1)
    reqs = {t: rng.standard_normal((5, prob.n)) for t in range(6)}   # 30 columns through an 8-column block
    out = _run(ses, {0: list(reqs.items())})
    for t, B in reqs.items():
        st, x, info = out[t]
        assert st == 0
        for j in range(5):
            assert info[j]["true_residual"] <= 10 * EPS
    assert ses.counts() == (0, 0)


def test_zero_right_hand_side_is_a_breakdown():
    prob = rs.diffusion(2, 16, seed=2)
    G = rs.GpuFactor(rs.Context(**PARAMS), prob.colptr, prob.rowind, prob.vals, prob.xyz)
    ses = rs.Session(G, max_columns=4)
    b = np.zeros((2, prob.n))
    b[1] = 1.0
    out = _run(ses, {0: [(5, b)]})
    st, x, info = out[5]
    assert st == 5   # RSCHOL_E_BREAKDOWN, as rschol_pcg reports a zero column
    assert np.all(x[0] == 0)
    assert info[1]["true_residual"] <= 10 * EPS


@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_graph_replayed_steps_match_direct_launches(precision, monkeypatch):
    """A session replays the iteration part of a step from a CUDA graph once
    two consecutive steps have the same width and buffers; with
    RSCHOL_SESSION_GRAPH=0 every step launches the same kernels directly.
    Staggered joins change the width (a new capture) and a long run of
    unchanged steps replays: bitwise the same x and iteration counts."""
    prob = rs.diffusion(3, 12, sigma=1.0, seed=4)
    rng = np.random.default_rng(11)
    reqs = {t: rng.standard_normal((int(rng.integers(1, 4)), prob.n)) for t in range(1, 6)}
    schedule = {0: [(1, reqs[1])], 1: [(2, reqs[2])], 5: [(3, reqs[3])], 6: [(4, reqs[4])], 20: [(5, reqs[5])]}
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("RSCHOL_SESSION_GRAPH", mode)
        G = rs.GpuFactor(rs.Context(precision=precision, **PARAMS), prob.colptr, prob.rowind, prob.vals, prob.xyz)
        out[mode] = _run(rs.Session(G, max_columns=8), schedule)
        del G
    for t in reqs:
        assert out["0"][t][0] == 0 and out["1"][t][0] == 0
        assert np.array_equal(out["0"][t][1], out["1"][t][1]), t
        assert [i["iterations"] for i in out["0"][t][2]] == [i["iterations"] for i in out["1"][t][2]]
