"""Serving loop: factor cache by matrix id, admission by device bytes,
concurrent workers, and the result of a request the same alone and in a mix.

The host-side logic (queueing, status reporting, argument checks) runs
without a GPU: every request then fails with RSCHOL_E_NO_DEVICE.  The GPU
tests check each request of a mixed stream against the same system solved
alone through GpuFactor.pcg.
"""
import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs

PARAMS = dict(max_dense_block=30, max_diag_block=60, nd_leaf=16)


def _mix():
    return {
        0: rs.diffusion(2, 40, sigma=1.0, seed=11, nrhs=3),
        1: rs.diffusion(3, 10, sigma=1.0, seed=12, nrhs=3),
        2: rs.elasticity(4, seed=13, nrhs=3),
    }


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_server_reports_no_device_without_gpu():
    srv = rs.Server(workers=2, hbm_budget_bytes=1e9, **PARAMS)
    probs = _mix()
    ids = [srv.submit(k, p.colptr, p.rowind, p.vals, np.stack(p.rhs[:1]), p.xyz) for k, p in probs.items()]
    for rid in ids:
        st, x, info, t = srv.wait(rid)
        assert st == 7   # RSCHOL_E_NO_DEVICE
        assert t["latency"] >= 0
    s = srv.stats()
    assert s["completed"] == 3 and s["misses"] == 3 and s["cached_factors"] == 0 and s["cached_bytes"] == 0
    srv.close()


def test_server_rejects_bad_requests():
    srv = rs.Server(workers=1, hbm_budget_bytes=1e9, **PARAMS)
    p = rs.diffusion(2, 8, seed=1, nrhs=1)
    with pytest.raises(rs.RscholError):
        srv.submit(0, p.colptr, p.rowind, p.vals, np.zeros((65, p.n)))
    with pytest.raises(rs.RscholError):
        srv.submit(0, p.colptr, p.rowind, p.vals, np.zeros((0, p.n)))
    srv.close()
    lib = rs.load_library()
    assert not lib.rschol_server_create(None, 1, 1e9)


def _alone(G, B):
    ses = rs.Session(G)
    ses.add(1, B, eps=1e-10)
    out = {}
    while not out:
        out = ses.step()
    return out[1]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_each_request_same_alone_and_in_the_mix(precision):
    probs = _mix()
    rng = np.random.default_rng(5)
    factors = {k: rs.GpuFactor(rs.Context(precision=precision, **PARAMS), p.colptr, p.rowind, p.vals, p.xyz)
               for k, p in probs.items()}
    srv = rs.Server(workers=3, hbm_budget_bytes=64e9, precision=precision, **PARAMS)
    reqs = []
    for i in range(24):
        k = int(rng.integers(0, 3))
        p = probs[k]
        B = rng.standard_normal((int(rng.integers(1, 6)), p.n))
        reqs.append((srv.submit(k, p.colptr, p.rowind, p.vals, B, p.xyz, eps=1e-10), k, B))
    worst = 0.0
    for rid, k, B in reqs:
        st, x, info, t = srv.wait(rid)
        assert st == 0
        st1, x1, info1 = _alone(factors[k], B)
        assert st1 == 0
        for j in range(B.shape[0]):
            assert info[j]["iterations"] == info1[j]["iterations"]
            assert info[j]["true_residual"] <= 1e-9
            worst = max(worst, np.linalg.norm(x[j] - x1[j]) / np.linalg.norm(x1[j]))
        assert t["latency"] >= t["pcg"] >= 0
    print("server: worst alone-vs-mix %.3e" % worst)
    assert worst <= 1e-12
    s = srv.stats()
    assert s["completed"] == 24 and s["misses"] == 3 and s["hits"] == 21
    srv.close()


def _footprint(k, p):
    srv = rs.Server(workers=1, hbm_budget_bytes=1e12, **PARAMS)
    st = srv.wait(srv.submit(k, p.colptr, p.rowind, p.vals, np.stack(p.rhs[:1]), p.xyz))[0]
    assert st == 0
    b = srv.stats()["cached_bytes"]
    srv.close()
    return b


@pytest.mark.gpu
def test_budget_evicts_least_recently_used():
    probs = _mix()
    size = {k: _footprint(k, probs[k]) for k in (0, 1)}
    # room for either factor alone, not for both: every switch of matrix evicts the idle one
    budget = max(size.values()) + 0.5 * min(size.values())
    srv = rs.Server(workers=1, hbm_budget_bytes=budget, **PARAMS)
    res = []
    for k in [0, 0, 1, 0]:
        p = probs[k]
        res.append(srv.wait(srv.submit(k, p.colptr, p.rowind, p.vals, np.stack(p.rhs[:1]), p.xyz)))
    assert [r[0] for r in res] == [0, 0, 0, 0]
    assert [r[3]["cache_hit"] for r in res] == [False, True, False, False]
    s = srv.stats()
    assert s["evictions"] == 2 and s["misses"] == 3 and s["hits"] == 1
    assert s["cached_bytes"] <= budget and s["cached_factors"] == 1
    srv.close()


@pytest.mark.gpu
def test_factor_above_the_budget_fails_with_oom():
    p = rs.diffusion(2, 32, seed=3)
    srv = rs.Server(workers=1, hbm_budget_bytes=1024.0, **PARAMS)
    st, x, info, t = srv.wait(srv.submit(0, p.colptr, p.rowind, p.vals, np.stack(p.rhs[:1]), p.xyz))
    assert st == 3   # RSCHOL_E_OOM
    assert srv.stats()["cached_factors"] == 0
    srv.close()
