"""Least-squares serving loop: continuous batching under an HBM budget."""

import numpy as np
import pytest

import later_gb300 as lg
from oracle import gen

pytestmark = pytest.mark.gpu


def _requests(count, seed, mmax=4096, nmax=384):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        m = int(np.exp(rng.uniform(np.log(512), np.log(mmax))))
        n = int(np.exp(rng.uniform(np.log(32), np.log(nmax))))
        if m < 2 * n:
            continue
        kappa = float(np.exp(rng.uniform(np.log(10), np.log(1e4))))
        A = gen.svd_matrix(m, n, kappa, seed=len(out) + 100 * seed)
        xs = rng.standard_normal((n, 1))
        B = (A.astype(np.float64) @ xs + 1e-3 * rng.standard_normal((m, 1))).astype(np.float32)
        out.append((A, B))
    return out


def test_same_result_alone_and_in_the_mix(cuda):
    reqs = _requests(8, seed=1)
    alone = []
    srv = lg.LsServer(slots=1, hbm_budget_gb=4)
    for A, B in reqs:
        X, res = srv.wait(srv.submit(A, B))
        assert res["status"] == 0 and res["backward_error"] <= 1e-6, res
        alone.append(X)
    srv.close()
    srv = lg.LsServer(slots=4, hbm_budget_gb=4)
    tickets = [srv.submit(A, B) for A, B in reqs]
    outs = [srv.wait(t) for t in tickets]
    srv.close()
    slots = {r["slot"] for _, r in outs}
    assert len(slots) > 1  # the mix really ran on several slots
    for (X, r), Xa in zip(outs, alone):
        assert r["status"] == 0 and r["backward_error"] <= 1e-6, r
        # Same algorithm, same kernels, per-request workspaces: identical to FP64 round-off.
        assert np.max(np.abs(X - Xa)) <= 1e-12 * max(1.0, np.max(np.abs(Xa))), np.max(np.abs(X - Xa))


def test_admission_respects_the_hbm_budget(cuda):
    reqs = _requests(6, seed=2, mmax=4096, nmax=256)
    budget_gb = 0.2
    srv = lg.LsServer(slots=4, hbm_budget_gb=budget_gb)
    tickets = [srv.submit(A, B) for A, B in reqs]
    outs = [srv.wait(t) for t in tickets]
    assert all(r["status"] == 0 for _, r in outs)
    # the pool's own high-water mark: something was admitted, never beyond the budget
    assert 0 < srv.hbm_peak() <= budget_gb * (1 << 30)
    assert srv.hbm_in_use() == 0
    # A request larger than the whole budget is refused up front.
    big = gen.normal(16384, 1024, seed=3)
    with pytest.raises(lg.LaterError) as e:
        srv.submit(big, np.ones((16384, 1), np.float32))
    assert e.value.status == 2
    srv.close()
