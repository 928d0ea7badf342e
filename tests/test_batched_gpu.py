"""Batched uneven tall-skinny QR in one persistent launch, against FP64 LAPACK and per-matrix rgsqrf."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import metrics

pytestmark = pytest.mark.gpu


def _shapes(count, seed, mmax=2048, nmax=128):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        m = int(np.exp(rng.uniform(np.log(256), np.log(mmax))))
        n = int(np.exp(rng.uniform(np.log(16), np.log(nmax))))
        if m >= 4 * n:
            out.append((m, n))
    return out


def _mats(shapes, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return [torch.randn(n, m, generator=g, device="cuda").t() for m, n in shapes]  # column-major m x n


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_batched_matches_lapack(cuda, variant):
    shapes = _shapes(96, seed=1)
    mats = _mats(shapes, seed=2)
    orig = [a.cpu().numpy() for a in mats]
    b = lg.BatchedQR(mats)
    b.run(variant)
    assert lg.device_status() == 0
    assert int(b.status.abs().sum()) == 0
    for a0, q, r in zip(orig, b.mats, b.rs):
        Q, R = q.cpu().numpy(), r.cpu().numpy()
        assert metrics.qr_backward_error(a0, Q, R) < 2e-6
        assert metrics.orthogonality(Q) < 2e-5
        _, Rx = metrics.lapack_qr_positive(a0)
        assert np.linalg.norm(R - Rx) / np.linalg.norm(Rx) < 2e-6
        assert np.all(np.tril(R, -1) == 0)


def test_batched_graph_capture_and_determinism(cuda):
    shapes = _shapes(64, seed=3, mmax=4096, nmax=256)
    mats = _mats(shapes, seed=4)
    orig = [a.clone() for a in mats]
    b = lg.BatchedQR(mats)
    b.run(0)
    torch.cuda.synchronize()
    ref = [r.clone() for r in b.rs]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            b.run(0, stream=s)
    for a, o in zip(mats, orig):
        a.copy_(o)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    for r, r0 in zip(b.rs, ref):
        assert torch.equal(r, r0)


def test_batched_agrees_with_rgsqrf_loop(cuda):
    shapes = [(1024, 64), (2048, 96), (512, 32), (4096, 256)]
    mats = _mats(shapes, seed=5)
    loop = [a.clone() for a in mats]
    b = lg.BatchedQR(mats)
    b.run(1)
    for a, rb in zip(loop, b.rs):
        R = lg.later_rgsqrf(a, precision="split3")
        assert torch.allclose(R, rb, rtol=1e-4, atol=1e-4 * float(rb.abs().max()))


def test_autotuner_picks_a_variant(cuda, tmp_path, monkeypatch):
    from later_gb300 import autotune
    monkeypatch.setenv("LATER_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    shapes = _shapes(128, seed=6)
    best, times = autotune.tune(shapes, sample=32, reps=1)
    assert best in times and len(times) == autotune.N_VARIANTS
    best2, _ = autotune.tune(shapes, sample=32, reps=1)  # cached
    assert best2 == best
