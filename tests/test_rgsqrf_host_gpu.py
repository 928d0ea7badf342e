"""later_c_rgsqrf_host: the factorisation with the matrix in host memory, copied in and out in column
chunks overlapped with the recursion. The result is bit-identical to the device-buffer call on the same
input (the copies change when things happen, not what is computed)."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics

pytestmark = pytest.mark.gpu


def _pinned(m, n):
    return torch.empty(n, m, pin_memory=True).t()  # column-major


@pytest.mark.parametrize("m,n,prec", [(4096, 1024, "fp16"), (16384, 2048, "split2"), (3000, 640, "split3"),
                                      (8192, 8192, "split2"), (2048, 96, "fp16")])
def test_host_variant_is_bit_identical(cuda, m, n, prec):
    A = gen.normal(m, n, seed=m + n)
    hA = _pinned(m, n)
    hA.copy_(torch.from_numpy(A))
    hQ = _pinned(m, n)
    hR = _pinned(n, n)
    hR.zero_()
    dA = lg.empty_colmajor(m, n)
    dR = lg.empty_colmajor(n, n)
    lg.later_rgsqrf_host(hA, hQ, hR, dA, dR, precision=prec)
    assert lg.device_status() == 0
    torch.cuda.synchronize()
    dA2 = lg.colmajor(torch.from_numpy(A).cuda())
    R2 = lg.later_rgsqrf(dA2, precision=prec)
    assert lg.device_status() == 0
    assert torch.equal(hQ, dA2.cpu())
    assert torch.equal(torch.triu(hR), torch.triu(R2.cpu()))
    assert torch.equal(dR.cpu(), R2.cpu())


def test_host_variant_in_place_and_repeated(cuda):
    """hQ may be hA (Q overwrites A on the host, like the reference's A -> Q); calls back to back on one
    stream reuse the copy streams and see each other's results in order."""
    m, n = 8192, 1024
    A = gen.normal(m, n, seed=3)
    dA = lg.empty_colmajor(m, n)
    dR = lg.empty_colmajor(n, n)
    outs = []
    for _ in range(3):
        hA = _pinned(m, n)
        hA.copy_(torch.from_numpy(A))
        hR = _pinned(n, n)
        hR.zero_()
        lg.later_rgsqrf_host(hA, hA, hR, dA, dR, precision="split2")
        outs.append((hA, hR))
    assert lg.device_status() == 0
    torch.cuda.synchronize()
    for hQ, hR in outs:
        assert torch.equal(hQ, outs[0][0]) and torch.equal(hR, outs[0][1])
    Q, R = outs[0][0].numpy(), np.triu(outs[0][1].numpy())
    assert metrics.qr_backward_error(A, Q, R) < 2e-6
