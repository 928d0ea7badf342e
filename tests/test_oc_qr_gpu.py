"""later_c_oc_rgsqrf: the out-of-core QR (QR/later_oc_qr.cu:29-121) with A, Q and R in host memory,
run through a small device region so that the matrix is processed in several in-core panels."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics

pytestmark = pytest.mark.gpu


def _pinned(m, n):
    return torch.empty(n, m, pin_memory=True).t()


@pytest.mark.parametrize("m,n,panel,prec,cgs2,bound", [(4096, 2048, 512, "split2", False, 2e-6),
                                                       (8192, 1024, 256, "fp16", False, 5e-4),
                                                       (3000, 640, 128, "split3", True, 2e-6),
                                                       (16384, 4096, 1024, "split2", False, 3e-6)])
def test_oc_qr_through_a_small_device_region(cuda, m, n, panel, prec, cgs2, bound):
    A = gen.normal(m, n, seed=m + n + panel)
    hA = _pinned(m, n)
    hA.copy_(torch.from_numpy(A))
    hR = _pinned(n, n)
    hR.fill_(float("nan"))
    nbytes = lg.oc_rgsqrf_bytes(m, panel, prec, cgs2)  # room for one panel, two Q slots and the panel's QR
    assert n > panel  # several panels pass through the region
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    lg.later_oc_rgsqrf(hA, hR, dev, panel, precision=prec, cgs2=cgs2)
    assert lg.device_status() == 0
    torch.cuda.synchronize()
    Q, R = hA.numpy(), hR.numpy()
    assert np.all(np.isfinite(R)) and np.all(np.tril(R, -1) == 0) and np.all(np.diag(R) > 0)
    bwd, orth = metrics.qr_backward_error(A, Q, R), metrics.orthogonality(Q)
    assert bwd <= bound, bwd
    assert orth / n <= (5e-5 if prec == "fp16" else 1e-5), orth
    # the in-core factorisation in the same precision gives the same R to its working accuracy
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    R2 = lg.later_rgsqrf(dA, precision=prec, cgs2=cgs2).cpu().numpy()
    tol = 5e-4 if prec in ("fp16", "split2") else 1e-5
    assert np.linalg.norm(R - R2) / np.linalg.norm(R2) <= tol
