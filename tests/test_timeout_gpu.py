"""Failure detection without a GPU fault: every device wait in the library is bounded, and a wait that
runs out is reported through the device status word as LATER_ERR_TIMEOUT while the context stays usable."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics

pytestmark = pytest.mark.gpu

TIMEOUT = 4  # LATER_ERR_TIMEOUT


def test_wait_that_never_completes_reports_timeout(cuda):
    # an mbarrier phase and a global flag that nothing completes; 100k cycles (about 50 us)
    lg.wait_selftest(timeout_cycles=100_000)
    assert lg.device_status() == TIMEOUT
    assert lg.device_status() == 0  # read and cleared
    # the context is still usable: an ordinary factorisation runs and is correct
    A = gen.normal(2048, 256, seed=3)
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    R = lg.later_rgsqrf(dA)
    assert lg.device_status() == 0
    assert metrics.qr_backward_error(A, dA.cpu().numpy(), R.cpu().numpy()) < 5e-4


def test_leaf_grid_barrier_budget_then_normal_call(cuda):
    """A 16384 x 128 rgsqrf is one fused-leaf launch whose CTAs meet at grid barriers. With a budget of
    a few cycles a CTA that waits at a barrier gives up, raises the abort flag that releases the others,
    and the launch ends with LATER_ERR_TIMEOUT (or completes if no CTA ever had to wait). Either way the
    barrier counters are reset by the last CTA out, so the next call with the default budget is exact."""
    A = gen.normal(16384, 128, seed=8)
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    lg.later_rgsqrf(dA, timeout_cycles=16)
    assert lg.device_status() in (0, TIMEOUT)
    dA.copy_(torch.from_numpy(A).cuda())
    R = lg.later_rgsqrf(dA)
    assert lg.device_status() == 0
    Q = dA.cpu().numpy()
    assert metrics.qr_backward_error(A, Q, R.cpu().numpy()) < 1e-5
    assert metrics.orthogonality(Q) < 1e-4
