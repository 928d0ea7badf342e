"""Programmatic dependent launch changes no result.

With it (the default) the GEMM, split-K reduction, conversion and BLAS-3 leaf
kernels may be scheduled while the previous kernel in the stream is still
running; each waits (griddepcontrol.wait) before its first global access. The
same calls in a process started with LATER_PDL=0 launch every kernel after the
previous one has ended. rgsqrf, rpotrf and a split-K GEMM must agree bit for
bit between the two: a missing wait would show up as a read of stale data.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

import later_gb300 as lg

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import sys
import numpy as np
import torch
import later_gb300 as lg

def spd(n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64)
    A = (X @ X.t()) / n + torch.eye(n, device="cuda", dtype=torch.float64)
    return lg.colmajor(A.float())

def run():
    out = {}
    g = torch.Generator(device="cuda").manual_seed(7)
    A = lg.colmajor(torch.randn(1024, 4096, generator=g, device="cuda").t())
    R = lg.later_rgsqrf(A, precision="split2")
    out["q"], out["r"] = A.cpu().numpy(), R.cpu().numpy()
    S = spd(4096, 8)
    lg.later_rpotrf("l", 4096, S)
    out["l"] = S.cpu().numpy()
    Ah = lg.empty_colmajor(16384, 256, dtype=torch.float16)
    Ah.copy_(torch.randn(16384, 256, generator=g, device="cuda"))
    work = torch.empty(1 << 24, device="cuda")
    out["g"] = lg.gemm16("T", "N", Ah, Ah, work=work).cpu().numpy()
    assert lg.device_status() == 0
    return out

if __name__ == "__main__":
    np.savez(sys.argv[1], **run())
"""


def test_results_identical_without_pdl(cuda, tmp_path):
    script = tmp_path / "pdl_case.py"
    script.write_text(SCRIPT)
    env = dict(os.environ, LATER_PDL="0", PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    off = tmp_path / "off.npz"
    r = subprocess.run([sys.executable, str(script), str(off)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    sys.path.insert(0, str(tmp_path))
    try:
        import pdl_case
        on = pdl_case.run()
    finally:
        sys.path.remove(str(tmp_path))
    ref = np.load(off)
    for k in ("q", "r", "l", "g"):
        assert np.array_equal(on[k], ref[k]), k
