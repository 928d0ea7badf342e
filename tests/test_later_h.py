"""Drop-in boundary: a client written against include/LATER.h builds, links and runs."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

import later_gb300 as lg

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "later_h_client.cu"


def _build(out: Path) -> Path:
    lib = lg.build.build()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", f"-I{ROOT / 'include'}",
           str(SRC), "-o", str(out), f"-L{lib.parent}", "-llater_gb300", f"-Xlinker=-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_later_h_client_compiles_and_links(tmp_path):
    exe = _build(tmp_path / "later_h_client")
    assert exe.exists()


def test_later_h_exports_cpp_symbols():
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-DC", str(lg.build.build())], capture_output=True, text=True).stdout
    for sym in ["later_rgsqrf(cudaCtxt", "later_rhouqr(cudaCtxt", "later_ormqr(int", "later_ormqr2(int", "later_bhouqr(int", "later_qdwh_polar(cudaCtxt", "later_sy2sb_rec(cudaCtxt", "ssytrd_sy2sb(cudaCtxt",
                "later_rtrsm(cublasContext*", "later_rsyrk(cublasContext*", "later_rtrmm(int", "later_rpotrf(char",
                "later_get_last_status()"]:
        assert sym in out, sym


@pytest.mark.gpu
def test_later_h_client_runs(cuda, tmp_path):
    exe = _build(tmp_path / "later_h_client")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
