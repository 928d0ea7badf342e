"""The C-ABI library builds, loads and exports every entry point the headers declare (no GPU needed)."""
import re
import subprocess
from pathlib import Path

import later_gb300 as lg

ROOT = Path(__file__).resolve().parent.parent


def _declared_c_symbols():
    text = (ROOT / "include" / "later_c.h").read_text()
    return sorted(set(re.findall(r"\b(later_c_\w+)\s*\(", text)))


def test_library_loads_and_exports_c_abi():
    l = lg.lib()
    names = _declared_c_symbols()
    assert names, "no declarations found"
    for name in names:
        assert hasattr(l, name), name


def test_default_options_and_status_strings():
    import ctypes
    l = lg.lib()
    o = lg.Options()
    l.later_c_default_options(ctypes.byref(o))
    assert (o.precision, o.cgs2, o.leaf) == (0, 0, 128)
    assert l.later_c_status_string(2) == b"workspace too small"


def test_bufsize_query_cpu():
    lw, lh = lg.rgsqrf_bufsize(4096, 1024)
    assert lh >= 4096 * 1024
    # The reference test's own work size (test/test_qr.cu:69) is enough to run.
    assert lw > 0


def test_split2_workspace_holds_the_lo_copy():
    # SPLIT2 keeps Q's lo copy for the A2 -= Q1 R12 update: the same 16-bit workspace as SPLIT3,
    # twice the FP16 one.
    _, h16 = lg.rgsqrf_bufsize(4096, 1024, precision="fp16")
    _, h2 = lg.rgsqrf_bufsize(4096, 1024, precision="split2")
    _, h3 = lg.rgsqrf_bufsize(4096, 1024, precision="split3")
    assert h2 == h3 == 2 * h16


def test_split2_is_rejected_outside_rgsqrf():
    import pytest
    # SPLIT2 is a trailing-update mode of the QR recursion; the BLAS3 / Cholesky routines refuse it.
    for op in ("s", "t", "m", "p"):
        with pytest.raises(lg.LaterError):
            lg.blas3_bufsize(op, 512, 512, precision="split2")
    lg.blas3_bufsize("p", 512, 512, precision="split3")  # the other modes stay valid
