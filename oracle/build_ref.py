"""Recipe for oracle/_ref: the reference LATER on the GPU (test infrastructure only).

Two outputs, both into oracle/_ref/ (git-ignored, carried to the GPU machine with
the rest of the tree):

1. Cubins of the reference's own device code, compiled for sm_103a from its
   sources where they lie (QR/panel.cu -> panel.cubin, util/util.cu ->
   util.cubin). This needs the reference tree and runs only where it is
   present; the GPU machine uses the cubins built here (device code, not host
   code, so they run there unchanged). The sources compile unmodified with
   three command-line shims, explained in oracle/ref_shim.h: a force-included
   stub of the texture-reference template that the vendored CUB 1.8.0 names,
   CUB_NS_QUALIFIER for CUDA 13's CUB, and a macro for the removed
   cudaDeviceProp::clockRate in util/util.cu's host-only print_env.
2. oracle/_ref/libref_harness.so from oracle/ref_harness.cu (this project's
   code: the reference's host recursion restated call for call around those
   kernels and cuBLAS / cuSOLVER). Built wherever nvcc and the CUDA libraries
   are, for the machine it runs on.

`load()` returns the harness bound to the current device and a stream, or
None when either output is missing.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REF = Path(os.environ.get("LATER_REFERENCE_DIR", "/root/reference"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUBINS = {"panel.cubin": "QR/panel.cu", "util.cubin": "util/util.cu"}
HARNESS = OUT / "libref_harness.so"


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def build_cubins(force: bool = False) -> bool:
    """Compiles the reference's device code (needs the reference tree). True if the cubins exist after."""
    OUT.mkdir(exist_ok=True)
    if not REF.is_dir():
        return all((OUT / c).exists() for c in CUBINS)
    for cubin, src in CUBINS.items():
        out = OUT / cubin
        if out.exists() and not force:
            continue
        cmd = [_nvcc(), "-cubin", *ARCH, "-O3", "-w", "-include", str(HERE / "ref_shim.h"),
               "-DCUB_NS_QUALIFIER=::cub", "-DclockRate=l2CacheSize",
               f"-I{REF / 'include'}", f"-I{REF / 'QR' / 'include'}", str(REF / src), "-o", str(out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference cubin {cubin} failed:\n{r.stderr[-4000:]}")
    return True


def build_harness(force: bool = False) -> bool:
    """Compiles oracle/ref_harness.cu for this machine. True on success."""
    OUT.mkdir(exist_ok=True)
    src = HERE / "ref_harness.cu"
    if HARNESS.exists() and not force and HARNESS.stat().st_mtime > src.stat().st_mtime:
        return True
    home = _cuda_home()
    libdirs = [p for p in (home / "lib64", home / "lib64" / "stubs", home / "lib", home / "lib" / "stubs")
               if p.is_dir()]
    cmd = [_nvcc(), *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", str(src), "-o", str(HARNESS),
           *[f"-L{p}" for p in libdirs], "-lcublas", "-lcusolver", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(f"reference harness not built: {r.stderr[-2000:]}", file=sys.stderr)
        return False
    return True


def build(force: bool = False) -> bool:
    ok = build_cubins(force)
    return build_harness(force) and ok


def available() -> bool:
    return HARNESS.exists() and all((OUT / c).exists() for c in CUBINS)


class RefLater:
    """The reference's rgsqrf / rpotrf on the GPU, and cuSOLVER's Sgeqrf / Spotrf, on torch tensors."""

    def __init__(self, lib, stream):
        self.lib = lib
        self.stream = stream

    def rgsqrf(self, A, R, work, hwork):
        """A (m x n, lda == m, column-major FP32) -> Q in place; R (n x n) upper part written."""
        m, n = A.shape
        assert A.stride(0) == 1 and A.stride(1) == m
        r = self.lib.ref_rgsqrf(m, n, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(R.data_ptr()), R.stride(1),
                                ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(hwork.data_ptr()))
        if r:
            raise RuntimeError(f"reference rgsqrf failed ({r})")

    @staticmethod
    def rgsqrf_bufsize(m, n):
        """(work floats, hwork halves) as the reference's QR test allocates them (test/test_qr.cu:75-80)."""
        return m // 256 * 32 * n, m * n

    def rpotrf(self, A, hwork):
        n = A.shape[0]
        assert A.stride(0) == 1 and A.stride(1) == n
        info = ctypes.c_int(0)
        r = self.lib.ref_rpotrf(n, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(hwork.data_ptr()),
                                ctypes.byref(info))
        if r:
            raise RuntimeError(f"reference rpotrf failed ({r})")
        return info.value

    def sgeqrf(self, A, tau, work, dinfo):
        m, n = A.shape
        r = self.lib.ref_sgeqrf(m, n, ctypes.c_void_p(A.data_ptr()), A.stride(1), ctypes.c_void_p(tau.data_ptr()),
                                ctypes.c_void_p(work.data_ptr()), work.numel(), ctypes.c_void_p(dinfo.data_ptr()))
        if r:
            raise RuntimeError(f"cusolverDnSgeqrf failed ({r})")

    def sgeqrf_bufsize(self, A):
        m, n = A.shape
        lw = ctypes.c_int(0)
        if self.lib.ref_sgeqrf_bufsize(m, n, ctypes.c_void_p(A.data_ptr()), A.stride(1), ctypes.byref(lw)):
            raise RuntimeError("cusolverDnSgeqrf_bufferSize failed")
        return lw.value

    def spotrf(self, A, work, dinfo):
        n = A.shape[0]
        r = self.lib.ref_spotrf(n, ctypes.c_void_p(A.data_ptr()), A.stride(1), ctypes.c_void_p(work.data_ptr()),
                                work.numel(), ctypes.c_void_p(dinfo.data_ptr()))
        if r:
            raise RuntimeError(f"cusolverDnSpotrf failed ({r})")

    def spotrf_bufsize(self, A):
        n = A.shape[0]
        lw = ctypes.c_int(0)
        if self.lib.ref_spotrf_bufsize(n, ctypes.c_void_p(A.data_ptr()), A.stride(1), ctypes.byref(lw)):
            raise RuntimeError("cusolverDnSpotrf_bufferSize failed")
        return lw.value


def load(stream=None):
    """The harness on the current device, bound to `stream` (torch's current stream by default), or None."""
    if not available():
        return None
    import torch
    lib = ctypes.CDLL(str(HARNESS))
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.ref_init.argtypes = [ctypes.c_char_p, vp]
    lib.ref_rgsqrf.argtypes = [i, i, vp, vp, i, vp, vp]
    lib.ref_rpotrf.argtypes = [i, vp, vp, ctypes.POINTER(i)]
    lib.ref_sgeqrf_bufsize.argtypes = [i, i, vp, i, ctypes.POINTER(i)]
    lib.ref_sgeqrf.argtypes = [i, i, vp, i, vp, vp, i, vp]
    lib.ref_spotrf_bufsize.argtypes = [i, vp, i, ctypes.POINTER(i)]
    lib.ref_spotrf.argtypes = [i, vp, i, vp, i, vp]
    st = stream if stream is not None else torch.cuda.current_stream()
    r = lib.ref_init(str(OUT).encode(), ctypes.c_void_p(st.cuda_stream))
    if r:
        raise RuntimeError(f"reference harness init failed ({r})")
    return RefLater(lib, st)


if __name__ == "__main__":
    print("cubins:", build_cubins(force="--force" in sys.argv), "harness:", build_harness(force="--force" in sys.argv))
