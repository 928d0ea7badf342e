"""Benchmark: recursive tensor-core QR (later_rgsqrf) on one GB300.

Workload (default): rgsqrf of a 16384 x 16384 FP32 matrix, entries N(0,1)
from a fixed seed, leaf panel width 128 — the square shape of the QR precision
sweep — with SPLIT2 tensor-core trailing updates (FP16 products, FP32
accumulation, the update's Q operand split hi + lo), the mode whose backward
error ||A - QR|| / ||A|| stays below 1e-5. The same matrix is also timed with
plain FP16 updates (the reference's only mode) and reported under
`alt_precision`. The metric is the reference's QR rate, 2 n^2 (m - n/3) / t
(test/test_qr.cu:85-86), in TFLOP/s, reported beside the backward error.

The same line carries, under `configs`, the QR precision sweep (rgsqrf and rhouqr
over SVD-built 16384 x 16384 and 65536 x 4096 inputs, kappa 1e1 / 1e3 / 1e5, every
precision mode, with probe-estimated FP64 errors), the Cholesky + refined SPD solve,
the batched QR and the least-squares serving loop; `--config sweep | spd | batched |
serve` runs one of them alone.

A step is one QR of the full matrix. The matrix (1 GiB) is larger than L2, and
it is restored from a pristine device copy before each step (outside the
per-step events). `value` is the device-timed rate with inputs resident in
HBM; `e2e` is the same QR through the public API with the matrix copied from
pinned host memory and Q and R copied back inside the timed region.

--impl reference times the reference LATER's own rgsqrf on the same GPU and
matrix (its kernels compiled from its sources into oracle/_ref, its host
recursion restated with the same cuBLAS calls), device time and end to end
with plain memcpys around the call; where oracle/_ref is not built, the
oracle's numpy restatement on the host cores, on a bounded sample.

Multi-GPU: a single QR does not shard (replicas only); under torchrun every
rank factors its own matrix and `value` sums the ranks' rates (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "QR TFLOP/s (LAPACK count 2n^2(m-n/3)) at stated ||A-QR||/||A||"
# Untimed end-to-end passes before the timed ones, in both arms: on GB300 the first passes over freshly
# pinned host buffers (2.6 GB per QR) take up to twice the steady time (55, 35, 28, 28 ms measured).
E2E_WARMUP = 4
# Timed end-to-end passes, in both arms, and the statistic reported: the median pass. On these boxes a
# pass now and then takes far longer in either arm (66 and 104 ms against 27 ms for ours; 168, 168 and
# 128 against 80 ms for the reference's, in one run; the SM clock steady and the measured copy rate
# unchanged): the host side of the copies, not the factorisation. Nine passes keep the median on a
# steady pass with up to four such outliers. Every pass and the mean are in the line as well.
E2E_PASSES = 9
E2E_STATISTIC = "median of the timed passes (pass_ms lists them; mean_ms_per_step is their mean)"


def qr_flops(m, n):
    return 2.0 * n * n * (m - n / 3.0)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--m", type=int, default=16384)
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--precision", default=None, choices=["fp16", "bf16", "split3", "split2"],
                   help="tensor-core precision (default: split2 for qr, fp16 for spd)")
    p.add_argument("--alt-precision", default="fp16", choices=["none", "fp16", "bf16", "split3", "split2"],
                   help="qr: also time this precision on the same matrix (reported under alt_precision)")
    p.add_argument("--leaf", type=int, default=128)
    p.add_argument("--panel", default="fused", choices=["fused", "wide", "mgs"],
                   help="rgsqrf leaf: fused 32-column CholQR2 panels (default), fused leaf-wide CholQR2 first, "
                        "or the reference's MGS-TSQR panels")
    p.add_argument("--cgs2", action="store_true")
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--e2e-steps", type=int, default=E2E_PASSES)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-ref", action="store_true", help="skip the same-GPU reference / cuSOLVER comparators")
    p.add_argument("--no-extras", action="store_true",
                   help="qr: skip the C2 sweep and the C3 / C4 / C5 configurations that follow the headline in "
                        "the same line")
    p.add_argument("--cpu-m", type=int, default=16384, help="CPU sample rows")
    p.add_argument("--cpu-n", type=int, default=1024, help="CPU sample columns")
    p.add_argument("--config", default="qr", choices=["qr", "spd", "batched", "serve", "sweep"],
                   help="qr: rgsqrf (default, the headline); spd: rpotrf + FP64-refined SPD solve; "
                        "batched: 4096 uneven tall-skinny QRs in one persistent launch; serve: LS serving loop; "
                        "sweep: rgsqrf / rhouqr precision sweep over SVD-built inputs")
    p.add_argument("--sweep-small", action="store_true", help="sweep: smaller shapes (a quick check)")
    p.add_argument("--kappa", type=float, default=1e2, help="spd: condition number")
    p.add_argument("--count", type=int, default=4096, help="batched: number of matrices")
    p.add_argument("--rates", type=float, nargs="*", default=None,
                   help="serve: arrival rates as multiples of the measured one-at-a-time rate")
    p.add_argument("--requests", type=int, default=1000, help="serve: requests per rate")
    p.add_argument("--slots", type=int, default=4, help="serve: server slots")
    p.add_argument("--gemm", type=int, nargs=3, metavar=("M", "N", "K"), default=None,
                   help="time only the tensor-core GEMM R12 = Q1^T A2 of this shape (TN, FP16) — the "
                        "top-level trailing-update product of rgsqrf; used for kernel profiling")
    return p.parse_args()


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, interval_ms=200):
        self.index = index
        self.interval_ms = interval_ms
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------- FP64 metrics
def qr_errors_fp64(A, Q, R, block=2048):
    """||A - QR||_F / ||A||_F and ||I - Q^T Q||_F with FP64 products on the GPU, in column blocks
    (R upper triangular: block J of A - QR needs Q[:, :J_end]; Q^T Q symmetric: blocks on and above
    the diagonal, off-diagonal ones counted twice)."""
    import torch
    m, n = Q.shape
    Qd = Q.double()
    num = torch.zeros((), dtype=torch.float64, device=Q.device)
    den = torch.zeros((), dtype=torch.float64, device=Q.device)
    orth = torch.zeros((), dtype=torch.float64, device=Q.device)
    for j0 in range(0, n, block):
        j1 = min(n, j0 + block)
        Ab = A[:, j0:j1].double()
        res = Ab - Qd[:, :j1] @ torch.triu(R[:j1, j0:j1].double(), diagonal=-j0)
        num += (res * res).sum()
        den += (Ab * Ab).sum()
        G = Qd[:, j0:j1].t() @ Qd[:, j0:]
        G[:, : j1 - j0] -= torch.eye(j1 - j0, dtype=torch.float64, device=Q.device)
        orth += (G[:, : j1 - j0] ** 2).sum() + 2.0 * (G[:, j1 - j0:] ** 2).sum()
    return float(torch.sqrt(num / den)), float(torch.sqrt(orth))


# ------------------------------------------------------------ CPU baselines
def cpu_oracle_rate(m, n, seed, prec="fp16"):
    """Times the oracle restatement of later_rgsqrf (numpy, all host threads) on an m x n sample;
    prec fp16 is the reference's own arithmetic."""
    import numpy as np
    from oracle import gen
    from oracle import later_oracle as lo
    A = gen.normal(m, n, seed)
    lo.rgsqrf(A[: min(m, 2048), : min(n, 256)], prec=prec)  # warm-up (BLAS threads, caches)
    t = time.perf_counter()
    lo.rgsqrf(A, prec=prec)
    dt = time.perf_counter() - t
    return qr_flops(m, n) / dt / 1e12, dt


def host_sgeqrf_rate(m, n, seed):
    """Host LAPACK sgeqrf (scipy's bundled OpenBLAS, all host cores) on an m x n sample."""
    try:
        import scipy.linalg.lapack as la
    except Exception:
        return None, None
    from oracle import gen
    A = gen.normal(m, n, seed)
    la.sgeqrf(A[:1024, :256].copy(order="F"))
    t = time.perf_counter()
    la.sgeqrf(A, overwrite_a=True)
    dt = time.perf_counter() - t
    return qr_flops(m, n) / dt / 1e12, dt


def flat(t):
    """The storage of a column-major (m x n, strides (1, m)) tensor as one contiguous vector: copies
    between such host and device tensors then run as single plain memcpys (about 200 GB/s each way on
    GB300), where copy_ on the transposed views takes a several times slower strided path."""
    v = t.t()
    assert v.is_contiguous()
    return v.reshape(-1)


def time_reference_gpu(a, A0, ref, steps, warmup, clocks=False):
    """The reference LATER's rgsqrf on this GPU (oracle/_ref: its kernels compiled from its sources,
    its host recursion restated call for call with the same cuBLAS calls) on the device matrix A0:
    device-timed steps, FP64 accuracy of the last one, and the end-to-end time with the matrix copied
    from pinned host memory and Q, R copied back."""
    import torch
    m, n = A0.shape
    dev = A0.device
    A = torch.empty(n, m, device=dev).t()
    R = torch.zeros(n, n, device=dev).t()
    lw, lh = ref.rgsqrf_bufsize(m, n)
    work = torch.zeros(max(lw, m // 256 * 32 * 64), device=dev)
    hwork = torch.zeros(lh, dtype=torch.float16, device=dev)
    st = torch.cuda.current_stream()
    for _ in range(warmup):
        A.copy_(A0)
        ref.rgsqrf(A, R, work, hwork)
    torch.cuda.synchronize()
    # end to end first, right after the warm-up (as in our arm)
    hA = torch.empty(n, m, pin_memory=True).t()
    hA.copy_(A0)
    hQ = torch.empty(n, m, pin_memory=True).t()
    hR = torch.empty(n, n, pin_memory=True).t()

    def step():
        flat(A).copy_(flat(hA), non_blocking=True)
        ref.rgsqrf(A, R, work, hwork)
        flat(hQ).copy_(flat(A), non_blocking=True)
        flat(hR).copy_(flat(R), non_blocking=True)

    # warm-up: the first passes over freshly pinned host buffers run slower (about 2x for the first
    # two on GB300) before the copies reach their steady rate
    for _ in range(E2E_WARMUP):
        step()
    torch.cuda.synchronize()
    k = E2E_PASSES
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
    marks[0].record(st)
    for i in range(k):
        step()
        marks[i + 1].record(st)
    torch.cuda.synchronize()
    e2e_pass_ms = [round(marks[i].elapsed_time(marks[i + 1]), 3) for i in range(k)]
    e2e_mean_ms = marks[0].elapsed_time(marks[k]) / k
    e2e_ms = statistics.median(e2e_pass_ms)
    evs = []
    clk = ClockSampler(dev.index or 0) if clocks else None
    if clk:
        clk.__enter__()
    for _ in range(steps):
        A.copy_(A0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ref.rgsqrf(A, R, work, hwork)
        e1.record(st)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if clk:
        clk.__exit__()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / steps
    bwd, orth = qr_errors_fp64(A0, A, torch.triu(R))
    out = {"ms_per_step": ms, "value": qr_flops(m, n) / ms / 1e9, "unit": "TFLOP/s",
           "backward_error": bwd, "orthogonality_over_n": orth / n, "e2e_ms": e2e_ms,
           "e2e": qr_flops(m, n) / e2e_ms / 1e9, "e2e_pass_ms": e2e_pass_ms, "e2e_mean_ms": e2e_mean_ms}
    if clk:
        out["clocks"] = clk.summary()
    return out


def time_cusolver_sgeqrf(A0, ref, steps=3):
    """cusolverDnSgeqrf on the same matrix: the reference QR test's own FP32 GPU comparator
    (test/test_qr.cu:184-206). Math mode default: FP32 arithmetic, no TF32."""
    import torch
    m, n = A0.shape
    A = torch.empty(n, m, device=A0.device).t()
    A.copy_(A0)
    tau = torch.empty(n, device=A0.device)
    lw = ref.sgeqrf_bufsize(A)
    work = torch.empty(max(1, lw), device=A0.device)
    info = torch.zeros(1, dtype=torch.int32, device=A0.device)
    st = torch.cuda.current_stream()
    ref.sgeqrf(A, tau, work, info)
    ts = []
    for _ in range(steps):
        A.copy_(A0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ref.sgeqrf(A, tau, work, info)
        e1.record(st)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ms = statistics.median(ts)
    return {"impl": "cusolverDnSgeqrf FP32 (test/test_qr.cu:184-206)", "ms_per_step": ms,
            "value": qr_flops(m, n) / ms / 1e9, "unit": "TFLOP/s", "info": int(info.item())}


def reference_gpu_harness():
    """The reference LATER on this GPU, or None (not built / no device)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        from oracle import build_ref
        if not build_ref.available():
            build_ref.build()
        return build_ref.load()
    except Exception as e:  # noqa: BLE001
        print(f"reference harness unavailable: {e}", file=sys.stderr)
        return None


def run_reference(a, rank, world):
    """The reference arm. On a GPU with oracle/_ref built: the reference LATER's own rgsqrf (its
    kernels and cuBLAS, FP16 tensor-core GEMMs, the only mode it has) on the same 16384^2 matrix,
    timed like our arm. Otherwise the oracle's port of it on the host cores, on a bounded sample."""
    if rank != 0:
        return
    ncores = os.cpu_count() or 1
    ref = reference_gpu_harness()
    if ref is not None:
        import torch
        torch.cuda.set_device(0)
        g = torch.Generator(device="cuda").manual_seed(a.seed)
        A0 = torch.randn(a.n, a.m, generator=g, device="cuda").t()
        r = time_reference_gpu(a, A0, ref, a.steps, a.warmup, clocks=True)
        cfg = workload_config(a)
        cfg = dict(cfg, workload=f"rgsqrf {a.m}x{a.n} fp32, N(0,1) seed {a.seed}, the reference's FP16 "
                                 f"tensor-core trailing updates (cuBLAS GemmEx), leaf 128", precision="fp16")
        sample = ("the reference LATER on this GPU: its mgs_kernel2 / s2h kernels compiled from its sources "
                  "(oracle/_ref cubins), its host recursion (QR/later_rgsqrf.cu, QR/panel.cu) restated call for "
                  "call with the same cuBLAS GemmEx / Sgemm / SgemmStridedBatched calls; full matrix")
        line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": "TFLOP/s", "n_gpus": 1,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp16", "data": "synthetic", "config": cfg,
                "accuracy": {"backward_error": r["backward_error"], "orthogonality_over_n": r["orthogonality_over_n"],
                             "computed": "FP64 on the GPU"},
                "cpu_baseline": {"value": r["value"], "unit": "TFLOP/s", "cores": ncores, "kind": "reference",
                                 "device": "GPU", "sample": sample},
                "e2e": {"value": r["e2e"], "unit": "TFLOP/s", "ms_per_step": r["e2e_ms"], "statistic": E2E_STATISTIC,
                        "mean_ms_per_step": r["e2e_mean_ms"], "pass_ms": r["e2e_pass_ms"],
                        "h2d_bytes_per_step": a.m * a.n * 4, "d2h_bytes_per_step": a.m * a.n * 4 + a.n * a.n * 4},
                "clocks": r.get("clocks")}
        print(json.dumps(line), flush=True)
        return
    rates = []
    for _ in range(a.warmup):
        cpu_oracle_rate(a.cpu_m, a.cpu_n, a.seed)
    for _ in range(a.steps):
        r, _ = cpu_oracle_rate(a.cpu_m, a.cpu_n, a.seed)
        rates.append(r)
    v = statistics.median(rates)
    sample = (f"oracle restatement of later_rgsqrf in the reference's own FP16 arithmetic (numpy, fp16-rounded "
              f"GEMM operands) on {a.cpu_m}x{a.cpu_n}, N(0,1) seed {a.seed}")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": qr_flops(a.cpu_m, a.cpu_n) / v / 1e9,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp16",
            "data": "synthetic",
            "config": {"workload": f"rgsqrf {a.cpu_m}x{a.cpu_n} fp32 sample, N(0,1) seed {a.seed}, FP16-rounded "
                                   f"GEMM operands (the reference's arithmetic), leaf 128, on the host cores",
                       "m": a.cpu_m, "n": a.cpu_n, "precision": "fp16", "leaf": 128,
                       "sample_of": workload_config(a)["workload"]},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": ncores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(a):
    return {"workload": f"rgsqrf {a.m}x{a.n} fp32, N(0,1) seed {a.seed}, {a.precision} tensor-core trailing "
                        f"updates, leaf {a.leaf}{', CGS2' if a.cgs2 else ''}",
            "m": a.m, "n": a.n, "precision": a.precision, "leaf": a.leaf, "cgs2": a.cgs2, "panel": a.panel,
            "l2": "inputs larger than L2 (matrix >= 1 GiB at the default size)"}


# ------------------------------------------------------------------ ours
def run_ours(a, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    import later_gb300 as lg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    m, n = a.m, a.n
    flops = qr_flops(m, n)
    g = torch.Generator(device=dev).manual_seed(a.seed + rank)
    A0 = torch.randn(n, m, generator=g, device=dev).t()  # column-major m x n
    A = lg.empty_colmajor(m, n, device=dev)
    R = lg.empty_colmajor(n, n, device=dev)
    lw, lh = lg.rgsqrf_bufsize(m, n, a.precision, a.cgs2, a.leaf)
    work = torch.empty(lw, dtype=torch.float32, device=dev)
    hwork = torch.empty(lh, dtype=torch.float16, device=dev)
    st = torch.cuda.current_stream()

    def qr():
        lg.later_rgsqrf(A, R, work, hwork, precision=a.precision, cgs2=a.cgs2, leaf=a.leaf, panel=a.panel)

    for _ in range(a.warmup):
        A.copy_(A0)
        qr()
    status = lg.device_status()
    if status != 0:
        raise RuntimeError(f"device status {status} during warm-up")

    # ---- end to end through the public API with host buffers: later_c_rgsqrf_host copies pinned host A
    # in and Q, R (upper triangle) out in column chunks overlapped with the factorisation. Measured first,
    # right after the warm-up, like the reference arm (a process of its own): after the FP64 accuracy
    # check and the same-GPU comparators one pass in three ran about 13 ms slower on some boxes, while in a
    # process doing nothing else every pass took 27.1-27.8 ms
    e2e = None
    if a.e2e_steps > 0:
        hA = torch.empty(n, m, pin_memory=True).t()  # column-major like A
        hA.copy_(A0)
        hQ = torch.empty(n, m, pin_memory=True).t()
        hR = torch.empty(n, n, pin_memory=True).t()

        def qr_host():
            lg.later_rgsqrf_host(hA, hQ, hR, A, R, work, hwork, precision=a.precision, cgs2=a.cgs2, leaf=a.leaf,
                                 panel=a.panel)

        for _ in range(E2E_WARMUP):  # fresh pinned buffers: the first passes run slower
            qr_host()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        marks = [torch.cuda.Event(enable_timing=True) for _ in range(a.e2e_steps + 1)]
        eclk = ClockSampler(dev.index or 0, interval_ms=20)
        eclk.__enter__()
        time.sleep(0.2)  # the sampler's first reading
        e0.record(st)
        marks[0].record(st)
        for i in range(a.e2e_steps):
            qr_host()
            marks[i + 1].record(st)
        e1.record(st)
        torch.cuda.synchronize()
        eclk.__exit__()
        mean_ms = e0.elapsed_time(e1) / a.e2e_steps
        pass_ms = [round(marks[i].elapsed_time(marks[i + 1]), 3) for i in range(a.e2e_steps)]
        e2e_ms = statistics.median(pass_ms)
        # bytes copied out: Q, and per column chunk of R the rows on and above the diagonal
        units = -(-n // a.leaf)
        chunk = max(1, -(-units // 64)) * a.leaf
        r_bytes = sum(min(chunk, n - c0) * min(n, c0 + chunk) * 4 for c0 in range(0, n, chunk))
        e2e = {"value": flops / e2e_ms / 1e9, "unit": "TFLOP/s", "ms_per_step": e2e_ms,
               "statistic": E2E_STATISTIC, "mean_ms_per_step": mean_ms,
               "api": "later_c_rgsqrf_host (pinned host A in; Q and R's upper triangle out; copies overlapped)",
               "h2d_bytes_per_step": m * n * 4, "d2h_bytes_per_step": m * n * 4 + r_bytes, "pass_ms": pass_ms,
               "clocks": eclk.summary()}
        # the same copies done serially around the device-buffer call, for comparison
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(a.e2e_steps):
            flat(A).copy_(flat(hA), non_blocking=True)
            qr()
            flat(hQ).copy_(flat(A), non_blocking=True)
            flat(hR).copy_(flat(R), non_blocking=True)
        e1.record(st)
        torch.cuda.synchronize()
        e2e["serial_copies_ms_per_step"] = e0.elapsed_time(e1) / a.e2e_steps
        # this host's pinned copy bandwidth (1 GiB each way, contiguous): the floor the copies sit on
        flat_d, flat_h = flat(A), flat(hQ)
        bw = {}
        for name, dst, src in (("h2d", flat_d, flat(hA)), ("d2h", flat_h, flat_d)):
            torch.cuda.synchronize()
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
            torch.cuda.synchronize()
            bw[name] = flat_d.numel() * 4 / (e0.elapsed_time(e1) * 1e6)
        e2e["pinned_copy_gbs"] = bw

    # ---- timed region (device events per step; restore copy outside the events)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lg.launch_count()
    evs = []
    with ClockSampler(local_rank) as clk:
        t_wall = time.perf_counter()
        for _ in range(a.steps):
            A.copy_(A0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            qr()
            e1.record(st)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    if world > 1:
        dist.barrier()
    launches = lg.launch_count() - launches0
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    ms_step = sum(ms) / len(ms)
    clocks = clk.summary()

    # ---- accuracy of the last step, in FP64 on the GPU (outside the timed region)
    t_acc = time.perf_counter()
    bwd, orth = qr_errors_fp64(A0, A, R)
    t_acc = time.perf_counter() - t_acc

    # ---- the same matrix in a second precision (the reference's FP16 by default)
    alt = None
    if a.alt_precision not in ("none", a.precision):
        lw2, lh2 = lg.rgsqrf_bufsize(m, n, a.alt_precision, a.cgs2, a.leaf)
        work2 = work if lw2 <= lw else torch.empty(lw2, dtype=torch.float32, device=dev)
        hwork2 = hwork if lh2 <= lh else torch.empty(lh2, dtype=torch.float16, device=dev)

        def qr_alt():
            lg.later_rgsqrf(A, R, work2, hwork2, precision=a.alt_precision, cgs2=a.cgs2, leaf=a.leaf,
                            panel=a.panel)

        for _ in range(2):
            A.copy_(A0)
            qr_alt()
        ms_alt = []
        for _ in range(a.steps):
            A.copy_(A0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            qr_alt()
            e1.record(st)
            torch.cuda.synchronize()
            ms_alt.append(e0.elapsed_time(e1))
        bwd_alt, orth_alt = qr_errors_fp64(A0, A, R)
        ma = sum(ms_alt) / len(ms_alt)
        alt = {a.alt_precision: {"value": flops / ma / 1e9, "unit": "TFLOP/s", "ms_per_step": ma,
                                 "steps": a.steps, "backward_error": bwd_alt, "orthogonality_over_n": orth_alt / n}}

    # ---- the reference LATER and cuSOLVER's Sgeqrf on the same matrix and GPU, in this process
    same_gpu = None
    if not a.no_ref:
        ref = reference_gpu_harness()
        if ref is not None:
            try:
                rr = time_reference_gpu(a, A0, ref, a.steps, 2)
                rr["impl"] = ("reference LATER rgsqrf: its kernels (compiled from its sources) + its host recursion "
                              "restated with the same cuBLAS calls, FP16 GemmEx")
                same_gpu = {"reference_rgsqrf": rr, "cusolver_sgeqrf": time_cusolver_sgeqrf(A0, ref)}
                same_gpu["speedup_vs_reference"] = rr["ms_per_step"] / ms_step
                same_gpu["e2e_speedup_vs_reference"] = None
            except Exception as e:  # noqa: BLE001
                same_gpu = {"error": str(e)}
        else:
            same_gpu = {"unavailable": "oracle/_ref not built"}

    # ---- the same QR replayed from a captured CUDA graph (launch overhead of the direct call)
    graph_replay = None
    try:
        cs = torch.cuda.Stream()
        cs.wait_stream(st)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(cs):
            A.copy_(A0)
            lg.later_rgsqrf(A, R, work, hwork, precision=a.precision, cgs2=a.cgs2, leaf=a.leaf, panel=a.panel,
                            stream=cs)
            torch.cuda.synchronize()
            with torch.cuda.graph(graph, stream=cs):
                lg.later_rgsqrf(A, R, work, hwork, precision=a.precision, cgs2=a.cgs2, leaf=a.leaf,
                                panel=a.panel, stream=cs)
        gts = []
        for _ in range(a.steps):
            A.copy_(A0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            graph.replay()
            e1.record(st)
            torch.cuda.synchronize()
            gts.append(e0.elapsed_time(e1))
        gms = statistics.median(gts)
        graph_replay = {"ms_per_step": gms, "value": flops / gms / 1e9, "unit": "TFLOP/s"}
        del graph
    except Exception as e:  # noqa: BLE001
        graph_replay = {"error": f"{type(e).__name__}: {e}"}

    # ---- per-class trace of one extra step (roofline of the dominant kernel)
    A.copy_(A0)
    lg.trace_begin()
    qr()
    tr = lg.trace_end()

    if same_gpu and e2e and "reference_rgsqrf" in same_gpu:
        same_gpu["e2e_speedup_vs_reference"] = same_gpu["reference_rgsqrf"]["e2e_ms"] / e2e["ms_per_step"]

    # ---- aggregate over ranks (max time)
    rate = flops / ms_step / 1e9
    if world > 1:
        t = torch.tensor([ms_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t)
        value = world * flops / ms_max / 1e9
    else:
        ms_max = ms_step
        value = rate
    if rank != 0:
        return

    import json as _j
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = _j.loads(pk.read_text())
    peak = peaks.get("bf16_tflops")
    peak_src = "measured bf16 burst (MEASURED_PEAKS.json)" if peak else "fallback 1900 TFLOP/s"
    peak = peak or 1900.0
    top_ach = tr["top_gemm_flops"] / tr["top_gemm_ms"] / 1e9 if tr["top_gemm_ms"] else None
    all_ach = tr["gemm_flops"] / tr["gemm_ms"] / 1e9 if tr["gemm_ms"] else None
    traffic = None
    prof = ROOT / "profiles" / f"tc_gemm_tn_{m // 2}x{n - n // 2}x{m}.md"
    if prof.exists():  # DRAM bytes of the same launch from the committed ncu capture
        for line in prof.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = int(line.split(":")[1])
    roof_gemm = {"bound": "tensor", "kernel": "tc_gemm_kernel (largest launch: top-level trailing update)",
                 "achieved": top_ach, "peak": peak, "unit": "TFLOP/s", "frac": (top_ach / peak) if top_ach else None,
                 "peak_source": peak_src, "traffic": traffic,
                 "traffic_source": str(prof.relative_to(ROOT)) if traffic else None,
                 "all_gemm_achieved": all_ach, "all_gemm_frac": (all_ach / peak) if all_ach else None}
    # The dominant kernel by time is the fused leaf (one cooperative launch per 128-column leaf).
    # Its algorithmic traffic: read the m x w leaf (FP32), write Q (FP32) and Q's 16-bit copy.
    hbm = peaks.get("hbm_gbs")
    hbm_src = "measured copy bandwidth (MEASURED_PEAKS.json)" if hbm else "fallback 6800 GB/s"
    hbm = hbm or 6800.0
    w = min(n, a.leaf)
    leaf_bytes = m * w * (4 + 4 + (4 if a.precision in ("split3", "split2") else 2))
    leaf_ms = tr["panel_ms"] / tr["panel_launches"] if tr["panel_launches"] else None
    leaf_ach = leaf_bytes / leaf_ms / 1e6 if leaf_ms else None
    leaf_traffic = None
    lprof = ROOT / "profiles" / f"leaf_res_kernel_{m}x{w}.md"
    if lprof.exists():
        for line in lprof.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                leaf_traffic = int(line.split(":")[1])
    roof = {"bound": "hbm", "kernel": "leaf_res_kernel (fused leaf; latency-bound, see profiles)",
            "achieved": leaf_ach, "peak": hbm, "unit": "GB/s", "frac": (leaf_ach / hbm) if leaf_ach else None,
            "peak_source": hbm_src, "algorithmic_bytes_per_launch": leaf_bytes, "launch_ms": leaf_ms,
            "launches": tr["panel_launches"], "traffic": leaf_traffic,
            "traffic_source": str(lprof.relative_to(ROOT)) if leaf_traffic else None}

    cpu = None
    if not a.no_cpu:
        r_or, dt_or = cpu_oracle_rate(a.cpu_m, a.cpu_n, a.seed)
        r_la, dt_la = host_sgeqrf_rate(a.cpu_m, a.cpu_n, a.seed)
        cpu = {"value": r_or, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"oracle restatement of later_rgsqrf (numpy, all host threads) on {a.cpu_m}x{a.cpu_n} "
                         f"N(0,1), {dt_or:.2f} s",
               "host_sgeqrf": {"value": r_la, "unit": "TFLOP/s", "seconds": dt_la,
                               "sample": f"scipy OpenBLAS sgeqrf {a.cpu_m}x{a.cpu_n}"}}

    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": a.precision, "data": "synthetic",
            "config": workload_config(a),
            "accuracy": {"backward_error": bwd, "orthogonality_fro": orth, "orthogonality_over_n": orth / n,
                         "computed": "FP64 on the GPU (the quantities of test/test_qr.cu:216-268 without the "
                                     "FP32 checker's own rounding)", "seconds": t_acc},
            "executed_tflops": 2.0 * m * n * n / ms_step / 1e9, "alt_precision": alt,
            "roofline": roof, "roofline_gemm": roof_gemm, "cpu_baseline": cpu, "e2e": e2e,
            "same_gpu_comparators": same_gpu, "graph_replay": graph_replay, "gpu_launches": launches,
            "launches_per_step": launches / max(1, a.steps), "clocks": clocks,
            "wall_s_timed_region": t_wall,
            "trace_ms": {"gemm": tr["gemm_ms"], "panel": tr["panel_ms"], "leaf_gemm": tr["leaf_gemm_ms"],
                         "other": tr["other_ms"]}}
    if world == 1 and not a.no_extras:
        # The other configurations of the reference's workload, measured in the same run (each with its
        # own roofline): C3 Cholesky + refined SPD solve, C4 batched uneven QR, C5 least-squares serving.
        del A, A0, R, work, hwork
        torch.cuda.empty_cache()
        ref = None if a.no_ref else reference_gpu_harness()
        extras = {}
        t_x = time.perf_counter()
        for name, fn in (("C2_sweep", lambda: sweep_summary(a)),
                         ("C3_spd_kappa1e2", lambda: spd_result(a, 16384, 1e2, "fp16", 3, 1, cpu=not a.no_cpu, ref=ref)),
                         ("C3_spd_kappa1e6", lambda: spd_result(a, 16384, 1e6, "fp16", 3, 1, cpu=False, ref=None)),
                         ("C4_batched", lambda: batched_result(a, 4096, 3, 2)),
                         ("C5_serve", lambda: serve_result(a, 1000, [0.5, 2.0, 8.0], 4, 200))):
            t1 = time.perf_counter()
            try:
                extras[name] = fn()
            except Exception as e:  # noqa: BLE001
                extras[name] = {"error": f"{type(e).__name__}: {e}"}
            extras[name]["wall_s"] = time.perf_counter() - t1
            torch.cuda.empty_cache()
        line["configs"] = extras
        line["configs_wall_s"] = time.perf_counter() - t_x
    print(json.dumps(line), flush=True)


def run_gemm_only(a):
    """One TN GEMM shape, FP16 operands, FP32 output, through later_c_gemm16."""
    import torch
    import later_gb300 as lg
    M, N, K = a.gemm
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A = lg.empty_colmajor(K, M, dtype=torch.float16)
    A.copy_(torch.randn(K, M, generator=g, device="cuda"))
    B = lg.empty_colmajor(K, N, dtype=torch.float16)
    B.copy_(torch.randn(K, N, generator=g, device="cuda"))
    D = lg.empty_colmajor(M, N)
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    for _ in range(a.warmup):
        lg.gemm16("T", "N", A, B, D=D, work=work)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        lg.gemm16("T", "N", A, B, D=D, work=work)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    print(json.dumps({"metric": "tensor-core GEMM TFLOP/s (2MNK)", "value": 2.0 * M * N * K / ms / 1e9,
                      "unit": "TFLOP/s", "ms_per_step": ms, "shape": [M, N, K], "op": "TN fp16->fp32"}), flush=True)


def _haar_gpu(n, k, g):
    import torch
    q, r = torch.linalg.qr(torch.randn(n, k, generator=g, device="cuda", dtype=torch.float64))
    return q * torch.sign(torch.diagonal(r))[None, :]


def _peaks():
    pk = ROOT / "MEASURED_PEAKS.json"
    return json.loads(pk.read_text()) if pk.exists() else {}


def spd_result(a, n, kappa, precision, steps, warmup, cpu=True, ref=None):
    """Config 3: n x n SPD A = Q diag(lambda) Q^T (Q Haar, lambda log-uniform in [1/kappa, 1]),
    rpotrf + FP64 iterative refinement on 16 FP32 right-hand sides to backward error 1e-12."""
    import numpy as np
    import torch
    import later_gb300 as lg
    k = 16
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    # Q from an FP32 QR (an FP64 QR of n=16384 is slow on GB300's FP64 units); A = Q diag(lam) Q^T is formed
    # in FP64, so A is a congruence of diag(lam) by a near-orthogonal Q (spectrum within ~1e-5 relative) and
    # only its final rounding to FP32 perturbs it. An FP32 product would add accumulation error far above
    # lam_min = 1/kappa at kappa = 1e6.
    t_gen = time.perf_counter()
    G = torch.randn(n, n, generator=g, device="cuda")
    try:
        q, r = torch.linalg.qr(G)
    except RuntimeError:  # torch's linalg library cannot be loaded (e.g. under a profiler): this library's QR
        q = lg.colmajor(G)
        r = lg.later_rgsqrf(q, precision="split3")
    q *= torch.sign(torch.diagonal(r))[None, :]
    del r, G
    q = q.double()
    lam = torch.exp(torch.empty(n, device="cuda", dtype=torch.float64).uniform_(-float(np.log(kappa)), 0.0,
                                                                                 generator=g))
    A = (q * lam[None, :]) @ q.t()
    del q
    A = lg.colmajor(((A + A.t()) / 2).float())
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen
    B = lg.colmajor(torch.randn(n, k, generator=g, device="cuda"))
    F = lg.empty_colmajor(n, n)
    lw, lh = lg.blas3_bufsize("p", n, n, precision=precision)
    work = torch.empty(lw, dtype=torch.float32, device="cuda")
    hwork = torch.empty(lh, dtype=torch.float16, device="cuda")
    ts = []
    st = 0
    for it in range(warmup + steps):
        F.copy_(A)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("rpotrf")  # lets a profiler select the factorisation's kernels
        e0.record()
        lg.later_rpotrf("l", n, F, precision=precision, work=work, hwork=hwork)
        e1.record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        st = lg.device_status()
        if it >= warmup:
            ts.append(e0.elapsed_time(e1))
    fact_ms = statistics.median(ts)
    # the same factorisation captured once in a CUDA graph and replayed (its ~1800 launches are small: the
    # graph shows how much of the direct call's time is launch overhead)
    graph_ms = None
    try:
        cs = torch.cuda.Stream()
        cs.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(cs):
            F.copy_(A)
            lg.later_rpotrf("l", n, F, precision=precision, work=work, hwork=hwork, stream=cs)
            torch.cuda.synchronize()
            with torch.cuda.graph(graph, stream=cs):
                lg.later_rpotrf("l", n, F, precision=precision, work=work, hwork=hwork, stream=cs)
        gts = []
        for _ in range(max(steps, 2)):
            F.copy_(A)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            graph.replay()
            e1.record()
            torch.cuda.synchronize()
            gts.append(e0.elapsed_time(e1))
        graph_ms = statistics.median(gts)
        del graph
    except Exception as e:  # noqa: BLE001
        graph_ms = f"not captured: {type(e).__name__}: {e}"
    del work, hwork
    t0 = time.perf_counter()
    X, info = lg.spd_solve(A, B, precision=precision, max_iter=60, tol=1e-12)
    torch.cuda.synchronize()
    solve_s = time.perf_counter() - t0
    flops = n ** 3 / 3.0
    peak = _peaks().get("bf16_tflops") or 1900.0
    # the factorisation is ~1800 small launches: replayed from a captured CUDA graph (the way to run it on
    # GB300 when it is repeated) it is reported as the value; the direct call is beside it
    best_ms = graph_ms if isinstance(graph_ms, float) else fact_ms
    ach = flops / best_ms / 1e9
    out = {"workload": f"rpotrf n={n} SPD kappa={kappa:g} ({precision} tensor-core updates) + FP64 refinement, "
                       f"{k} RHS to backward error 1e-12",
           "value": ach, "unit": "TFLOP/s (n^3/3)", "ms_per_step": best_ms,
           "timed_as": "CUDA graph replay" if isinstance(graph_ms, float) else "direct call",
           "direct_call": {"ms_per_step": fact_ms, "value": flops / fact_ms / 1e9}, "steps": steps,
           "factor_status": st, "solve": {"seconds_incl_factor": solve_s, **info},
           "graph_replay": ({"ms_per_step": graph_ms, "value": flops / graph_ms / 1e9}
                            if isinstance(graph_ms, float) else graph_ms),
           "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                        "peak_source": "measured bf16 burst (MEASURED_PEAKS.json)"},
           "input_build_s": t_gen}
    if ref is not None:  # the reference's l_potrf (cuSOLVER Spotrf leaves + its rtrsm / rsyrk) and cuSOLVER
        try:
            Fr = lg.empty_colmajor(n, n)
            hw = torch.zeros(n // 2 * n, dtype=torch.float16, device="cuda")
            rts = []
            for it in range(3):
                Fr.copy_(A)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                infor = ref.rpotrf(Fr, hw)
                e1.record()
                torch.cuda.synchronize()
                if it:
                    rts.append(e0.elapsed_time(e1))
            rms = statistics.median(rts)
            lwc = ref.spotrf_bufsize(Fr)
            wc = torch.empty(max(1, lwc), device="cuda")
            dinfo = torch.zeros(1, dtype=torch.int32, device="cuda")
            cts = []
            for it in range(3):
                Fr.copy_(A)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                ref.spotrf(Fr, wc, dinfo)
                e1.record()
                torch.cuda.synchronize()
                if it:
                    cts.append(e0.elapsed_time(e1))
            cms = statistics.median(cts)
            out["same_gpu_comparators"] = {
                "reference_rpotrf": {"ms_per_step": rms, "value": flops / rms / 1e9, "info": infor,
                                     "impl": "reference l_potrf: cusolverDnSpotrf leaves of 2048 (LWORK 65536), "
                                             "its recursive trsm / syrk with FP16 GemmEx"},
                "cusolver_spotrf": {"ms_per_step": cms, "value": flops / cms / 1e9, "info": int(dinfo.item()),
                                    "impl": "cusolverDnSpotrf FP32"}}
            del Fr, hw, wc
        except Exception as e:  # noqa: BLE001
            out["same_gpu_comparators"] = {"error": str(e)}
    if cpu:
        import scipy.linalg.lapack as la
        As = np.asfortranarray(A.cpu().numpy())
        la.spotrf(As[:512, :512].copy(order="F"))
        t = time.perf_counter()
        la.spotrf(As, lower=1, overwrite_a=1)
        dt = time.perf_counter() - t
        out["cpu_baseline"] = {"value": flops / dt / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"host LAPACK spotrf (scipy's OpenBLAS, all host cores) on "
                                                         f"the same {n}x{n} matrix, {dt:.2f} s"}
    return out


def run_spd(a):
    r = spd_result(a, a.n, a.kappa, a.precision, a.steps, a.warmup, cpu=not a.no_cpu,
                   ref=None if a.no_ref else reference_gpu_harness())
    print(json.dumps({"metric": "Cholesky TFLOP/s (n^3/3) + refined SPD solve", "value": r["value"],
                      "unit": "TFLOP/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
                      "ms_per_step": r["ms_per_step"], "higher_is_better": True, "dtype": a.precision,
                      "data": "synthetic", "config": {"workload": r["workload"], "n": a.n, "kappa": a.kappa,
                                                      "precision": a.precision}, **{k: v for k, v in r.items()
                                                      if k not in ("value", "ms_per_step", "workload")}}),
          flush=True)


def batched_shapes(count, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    shapes = []
    while len(shapes) < count:
        m = int(np.exp(rng.uniform(np.log(256), np.log(8192))))
        n = int(np.exp(rng.uniform(np.log(16), np.log(256))))
        if m >= 4 * n:
            shapes.append((m, n))
    return shapes


def batched_result(a, count, steps, warmup):
    """Config 4: `count` N(0,1) matrices, m log-uniform [256, 8192], n log-uniform [16, 256], m >= 4n;
    one persistent launch under a captured CUDA graph, tile variant from the autotuner; compared with
    looping plain rgsqrf per matrix (timed on a sample of the same distribution)."""
    import torch
    import later_gb300 as lg
    from later_gb300 import autotune
    shapes = batched_shapes(count, a.seed)
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    orig = [torch.randn(n, m, generator=g, device="cuda").t() for m, n in shapes]
    mats = [o.clone() for o in orig]
    flops = sum(2.0 * n * n * (m - n / 3.0) for m, n in shapes)
    nbytes = sum(4.0 * (2 * m * n + n * n) for m, n in shapes)  # read A, write Q, write R
    best, tune_ms = autotune.tune(shapes, use_cache=True)
    b = lg.BatchedQR(mats)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        b.run(best, stream=s)
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=s):
            b.run(best, stream=s)
    ts = []
    for it in range(warmup + steps):
        for x, o in zip(mats, orig):
            x.copy_(o)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize()
        if it >= warmup:
            ts.append(e0.elapsed_time(e1))
    ms = statistics.median(ts)
    bad = int((b.status != 0).sum())
    # comparator: plain rgsqrf per matrix on a sample of 256, scaled by flops
    idx = list(range(0, count, max(1, count // 256)))
    sub = [orig[i].clone() for i in idx]
    for x in sub[:4]:
        lg.later_rgsqrf(x.clone())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for x in sub:
        lg.later_rgsqrf(x)
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t0
    sub_flops = sum(2.0 * shapes[i][1] ** 2 * (shapes[i][0] - shapes[i][1] / 3.0) for i in idx)
    hbm = _peaks().get("hbm_gbs") or 6800.0
    gbs = nbytes / ms / 1e6
    return {"workload": f"{count} N(0,1) matrices, m in [256,8192], n in [16,256], m>=4n; one persistent launch "
                        f"in a captured CUDA graph", "value": flops / ms / 1e9, "unit": "TFLOP/s (sum 2n^2(m-n/3))",
            "matrices_per_s": count / ms * 1e3, "ms_per_step": ms, "steps": steps, "graph": True, "variant": best,
            "autotune_ms": tune_ms, "matrices_failed": bad,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                         "algorithmic_bytes": nbytes, "note": "read A, write Q and R once; FP32 SIMT arithmetic"},
            "comparator_rgsqrf_loop": {"value": sub_flops / loop_s / 1e12, "unit": "TFLOP/s",
                                       "matrices_per_s": len(sub) / loop_s,
                                       "sample": f"{len(sub)} matrices of the same distribution"}}


def qr_errors_probe(A0d, AX, X, Q, R):
    """||A - QR||_F / ||A||_F and ||I - Q^T Q||_F estimated in FP64 from k Gaussian probe vectors X (n x k):
    E[||E X||_F^2] = k ||E||_F^2 for X with i.i.d. N(0,1) entries (relative spread about sqrt(2 / k)).
    A0d: A in FP64; AX = A0d X, computed once per input."""
    import torch
    k = X.shape[1]
    Qd = Q.double()
    E = AX - Qd @ (torch.triu(R).double() @ X)
    bwd = float(torch.sqrt((E * E).sum() / k) / torch.linalg.norm(A0d))
    F = Qd.t() @ (Qd @ X) - X
    orth = float(torch.sqrt((F * F).sum() / k))
    return bwd, orth


def sweep_result(a, probes=64):
    """The QR precision sweep: A = U diag(sigma) V^T (U, V orthonormal from Gaussian QR with the signs of R's
    diagonal moved into Q, sigma geometric from 1 to 1/kappa), 16384 x 16384 and 65536 x 4096, kappa in
    {1e1, 1e3, 1e5}; rgsqrf in FP16, BF16, SPLIT3 and SPLIT2, with and without CGS2 for FP16 and SPLIT2, and
    rhouqr in FP16, BF16 and SPLIT3. Per run: the median of two timed calls after one untimed one (device
    time, workspaces preallocated, the input restored before each call outside the events), and the
    backward error and orthogonality estimated in FP64 from Gaussian probes."""
    import torch
    import later_gb300 as lg
    shapes = [(16384, 16384), (65536, 4096)] if not a.sweep_small else [(4096, 2048), (16384, 1024)]
    kappas = [1e1, 1e3, 1e5]
    rg_modes = [("fp16", False), ("bf16", False), ("split3", False), ("split2", False), ("fp16", True),
                ("split2", True)]
    rh_modes = ["fp16", "bf16", "split3"]
    results = []

    def timed(restore, call, warm=1, reps=2):
        ts = []
        for it in range(warm + reps):
            restore()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call()
            e1.record()
            torch.cuda.synchronize()
            if it >= warm:
                ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    for m, n in shapes:
        g = torch.Generator(device="cuda").manual_seed(a.seed + m + n)

        def haar(rows, cols):
            q, r = torch.linalg.qr(torch.randn(rows, cols, generator=g, device="cuda"))
            return q * torch.sign(torch.diagonal(r))[None, :]

        U, V = haar(m, n), haar(n, n)
        X = torch.randn(n, probes, generator=g, device="cuda", dtype=torch.float64)
        flops = qr_flops(m, n)
        for kappa in kappas:
            sig = torch.logspace(0.0, -math.log10(kappa), n, device="cuda")
            A0 = lg.empty_colmajor(m, n)
            A0.copy_((U * sig[None, :]) @ V.t())
            A0d = A0.double()
            AX = A0d @ X
            A = lg.empty_colmajor(m, n)
            for prec, cgs2 in rg_modes:
                R = lg.empty_colmajor(n, n)
                lw, lh = lg.rgsqrf_bufsize(m, n, prec, cgs2)
                work = torch.empty(lw, device="cuda")
                hwork = torch.empty(lh, dtype=torch.float16, device="cuda")
                row = {"routine": "rgsqrf", "m": m, "n": n, "kappa": kappa, "precision": prec, "cgs2": cgs2}
                try:
                    ms = timed(lambda: A.copy_(A0),
                               lambda: lg.later_rgsqrf(A, R, work, hwork, precision=prec, cgs2=cgs2))
                    st = lg.device_status()
                    bwd, orth = qr_errors_probe(A0d, AX, X, A, R)
                    row.update({"ms": round(ms, 3), "tflops": round(flops / ms / 1e9, 1), "backward_error": bwd,
                                "orthogonality_fro": orth, "orthogonality_over_n": orth / n, "status": st})
                except lg.LaterError as e:
                    row["error"] = str(e)
                results.append(row)
                del R, work, hwork
            for prec in rh_modes:
                W, R = lg.empty_colmajor(m, n), lg.empty_colmajor(n, n)
                lw, lh = lg.rhouqr_bufsize(m, n, prec)
                work = torch.empty(lw, device="cuda")
                hwork = torch.empty(lh, dtype=torch.float16, device="cuda")
                row = {"routine": "rhouqr", "m": m, "n": n, "kappa": kappa, "precision": prec, "cgs2": False}
                try:
                    ms = timed(lambda: A.copy_(A0), lambda: lg.later_rhouqr(A, W, R, work, hwork, precision=prec))
                    st = lg.device_status()
                    lg.later_ormqr(W, A)  # Q = I - W Y^T over W, for the errors (not timed)
                    st = st or lg.device_status()
                    bwd, orth = qr_errors_probe(A0d, AX, X, W, R)
                    row.update({"ms": round(ms, 3), "tflops": round(flops / ms / 1e9, 1), "backward_error": bwd,
                                "orthogonality_fro": orth, "orthogonality_over_n": orth / n, "status": st})
                except lg.LaterError as e:
                    row["error"] = str(e)
                results.append(row)
                del W, R, work, hwork
            del A0, A0d, AX, A
            torch.cuda.empty_cache()
        del U, V
    return results


def sweep_summary(a):
    res = sweep_result(a)
    head = [r for r in res if r["routine"] == "rgsqrf" and r["precision"] == "split2" and not r["cgs2"]
            and "tflops" in r]
    shapes = list(dict.fromkeys(f"{r['m']}x{r['n']}" for r in res))
    return {"workload": "A = U diag(sigma) V^T, sigma geometric 1..1/kappa, kappa 1e1, 1e3, 1e5; shapes "
                        + ", ".join(shapes) + "; rgsqrf fp16 / bf16 / split3 / split2 (+ CGS2 for fp16, split2), "
                        "rhouqr fp16 / bf16 / split3",
            "value": min(r["tflops"] for r in head) if head else None, "unit": "TFLOP/s (2n^2(m-n/3))",
            "value_is": "the lowest rgsqrf SPLIT2 rate over the sweep's shapes and kappas",
            "errors": "estimated in FP64 from 64 Gaussian probe vectors (relative spread about 18%)",
            "timing": "device time, median of 2 calls after 1 untimed, through the Python API with "
                      "preallocated workspaces",
            "results": res}


def run_sweep(a):
    t0 = time.perf_counter()
    r = sweep_summary(a)
    print(json.dumps({"metric": "QR precision sweep: TFLOP/s (2n^2(m-n/3)) with backward error and orthogonality",
                      "n_gpus": 1, "higher_is_better": True, "data": "synthetic",
                      "config": {"workload": r.pop("workload")}, **r,
                      "wall_s": round(time.perf_counter() - t0, 1)}), flush=True)


def run_batched(a):
    r = batched_result(a, a.count, a.steps, a.warmup)
    print(json.dumps({"metric": "batched QR TFLOP/s (sum 2n^2(m-n/3)) and matrices/s", "n_gpus": 1,
                      "warmup": a.warmup, "higher_is_better": True, "dtype": "fp32", "data": "synthetic",
                      "config": {"workload": r["workload"]}, **r}), flush=True)


def serve_result(a, requests, rates_factors, slots, base_requests):
    """Config 5: Poisson arrivals of LS requests, m log-uniform [512, 32768], n log-uniform [32, 2048],
    m >= 2n, kappa log-uniform [1e1, 1e4] (SVD construction), b = A x* + 1e-3 noise; refinement to
    backward error 1e-6; solves/s and p50/p99 latency at each swept rate, against an FP32 QR least-squares
    (torch.linalg.lstsq on the GPU: cuSOLVER, TF32 off) on the same request stream."""
    import numpy as np
    import torch
    import later_gb300 as lg
    torch.backends.cuda.matmul.allow_tf32 = False
    rng = np.random.default_rng(a.seed)
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    pool = []
    npool = min(requests, 32)
    while len(pool) < npool:
        m = int(np.exp(rng.uniform(np.log(512), np.log(32768))))
        n = int(np.exp(rng.uniform(np.log(32), np.log(2048))))
        if m < 2 * n:
            continue
        kappa = float(np.exp(rng.uniform(np.log(10), np.log(1e4))))
        u = _haar_gpu(m, n, g)
        v = _haar_gpu(n, n, g)
        sig = torch.logspace(0, -np.log10(kappa), n, device="cuda", dtype=torch.float64)
        A = ((u * sig[None, :]) @ v.t()).float()
        xs = torch.randn(n, 1, generator=g, device="cuda", dtype=torch.float64)
        B = (A.double() @ xs + 1e-3 * torch.randn(m, 1, generator=g, device="cuda", dtype=torch.float64)).float()
        pool.append((np.asfortranarray(A.cpu().numpy()), np.asfortranarray(B.cpu().numpy())))
    req_flops = [2.0 * A.shape[1] ** 2 * (A.shape[0] - A.shape[1] / 3.0) for A, _ in pool]
    srv = lg.LsServer(slots=slots, hbm_budget_gb=64, precision="split3", tol=1e-6)
    for A, B in pool[:2]:
        srv.wait(srv.submit(A, B))
    t0 = time.perf_counter()
    for A, B in pool[:8]:
        srv.wait(srv.submit(A, B))
    serial = (time.perf_counter() - t0) / 8
    rates = [f / serial for f in rates_factors]
    results = []
    for lam in rates:
        arr = np.cumsum(rng.exponential(1.0 / lam, requests))
        t_start = time.perf_counter()
        tickets = []
        for i, t_arr in enumerate(arr):
            now = time.perf_counter() - t_start
            if t_arr > now:
                time.sleep(t_arr - now)
            A, B = pool[i % len(pool)]
            tickets.append(srv.submit(A, B))
        outs = [srv.wait(t) for t in tickets]
        wall = time.perf_counter() - t_start
        lat = np.array([r["latency_ms"] for _, r in outs])
        bwd = max(r["backward_error"] for _, r in outs)
        results.append({"rate": lam, "requests": requests, "solves_per_s": len(outs) / wall,
                        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                        "max_backward_error": bwd, "failed": sum(1 for _, r in outs if r["status"] != 0),
                        "qr_tflops": sum(req_flops[i % len(pool)] for i in range(requests)) / wall / 1e12})
    peak_hbm = srv.hbm_peak()
    srv.close()
    # FP32 QR baseline on the same GPU, same request pool, one request at a time
    for A, B in pool[:2]:
        torch.linalg.lstsq(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat = []
    for i in range(base_requests):
        A, B = pool[i % len(pool)]
        t1 = time.perf_counter()
        x = torch.linalg.lstsq(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()).solution
        x.cpu()
        lat.append((time.perf_counter() - t1) * 1e3)
    wall = time.perf_counter() - t0
    base = {"solves_per_s": base_requests / wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "requests": base_requests,
            "impl": "torch.linalg.lstsq FP32 on the GPU (cuSOLVER QR), serial"}
    best = max(results, key=lambda r: r["solves_per_s"])
    peak = _peaks().get("bf16_tflops") or 1900.0
    return {"workload": f"{requests} LS requests per rate from a pool of {len(pool)}, m in [512,32768], "
                        f"n in [32,2048], m>=2n, kappa in [1e1,1e4], {slots} slots",
            "value": best["solves_per_s"], "unit": "solves/s", "slots": slots, "sweep": results,
            "fp32_qr_baseline": base, "speedup_vs_fp32_qr": best["solves_per_s"] / base["solves_per_s"],
            "hbm_peak_bytes": peak_hbm,
            "roofline": {"bound": "tensor", "achieved": best["qr_tflops"], "peak": peak, "unit": "TFLOP/s",
                         "frac": best["qr_tflops"] / peak,
                         "note": "QR flops 2n^2(m-n/3) of the solved requests per second at the best rate; "
                                 "small requests are launch- and latency-bound"}}


def run_serve(a):
    factors = [r for r in a.rates] if a.rates else [0.5, 1.0, 2.0, 4.0, 8.0, 16.0]
    r = serve_result(a, a.requests, factors, a.slots, min(a.requests, 200))
    print(json.dumps({"metric": "LS solves/s at backward error <= 1e-6, p50/p99 latency", "n_gpus": 1,
                      "higher_is_better": True, "dtype": "split3", "data": "synthetic",
                      "config": {"workload": r["workload"]}, **r}), flush=True)


def main():
    a = parse()
    if a.precision is None:
        a.precision = "split2" if a.config == "qr" else "fp16"
    if a.gemm:
        run_gemm_only(a)
        return
    if a.config != "qr" and a.impl == "ours":
        {"spd": run_spd, "batched": run_batched, "serve": run_serve, "sweep": run_sweep}[a.config](a)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        run_ours(a, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
