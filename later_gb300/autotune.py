"""Autotuner for the batched QR tile shape.

The persistent batched kernel has tile variants (rows per streamed chunk x
CTAs per SM, `later_c_batched_qr_run(..., variant)`). For a batch the tuner
builds a sample with the same size distribution (the shapes of every k-th
matrix, random N(0,1) contents), times each variant with CUDA events after a
warm-up, and returns the fastest. Results are cached per GPU name and size
histogram in a JSON table (LATER_GB300_TUNE_CACHE or
~/.cache/later_gb300/batched_tune.json), so a serving process tunes once.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

N_VARIANTS = 4


def _cache_path() -> Path:
    p = os.environ.get("LATER_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "later_gb300" / "batched_tune.json"


def _key(shapes, device_name: str) -> str:
    # log2 histogram of (m, n): batches with the same mix share a tuning result, within a factor-of-4
    # bucket of the batch count (the variants change CTAs per SM, so the count against the SMs matters)
    hist = {}
    for m, n in shapes:
        k = f"{int(math.log2(max(m, 1)))}x{int(math.log2(max(n, 1)))}"
        hist[k] = hist.get(k, 0) + 1
    tot = sum(hist.values())
    sig = ",".join(f"{k}:{round(v / tot, 2)}" for k, v in sorted(hist.items()))
    count = int(math.log2(max(tot, 1))) // 2
    return f"{device_name}|n{count}|{sig}"


def tune(shapes, sample=256, reps=3, use_cache=True, seed=0):
    """Returns (best_variant, {variant: ms}) for a batch with these (m, n) shapes."""
    import torch
    import later_gb300 as lg
    dev_name = torch.cuda.get_device_name()
    key = _key(shapes, dev_name)
    path = _cache_path()
    table = {}
    if use_cache and path.exists():
        try:
            table = json.loads(path.read_text())
        except Exception:
            table = {}
        if key in table:
            return table[key]["best"], {int(k): v for k, v in table[key]["ms"].items()}
    step = max(1, len(shapes) // sample)
    sub = shapes[::step][:sample]
    g = torch.Generator(device="cuda").manual_seed(seed)
    orig = [torch.randn(n, m, generator=g, device="cuda").t() for m, n in sub]
    work = [lg.empty_colmajor(m, n) for m, n in sub]
    b = lg.BatchedQR(work)
    times = {}
    for v in range(N_VARIANTS):
        for w, o in zip(work, orig):
            w.copy_(o)
        b.run(v)  # warm-up
        ms = []
        for _ in range(reps):
            for w, o in zip(work, orig):
                w.copy_(o)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            b.run(v)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        times[v] = min(ms)
    best = min(times, key=times.get)
    if use_cache:
        table[key] = {"best": best, "ms": times}
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(table, indent=1))
    return best, times
