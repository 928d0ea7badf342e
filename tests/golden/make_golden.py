"""Generates the golden vectors in tests/golden/ from the reference LATER run on a GPU.

Needs a CUDA device and oracle/_ref (the reference's kernels compiled from its
sources plus the harness that drives them; see oracle/build_ref.py). Each
fixture holds the seeded input's recipe (generator, shape, seed) and the
reference's outputs on it; tests/test_golden.py rebuilds the input on the CPU
and checks the oracle against them.

    python tests/golden/make_golden.py [OUTDIR]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main(out: Path):
    import torch

    from oracle import build_ref, gen, metrics
    build_ref.build()
    ref = build_ref.load()
    assert ref is not None, "oracle/_ref is not available"
    out.mkdir(parents=True, exist_ok=True)

    def rgsqrf(A):
        m, n = A.shape
        dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()
        R = torch.zeros(n, n, device="cuda").t()
        lw, lh = ref.rgsqrf_bufsize(m, n)
        work = torch.zeros(max(lw, m // 256 * 32 * 64), device="cuda")
        hwork = torch.zeros(lh, dtype=torch.float16, device="cuda")
        ref.rgsqrf(dA, R, work, hwork)
        torch.cuda.synchronize()
        return dA.cpu().numpy(), np.triu(R.cpu().numpy())

    for name, (m, n, seed) in {"rgsqrf_leaf_512x128": (512, 128, 101),
                               "rgsqrf_fp16_512x256": (512, 256, 102),
                               "rgsqrf_leaf_2600x128": (2600, 128, 103)}.items():
        A = gen.normal(m, n, seed)
        Q, R = rgsqrf(A)
        np.savez_compressed(out / f"{name}.npz", generator="normal", m=m, n=n, seed=seed, Q=Q, R=R,
                            backward_error=metrics.qr_backward_error(A, Q, R),
                            orthogonality=metrics.orthogonality(Q))
        print(name, metrics.qr_backward_error(A, Q, R), metrics.orthogonality(Q))

    n, kappa, seed = 4096, 1e2, 12
    A = gen.spd_matrix(n, kappa, seed)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()
    hwork = torch.zeros(n // 2 * n, dtype=torch.float16, device="cuda")
    info = ref.rpotrf(dA, hwork)
    L = np.tril(dA.cpu().numpy())
    np.savez_compressed(out / "rpotrf_fp16_4096.npz", generator="spd_matrix", n=n, kappa=kappa, seed=seed, info=info,
                        L_sample=L[::64, ::64], L_col_norms=np.linalg.norm(L.astype(np.float64), axis=0),
                        backward_error=metrics.chol_backward_error(A, L))
    print("rpotrf", info, metrics.chol_backward_error(A, L))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
