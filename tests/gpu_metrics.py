"""FP64 accuracy figures computed on the GPU (test and benchmark infrastructure).

For matrices too large for the host oracle in reasonable time (16384^2,
65536 x 4096) the backward error ||A - QR||_F / ||A||_F and the orthogonality
||I - Q^T Q||_F are formed with FP64 products on the device, in column blocks
so that only one FP64 copy of Q is held. R is upper triangular, so column
block J of A - QR needs only Q[:, :J_end]; Q^T Q is symmetric, so only the
blocks on and above the diagonal are formed. These are the quantities the
reference prints in FP32 (test/test_qr.cu:216-268), here without the FP32
checker's own rounding (about sqrt(n) u_fp32).
"""
from __future__ import annotations


def qr_errors_fp64(A, Q, R, block: int = 2048):
    """(backward error, orthogonality) of a thin QR, FP64 on the GPU.

    A, Q: m x n FP32 device tensors (any strides); R: n x n FP32 device tensor
    (entries below the diagonal ignored).
    """
    import torch
    m, n = Q.shape
    Qd = Q.double()
    num = torch.zeros((), dtype=torch.float64, device=Q.device)
    den = torch.zeros((), dtype=torch.float64, device=Q.device)
    orth = torch.zeros((), dtype=torch.float64, device=Q.device)
    for j0 in range(0, n, block):
        j1 = min(n, j0 + block)
        Rb = torch.triu(R[:j1, j0:j1].double(), diagonal=-j0)
        Ab = A[:, j0:j1].double()
        res = Ab - Qd[:, :j1] @ Rb
        num += (res * res).sum()
        den += (Ab * Ab).sum()
        # rows j0:j1 of Q^T Q - I, columns j0: (upper part; off-diagonal blocks counted twice)
        G = Qd[:, j0:j1].t() @ Qd[:, j0:]
        G[:, : j1 - j0] -= torch.eye(j1 - j0, dtype=torch.float64, device=Q.device)
        d = G[:, : j1 - j0]
        o = G[:, j1 - j0:]
        orth += (d * d).sum() + 2.0 * (o * o).sum()
    return float(torch.sqrt(num / den)), float(torch.sqrt(orth))
