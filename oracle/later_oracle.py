"""Numpy restatement of the reference's recursive QR algorithms (CPU oracle).

Test infrastructure only: the CUDA library is checked against this code on the
same seeded inputs; nothing in the product path imports it.

Precision model (the reference's): matrices are stored in FP32; the trailing
updates are cublasGemmEx calls on FP16 copies (s2h) with FP32 accumulation,
restated as FP32 matmuls of FP16-rounded operands (a product of two FP16
numbers is exact in FP32); panels and their small GEMMs are FP32.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def round16(x: np.ndarray, prec: str = "fp16") -> np.ndarray:
    """FP32 value of the 16-bit operand the tensor core sees (s2h, util/util.cu:24-32)."""
    if prec == "fp16":
        return x.astype(np.float16).astype(F32)
    if prec == "bf16":
        # round-to-nearest-even to 8 significand bits
        u = np.ascontiguousarray(x, dtype=F32).view(np.uint32)
        r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
        return r.view(F32).reshape(x.shape)
    if prec == "split3":
        hi = x.astype(np.float16).astype(F32)
        lo = ((x - hi) * F32(2048)).astype(np.float16).astype(F32) / F32(2048)
        return hi + lo
    raise ValueError(prec)


def tc_gemm(a: np.ndarray, b: np.ndarray, prec: str = "fp16") -> np.ndarray:
    """FP32-accumulated product of 16-bit-rounded operands (cublasGemmEx, CUDA_R_16F in, CUDA_R_32F out)."""
    if prec == "split3":
        ah = a.astype(np.float16).astype(F32)
        bh = b.astype(np.float16).astype(F32)
        al = ((a - ah) * F32(2048)).astype(np.float16).astype(F32)
        bl = ((b - bh) * F32(2048)).astype(np.float16).astype(F32)
        return (ah @ bh) + (ah @ bl + al @ bh) * F32(1.0 / 2048)
    return round16(a, prec) @ round16(b, prec)


# ------------------------------------------------------------------ panels
def mgs_block(a: np.ndarray):
    """MGS of a (<=256) x k block in FP32 — mgs_kernel2, QR/panel.cu:246-325.

    R_kk = ||a_k|| (positive), q_k = a_k / R_kk, then for j > k:
    R_kj = q_k^T a_j and a_j -= R_kj q_k. Columns beyond the row count are
    exactly dependent; they are returned as zero columns with a zero R row
    (the reference leaves them unprocessed, :254,:273).
    """
    a = np.array(a, dtype=F32, order="F")
    mm, k = a.shape
    r = np.zeros((k, k), dtype=F32)
    for c in range(k):
        nrm = F32(np.sqrt(np.dot(a[:, c], a[:, c]))) if c < mm else F32(0)
        if nrm > 0:
            a[:, c] *= F32(1) / nrm
        else:
            a[:, c] = 0
        r[c, c] = nrm
        if c + 1 < k:
            d = a[:, c] @ a[:, c + 1:]
            r[c, c + 1:] = d
            a[:, c + 1:] -= np.outer(a[:, c], d).astype(F32)
    return a, r


def tsqr32(a: np.ndarray, block: int = 256):
    """TSQR of an m x 32 panel — mgs_caqr_panel_256x32, QR/panel.cu:65-134.

    MGS on each 256-row block, the 32x32 R factors stacked (32 rows per block)
    and factored recursively, then each block's Q multiplied by its 32x32 slice
    of the stacked Q (cublasSgemmStridedBatched, :97-102).
    """
    m, k = a.shape
    if m <= block:
        return mgs_block(a)
    nb = (m + block - 1) // block
    q = np.empty_like(a, dtype=F32)
    stack = np.zeros((nb * k, k), dtype=F32)
    for i in range(nb):
        qi, ri = mgs_block(a[i * block:(i + 1) * block])
        q[i * block:(i + 1) * block] = qi
        stack[i * k:(i + 1) * k] = ri
    qs, r = tsqr32(stack, block)
    for i in range(nb):
        q[i * block:(i + 1) * block] = q[i * block:(i + 1) * block] @ qs[i * k:(i + 1) * k]
    return q, r


def split_half(n: int) -> int:
    """Split point of a width-n recursion step (n/2 for the reference's powers of two)."""
    return ((n // 32 + 1) // 2) * 32


def leaf_qr(a: np.ndarray, r: np.ndarray, cgs2: bool = False):
    """128-wide leaf — mgs_caqr_panel_256x128, QR/panel.cu:10-63: halves down to
    32-column TSQR panels, glued by FP32 block-CGS updates (cublasSgemm)."""
    w = a.shape[1]
    if w <= 32:
        q, rr = tsqr32(a)
        a[:] = q
        r[:w, :w] = rr
        return
    w1 = split_half(w)
    leaf_qr(a[:, :w1], r[:w1, :w1], cgs2)
    s = a[:, :w1].T @ a[:, w1:]
    a[:, w1:] -= a[:, :w1] @ s
    if cgs2:
        s2 = a[:, :w1].T @ a[:, w1:]
        a[:, w1:] -= a[:, :w1] @ s2
        s = s + s2
    r[:w1, w1:] = s
    leaf_qr(a[:, w1:], r[w1:, w1:], cgs2)


def rgsqrf(A: np.ndarray, leaf: int = 128, prec: str = "fp16", cgs2: bool = False):
    """Recursive Gram-Schmidt QR — later_rgsqrf / qr, QR/later_rgsqrf.cu:25-79.

    Returns (Q, R) in FP32. Trailing update: R12 = Q1^T A2 (FP16 GemmEx, :45-49),
    A2 -= Q1 fp16(R12) (:51-56); R12 itself is kept in FP32.

    prec "split2" (no reference counterpart): R12 = fp16(Q1)^T fp16(A2) kept at
    its FP16-rounded value, and A2 -= (Q1hi + Q1lo/2^11) fp16(R12), so the
    factor that is subtracted is the one stored (backward error at FP32 level).
    """
    a = np.array(A, dtype=F32, order="F")
    m, n = a.shape
    r = np.zeros((n, n), dtype=F32)

    def rec(a, r):
        nn = a.shape[1]
        if nn <= leaf:
            leaf_qr(a, r, cgs2)
            return
        n1 = split_half(nn)
        rec(a[:, :n1], r[:n1, :n1])
        q1 = a[:, :n1]
        passes = 2 if cgs2 else 1
        r12 = np.zeros((n1, nn - n1), dtype=F32)
        for _ in range(passes):
            if prec == "split2":
                s = round16(round16(q1.T) @ round16(a[:, n1:]))
                qh = round16(q1)
                ql = ((q1 - qh) * F32(2048)).astype(np.float16).astype(F32)
                r12 += s
                a[:, n1:] -= qh @ s + (ql @ s) * F32(1.0 / 2048)
                continue
            s = tc_gemm(q1.T, a[:, n1:], prec)
            r12 += s
            a[:, n1:] -= tc_gemm(q1, s, prec)
        r[:n1, n1:] = r12
        rec(a[:, n1:], r[n1:, n1:])

    rec(a, r)
    return a, r


# ------------------------------------------------------------ Householder QR
def householder_reconstruct(q: np.ndarray, r: np.ndarray, signs: bool = True):
    """Compact-WY form of an explicit TSQR factor — reconstructY + leaf W,
    QR/later_rhouqr.cu:56-78, 233-276.

    LU without pivoting of (I - Q S): Y = L (unit lower trapezoidal), U upper;
    W = (I - Q S) Y1^{-T} = Y T with T = U Y1^{-T}; R' = S R. With signs=True,
    s_k = -sign of the k-th pivot candidate (Ballard et al., IPDPS 2014), which
    makes every pivot >= 1 and gives LAPACK's Householder vectors; signs=False
    is the reference's literal S = I (cusolverDnSgetrf on I - Q, :251-260).
    """
    q = np.array(q, dtype=F32)
    m, k = q.shape
    g = q[:k, :].copy()
    L = np.eye(k, dtype=F32)
    U = np.zeros((k, k), dtype=F32)
    s = np.ones(k, dtype=F32)
    for j in range(k):
        # eliminate column j with the previous pivots (lower part of L known)
        col = g[:, j].copy()
        for i in range(j):
            col[i + 1:] -= L[i + 1:, i] * col[i]
        gk = col[j]
        sj = F32(-1.0 if gk >= 0 else 1.0) if signs else F32(1.0)
        s[j] = sj
        v = -sj * col
        v[j] += F32(1.0)
        U[: j + 1, j] = v[: j + 1]
        L[j + 1:, j] = v[j + 1:] / v[j]
        g[:, j] = col
    y = np.zeros((m, k), dtype=F32)
    y[:k] = np.tril(L)
    # bottom rows: y U = -(q S)
    b = -(q[k:] * s[None, :])
    y[k:] = np.linalg.solve(U.T.astype(np.float64), b.T.astype(np.float64)).T.astype(F32)
    t = (U.astype(np.float64) @ np.linalg.inv(np.tril(L).astype(np.float64)).T).astype(F32)
    t = np.triu(t)
    w = (y @ t).astype(F32)
    return y, w, (s[:, None] * np.asarray(r, dtype=F32)).astype(F32), t


def rhouqr(A: np.ndarray, prec: str = "fp16", signs: bool = True):
    """Recursive Householder QR — later_rhouqr / qr, QR/later_rhouqr.cu:27-201.

    Returns (Y, W, R) with Q = I - W Y^T. Leaf n <= 32: TSQR then Householder
    reconstruction. Trailing update A2 <- (I - Y1 W1^T) A2 and the W merge
    W2 <- W2 - W1 (Y1^T W2) run in FP32 when n/2 <= 128 or m <= 128 (:83-102),
    else with FP16-rounded operands (:104-135). The top n/2 rows of W2 are
    zero before the merge.
    """
    a = np.array(A, dtype=F32, order="F")
    m, n = a.shape
    w = np.zeros((m, n), dtype=F32)
    r = np.zeros((n, n), dtype=F32)

    def gemm(x, y, use_tc):
        return tc_gemm(x, y, prec) if use_tc else (x @ y).astype(F32)

    def rec(a, w, r):
        mr, nn = a.shape
        if nn <= 32:
            q, rr = tsqr32(a)
            y, ww, rr2, _ = householder_reconstruct(q, rr, signs)
            a[:] = y
            w[:] = ww
            r[:nn, :nn] = rr2
            return
        n1 = split_half(nn)
        rec(a[:, :n1], w[:, :n1], r[:n1, :n1])
        tc = n1 > 128 and mr > 128
        work = gemm(w[:, :n1].T, a[:, n1:], tc)
        a[:, n1:] -= gemm(a[:, :n1], work, tc)
        rec(a[n1:, n1:], w[n1:, n1:], r[n1:, n1:])
        r[:n1, n1:] = a[:n1, n1:]
        a[:n1, n1:] = 0
        w[:n1, n1:] = 0
        work = gemm(a[:, :n1].T, w[:, n1:], tc)
        w[:, n1:] -= gemm(w[:, :n1], work, tc)

    rec(a, w, r)
    return a, w, r


def bhouqr(A: np.ndarray, prec: str = "fp32", nb: int = 128, signs: bool = True):
    """Blocked Householder QR — later_bhouqr, QR/later_bhouqr.cu:88-189.

    For each block of nb columns at column i: rhouqr of A[i:, i:i+nb] (its own
    updates in FP32 at nb = 128), the trailing update A2 -= Y_i (W_i^T A2)
    (cublasSgemm, :117-136), R12 taken from A2's top rows and zeroed
    (copyAndClear, :138-140), then the W merge W_i -= W[:, :i] (Y[:, :i]^T W_i)
    (:143-165) over full-height columns whose rows above i are zero.
    prec "fp32" is the reference's arithmetic; "fp16" / "bf16" / "split3" model
    the same GEMMs on 16-bit operands.
    """
    a = np.array(A, dtype=F32, order="F")
    m, n = a.shape
    w = np.zeros((m, n), dtype=F32)
    r = np.zeros((n, n), dtype=F32)

    def gemm(x, y):
        return (x @ y).astype(F32) if prec == "fp32" else tc_gemm(x, y, prec)

    for i in range(0, n, nb):
        b = min(nb, n - i)
        y, wi, ri = rhouqr(a[i:, i:i + b], prec="fp16", signs=signs)
        a[i:, i:i + b] = y
        w[i:, i:i + b] = wi
        r[i:i + b, i:i + b] = ri
        if n - i > b:
            t = gemm(w[i:, i:i + b].T, a[i:, i + b:])
            a[i:, i + b:] -= gemm(a[i:, i:i + b], t)
            r[i:i + b, i + b:] = a[i:i + b, i + b:]
            a[i:i + b, i + b:] = 0
        if i > 0:
            t2 = gemm(a[:, :i].T, w[:, i:i + b])
            w[:, i:i + b] -= gemm(w[:, :i], t2)
    return a, w, r


def ormqr(W: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Q = I - W Y1^T (first n columns) — QR/later_ormqr.cu:50-58, in FP32."""
    m, n = W.shape
    y1 = np.tril(np.asarray(Y, dtype=F32)[:n, :n], -1) + np.eye(n, dtype=F32)
    return (np.eye(m, n, dtype=F32) - W.astype(F32) @ y1.T).astype(F32)


# --------------------------------------------------------- BLAS-3 / Cholesky
def _solve_tri(L, B, lower=True, trans=False, side="left"):
    import scipy.linalg as sl
    L = np.asarray(L, dtype=F32)
    B = np.asarray(B, dtype=F32)
    if side == "left":
        return sl.solve_triangular(L, B, lower=lower, trans=1 if trans else 0).astype(F32)
    # X op(L) = B  <=>  op(L)^T X^T = B^T
    return sl.solve_triangular(L, B.T, lower=lower, trans=0 if trans else 1).T.astype(F32)


def rsyrk(alpha, A, beta, C, prec="fp16"):
    """C <- alpha A A^T + beta C, lower triangle — syrk, BLAS/later_rsyrk.cu:12-77
    (every block is a GemmEx of FP16-rounded A with FP32 accumulation)."""
    a = round16(np.asarray(A, dtype=F32), prec)
    out = np.array(C, dtype=F32)
    full = (F32(alpha) * (a @ a.T) + F32(beta) * out).astype(F32)
    il = np.tril_indices(out.shape[0])
    out[il] = full[il]
    return out


def rtrsm(side, L, B, prec="fp16", leaf=256):
    """Recursive TRSM with a lower L — trsm_l_l_n / trsm_l_r_t, BLAS/later_rtrsm.cu:75-163.
    side 'l': L X = B (split on rows); side 'r': X L^T = B (split on columns).
    Leaf (<= leaf): FP32 substitution (cublasStrsm); updates: FP16 GemmEx."""
    L = np.asarray(L, dtype=F32)
    X = np.array(B, dtype=F32)

    def rec_l(L, X):
        m = L.shape[0]
        if m <= leaf:
            X[:] = _solve_tri(L, X, lower=True, side="left")
            return
        h = m // 2
        rec_l(L[:h, :h], X[:h])
        X[h:] -= tc_gemm(L[h:, :h], X[:h], prec)
        rec_l(L[h:, h:], X[h:])

    def rec_r(L, X):
        n = L.shape[0]
        if n <= leaf:
            X[:] = _solve_tri(L, X, lower=True, trans=True, side="right")
            return
        h = n // 2
        rec_r(L[:h, :h], X[:, :h])
        X[:, h:] -= tc_gemm(X[:, :h], L[h:, :h].T, prec)
        rec_r(L[h:, h:], X[:, h:])

    (rec_l if side == "l" else rec_r)(L, X)
    return X


def rtrmm(L, B, prec="fp16", leaf=256):
    """C = L B, L lower — trmm, BLAS/later_rtrmm.cu:14-71 (leaf cublasStrmm in FP32,
    off-diagonal GemmEx into tempC, then C2 += tempC)."""
    L = np.asarray(L, dtype=F32)
    B = np.asarray(B, dtype=F32)
    C = np.zeros_like(B)

    def rec(L, B, C):
        m = L.shape[0]
        if m <= leaf:
            C[:] = (np.tril(L) @ B).astype(F32)
            return
        h = m // 2
        rec(L[:h, :h], B[:h], C[:h])
        tmp = tc_gemm(L[h:, :h], B[:h], prec)
        rec(L[h:, h:], B[h:], C[h:])
        C[h:] += tmp

    rec(L, B, C)
    return C


def rpotrf(A, prec="fp16", leaf=2048):
    """Recursive lower Cholesky — l_potrf, Cholesky/later_rpotrf.cu:22-66: leaf spotrf
    (<= 2048), off-diagonal later_rtrsm('l','r','t'), trailing later_rsyrk(-1, 1)."""
    a = np.array(A, dtype=F32)

    def rec(a):
        n = a.shape[0]
        if n <= leaf:
            a[:] = np.linalg.cholesky(a.astype(F32)).astype(F32)
            return
        h = n // 2
        rec(a[:h, :h])
        a[h:, :h] = rtrsm("r", a[:h, :h], a[h:, :h], prec)
        a[h:, h:] = rsyrk(-1.0, a[h:, :h], 1.0, a[h:, h:], prec)
        rec(a[h:, h:])

    rec(a)
    return np.tril(a)


# ---------------------------------------------------------------- QDWH polar
def qdwh_coeffs(l: float):
    """Dynamically weighted Halley coefficients (a, b, c) and the next lower bound, as
    EVD/later_qdwh_polar.cu:58-65 computes them (Nakatsukasa, Bai and Gygi, SIAM J. Matrix
    Anal. Appl. 31(5), 2010, eqs. (3.3)-(3.4))."""
    l2 = l * l
    dd = (4.0 * (1.0 - l2) / (l2 * l2)) ** (1.0 / 3.0)
    sqd = np.sqrt(1.0 + dd)
    a = sqd + np.sqrt(8.0 - 4.0 * dd + 8.0 * (2.0 - l2) / (l2 * sqd)) / 2.0
    b = (a - 1.0) ** 2 / 4.0
    c = a + b - 1.0
    return a, b, c, l * (a + b * l2) / (1.0 + c * l2)


def qdwh_polar(A: np.ndarray, prec: str = "split3", l0: float | None = None, symmetrize: bool = False,
               tol: float = 1e-6, max_iter: int = 10):
    """Polar decomposition A = U H by the QR-based QDWH iteration — later_qdwh_polar,
    EVD/later_qdwh_polar.cu:24-110:
      X0 = A / ||A||_F;  while not converged:
        [sqrt(c) X; I] = [Q1; Q2] R   (rgsqrf of the (m + n) x n stack)
        X <- (b/c) X + (a - b/c)/sqrt(c) Q1 Q2^T
    stopping when 1 - l < 10 eps and ||X_new - X||_F < (10 eps)^(1/3) (the reference's tol1 / tol3,
    with its eps = 2e-4 replaced by `tol`). H = (U^T A + (U^T A)^T) / 2. l0 defaults to
    1 / ||R0^{-1}||_F for X0 = Q0 R0, a guaranteed lower bound on sigma_min(X0).
    The stack's QR must be orthonormal to working accuracy although its condition number is about
    sqrt(c) (1e4 in the first step at kappa 1e5): Gram-Schmidt needs the second projection pass
    (CGS2) for that, and FP32-level projections (SPLIT3); with the reference's FP16 products the
    iterate stalls at FP16-level orthogonality."""
    A = np.asarray(A, dtype=F32)
    m, n = A.shape
    alpha = np.linalg.norm(A.astype(np.float64))
    X = (A / F32(alpha)).astype(F32)
    if l0 is None:
        _, R0 = rgsqrf(X, prec=prec)
        l0 = 1.0 / np.linalg.norm(np.linalg.inv(np.triu(R0).astype(np.float64)))
    l = float(l0)
    tol1 = 10.0 * tol / 2.0
    tol3 = tol1 ** (1.0 / 3.0)
    it = 0
    for it in range(1, max_iter + 1):
        a, b, c, l = qdwh_coeffs(min(l, 1.0))
        S = np.vstack([F32(np.sqrt(c)) * X, np.eye(n, dtype=F32)]).astype(F32)
        Q, _ = rgsqrf(S, prec=prec, cgs2=True)
        gp = "split3" if prec in ("split2", "split3") else prec
        Xn = (F32(b / c) * X + F32((a - b / c) / np.sqrt(c)) * tc_gemm(Q[:m], Q[m:].T, gp)).astype(F32)
        if symmetrize:
            Xn = ((Xn + Xn.T) / 2).astype(F32)
        diff = np.linalg.norm((Xn - X).astype(np.float64))
        X = Xn
        if diff < tol3 and 1.0 - l < tol1:
            break
    H = (X.astype(np.float64).T @ A.astype(np.float64))
    H = ((H + H.T) / 2).astype(F32)
    return X, H, it


# --------------------------------------------------------------- sy2sb
def sy2sb(A: np.ndarray, nb: int = 128, prec: str = "fp32"):
    """Symmetric to band reduction B = Q^T A Q (bandwidth nb) — ssytrd_sy2sb,
    EVD/later_sy2sb_blocked.cu:23-186, on one matrix updated in place. Per block
    column i: rhouqr of the panel A[i+nb:, i:i+nb] (FP32 at nb <= 128), the panel
    becomes [R; 0] (and its mirror above the diagonal), then the two-sided ZY
    update of A22 = A[i+nb:, i+nb:]: P = A22 W, T = W^T P, Z = P - T-weighted Y / 2,
    A22 -= Y Z^T + Z Y^T. Returns (B, Y, W) with the reflectors of each block
    column in place (Q = prod_i (I - W_i Y_i^T))."""
    a = np.array(A, dtype=F32)
    n = a.shape[0]
    Y = np.zeros((n, n), dtype=F32)
    Wf = np.zeros((n, n), dtype=F32)

    def gemm(x, y):
        return (x @ y).astype(F32) if prec == "fp32" else tc_gemm(x, y, prec)

    for i in range(0, n - nb, nb):
        r0 = i + nb
        y, w, r = rhouqr(a[r0:, i:i + nb], prec="fp16")
        Y[r0:, i:i + nb] = y
        Wf[r0:, i:i + nb] = w
        pan = np.zeros_like(y)
        pan[:nb] = np.triu(r)
        a[r0:, i:i + nb] = pan
        a[i:i + nb, r0:] = pan.T
        a22 = a[r0:, r0:]
        P = gemm(a22, w)
        T = gemm(w.T, P)
        Z = (P - F32(0.5) * gemm(y, T)).astype(F32)
        a22 -= gemm(y, Z.T)
        a22 -= gemm(Z, y.T)
    return a, Y, Wf
