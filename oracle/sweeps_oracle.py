"""CPU oracle of the batched banded kernels of the 1D3V finite-volume path — TEST
INFRASTRUCTURE ONLY.

A NumPy restatement of the reference's CuPy raw kernels (ut-padas/boltzmann,
`BESolver/python/rawkernel.py`) and of its unit upper BSR triangular solve
(`BESolver/cuda/spsm_bsr_upper_tri_solve.cu`), used by `tests/` as the checker of the
library's kernels (`boltzmann_gb300.native_kernels`). Each function states the recurrence
of the reference kernel it follows, vectorised over the batch of systems. The tests also
pin these recurrences to dense linear algebra (the matrices the band storage describes).
"""
from __future__ import annotations

import numpy as np


def bidiagonal_solve(diag, sdiag, b, lower):
    """rawkernel.py:5-33: lower x0 = b0/d0, xi = (bi - s[i-1] x[i-1]) / di; upper from the end
    with s[i] x[i+1]."""
    d = diag.reshape(-1, diag.shape[-1])
    s = sdiag.reshape(-1, sdiag.shape[-1])
    bb = b.reshape(-1, b.shape[-1])
    N = d.shape[1]
    x = np.zeros_like(bb)
    if lower:
        x[:, 0] = bb[:, 0] / d[:, 0]
        for i in range(1, N):
            x[:, i] = (bb[:, i] - s[:, i - 1] * x[:, i - 1]) / d[:, i]
    else:
        x[:, N - 1] = bb[:, N - 1] / d[:, N - 1]
        for i in range(N - 2, -1, -1):
            x[:, i] = (bb[:, i] - s[:, i] * x[:, i + 1]) / d[:, i]
    return x.reshape(b.shape)


def banded_tri_solve(diags, b, lower):
    """rawkernel.py:34-74 (row storage: lower L[i][i-k] = D[k][i], upper U[i][i+k] = D[k][i])."""
    D = diags.reshape(-1, diags.shape[-2], diags.shape[-1])
    bb = b.reshape(-1, b.shape[-1])
    nd, N = D.shape[1], D.shape[2]
    x = np.zeros_like(bb)
    order = range(N) if lower else range(N - 1, -1, -1)
    for i in order:
        s = np.zeros(bb.shape[0])
        for k in range(1, nd):
            j = i - k if lower else i + k
            if 0 <= j < N:
                s += D[:, k, i] * x[:, j]
        x[:, i] = (bb[:, i] - s) / D[:, 0, i]
    return x.reshape(b.shape)


def banded_tri_mv(diags, b, lower):
    """rawkernel.py:75-115."""
    D = diags.reshape(-1, diags.shape[-2], diags.shape[-1])
    bb = b.reshape(-1, b.shape[-1])
    nd, N = D.shape[1], D.shape[2]
    y = np.zeros_like(bb)
    for i in range(N):
        for k in range(nd):
            j = i - k if lower else i + k
            if 0 <= j < N:
                y[:, i] += D[:, k, i] * bb[:, j]
    return y.reshape(b.shape)


def band_by_column_to_dense(Dc, lower):
    """The matrix of a column-stored band (the sweeps' D_LtoR / D_RtoL): lower M[i][i-k] =
    Dc[k][i-k], upper M[i][i+k] = Dc[k][i+k]."""
    nd, N = Dc.shape
    M = np.zeros((N, N))
    for k in range(nd):
        for i in range(N):
            j = i - k if lower else i + k
            if 0 <= j < N:
                M[i, j] = Dc[k, j]
    return M


def _be_lines(L, R, a, ltr, dt, b):
    """(I + a dt D) x = b per line, D = the column-stored lower band L when ltr else the upper
    band R (rawkernel.py:168-375): lines in rows of b, a and ltr per line."""
    nd, N = L.shape
    x = np.zeros_like(b)
    ad = a * dt
    for line in range(b.shape[0]):
        if ltr[line]:
            for i in range(N):
                s = sum(L[k, i - k] * x[line, i - k] for k in range(1, nd) if i - k >= 0)
                x[line, i] = (b[line, i] - ad[line] * s) / (1.0 + ad[line] * L[0, i])
        else:
            for i in range(N - 1, -1, -1):
                s = sum(R[k, i + k] * x[line, i + k] for k in range(1, nd) if i + k < N)
                x[line, i] = (b[line, i] - ad[line] * s) / (1.0 + ad[line] * R[0, i])
    return x


def adv_vr_BE(D_LtoR, D_RtoL, Ex, cos_vt, dt, b, Nr, Nvt, Nx):
    """rawkernel.py:168-230: lines (x, j) of Nr cells, a = -E[x] cos(theta_j), left to right
    when a >= 0."""
    a = (-Ex[:, None] * cos_vt[None, :]).reshape(-1)
    return _be_lines(D_LtoR, D_RtoL, a, a >= 0, dt, b.reshape(Nx * Nvt, Nr)).reshape(b.shape)


def adv_vt_BE(D_LtoR, D_RtoL, Ex, vr, dt, b, Nr, Nvt, Nx):
    """rawkernel.py:232-296: lines (x, r) of Nvt cells, a = E[x] / v_r, left to right when
    -a >= 0."""
    a = (Ex[:, None] / vr[None, :]).reshape(-1)
    return _be_lines(D_LtoR, D_RtoL, a, -a >= 0, dt, b.reshape(Nx * Nr, Nvt)).reshape(b.shape)


def adv_x_BE(D_LtoR, D_RtoL, vr, cos_vt, dt, b, Nr, Nvt, Nx):
    """rawkernel.py:298-375: lines (r, j) of Nx cells, a = v_r cos(theta_j), left to right
    when a >= 0."""
    a = (vr[:, None] * cos_vt[None, :]).reshape(-1)
    return _be_lines(D_LtoR, D_RtoL, a, a >= 0, dt, b.reshape(Nr * Nvt, Nx)).reshape(b.shape)


def bsr_upper_unit_solve(data, indptr, indices, bs, b):
    """spsm_bsr_upper_tri_solve.cu:1-61: block rows from the last, x_i = b_i - sum_{j > i}
    A_ij x_j (blocks on or below the diagonal ignored: unit diagonal). b (nrhs, n)."""
    nbr = len(indptr) - 1
    bb = b.reshape(-1, nbr * bs)
    x = np.zeros_like(bb)
    for i in range(nbr - 1, -1, -1):
        xi = bb[:, i * bs:(i + 1) * bs].copy()
        for e in range(indptr[i], indptr[i + 1]):
            j = indices[e]
            if j <= i:
                continue
            xi -= x[:, j * bs:(j + 1) * bs] @ data[e].T
        x[:, i * bs:(i + 1) * bs] = xi
    return x.reshape(b.shape)
