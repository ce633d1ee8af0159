"""The split FP64 factorization's launch geometry and index arithmetic (k_lus_panel, k_lus_trsm,
k_lus_update in boltzmann_gb300/csrc/lu.cu), restated on the CPU with the kernels' own loops,
bounds tests and block decomposition: every read and write stays inside the caller's
[N x ld] matrix and [N] permutation, and the result is an LU factorization with partial
pivoting of [A | b] (rows kept in place, pivot order in perm). No GPU."""
import numpy as np
import pytest

SP_T = 64  # trailing tile edge of the kernels


def _panel_nb(N):
    """factor_split's panel width: as wide as the panel's shared memory allows (200 KB)."""
    for nb in (32, 16, 8):
        if ((N * 4 + 15) // 16) * 16 + (N | 1) * nb * 8 <= 200 * 1024:
            return nb
    return 8


class Checked:
    """A matrix [N x ld] that asserts every access is in bounds."""

    def __init__(self, a):
        self.a = a

    def get(self, r, c):
        assert 0 <= r < self.a.shape[0] and 0 <= c < self.a.shape[1], (r, c)
        return self.a[r, c]

    def set(self, r, c, v):
        assert 0 <= r < self.a.shape[0] and 0 <= c < self.a.shape[1], (r, c)
        self.a[r, c] = v


def split_factor(A, N, NC, NB):
    M = Checked(A)
    perm = np.zeros(N, dtype=np.int64)
    info = 0
    for k0 in range(0, N, NB):
        mrows, kb = N - k0, min(NB, N - k0)
        # k_lus_panel: one CTA; ps = perm[k0:], panel rows ps[r], columns k0 .. k0+kb-1
        ps = np.arange(mrows) if k0 == 0 else perm[k0:].copy()
        P = np.array([[M.get(ps[r], k0 + c) for c in range(kb)] for r in range(mrows)])
        inf = 0
        for j in range(kb):
            col = np.abs(P[j:, j])
            pr = j + int(np.argmax(col))  # first index of the maximum, as the kernel's reduction
            if pr != j:
                P[[j, pr], :] = P[[pr, j], :]
                ps[[j, pr]] = ps[[pr, j]]
            if col.max() == 0 and inf == 0:
                inf = j + 1
            d = P[j, j]
            P[j + 1:, j] *= (1.0 / d) if d != 0 else 0.0
            P[j + 1:, j + 1:kb] -= np.outer(P[j + 1:, j], P[j, j + 1:kb])
        for r in range(mrows):
            for c in range(kb):
                M.set(ps[r], k0 + c, P[r, c])
        perm[k0:] = ps
        if info == 0 and inf:
            info = k0 + inf
        c0g = k0 + kb
        ncol, mr = NC - c0g, N - c0g
        if ncol <= 0:
            break
        ncb = (ncol + SP_T - 1) // SP_T
        # k_lus_trsm: grid P * ncb, SP_T threads, thread = one column c < NC
        pr_ = [perm[k0 + t] if t < kb else 0 for t in range(NB)]
        L = np.array([[M.get(pr_[i], k0 + j) if (i < kb and j < kb) else 0.0 for j in range(NB)]
                      for i in range(NB)])
        for cb in range(ncb):
            for tid in range(SP_T):
                c = c0g + cb * SP_T + tid
                if c >= NC:
                    continue
                x = [M.get(pr_[j], c) if j < kb else 0.0 for j in range(NB)]
                for j in range(1, NB):
                    for i in range(j):
                        x[j] -= L[j, i] * x[i]
                for j in range(kb):
                    M.set(pr_[j], c, x[j])
        if mr <= 0:
            continue
        # k_lus_update: grid P * nrb * ncb, tile (rb, cb) of 64 x 64
        nrb = (mr + SP_T - 1) // SP_T
        pk = [perm[k0 + t] if t < kb else 0 for t in range(NB)]
        for rb in range(nrb):
            prow = [perm[c0g + rb * SP_T + t] if rb * SP_T + t < mr else -1 for t in range(SP_T)]
            Ls = np.array([[M.get(prow[r], k0 + k) if (prow[r] >= 0 and k < kb) else 0.0 for r in range(SP_T)]
                           for k in range(NB)])
            for cb in range(ncb):
                Us = np.array([[M.get(pk[k], c0g + cb * SP_T + c) if (k < kb and cb * SP_T + c < ncol) else 0.0
                                for c in range(SP_T)] for k in range(NB)])
                acc = Ls.T @ Us
                for r in range(SP_T):
                    if prow[r] < 0:
                        continue
                    for c in range(SP_T):
                        if cb * SP_T + c < ncol:
                            cg = c0g + cb * SP_T + c
                            M.set(prow[r], cg, M.get(prow[r], cg) - acc[r, c])
    return perm, info


@pytest.mark.parametrize("N", [5, 33, 70, 97])
def test_split_factor_geometry_and_result(N):
    rng = np.random.default_rng(N)
    NC = N + 1
    ld = (NC + 3) & ~3  # the solver's 16-byte aligned rows
    A0 = rng.standard_normal((N, ld))
    A = A0.copy()
    perm, info = split_factor(A, N, NC, 32)
    assert info == 0
    assert sorted(perm.tolist()) == list(range(N))
    LU = A[perm, :]
    L = np.tril(LU[:, :N], -1) + np.eye(N)
    U = np.triu(LU[:, :N])
    assert np.abs(L @ U - A0[perm, :N]).max() < 1e-12 * N
    # the appended right-hand side column is eliminated with the matrix: L y = b
    assert np.abs(L @ LU[:, N] - A0[perm, N]).max() < 1e-12 * N


@pytest.mark.parametrize("N,NB", [(40, 16), (29, 8)])
def test_narrow_panels(N, NB):
    rng = np.random.default_rng(N + NB)
    A0 = rng.standard_normal((N, N + 1))
    A = A0.copy()
    perm, info = split_factor(A, N, N + 1, NB)
    LU = A[perm, :]
    L = np.tril(LU[:, :N], -1) + np.eye(N)
    assert np.abs(L @ np.triu(LU[:, :N]) - A0[perm, :N]).max() < 1e-12 * N


def test_zero_pivot_reported_in_a_later_panel():
    N = 40
    A = np.eye(N, N + 1)
    A[35, 35] = 0.0
    _, info = split_factor(A, N, N + 1, 32)
    assert info == 36


def test_panel_width_rule():
    """The panel (rows x width doubles plus the row permutation) fits 200 KB of shared memory."""
    assert _panel_nb(385) == 32 and _panel_nb(1281) == 16 and _panel_nb(2048) == 8
