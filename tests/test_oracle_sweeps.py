"""The oracle of the batched banded kernels (rawkernel.py recurrences) against dense linear
algebra on the matrices the band storage describes, on the CPU."""
import numpy as np
import pytest

from oracle import sweeps_oracle as S


def dense_rowband(D, lower):
    nd, N = D.shape
    M = np.zeros((N, N))
    for k in range(nd):
        for i in range(N):
            j = i - k if lower else i + k
            if 0 <= j < N:
                M[i, j] = D[k, i]
    return M


@pytest.mark.parametrize("lower", [True, False])
def test_bidiagonal_and_banded(lower):
    rng = np.random.default_rng(5)
    bsz, N, nd = 7, 13, 4
    d = rng.uniform(1.0, 2.0, (bsz, N))
    s = rng.standard_normal((bsz, N - 1))
    b = rng.standard_normal((bsz, N))
    x = S.bidiagonal_solve(d, s, b, lower)
    for q in range(bsz):
        M = np.diag(d[q]) + (np.diag(s[q], -1) if lower else np.diag(s[q], 1))
        np.testing.assert_allclose(M @ x[q], b[q], rtol=1e-12, atol=1e-12)
    D = rng.standard_normal((bsz, nd, N))
    D[:, 0] = rng.uniform(1.0, 2.0, (bsz, N))
    x = S.banded_tri_solve(D, b, lower)
    y = S.banded_tri_mv(D, b, lower)
    for q in range(bsz):
        M = dense_rowband(D[q], lower)
        np.testing.assert_allclose(M @ x[q], b[q], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(y[q], M @ b[q], rtol=1e-12, atol=1e-12)


def test_sweeps_solve_their_backward_euler_systems():
    rng = np.random.default_rng(6)
    Nr, Nvt, Nx, nd, dt = 9, 6, 5, 3, 0.3
    L = rng.uniform(0.1, 1.0, (nd, max(Nr, Nvt, Nx)))
    R = rng.uniform(0.1, 1.0, (nd, max(Nr, Nvt, Nx)))
    Ex = rng.standard_normal(Nx)
    cos_vt = np.cos(np.linspace(0.1, np.pi - 0.1, Nvt))
    vr = rng.uniform(0.5, 2.0, Nr)
    for kind, (c1, c2, N, shape, coef, ltr) in enumerate([
            (Ex, cos_vt, Nr, (Nx * Nvt, Nr), lambda: (-Ex[:, None] * cos_vt[None, :]).ravel(), lambda a: a >= 0),
            (Ex, vr, Nvt, (Nx * Nr, Nvt), lambda: (Ex[:, None] / vr[None, :]).ravel(), lambda a: -a >= 0),
            (vr, cos_vt, Nx, (Nr * Nvt, Nx), lambda: (vr[:, None] * cos_vt[None, :]).ravel(), lambda a: a >= 0)]):
        LL, RR = L[:, :N].copy(), R[:, :N].copy()
        b = rng.standard_normal(shape)
        fn = [S.adv_vr_BE, S.adv_vt_BE, S.adv_x_BE][kind]
        x = fn(LL, RR, c1, c2, dt, b, Nr, Nvt, Nx)
        a = coef()
        for line in range(shape[0]):
            Dm = S.band_by_column_to_dense(LL if ltr(a[line]) else RR, ltr(a[line]))
            M = np.eye(N) + a[line] * dt * Dm
            np.testing.assert_allclose(M @ x[line], b[line], rtol=1e-10, atol=1e-10)


def test_bsr_upper_unit():
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(7)
    nbr, bs, nrhs = 6, 4, 3
    A = rng.standard_normal((nbr * bs, nbr * bs)) * (rng.random((nbr * bs, nbr * bs)) < 0.3)
    Ab = sp.bsr_matrix(A, blocksize=(bs, bs))
    Ab.sort_indices()
    b = rng.standard_normal((nrhs, nbr * bs))
    x = S.bsr_upper_unit_solve(Ab.data, Ab.indptr, Ab.indices, bs, b)
    U = np.triu(A, 0)
    for i in range(nbr):  # unit diagonal blocks, strictly upper block part only
        U[i * bs:(i + 1) * bs, :(i + 1) * bs] = 0.0
        U[i * bs:(i + 1) * bs, i * bs:(i + 1) * bs] = np.eye(bs)
    np.testing.assert_allclose(x @ U.T, b, rtol=1e-10, atol=1e-10)
