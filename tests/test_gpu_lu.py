"""Batched LU through the C ABI against numpy.linalg.solve."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [1, 7, 31, 64, 129, 385, 600, 1281])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("kernel", [0, 1, 2, 4, 5, 6], ids=["auto", "right", "tc", "tc1", "tc128", "split"])
def test_lu_factor_solve(N, dtype, kernel):
    if kernel == 6 and dtype != "f64":
        pytest.skip("the split kernel is FP64")
    if kernel in (2, 4, 5) and (dtype == "f64" or N > 512):
        pytest.skip("the tensor-core factorization is FP32 with N <= 512")
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(N)
    P = 5
    A = rng.standard_normal((P, N, N)) + np.eye(N) * 0.1
    b = rng.standard_normal((P, N))
    tdt = torch.float64 if dtype == "f64" else torch.float32
    dA = torch.as_tensor(A, dtype=tdt, device="cuda").contiguous()
    db = torch.as_tensor(b, dtype=tdt, device="cuda").contiguous()
    piv = torch.empty((P, N), dtype=torch.int32, device="cuda")
    info = torch.empty(P, dtype=torch.int32, device="cuda")
    dt = 0 if dtype == "f64" else 1
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.bte_lu_factor_ex(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                    C.c_void_p(info.data_ptr()), kernel, st), "lu_factor")
    _lib.check(lib.bte_lu_solve(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                C.c_void_p(db.data_ptr()), st), "lu_solve")
    torch.cuda.synchronize()
    x = db.cpu().numpy().astype(np.float64)
    # normwise backward error ||A x - b|| / (||A|| ||x|| + ||b||), bounded by c N eps for LU with partial pivoting
    Ad = A.astype(np.float32).astype(np.float64) if dtype == "f32" else A
    bd = b.astype(np.float32).astype(np.float64) if dtype == "f32" else b
    res = np.einsum("pij,pj->pi", Ad, x) - bd
    berr = np.linalg.norm(res, axis=1) / (np.linalg.norm(Ad, ord=2, axis=(1, 2)) * np.linalg.norm(x, axis=1)
                                           + np.linalg.norm(bd, axis=1))
    eps = np.finfo(np.float64 if dtype == "f64" else np.float32).eps
    assert np.all(info.cpu().numpy() == 0)
    assert np.max(berr) < 2 * N * eps, (berr, N * eps)
    if dtype == "f64":
        ref = np.linalg.solve(A, b[..., None])[..., 0]
        assert np.max(np.linalg.norm(x - ref, axis=1) / np.linalg.norm(ref, axis=1)) < 1e-9


def test_lu_zero_pivot_reported():
    """A singular matrix reports the first zero pivot instead of faulting or returning NaN silently."""
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    N = 40
    A = np.eye(N)
    A[17, 17] = 0.0
    dA = torch.as_tensor(A[None], device="cuda").contiguous()
    piv = torch.empty((1, N), dtype=torch.int32, device="cuda")
    info = torch.empty(1, dtype=torch.int32, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.bte_lu_factor(0, 1, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                 C.c_void_p(info.data_ptr()), st), "lu_factor")
    torch.cuda.synchronize()
    assert int(info.item()) == 18


@pytest.mark.parametrize("kernel", [0, 6], ids=["auto", "split"])
def test_lu_zero_pivot_reported_fp64_kernels(kernel):
    """The first zero pivot (1-based) in a later panel, from the one-CTA and the split FP64 kernels."""
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    N = 100
    A = np.eye(N)
    A[70, 70] = 0.0
    dA = torch.as_tensor(np.stack([A, np.eye(N)]), device="cuda").contiguous()
    piv = torch.empty((2, N), dtype=torch.int32, device="cuda")
    info = torch.empty(2, dtype=torch.int32, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.bte_lu_factor_ex(0, 2, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                    C.c_void_p(info.data_ptr()), kernel, st), "lu_factor")
    torch.cuda.synchronize()
    assert info.cpu().numpy().tolist() == [71, 0]


@pytest.mark.parametrize("N", [129, 385, 1281])
def test_lu_split_matches_one_cta_kernel(N):
    """The split FP64 factorization (kernel 6) of many matrices with the solver's padded rows
    and appended right-hand side (NC = N + 1): the same pivots as the one-CTA kernel on
    well-separated pivots, and factors that agree to FP64 rounding."""
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    P = 40
    ld = N + 4
    rng = np.random.default_rng(N + 5)
    A = rng.standard_normal((P, N, ld))
    out = []
    for kernel in (1, 6):
        dA = torch.as_tensor(A, device="cuda").contiguous()
        piv = torch.empty((P, N), dtype=torch.int32, device="cuda")
        info = torch.empty(P, dtype=torch.int32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(lib.bte_lu_factor_ex(0, P, N, C.c_void_p(dA.data_ptr()), ld, N * ld, C.c_void_p(piv.data_ptr()),
                                        C.c_void_p(info.data_ptr()), kernel, C.c_void_p(st)), "lu_factor")
        torch.cuda.synchronize()
        assert np.all(info.cpu().numpy() == 0)
        out.append((dA.cpu().numpy(), piv.cpu().numpy()))
    (a1, p1), (a6, p6) = out
    assert np.array_equal(p1, p6)
    # columns 0..N-1 hold L\U; the appended column is outside the factorization here (NC = N)
    d = np.abs(a1[:, :, :N] - a6[:, :, :N]).max() / np.abs(a1[:, :, :N]).max()
    assert d < 1e-11, d
    for i in range(3):
        LU = a6[i][p6[i], :N]
        L = np.tril(LU, -1) + np.eye(N)
        U = np.triu(LU)
        berr = np.abs(L @ U - A[i][p6[i], :N]).max() / np.abs(A[i]).max()
        assert berr < 50 * N * np.finfo(np.float64).eps, berr


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("N", [32, 64, 200])
def test_lu_negative_zero_is_not_a_pivot(dtype, N):
    """-0.0 entries below a nonzero diagonal (as -dt * 0 produces) must never be chosen as
    pivots: an identity with -0.0 below the diagonal factors with the identity permutation."""
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    P = 3
    A = np.eye(N)
    A[np.tril_indices(N, -1)] = -0.0  # assigned, not added: -0.0 + 0.0 is +0.0
    A = np.broadcast_to(A, (P, N, N)).copy()
    tdt = torch.float64 if dtype == "f64" else torch.float32
    dA = torch.as_tensor(A, dtype=tdt, device="cuda").contiguous()
    assert bool(torch.signbit(dA[0, 1, 0]))
    piv = torch.empty((P, N), dtype=torch.int32, device="cuda")
    info = torch.empty(P, dtype=torch.int32, device="cuda")
    b = torch.arange(P * N, dtype=tdt, device="cuda").reshape(P, N).contiguous()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    dt = 0 if dtype == "f64" else 1
    _lib.check(lib.bte_lu_factor(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                 C.c_void_p(info.data_ptr()), st), "lu_factor")
    x = b.clone()
    _lib.check(lib.bte_lu_solve(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                C.c_void_p(x.data_ptr()), st), "lu_solve")
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == 0)
    assert np.array_equal(piv.cpu().numpy(), np.broadcast_to(np.arange(N), (P, N)))
    assert torch.equal(x, b)


@pytest.mark.parametrize("N", [33, 128, 385, 512])
@pytest.mark.parametrize("kernel", [0, 2, 4, 5], ids=["auto", "tc", "tc1", "tc128"])
def test_lu_padded_rows_against_fp64(N, kernel):
    """FP32 factors with 16-byte aligned rows (the Newton solver's layout, vectorised path of
    the tensor-core kernel): backward error at FP32 level, and the tensor-core factors'
    solution as accurate as the SIMT kernel's (the split-TF32 products keep FP32 accuracy)."""
    import torch
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(1000 + N)
    P, ld = 7, (N + 3) & ~3
    A = rng.standard_normal((P, N, N)) + np.eye(N) * 0.5
    b = rng.standard_normal((P, N))
    Ap = np.zeros((P, N, ld), dtype=np.float32)
    Ap[:, :, :N] = A
    dA = torch.as_tensor(Ap, device="cuda").contiguous()
    db = torch.as_tensor(b, dtype=torch.float32, device="cuda").contiguous()
    piv = torch.empty((P, N), dtype=torch.int32, device="cuda")
    info = torch.empty(P, dtype=torch.int32, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.bte_lu_factor_ex(1, P, N, C.c_void_p(dA.data_ptr()), ld, N * ld, C.c_void_p(piv.data_ptr()),
                                    C.c_void_p(info.data_ptr()), kernel, st), "lu_factor")
    _lib.check(lib.bte_lu_solve(1, P, N, C.c_void_p(dA.data_ptr()), ld, N * ld, C.c_void_p(piv.data_ptr()),
                                C.c_void_p(db.data_ptr()), st), "lu_solve")
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == 0)
    x = db.cpu().numpy().astype(np.float64)
    Ad = A.astype(np.float32).astype(np.float64)
    bd = b.astype(np.float32).astype(np.float64)
    res = np.einsum("pij,pj->pi", Ad, x) - bd
    berr = np.linalg.norm(res, axis=1) / (np.linalg.norm(Ad, ord=2, axis=(1, 2)) * np.linalg.norm(x, axis=1)
                                           + np.linalg.norm(bd, axis=1))
    eps = np.finfo(np.float32).eps
    assert np.max(berr) < 2 * N * eps, (berr, N * eps)


def test_autotuner_picks_a_measured_kernel(tmp_path, monkeypatch):
    """The autotuner times every FP32 candidate for a size, keeps the fastest, and caches the
    choice on disk; a second call reads it back without timing."""
    from boltzmann_gb300 import autotune
    monkeypatch.setenv("BOLTZMANN_GB300_CACHE", str(tmp_path))
    monkeypatch.setattr(autotune, "_mem", {})
    rec = autotune.tune_lu(129, P=256)
    assert rec["kernel"] in autotune.CANDIDATES_SMALL
    assert rec["ms"][str(rec["kernel"])] == min(rec["ms"].values())
    assert (tmp_path / "lu_autotune.json").exists()
    monkeypatch.setattr(autotune, "_mem", {})
    monkeypatch.setattr(autotune, "time_lu", lambda *a, **k: pytest.fail("timed again"))
    assert autotune.tune_lu(129)["kernel"] == rec["kernel"]
