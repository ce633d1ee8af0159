"""Batched LU through the C ABI against numpy.linalg.solve."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [1, 7, 31, 64, 129, 385, 600, 1281])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_lu_factor_solve(N, dtype):
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
    _lib.check(lib.bte_lu_factor(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                 C.c_void_p(info.data_ptr()), st), "lu_factor")
    _lib.check(lib.bte_lu_solve(dt, P, N, C.c_void_p(dA.data_ptr()), N, N * N, C.c_void_p(piv.data_ptr()),
                                C.c_void_p(db.data_ptr()), st), "lu_solve")
    torch.cuda.synchronize()
    x = db.cpu().numpy().astype(np.float64)
    ref = np.linalg.solve(A, b[..., None])[..., 0]
    tol = 1e-10 if dtype == "f64" else 2e-3
    err = np.linalg.norm(x - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.all(info.cpu().numpy() == 0)
    assert np.max(err) < tol, err
