"""The finite-volume 1D3V op-split step on the GPU (boltzmann_gb300.bte_1d3v_fvm) against the
reference's own step (tests/golden/fvm_reference.npz), and its building blocks (FP64 GEMM,
axis permutation) against NumPy."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fvm_reference.npz")


def _t(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_gemm_and_permute():
    import ctypes as C
    import torch
    from boltzmann_gb300 import _lib
    from boltzmann_gb300.native_kernels import _ptr, _stream
    lib = _lib.load()
    rng = np.random.default_rng(21)
    M, K, N = 70, 45, 33
    A, B = rng.standard_normal((M, K)), rng.standard_normal((K, N))
    Cd = torch.empty(M, N, dtype=torch.float64, device="cuda")
    assert lib.bte_dgemm_nn(M, N, K, _ptr(_t(A)), K, _ptr(_t(B)), N, _ptr(Cd), N, _stream()) == 0
    np.testing.assert_allclose(Cd.cpu().numpy(), A @ B, rtol=1e-13, atol=1e-13)
    x = rng.standard_normal((3, 5, 7))
    for p in [(2, 1, 0), (0, 2, 1), (1, 2, 0)]:
        out = torch.empty(x.size, dtype=torch.float64, device="cuda")
        assert lib.bte_permute3(3, 5, 7, p[0], p[1], p[2], _ptr(_t(x)), _ptr(out), _stream()) == 0
        np.testing.assert_array_equal(out.cpu().numpy().reshape(np.transpose(x, p).shape), np.transpose(x, p))


def test_op_split_step_matches_the_reference():
    from boltzmann_gb300.bte_1d3v_fvm import FvmOpSplit
    g = dict(np.load(GOLDEN))
    st = FvmOpSplit(g["PmatC"], g["vr_diag_l2r"], g["vr_diag_r2l"], g["vt_diag_l2r"], g["vt_diag_r2l"],
                    g["x_diag_l2r"], g["x_diag_r2l"], g["vr"], g["vt"], int(g["Nx"]), float(g["tau"]),
                    float(g["qe"]), float(g["me"]), float(g["vth"]), float(g["L"]))
    y = st.step(g["E"], _t(g["v0"]), float(g["dt"])).cpu().numpy()
    ref = g["step"]
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
