"""Batched banded kernels of the 1D3V finite-volume path, with the reference's Python API.

Drop-ins for the functions of the reference's `BESolver/python/rawkernel.py` (CuPy raw
kernels) and for the unit upper BSR triangular solve of `cusparse_spsolve.py`
(`SpSMSolver(A, lower=False, unit_diagonal=True)`), running the library's sm_103a kernels
(`include/bte_sweeps_gb300.h`). Arrays are CUDA tensors (float64, contiguous) in the
reference's layouts; results are new tensors, as the reference returns new CuPy arrays
(the adv_*_BE functions write into the given `out`, as the reference's do). There is no CPU
path: a missing library or a CPU tensor raises.
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def _torch():
    import torch
    return torch


def _dev(t, name):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != torch.float64:
        raise TypeError("%s must be float64" % name)
    return t.contiguous()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (code %d): %s" % (what, rc, _lib.load().bte_sweep_last_error().decode()))


def bidiagonal_solve_batched(diag, sdiag, b, lower):
    """rawkernel.bidiagonal_solve_batched (rawkernel.py:389-413): diag (..., N), sdiag
    (..., N-1) the sub- (lower) or super-diagonal, b (..., N) -> x."""
    diag, sdiag, b = _dev(diag, "diag"), _dev(sdiag, "sdiag"), _dev(b, "b")
    N = diag.shape[-1]
    bsz = diag.numel() // N
    if sdiag.shape[-1] != N - 1 or sdiag.numel() // max(N - 1, 1) != bsz or b.numel() != bsz * N:
        raise ValueError("shape mismatch")
    out = _torch().empty_like(b)
    _check(_lib.load().bte_bidiag_solve(bsz, N, _ptr(diag), _ptr(sdiag), _ptr(b), _ptr(out), int(bool(lower)),
                                        _stream()), "bidiagonal_solve_batched")
    return out.reshape(diag.shape)


def banded_tri_solve_batched(diags, b, lower):
    """rawkernel.banded_tri_solve_batched (rawkernel.py:415-439): diags (..., ndiags, N)
    stored by row (lower L[i][i-k] = diags[k][i]; upper U[i][i+k] = diags[k][i]), b (..., N)."""
    diags, b = _dev(diags, "diags"), _dev(b, "b")
    nd, N = diags.shape[-2], diags.shape[-1]
    bsz = diags.numel() // (nd * N)
    if b.numel() != bsz * N:
        raise ValueError("shape mismatch")
    out = _torch().empty_like(b)
    _check(_lib.load().bte_banded_tri_solve(bsz, nd, N, _ptr(diags), _ptr(b), _ptr(out), int(bool(lower)), _stream()),
           "banded_tri_solve_batched")
    return out.reshape(b.shape)


def banded_tri_mv_batched(diags, b, lower):
    """rawkernel.banded_tri_mv_batched (rawkernel.py:441-466): out = L b or U b."""
    diags, b = _dev(diags, "diags"), _dev(b, "b")
    nd, N = diags.shape[-2], diags.shape[-1]
    bsz = diags.numel() // (nd * N)
    if b.numel() != bsz * N:
        raise ValueError("shape mismatch")
    out = _torch().empty_like(b)
    _check(_lib.load().bte_banded_tri_mv(bsz, nd, N, _ptr(diags), _ptr(b), _ptr(out), int(bool(lower)), _stream()),
           "banded_tri_mv_batched")
    return out.reshape(b.shape)


def _adv(kind, D_LtoR, D_RtoL, c1, c2, dt, b, out, ndiags, Nr, Nvt, Nx, name):
    D_LtoR, D_RtoL = _dev(D_LtoR, "D_LtoR"), _dev(D_RtoL, "D_RtoL")
    c1, c2, b = _dev(c1, "c1"), _dev(c2, "c2"), _dev(b, "b")
    if not (out.is_cuda and out.is_contiguous() and out.dtype == b.dtype and out.numel() == b.numel()):
        raise ValueError("out must be a contiguous float64 CUDA tensor of b's size")
    if b.numel() != Nr * Nvt * Nx:
        raise ValueError("b must hold Nr * Nvt * Nx values")
    N = (Nr, Nvt, Nx)[kind]
    if D_LtoR.numel() != ndiags * N or D_RtoL.numel() != ndiags * N:
        raise ValueError("D_LtoR and D_RtoL must be (ndiags, %d)" % N)
    if c1.numel() != (Nx, Nx, Nr)[kind] or c2.numel() != (Nvt, Nr, Nvt)[kind]:
        raise ValueError("coefficient vectors of the wrong length")
    _check(_lib.load().bte_adv_be_sweep(kind, _ptr(D_LtoR), _ptr(D_RtoL), _ptr(c1), _ptr(c2), float(dt), _ptr(b),
                                        _ptr(out), int(ndiags), int(Nr), int(Nvt), int(Nx), _stream()), name)


def adv_vr_BE(D_LtoR, D_RtoL, Ex, cos_vt, dt, b, out, ndiags, Nr, Nvt, Nx):
    """rawkernel.adv_vr_BE (rawkernel.py:468-479): b, out (Nx * Nvt, Nr)."""
    _adv(0, D_LtoR, D_RtoL, Ex, cos_vt, dt, b, out, ndiags, Nr, Nvt, Nx, "adv_vr_BE")


def adv_vt_BE(D_LtoR, D_RtoL, Ex, vr, dt, b, out, ndiags, Nr, Nvt, Nx):
    """rawkernel.adv_vt_BE (rawkernel.py:481-492): b, out (Nx * Nr, Nvt)."""
    _adv(1, D_LtoR, D_RtoL, Ex, vr, dt, b, out, ndiags, Nr, Nvt, Nx, "adv_vt_BE")


def adv_x_BE(D_LtoR, D_RtoL, vr, cos_vt, dt, b, out, ndiags, Nr, Nvt, Nx):
    """rawkernel.adv_x_BE (rawkernel.py:494-505): b, out (Nr * Nvt, Nx)."""
    _adv(2, D_LtoR, D_RtoL, vr, cos_vt, dt, b, out, ndiags, Nr, Nvt, Nx, "adv_x_BE")


class BsrUpperUnitSolver:
    """Unit upper block-triangular solves with a fixed BSR matrix, as the reference's
    cusparse_spsolve.SpSMSolver(A, lower=False, unit_diagonal=True) (cusparse_spsolve.py:71-
    300, spsm_bsr_upper_tri_solve.cu): A a scipy.sparse BSR matrix (sorted indices), solve(b)
    with b (nrhs, n) on the device -> x."""

    def __init__(self, A_bsr, device=None):
        torch = _torch()
        if A_bsr.format != "bsr":
            raise ValueError("A must be a BSR matrix")
        r, c = A_bsr.blocksize
        if r != c:
            raise ValueError("square blocks required")
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.bs = r
        self.nbr = A_bsr.shape[0] // r
        self.n = A_bsr.shape[0]
        self.data = torch.as_tensor(A_bsr.data, dtype=torch.float64, device=dev).contiguous()
        self.indptr = torch.as_tensor(A_bsr.indptr, dtype=torch.int32, device=dev).contiguous()
        self.indices = torch.as_tensor(A_bsr.indices, dtype=torch.int32, device=dev).contiguous()

    def solve(self, b):
        b = _dev(b, "b")
        nrhs = b.numel() // self.n
        if b.numel() != nrhs * self.n:
            raise ValueError("b must hold whole right-hand sides of length %d" % self.n)
        out = _torch().empty_like(b)
        _check(_lib.load().bte_bsr_upper_unit_solve(self.nbr, self.bs, nrhs, _ptr(self.data), _ptr(self.indptr),
                                                    _ptr(self.indices), _ptr(b), _ptr(out), _stream()),
               "BsrUpperUnitSolver.solve")
        return out
