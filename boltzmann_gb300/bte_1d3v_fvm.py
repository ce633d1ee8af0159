"""The finite-volume 1D3V op-split step on the GPU.

Counterpart of the reference's `bte_1d3v.step_op_split` with type XVTVRC
(BESolver/python/bte_1d3v_solver.py:1745-1870), the preconditioner step of its fully implicit
FVM solver, composed from the library's kernels (`include/bte_sweeps_gb300.h`):
1. collisions: yc = PmatC v (bte_dgemm_nn);
2. v_r advection sweeps on (Nx, Nvt, Nr) (bte_adv_be_sweep kind 0, aE = tau qe / (me vth) E);
3. v_theta advection sweeps on (Nx, Nr, Nvt) (kind 1);
4. inflow zeroing and x advection sweeps on (Nr, Nvt, Nx) (kind 2, a = vth tau / L v_r cos theta).
The layout swaps between the stages run through bte_permute3. Layouts are the reference's: v is
(Nr * Nvt, Nx), radial cell major.

The operators come from the reference's FVM set-up (`init()`): the dense collision inverse
PmatC and the column-stored upwind bands of v_r, v_theta and x (bte_1d3v_solver.py:1346-1470).
This module does not assemble them; the FVM operator set-up is the path's next item.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .native_kernels import _check, _ptr, _stream


class FvmOpSplit:
    """PmatC (dof_v x dof_v), band arrays (p+1, N) of the three directions, grids vr (Nr),
    vt (Nvt), and the coefficients tau, qe, me, vth, L of the reference's parameters."""

    def __init__(self, PmatC, vr_diag_l2r, vr_diag_r2l, vt_diag_l2r, vt_diag_r2l, x_diag_l2r, x_diag_r2l, vr, vt,
                 Nx, tau, qe, me, vth, L, device=None):
        import torch
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
        self.Nr, self.Nvt, self.Nx = len(vr), len(vt), int(Nx)
        if np.shape(PmatC) != (self.Nr * self.Nvt, self.Nr * self.Nvt):
            raise ValueError("PmatC must be (Nr * Nvt) x (Nr * Nvt)")
        self.P = t(PmatC)
        self.bands = [(t(vr_diag_l2r), t(vr_diag_r2l)), (t(vt_diag_l2r), t(vt_diag_r2l)), (t(x_diag_l2r), t(x_diag_r2l))]
        for (l, r), n in zip(self.bands, (self.Nr, self.Nvt, self.Nx)):
            if l.shape[1] != n or r.shape[1] != n or l.shape[0] != r.shape[0]:
                raise ValueError("band arrays must be (p + 1, N) for their direction")
        self.vr, self.vt = t(vr), t(vt)
        self.cos_vt = t(np.cos(np.asarray(vt)))
        self.cE = float(tau) * float(qe) / float(me) / float(vth)
        self.ax = float(vth) * (float(tau) / float(L))
        self.ax_vr = t(self.ax * np.asarray(vr))
        n = self.Nr * self.Nvt * self.Nx
        self._a = torch.empty(n, dtype=torch.float64, device=dev)
        self._b = torch.empty(n, dtype=torch.float64, device=dev)
        self.dev = dev

    def step(self, E, v, dt, alpha=1.0):
        """One op-split step: v (Nr * Nvt, Nx) CUDA float64, E (Nx) the field -> new v."""
        import torch
        lib, s = _lib.load(), _stream()
        Nr, Nvt, Nx = self.Nr, self.Nvt, self.Nx
        dof = Nr * Nvt
        v = v.contiguous()
        if v.numel() != dof * Nx or not v.is_cuda or v.dtype != torch.float64:
            raise ValueError("v must be a (Nr * Nvt, Nx) float64 CUDA tensor")
        aE = torch.as_tensor(np.asarray(E), dtype=torch.float64, device=self.dev) * self.cE
        h = float(alpha) * float(dt)
        a, b = self._a, self._b
        _check(lib.bte_dgemm_nn(dof, Nx, dof, _ptr(self.P), dof, _ptr(v), Nx, _ptr(a), Nx, s), "collision solve")
        # (Nr, Nvt, Nx) -> (Nx, Nvt, Nr)
        _check(lib.bte_permute3(Nr, Nvt, Nx, 2, 1, 0, _ptr(a), _ptr(b), s), "layout")
        (l, r) = self.bands[0]
        _check(lib.bte_adv_be_sweep(0, _ptr(l), _ptr(r), _ptr(aE), _ptr(self.cos_vt), h, _ptr(b), _ptr(a), l.shape[0],
                                    Nr, Nvt, Nx, s), "v_r sweep")
        # (Nx, Nvt, Nr) -> (Nx, Nr, Nvt)
        _check(lib.bte_permute3(Nx, Nvt, Nr, 0, 2, 1, _ptr(a), _ptr(b), s), "layout")
        (l, r) = self.bands[1]
        _check(lib.bte_adv_be_sweep(1, _ptr(l), _ptr(r), _ptr(aE), _ptr(self.vr), h, _ptr(b), _ptr(a), l.shape[0],
                                    Nr, Nvt, Nx, s), "v_theta sweep")
        # (Nx, Nr, Nvt) -> (Nr, Nvt, Nx)
        _check(lib.bte_permute3(Nx, Nr, Nvt, 1, 2, 0, _ptr(a), _ptr(b), s), "layout")
        _check(lib.bte_fvm_inflow_zero(Nr, Nvt, Nx, _ptr(self.vt), _ptr(b), s), "inflow")
        (l, r) = self.bands[2]
        out = torch.empty(dof, Nx, dtype=torch.float64, device=self.dev)
        _check(lib.bte_adv_be_sweep(2, _ptr(l), _ptr(r), _ptr(self.ax_vr), _ptr(self.cos_vt), h, _ptr(b), _ptr(out),
                                    l.shape[0], Nr, Nvt, Nx, s), "x sweep")
        return out
