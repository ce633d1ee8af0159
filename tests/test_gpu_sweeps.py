"""The library's batched banded kernels (include/bte_sweeps_gb300.h, through
boltzmann_gb300.native_kernels) against the oracle restating the reference's raw kernels
(rawkernel.py) and BSR triangular solve. Same recurrences in FP64: agreement to 1e-12
relative, both advection directions exercised."""
import numpy as np
import pytest

from oracle import sweeps_oracle as S

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _t(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _close(got, ref):
    got = got.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= TOL * max(np.max(np.abs(ref)), 1e-300)


@pytest.mark.parametrize("lower", [True, False])
def test_bidiagonal_banded_solve_and_mv(lower):
    from boltzmann_gb300 import native_kernels as K
    rng = np.random.default_rng(11)
    bsz, N, nd = 300, 48, 5
    d = rng.uniform(1.0, 2.0, (bsz, N))
    s = rng.standard_normal((bsz, N - 1)) * 0.5
    b = rng.standard_normal((bsz, N))
    _close(K.bidiagonal_solve_batched(_t(d), _t(s), _t(b), lower), S.bidiagonal_solve(d, s, b, lower))
    D = rng.standard_normal((bsz, nd, N)) * 0.3
    D[:, 0] = rng.uniform(1.0, 2.0, (bsz, N))
    _close(K.banded_tri_solve_batched(_t(D), _t(b), lower), S.banded_tri_solve(D, b, lower))
    _close(K.banded_tri_mv_batched(_t(D), _t(b), lower), S.banded_tri_mv(D, b, lower))


def test_advection_sweeps():
    import torch
    from boltzmann_gb300 import native_kernels as K
    rng = np.random.default_rng(12)
    Nr, Nvt, Nx, nd, dt = 24, 8, 30, 3, 0.05
    Ex = rng.standard_normal(Nx) * 3.0          # both signs: both sweep directions
    cos_vt = np.cos(np.linspace(0.05, np.pi - 0.05, Nvt))
    vr = rng.uniform(0.3, 3.0, Nr)
    for kind, (c1, c2, N, shape) in enumerate([(Ex, cos_vt, Nr, (Nx * Nvt, Nr)), (Ex, vr, Nvt, (Nx * Nr, Nvt)),
                                               (vr, cos_vt, Nx, (Nr * Nvt, Nx))]):
        L = rng.uniform(0.1, 1.0, (nd, N))
        R = rng.uniform(0.1, 1.0, (nd, N))
        b = rng.standard_normal(shape)
        out = torch.empty(shape, dtype=torch.float64, device="cuda")
        fn = [K.adv_vr_BE, K.adv_vt_BE, K.adv_x_BE][kind]
        ref = [S.adv_vr_BE, S.adv_vt_BE, S.adv_x_BE][kind](L, R, c1, c2, dt, b, Nr, Nvt, Nx)
        fn(_t(L), _t(R), _t(c1), _t(c2), dt, _t(b), out, nd, Nr, Nvt, Nx)
        _close(out, ref)


def test_bsr_upper_unit_solve():
    sp = pytest.importorskip("scipy.sparse")
    from boltzmann_gb300 import native_kernels as K
    rng = np.random.default_rng(13)
    nbr, bs, nrhs = 20, 16, 12        # the reference pairs blocks of Nvt with Nx right-hand sides
    A = rng.standard_normal((nbr * bs, nbr * bs)) * (rng.random((nbr * bs, nbr * bs)) < 0.2) * 0.2
    Ab = sp.bsr_matrix(A, blocksize=(bs, bs))
    Ab.sort_indices()
    b = rng.standard_normal((nrhs, nbr * bs))
    solver = K.BsrUpperUnitSolver(Ab)
    _close(solver.solve(_t(b)), S.bsr_upper_unit_solve(Ab.data, Ab.indptr, Ab.indices, bs, b))


def test_argument_errors():
    import torch
    from boltzmann_gb300 import native_kernels as K
    b = torch.zeros(4, 8, dtype=torch.float64, device="cuda")
    with pytest.raises(TypeError):
        K.bidiagonal_solve_batched(b.cpu(), b[:, :7], b, True)
    with pytest.raises(ValueError):
        K.banded_tri_solve_batched(torch.ones(4, 2, 8, dtype=torch.float64, device="cuda"), b[:, :5], True)
