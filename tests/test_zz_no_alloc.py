"""bte_initialize_noalloc: the Maxwellian initial state from a call that allocates no device memory.

The entry point exists for callers that cannot allocate device memory when they set up
points (for instance a serving process whose device memory is all held by another
allocator), so it keeps its scratch in a static device array of the library. These tests
call it through the C ABI and compare it with bte_initialize, the allocating entry point,
on two calls in a row (the second on a different grid, so that contents the first call left
in the shared scratch would show up), and check that a grid beyond the scratch's limit is
refused with a clear error. This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import gpu_solver, relmax

pytestmark = pytest.mark.gpu

TOL = 1e-13  # the two entry points differ only in how the 2-point angular rule's nodes are rounded


def _init(lib_fn, s, P):
    import torch
    n = s._grid_info[0]["n"]
    f = torch.full((P, n), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib_fn(s._grid[0], P, C.c_void_p(f.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, f


def test_noalloc_matches_initialize_on_two_calls(synthetic_xs):
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    grids = [gpu_solver(synthetic_xs, 64, 1, False, 3)[0], gpu_solver(synthetic_xs, 40, 2, False, 3)[0]]
    for s in grids:  # two calls in a row, on different grids
        rc, ref = _init(lib.bte_initialize, s, 3)
        _lib.check(rc, "bte_initialize")
        rc, got = _init(lib.bte_initialize_noalloc, s, 3)
        _lib.check(rc, "bte_initialize_noalloc")
        got, ref = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert relmax(got, ref) < TOL


def test_noalloc_rejects_grid_beyond_scratch(synthetic_xs):
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    s = gpu_solver(synthetic_xs, 520, 0, False, 1)[0]
    rc, f = _init(lib.bte_initialize_noalloc, s, 1)
    assert rc == -1
    assert b"n_sp <= 512" in lib.bte_last_error()
    assert bool(f.isnan().all())  # nothing written
    rc, _ = _init(lib.bte_initialize, s, 1)  # the allocating entry point takes the same grid
    _lib.check(rc, "bte_initialize")
