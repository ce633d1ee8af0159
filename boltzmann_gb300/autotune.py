"""Autotuner of the batched FP32 Newton factorization.

For a bordered system size N the library has several FP32 LU kernels (`bte_lu_factor_ex`):
  2  split-TF32 trailing updates on the tcgen05 tensor cores, two CTAs per SM;
  4  the same kernel with one CTA per SM (half the matrices in flight, so that their trailing
     matrices stay in L2);
  5  the same kernel with 128 threads per CTA (4 warps share the per-column pivot search);
  3  the left-looking SIMT kernel (blocks held in registers);
  1  the right-looking SIMT kernel (any N; the only choice above N = 512).
`tune_lu(N)` times every candidate on seeded synthetic systems of that size (diagonally shifted
normal matrices, the solver's 16-byte aligned row layout), one matrix per CTA in waves like
the solve's, and keeps the fastest; the choice is cached in memory and on disk per (GPU name,
N), in `$BOLTZMANN_GB300_CACHE` or `~/.cache/boltzmann_gb300/lu_autotune.json`. The solver
passes it as `bte_solve_opts.lu_kernel`. The reference has no counterpart: it calls one
library inverse (xp.linalg.inv, bte_0d3v_batched.py:856-880).
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading

from . import _lib

CANDIDATES_SMALL = (2, 4, 5, 3, 1)
CANDIDATES_LARGE = (1,)
_mem: dict = {}
_lock = threading.Lock()


def cache_path() -> str:
    d = os.environ.get("BOLTZMANN_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "boltzmann_gb300")
    return os.path.join(d, "lu_autotune.json")


def _load_disk() -> dict:
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_disk(key, rec) -> None:
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load_disk()
        data[key] = rec
        tmp = path + ".%d.tmp" % os.getpid()
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: the choice stays in memory


def _key(N, device):
    import torch
    return "%s|N=%d" % (torch.cuda.get_device_name(device), int(N))


def time_lu(N, kernel, P=1024, reps=3, device=0, seed=17):
    """Median device time (ms) of one bte_lu_factor_ex launch of `kernel` on P systems of size N."""
    import torch
    torch.cuda.set_device(device)
    lib = _lib.load()
    ld = (N + 1 + 3) & ~3
    g = torch.Generator(device="cuda").manual_seed(seed + N)
    A0 = torch.randn((P, N, ld), device="cuda", generator=g, dtype=torch.float32)
    A0[:, :, :N] += 2.0 * torch.eye(N, device="cuda")
    A = torch.empty_like(A0)
    piv = torch.empty((P, N), dtype=torch.int32, device="cuda")
    info = torch.empty(P, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    times = []
    for r in range(reps + 1):
        A.copy_(A0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        _lib.check(lib.bte_lu_factor_ex(1, P, N, C.c_void_p(A.data_ptr()), ld, N * ld, C.c_void_p(piv.data_ptr()),
                                        C.c_void_p(info.data_ptr()), kernel, C.c_void_p(st.cuda_stream)),
                   "bte_lu_factor_ex")
        e1.record(st)
        torch.cuda.synchronize()
        if r > 0:
            times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def tune_lu(N, P=1024, device=0, force=False):
    """The fastest FP32 factorization kernel for bordered size N: {"kernel", "ms" per candidate}."""
    key = _key(N, device)
    with _lock:
        if not force and key in _mem:
            return _mem[key]
        if not force:
            rec = _load_disk().get(key)
            if rec and rec.get("kernel") in (CANDIDATES_SMALL if N <= 512 else CANDIDATES_LARGE):
                _mem[key] = rec
                return rec
        cands = CANDIDATES_SMALL if N <= 512 else CANDIDATES_LARGE
        ms = {str(k): time_lu(N, k, P=P, device=device) for k in cands}
        best = min(cands, key=lambda k: ms[str(k)])
        rec = {"kernel": int(best), "ms": ms, "P": int(P)}
        _mem[key] = rec
        _store_disk(key, rec)
        return rec


def lu_kernel_for(N, device=0) -> int:
    """bte_solve_opts.lu_kernel for bordered size N (tuned on first use)."""
    return int(tune_lu(N, device=device)["kernel"])


def choices() -> dict:
    """The choices made in this process, for reports."""
    with _lock:
        return dict(_mem)
