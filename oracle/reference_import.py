"""Import the reference's CPU path in this container (test infrastructure only).

Used by `tests/golden/make_golden.py` to run the unmodified reference (NumPy path,
`use_gpu=0`) and record golden vectors. It never runs on the GPU host and nothing in
the product imports it. The recipe:

1. put `oracle/ref_shim` (stand-ins for cupy, multiprocess, lxcat_data_parser,
   matplotlib, h5py, findiff, toml) first on `sys.path`, then the reference's
   `BESolver/python` directory;
2. while importing, make `np.load` / `np.genfromtxt` return zeros for the polynomial
   tables that the reference checkout lacks (they only feed the non-spline bases);
3. `chdir` into `BESolver/python`, as the reference's drivers assume.
"""
import os
import sys
import contextlib

import numpy as np

REF_ROOT = os.environ.get("BOLTZ_REFERENCE_ROOT", "/root/reference")
REF_PY = os.path.join(REF_ROOT, "BESolver", "python")
SHIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_shim")


@contextlib.contextmanager
def _missing_tables_as_zeros():
    real_load, real_gft = np.load, np.genfromtxt

    def load(path, *a, **k):
        try:
            return real_load(path, *a, **k)
        except (FileNotFoundError, OSError, ValueError):
            return np.zeros((8, 8, 8))

    def gft(path, *a, **k):
        try:
            return real_gft(path, *a, **k)
        except (FileNotFoundError, OSError, ValueError):
            return np.zeros((8, 8))

    np.load, np.genfromtxt = load, gft
    try:
        yield
    finally:
        np.load, np.genfromtxt = real_load, real_gft


def available() -> bool:
    return os.path.isdir(REF_PY)


def import_reference():
    """Return the reference's `bte_0d3v_batched` module (CPU path)."""
    if not available():
        raise RuntimeError("reference checkout not found at %s" % REF_ROOT)
    for p in (REF_PY, SHIM):
        if p in sys.path:
            sys.path.remove(p)
    sys.path.insert(0, REF_PY)
    sys.path.insert(0, SHIM)
    os.chdir(REF_PY)
    with _missing_tables_as_zeros():
        import bte_0d3v_batched  # noqa: F401
    return sys.modules["bte_0d3v_batched"]
