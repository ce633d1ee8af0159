"""CPU stand-in for the `cupy` names the reference imports (test infrastructure only).

The reference's batched 0D3V class falls back to NumPy when `use_gpu=0`; it still
calls `cp.get_array_module`, `cp.asnumpy` and a few attributes at import time.
"""
import numpy as _np


def get_array_module(*args):
    return _np


def asnumpy(a):
    return _np.asarray(a)


def asarray(a):
    return _np.asarray(a)


class ndarray(_np.ndarray):
    pass


class RawKernel:
    def __init__(self, *a, **k):
        self.args = a

    def __call__(self, *a, **k):
        raise RuntimeError("cupy RawKernel is not available in the CPU oracle")


class _Cuda:
    class runtime:
        @staticmethod
        def deviceSynchronize():
            return None

    class nvtx:
        @staticmethod
        def RangePush(*a):
            return None

        @staticmethod
        def RangePop():
            return None

    class Device:
        def __init__(self, *a):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False


cuda = _Cuda()
