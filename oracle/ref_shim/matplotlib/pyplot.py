"""No-op stand-in for matplotlib.pyplot."""


class _Any:
    def __getattr__(self, name):
        return _noop

    def __call__(self, *a, **k):
        return _Any()


def _noop(*a, **k):
    return _Any()


rcParams = {}


def __getattr__(name):
    return _noop
