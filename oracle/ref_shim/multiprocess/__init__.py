"""Serial stand-in for `multiprocess.Pool` (test infrastructure only)."""


class Pool:
    def __init__(self, *a, **k):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def starmap(self, fn, it):
        return [fn(*args) for args in it]

    def map(self, fn, it):
        return [fn(a) for a in it]

    def close(self):
        pass

    def join(self):
        pass
