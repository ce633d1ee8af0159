"""No-op stand-in for matplotlib (the oracle draws nothing)."""
rcParams = {}


def use(*a, **k):
    pass
