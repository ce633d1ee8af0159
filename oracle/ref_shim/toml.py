"""`toml.load` on top of the standard library's tomllib."""
import tomllib


def load(f):
    if isinstance(f, str):
        with open(f, "rb") as fh:
            return tomllib.load(fh)
    return tomllib.load(f)
