"""Stand-in for the un-vendored `lxcat_data_parser` package (test infrastructure only).

Backed by the project's own LXCat reader so that the reference, the oracle and the
product all read the same tabulated file the same way.
"""
import os as _os
import sys as _sys

_sys.path.insert(0, _os.path.abspath(_os.path.join(_os.path.dirname(__file__), "..", "..", "..")))
from boltzmann_gb300.lxcat import parse_lxcat as _parse  # noqa: E402


class CrossSectionSet:
    def __init__(self, file, imposed_species=None):
        blocks = _parse(file)
        if imposed_species is not None:
            blocks = [b for b in blocks if b.species == imposed_species]
        self.cross_sections = blocks
        self.species = imposed_species
