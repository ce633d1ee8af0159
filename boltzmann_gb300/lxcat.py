"""LXCat cross-section file reader.

The reference reads tabulated electron-heavy cross sections through the third-party
`lxcat_data_parser` package (unpinned, not vendored): `BESolver/python/cross_section.py:31-69`
calls `CrossSectionSet(file, imposed_species=s)` once per species named on the file's
`SPECIES:` lines and keys the result by the text before the first comma of `PROCESS:`.
This module restates the published LXCat text format so that the product and the CPU
oracle read the same file through the same code:

    KEYWORD            ELASTIC | EFFECTIVE | EXCITATION | IONIZATION | ATTACHMENT
    target line        "Ar" or "Ar -> Ar*" (the species is the text before "->")
    parameter line     m/M for ELASTIC/EFFECTIVE, threshold (eV) for EXCITATION/IONIZATION;
                       ATTACHMENT has none
    KEY: value lines   SPECIES:, PROCESS:, PARAM.:, COMMENT:, UPDATED:, COLUMNS: ...
    -----              start of the table
    energy  sigma      two columns (eV, m^2)
    -----              end of the table

`read_available_species` and `read_cross_section_data` mirror the reference's
functions of the same names (`cross_section.py:31-41`, `:42-69`); errors raise
`ValueError` instead of calling `sys.exit`.
"""
from __future__ import annotations

import numpy as np

KEYWORDS = ("ELASTIC", "EFFECTIVE", "EXCITATION", "IONIZATION", "ATTACHMENT")


class CrossSection:
    """One tabulated process: `.info`, `.data`, `.threshold`, `.mass_ratio`, `.species`, `.type`."""

    def __init__(self, kind, species, param, info, energy, sigma):
        self.type = kind
        self.species = species
        self.info = info
        self.data = {"energy": energy, "cross section": sigma}
        self.threshold = param if kind in ("EXCITATION", "IONIZATION") else None
        self.mass_ratio = param if kind in ("ELASTIC", "EFFECTIVE") else None


def parse_lxcat(path: str) -> list[CrossSection]:
    """Parse every process block of an LXCat file, in file order."""
    with open(path, "r") as f:
        lines = [ln.rstrip("\n") for ln in f]
    out: list[CrossSection] = []
    i, n = 0, len(lines)
    while i < n:
        kw = lines[i].strip()
        if kw not in KEYWORDS:
            i += 1
            continue
        target = lines[i + 1].strip()
        species = target.split("->")[0].split("<")[0].strip()
        j = i + 2
        param = None
        if kw != "ATTACHMENT":
            tok = lines[j].strip().split()
            param = float(tok[0]) if tok else None
            j += 1
        info: dict[str, str] = {}
        while j < n and not lines[j].startswith("-----"):
            ln = lines[j]
            if ":" in ln:
                key, val = ln.split(":", 1)
                info[key.strip()] = val.strip()
            j += 1
        if j >= n:
            raise ValueError(f"{path}: table of '{kw}' block at line {i + 1} never starts")
        j += 1
        rows = []
        while j < n and not lines[j].startswith("-----"):
            tok = lines[j].split()
            if len(tok) >= 2:
                rows.append((float(tok[0]), float(tok[1])))
            j += 1
        if j >= n:
            raise ValueError(f"{path}: table of '{kw}' block at line {i + 1} never ends")
        arr = np.array(rows, dtype=np.float64).reshape(-1, 2)
        out.append(CrossSection(kw, species, param, info, arr[:, 0].copy(), arr[:, 1].copy()))
        i = j + 1
    return out


def read_available_species(path: str) -> list[str]:
    """Species named on `SPECIES: e / X` lines, first-seen order (`cross_section.py:31-41`)."""
    species = []
    with open(path, "r") as f:
        for line in f:
            if "SPECIES:" in line:
                species.append(line.split(":")[1].split("/")[1].strip())
    seen = []
    for s in species:
        if s not in seen:
            seen.append(s)
    return seen


def read_cross_section_data(path: str) -> dict:
    """process -> {info, type, species, energy, cross section, threshold, mass_ratio}.

    Iterates species in `read_available_species` order and, within a species, the
    file order of its processes, as `cross_section.py:42-69` does.
    """
    blocks = parse_lxcat(path)
    out: dict = {}
    for s in read_available_species(path):
        for b in blocks:
            if b.species != s:
                continue
            proc = b.info["PROCESS"].split(",")[0].strip()
            kind = b.info["PROCESS"].split(",")[1].strip().upper()
            out[proc] = {
                "info": b.info,
                "type": kind,
                "species": b.species,
                "energy": b.data["energy"],
                "cross section": b.data["cross section"],
                "threshold": b.threshold,
                "mass_ratio": b.mass_ratio,
            }
    return out


def write_lxcat(path: str, processes: list[dict]) -> None:
    """Write processes ({kind, species, target, param, process, energy, sigma}) as an LXCat file."""
    with open(path, "w") as f:
        for p in processes:
            f.write(p["kind"] + "\n")
            f.write(p.get("target", p["species"]) + "\n")
            if p["kind"] != "ATTACHMENT":
                f.write("%.10E\n" % p["param"])
            f.write("SPECIES: e / %s\n" % p["species"])
            f.write("PROCESS: %s, %s\n" % (p["process"], p["kind"].capitalize()))
            if p["kind"] in ("ELASTIC", "EFFECTIVE"):
                f.write("PARAM.:  m/M = %.10E\n" % p["param"])
            else:
                f.write("PARAM.:  E = %.10E eV\n" % p["param"])
            f.write("COMMENT: analytic synthetic cross section, tabulated\n")
            f.write("COLUMNS: Energy (eV) | Cross section (m2)\n")
            f.write("-----------------------------\n")
            for e, s in zip(p["energy"], p["sigma"]):
                f.write("%.17E\t%.17E\n" % (e, s))
            f.write("-----------------------------\n\n")
