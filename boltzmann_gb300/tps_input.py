"""Request ingestion from the TPS-style CSV of the reference's batched driver.

The reference driver reads one row per spatial point from a CSV (`-input`), with columns
`Tg`, `n0`, `ne/n0`, `E` and one `(<species>)/n0` column per species of the collision file
(bte_0d3v_batched_driver.py:79-122). This module restates that reading with the standard
`csv` module (the reference uses pandas) and turns the rows into `SolveRequest`s for the
serving loop, so that a plasma code writing that file can drive the GB300 server directly.

Semantics kept from the reference:
* ne = (ne/n0) * n0; the species fractions are normalised to sum to one per point
  (`:96`); a species named `Ar+` is then replaced by (ne/n0)^2 * n0, the reference's
  two-body recombination rule (`:98-102`);
* E/N = E / n0 / 1e-21 Td (`:108`); the normalisation temperature is
  Te = max(0.1, mean(Tg) / TEMP_K_1EV) eV and the grid's energy range ev_max =
  36 * mean(Tg) / TEMP_K_1EV eV (`:109-119`); the field handed to the solver is
  E/N * n0 * 1e-21 (`:121`).
Where the reference prints an unreadable file's error and carries on (`:104-106`), this
reader raises ValueError naming the file and the missing column.
"""
from __future__ import annotations

import csv

import numpy as np

QE = 1.602176634e-19
KB = 1.380649e-23
TEMP_K_1EV = QE / KB  # collisions.TEMP_K_1EV
TD = 1e-21


def read_tps_csv(path: str, species: list[str]) -> dict:
    """Point parameters from a TPS CSV (bte_0d3v_batched_driver.py:79-122).

    species: the species of the collision file in file order
    (lxcat.read_available_species). Returns n0, ne, Tg, E (P,), ns_by_n0 (n_species, P),
    EbyN (P,) in Td, and the grid settings Te and ev_max (eV)."""
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    if not rows:
        raise ValueError("%s: no data rows" % path)
    names = [c.strip() for c in rows[0].keys()]

    def column(name: str) -> np.ndarray:
        for key in rows[0].keys():
            if key.strip() == name:
                try:
                    return np.array([float(r[key]) for r in rows], dtype=np.float64)
                except (TypeError, ValueError) as e:
                    raise ValueError("%s: column %r is not numeric (%s)" % (path, name, e)) from None
        raise ValueError("%s: missing column %r (columns: %s)" % (path, name, ", ".join(names)))

    Tg = column("Tg")
    n0 = column("n0")
    ne = column("ne/n0") * n0
    E = column("E")
    ns_by_n0 = np.zeros((len(species), len(Tg)))
    for i, sp in enumerate(species):
        ns_by_n0[i] = column("(%s)/n0" % sp)
    tot = np.sum(ns_by_n0, axis=0)
    if np.any(tot <= 0):
        raise ValueError("%s: species fractions sum to zero at row(s) %s" % (path, np.where(tot <= 0)[0].tolist()))
    ns_by_n0 = ns_by_n0 / tot
    for i, sp in enumerate(species):
        if sp == "Ar+":
            ns_by_n0[i, :] = (ne / n0) ** 2 * n0
    EbyN = E / n0 / TD
    Tmean = float(np.mean(Tg / TEMP_K_1EV))
    return dict(n0=n0, ne=ne, Tg=Tg, E=EbyN * n0 * TD, ns_by_n0=ns_by_n0, EbyN=EbyN,
                Te=max(1e-1, Tmean), ev_max=36.0 * Tmean)


def requests_from_tps(params: dict, n_sp: int, l_max: int, max_points: int = 512, ee: bool = True) -> list:
    """Split the CSV's points into SolveRequests of at most max_points points each, in row
    order, for BteServer.submit."""
    from .serving import SolveRequest
    if max_points < 1:
        raise ValueError("max_points must be positive")
    P = len(params["n0"])
    out = []
    for k, a in enumerate(range(0, P, max_points)):
        b = min(P, a + max_points)
        out.append(SolveRequest(n_sp=n_sp, l_max=l_max, n0=params["n0"][a:b].copy(), ne=params["ne"][a:b].copy(),
                                Tg=params["Tg"][a:b].copy(), E=params["E"][a:b].copy(),
                                ns_by_n0=np.ascontiguousarray(params["ns_by_n0"][:, a:b]), ee=ee, rid=k))
    return out


def write_qoi_csv(fname: str, n0, ne, ni, Tg, E, qoi: dict, collision_names) -> str:
    """The QoI output of the reference's batched driver script (bte_0d3v_batched_driver.py:215-232):
    `fname`_qoi.csv with the header n0, ne, ni, Tg, E, energy, mobility, diffusion and one column
    per collision name, one row per point, numbers written as that script's csv writer writes
    its NumPy rows. qoi holds "energy", "mobility", "diffusion" (P,) and "rates" (n_proc, P), as
    the solver returns them (device tensors are copied to the host). Returns the path."""
    host = lambda a: np.asarray(a.cpu().numpy() if hasattr(a, "cpu") else a, dtype=np.float64)
    cols = [host(v).reshape(-1, 1) for v in (n0, ne, ni, Tg, E, qoi["energy"], qoi["mobility"], qoi["diffusion"])]
    rates = host(qoi["rates"])
    if rates.shape[0] != len(collision_names):
        raise ValueError("rates has %d rows for %d collisions" % (rates.shape[0], len(collision_names)))
    cols += [rates[i].reshape(-1, 1) for i in range(rates.shape[0])]
    data = np.concatenate(cols, axis=1)
    path = "%s_qoi.csv" % fname
    with open(path, "w", encoding="UTF8") as fh:
        w = csv.writer(fh, delimiter=",")
        w.writerow(["n0", "ne", "ni", "Tg", "E", "energy", "mobility", "diffusion"] + [str(g) for g in collision_names])
        w.writerows(data)
    return path
