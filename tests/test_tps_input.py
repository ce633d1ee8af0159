"""TPS CSV ingestion (the reference driver's `-input` file, bte_0d3v_batched_driver.py:79-122)."""
import numpy as np
import pytest

from boltzmann_gb300.tps_input import TEMP_K_1EV, read_tps_csv, requests_from_tps


def _write(path, header, rows):
    with open(path, "w") as f:
        f.write(",".join(header) + "\n")
        for r in rows:
            f.write(",".join(repr(float(v)) for v in r) + "\n")


def test_reads_and_normalises_like_the_driver(tmp_path):
    species = ["Ar", "Ar*", "Ar+"]
    header = ["Tg", "n0", "ne/n0", "E", "(Ar)/n0", "(Ar*)/n0", "(Ar+)/n0"]
    rows = [[300.0, 3.2e22, 1e-6, 2.0, 0.9, 0.1, 0.0],
            [900.0, 1.1e22, 1e-4, 5.0, 2.0, 2.0, 0.5]]
    p = tmp_path / "tps.csv"
    _write(p, header, rows)
    out = read_tps_csv(str(p), species)
    a = np.array(rows)
    n0, ne = a[:, 1], a[:, 2] * a[:, 1]
    # the driver's arithmetic, step by step (:88-121)
    ns = a[:, 4:7].T / np.sum(a[:, 4:7].T, axis=0)
    ns[2] = (ne / n0) ** 2 * n0
    ebyn = a[:, 3] / n0 / 1e-21
    tmean = np.mean(a[:, 0] / TEMP_K_1EV)
    np.testing.assert_array_equal(out["n0"], n0)
    np.testing.assert_array_equal(out["ne"], ne)
    np.testing.assert_array_equal(out["Tg"], a[:, 0])
    np.testing.assert_allclose(out["ns_by_n0"], ns, rtol=0, atol=0)
    np.testing.assert_allclose(out["EbyN"], ebyn, rtol=1e-15)
    np.testing.assert_allclose(out["E"], ebyn * n0 * 1e-21, rtol=1e-15)
    assert out["Te"] == pytest.approx(max(0.1, tmean), rel=1e-15)
    assert out["ev_max"] == pytest.approx(36 * tmean, rel=1e-15)
    # TEMP_K_1EV = e / k_B as scipy.constants gives it
    assert TEMP_K_1EV == pytest.approx(11604.518121550082, rel=1e-15)


def test_missing_column_and_empty_file(tmp_path):
    p = tmp_path / "bad.csv"
    _write(p, ["Tg", "n0", "ne/n0", "E"], [[300.0, 3.2e22, 1e-6, 2.0]])
    with pytest.raises(ValueError, match=r"\(Ar\)/n0"):
        read_tps_csv(str(p), ["Ar"])
    q = tmp_path / "empty.csv"
    q.write_text("Tg,n0,ne/n0,E,(Ar)/n0\n")
    with pytest.raises(ValueError, match="no data rows"):
        read_tps_csv(str(q), ["Ar"])


def test_requests_split_in_row_order(tmp_path):
    P = 1100
    rng = np.random.default_rng(3)
    header = ["Tg", "n0", "ne/n0", "E", "(Ar)/n0"]
    rows = np.column_stack([np.full(P, 300.0), np.full(P, 3.2e22), 10 ** rng.uniform(-8, -3, P),
                            10 ** rng.uniform(0, 3, P) * 3.2e22 * 1e-21, np.ones(P)])
    p = tmp_path / "big.csv"
    _write(p, header, rows)
    prm = read_tps_csv(str(p), ["Ar"])
    reqs = requests_from_tps(prm, n_sp=64, l_max=1, max_points=512)
    assert [r.P for r in reqs] == [512, 512, 76]
    assert [r.rid for r in reqs] == [0, 1, 2]
    np.testing.assert_array_equal(np.concatenate([r.E for r in reqs]), prm["E"])
    np.testing.assert_array_equal(np.concatenate([r.ns_by_n0 for r in reqs], axis=1), prm["ns_by_n0"])
    assert all(r.n_sp == 64 and r.l_max == 1 and r.ee for r in reqs)


def test_qoi_csv_has_the_driver_layout(tmp_path):
    """write_qoi_csv: the driver's header and one row per point, values read back exactly."""
    import csv
    from boltzmann_gb300.tps_input import write_qoi_csv
    rng = np.random.default_rng(4)
    P = 5
    n0, ne, Tg, E = rng.uniform(1e22, 4e22, P), rng.uniform(1e14, 1e16, P), np.full(P, 300.0), rng.uniform(1, 1e3, P)
    qoi = {"energy": rng.random(P), "mobility": rng.random(P), "diffusion": rng.random(P), "rates": rng.random((3, P))}
    path = write_qoi_csv(str(tmp_path / "run"), n0, ne, ne, Tg, E, qoi, ["C0", "C1", "C2"])
    rows = list(csv.reader(open(path)))
    assert rows[0] == ["n0", "ne", "ni", "Tg", "E", "energy", "mobility", "diffusion", "C0", "C1", "C2"]
    got = np.array(rows[1:], dtype=np.float64)
    want = np.column_stack([n0, ne, ne, Tg, E, qoi["energy"], qoi["mobility"], qoi["diffusion"], qoi["rates"].T])
    assert got.shape == (P, 11) and np.array_equal(got, want)
    with pytest.raises(ValueError):
        write_qoi_csv(str(tmp_path / "bad"), n0, ne, ne, Tg, E, qoi, ["C0"])
