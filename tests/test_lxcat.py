"""The project's LXCat reader and the synthetic workload tables."""
import numpy as np

from boltzmann_gb300.lxcat import parse_lxcat, read_available_species, read_cross_section_data
from boltzmann_gb300.workloads import synthetic_processes, batch_parameters


def test_roundtrip(synthetic_xs):
    data = read_cross_section_data(synthetic_xs)
    assert list(data) == ["E + Ar -> E + Ar", "E + Ar -> E + Ar*", "E + Ar -> E + E + Ar+"]
    assert read_available_species(synthetic_xs) == ["Ar"]
    for p, (k, v) in zip(synthetic_processes(), data.items()):
        assert v["type"] == p["kind"]
        np.testing.assert_array_equal(v["energy"], p["energy"])
        np.testing.assert_array_equal(v["cross section"], p["sigma"])
    assert data["E + Ar -> E + Ar"]["mass_ratio"] == 1.36e-5
    assert data["E + Ar -> E + Ar*"]["threshold"] == 11.55
    assert data["E + Ar -> E + E + Ar+"]["threshold"] == 15.76


def test_analytic_values():
    el, ex, io = synthetic_processes()
    e = np.array([0.0, 1.0, 10.0])
    np.testing.assert_allclose(np.interp(e, el["energy"], el["sigma"]), 1e-19 * np.sqrt(0.1 + e), rtol=1e-6)
    assert np.interp(30.0, ex["energy"], ex["sigma"]) == 1e-21
    assert np.interp(11.0, ex["energy"], ex["sigma"]) == 0.0
    assert np.interp(100.0, io["energy"], io["sigma"]) == 3e-20


def test_batch_parameters_are_seeded():
    a = batch_parameters(64, 20261203)
    b = batch_parameters(64, 20261203)
    np.testing.assert_array_equal(a["E"], b["E"])
    assert a["EbyN"].min() >= 1.0 and a["EbyN"].max() <= 1000.0
    ion = a["ne"] / a["n0"]
    assert ion.min() >= 1e-8 and ion.max() <= 1e-3


def test_reference_data_file_parses():
    import os
    f = "/root/reference/BESolver/python/lxcat_data/eAr_crs.6sp_Tg_0.5eV"
    if not os.path.exists(f):
        return
    d = read_cross_section_data(f)
    assert len(d) == 8
    assert read_available_species(f) == ["Ar", "Ar*(1)", "Ar*(2)", "Ar*(3)"]
