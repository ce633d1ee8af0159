"""Golden values of the reference's 1D3V quantities of interest (`bte_1d3v.compute_qoi`,
BESolver/python/bte_1d3v_solver.py:1179-1215) for both v-spaces, generated by running the
reference's own `bte_1d3v` on CPU:

* spectral (the table of `make_golden_1d3v.py`): the QoIs of the initial condition and of the
  step states v1 and v3 recorded in `bte1d_reference.npz`;
* finite-volume (the table of `make_golden_fvm.py`): the QoIs of the initial condition and of
  a seeded perturbation of it (so that the rates see a non-Maxwellian distribution), with the
  reference's QoI functionals op_mass, op_temp and op_rate (:493-502);
* for both, the radial components f_l(eps) of the last state at 50 energies
  (`compute_radial_components`, :1139-1177) and, for the FVM one, its harmonics
  (`ords_to_sph`, :678-685).

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script.
Writes `qoi_1d3v_reference.npz`. Usage:  python tests/golden/make_golden_1d3v_qoi.py
"""
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402
import make_golden_1d3v as G  # noqa: E402
import make_golden_fvm as GF  # noqa: E402


def _qoi(b, v):
    q = b.compute_qoi(np.copy(v), 0.0, b.params.dt)
    return np.asarray(q["rates"]), np.asarray(q["ne"]), np.asarray(q["Te"])


def main():
    tmp = tempfile.mkdtemp(prefix="qoi_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    out = {}
    try:
        S.cusparse_spsolve = types.SimpleNamespace(SpSMSolver=lambda *a, **k: None)
        spec = dict(np.load(os.path.join(HERE, "bte1d_reference.npz")))
        par = os.path.join(tmp, "spec.toml")
        G.write_toml(par, G.PARAMS, xs, os.path.join(tmp, "run_s"))
        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        for k in ("v0", "v1", "v3"):
            r, ne, te = _qoi(b, spec[k])
            out.update({"spec_%s_rates" % k: r, "spec_%s_ne" % k: ne, "spec_%s_Te" % k: te})
        ev = np.linspace(0.1, 70.0, 50)
        out.update(ev=ev, spec_v3_radial=np.asarray(b.compute_radial_components(ev, np.copy(spec["v3"]))))
        par = os.path.join(tmp, "fvm.toml")
        G.write_toml(par, GF.PARAMS, xs, os.path.join(tmp, "run_f"))
        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        v0 = np.asarray(b.initial_condition(0))
        vp = v0 * (1.0 + 0.3 * np.random.default_rng(11).random(v0.shape))
        for k, v in (("v0", v0), ("vp", vp)):
            r, ne, te = _qoi(b, v)
            out.update({"fvm_%s" % k: v, "fvm_%s_rates" % k: r, "fvm_%s_ne" % k: ne, "fvm_%s_Te" % k: te})
        out.update(fvm_op_mass=np.asarray(b.op_mass), fvm_op_temp=np.asarray(b.op_temp),
                   fvm_op_rate=np.asarray(b.op_rate), fvm_vp_sph=np.asarray(b.ords_to_sph(np.copy(vp))),
                   fvm_vp_radial=np.asarray(b.compute_radial_components(ev, np.copy(vp))))
        np.savez_compressed(os.path.join(HERE, "qoi_1d3v_reference.npz"), **out)
        print("wrote qoi_1d3v_reference.npz:", sorted(out))
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
