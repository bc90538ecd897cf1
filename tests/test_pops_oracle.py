"""The population-stage oracle against the reference converter's own outputs (CPU).

The golden atmospheres ``tests/golden/atm_*.npz`` were written by the
reference's converter (``synthe_py/tools/convert_atm_to_npz.py``) from the
``.atm`` models beside them (the batch models are regenerated from their
seeds in ``batch_atmospheres.json``).  The oracle (``oracle/pops.py``)
restates the converter's population stage and must reproduce those fields.

Tolerances (relative):
* electron and mass density, hc/kT, neutral H/He and H2 densities: 1e-12;
* Doppler widths: 1e-15 (the same operations);
* populations of elements outside the molecular equilibrium (Saha on the
  converged XNE and XNATOM): 1e-9;
* populations of the elements in the molecular equilibrium: 1e-5.  The
  Newton iteration stops when every step is below 1e-3 of its unknown, and
  in the hottest layers the step of a trace element (V, Ti at 35,000 K) is
  set by the rounding of the Gauss-Jordan elimination over a Jacobian whose
  entries span ~30 decades, so two correct FP64 evaluations differ there by
  up to a few 1e-6 (1e-10 elsewhere).
"""

import json

import numpy as np
import pytest

from _cases import GOLDEN
from kurucz_py_joss_submission_gb300 import workloads
from oracle import pops

SCALAR_FIELDS = ("electron_density", "mass_density", "xnf_h", "xnf_he1", "xnf_h2")
TOL_SCALAR = 1e-12
TOL_DOPPLER = 1e-15
TOL_SAHA = 1e-9
TOL_MOLECULAR = 1e-5

NAMED = ["t5800g444", "t2500gm10", "t6000g430"]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    m = (a != 0) | (b != 0)
    if not m.any():
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.maximum(np.abs(b[m]), 1e-300)))


def molecular_elements():
    codes = pops.readmol()[0]
    return {int(c) for c in codes if c < 100}


def check_fields(out, ref):
    for f in SCALAR_FIELDS:
        assert rel(out[f], ref[f]) <= TOL_SCALAR, (f, rel(out[f], ref[f]))
    if "hckt" in ref:
        assert rel(out["hckt"], ref["hckt"]) <= TOL_SCALAR
    assert rel(out["doppler_per_ion"], ref["doppler_per_ion"]) <= TOL_DOPPLER
    mol = molecular_elements()
    p, pr = out["population_per_ion"], ref["population_per_ion"]
    assert p.shape == pr.shape
    for z in range(1, 100):
        tol = TOL_MOLECULAR if z in mol else TOL_SAHA
        e = rel(p[:, :, z - 1], pr[:, :, z - 1])
        assert e <= tol, (z, e)
    assert not np.any(p[:, :, 99:])


def batch_atm(tmp_path, k):
    spec = json.loads((GOLDEN / "batch_atmospheres.json").read_text())["kept"][k]
    p = tmp_path / f"batch_{k}.atm"
    workloads.grey_atmosphere_atm(p, spec["teff"], spec["logg"], spec["metallicity"],
                                  n_layers=spec["n_layers"])
    return p, GOLDEN / spec["file"]


@pytest.mark.parametrize("name", NAMED)
def test_oracle_matches_converter(name):
    out = pops.convert(GOLDEN / f"atm_{name}.atm")
    ref = np.load(GOLDEN / f"atm_{name}.npz")
    assert np.array_equal(out["temperature"], ref["temperature"])
    assert np.array_equal(out["depth"], ref["depth"])
    check_fields(out, ref)


@pytest.mark.parametrize("k", range(8))
def test_oracle_matches_converter_batch_models(tmp_path, k):
    atm, ref_path = batch_atm(tmp_path, k)
    out = pops.convert(atm)
    ref = np.load(ref_path)
    assert np.array_equal(out["temperature"], ref["temperature"])
    check_fields(out, ref)


def test_readmol_system():
    """READMOL on the molecule table: 190 entries, the element equations in Z order, electrons last."""
    codes, equil, locj, kcomps, idequa, nequa = pops.readmol()
    assert len(codes) == 190 and equil.shape == (7, 190)
    ids = list(idequa[:nequa])
    assert ids[0] == 0 and ids[-1] == 100 and ids[1:-1] == sorted(ids[1:-1])
    assert kcomps.max() == nequa          # inverse electrons
    # CO (608.00): C and O; H- (100.00): H and an electron
    m = int(np.nonzero(np.abs(codes - 608.0) < 1e-9)[0][0])
    assert [idequa[k] for k in kcomps[locj[m]:locj[m + 1]]] == [6, 8]
    m = int(np.nonzero(np.abs(codes - 100.0) < 1e-9)[0][0])
    assert [idequa[k] for k in kcomps[locj[m]:locj[m + 1]]] == [1, 100]


def test_native_molecular_system_matches_oracle():
    """The library's READMOL (built when the tables are loaded; no GPU needed) equals the oracle's."""
    from kurucz_py_joss_submission_gb300.physics import populations as P

    sysm = P.molecular_system()
    codes, equil, locj, kcomps, idequa, nequa = pops.readmol()
    assert sysm["n_molecules"] == len(codes)
    assert sysm["n_equations"] == nequa
    assert list(sysm["equation_element"]) == list(idequa[:nequa])
    assert {z + 1 for z in np.nonzero(sysm["element_molecular"])[0]} == molecular_elements()


def test_parse_atm_matches_oracle():
    from kurucz_py_joss_submission_gb300.physics import populations as P

    for name in NAMED:
        d = P.parse_atm_file(GOLDEN / f"atm_{name}.atm")
        o = pops.parse_atm(GOLDEN / f"atm_{name}.atm")
        assert np.array_equal(P.abundance_vector(d), pops.abundances(o))
        cols = P.layer_columns(d)
        st = pops.derived(o)
        assert np.array_equal(cols["temperature"], st["temperature"])
        assert np.array_equal(cols["gas_pressure"], st["gas_pressure"])
        assert np.array_equal(cols["rhox"], st["rhox"])
