"""FP64 populations on the GPU (``ks_populations``) against the reference
converter's outputs and the oracle (needs a GPU).

Tolerances are those of ``tests/test_pops_oracle.py`` (relative): 1e-12 for
the electron and mass densities, hc/kT and the H/He/H2 densities; 1e-15 for
the Doppler widths; 1e-9 for the populations of elements outside the
molecular equilibrium and 1e-5 for those inside it (the reference's Newton
stop leaves trace elements of the hottest layers at the rounding of its
elimination, a few 1e-6).  Batched and single calls, and repeated calls,
give the same bits.  A synthesis on GPU populations reproduces the
reference's golden spectrum.
"""

import numpy as np
import pytest
import torch

from _cases import GOLDEN, gfall_path, golden, window
from test_pops_oracle import (NAMED, TOL_DOPPLER, TOL_MOLECULAR, TOL_SAHA, TOL_SCALAR, batch_atm,
                              molecular_elements, rel)
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic
from kurucz_py_joss_submission_gb300.physics import populations as P
from oracle import pops

pytestmark = pytest.mark.gpu

FIELDS = ("electron_density", "mass_density", "hckt", "xnf_h", "xnf_he1", "xnf_h2")


def check(out, ref):
    for f in FIELDS:
        assert rel(out[f], ref[f]) <= TOL_SCALAR, (f, rel(out[f], ref[f]))
    assert rel(out["doppler_per_ion"], ref["doppler_per_ion"]) <= TOL_DOPPLER
    mol = molecular_elements()
    for z in range(1, 100):
        tol = TOL_MOLECULAR if z in mol else TOL_SAHA
        e = rel(out["population_per_ion"][:, :, z - 1], ref["population_per_ion"][:, :, z - 1])
        assert e <= tol, (z, e)
    assert not np.any(out["population_per_ion"][:, :, 99:])


def all_models(tmp_path):
    paths = [GOLDEN / f"atm_{n}.atm" for n in NAMED]
    refs = [GOLDEN / f"atm_{n}.npz" for n in NAMED]
    for k in range(8):
        a, r = batch_atm(tmp_path, k)
        paths.append(a)
        refs.append(r)
    return paths, refs


def test_gpu_populations_match_converter_and_oracle(tmp_path):
    paths, refs = all_models(tmp_path)
    dp = P.DevicePopulations(paths).run()
    for k, (p, r) in enumerate(zip(paths, refs)):
        out = dp.host(k)
        ref = np.load(r)
        assert np.array_equal(out["temperature"], ref["temperature"])
        check(out, ref)
        orc = pops.convert(p)
        check(out, orc)
        assert np.array_equal(out["xnatm"] > 0, np.ones_like(out["xnatm"], dtype=bool))
        assert out["nmolec_iterations"].min() >= 1 and out["nmolec_iterations"].max() < 200


def test_gpu_populations_batch_equals_single_and_repeats(tmp_path):
    paths, _ = all_models(tmp_path)
    batch = P.DevicePopulations(paths).run()
    again = P.DevicePopulations(paths).run()
    for k, p in enumerate(paths):
        single = P.DevicePopulations([p]).run()
        a, b, c = batch.host(k), single.host(0), again.host(k)
        for f in FIELDS + ("population_per_ion", "doppler_per_ion", "xnatm", "nmolec_iterations"):
            assert np.array_equal(a[f], b[f]), (k, f)
            assert np.array_equal(a[f], c[f]), (k, f)


def test_synthesis_on_gpu_populations_matches_reference():
    """.atm -> GPU populations -> FP64 synthesis against the reference's golden
    spectrum of the same model (continuum tables from its converted model)."""
    name = "tiny_500_501"
    g = golden(name)
    base = atm_io.load_cached(GOLDEN / "atm_t5800g444.npz")
    dp = P.DevicePopulations([GOLDEN / "atm_t5800g444.atm"]).run()
    atm = dp.atmosphere(0, continuum=base)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    syn = Synthesizer(DeviceCatalog(cat), DeviceAtmosphere(atm), DeviceGrid(g["wavelength"]),
                      make_options(precision="fp64"))
    st = syn.run(stats=True)
    torch.cuda.synchronize()
    assert st["device_flags"] == 0
    ft, fc = syn.flux_total.cpu().numpy(), syn.flux_cont.cpu().numpy()
    assert rel(fc, g["flux_cont_hz"]) < 1e-9
    assert float(np.max(np.abs(ft - g["flux_total_hz"]) / g["flux_cont_hz"])) < 1e-8


def test_rejects_bad_models():
    with pytest.raises(ValueError):
        P.layer_columns({"glog": 4.0, "layers": [
            {"RHOX": 2.0, "T": 5000.0, "P": 1e4, "XNE": 1e12, "ABROSS": 0, "ACCRAD": 0, "VTURB": 0},
            {"RHOX": 1.0, "T": 5000.0, "P": 1e4, "XNE": 1e12, "ABROSS": 0, "ACCRAD": 0, "VTURB": 0}]})


def test_cli_gpu_populations_spec(tmp_path):
    """``cli.main MODEL.atm LINES.gf --populations gpu``: populations from the
    .atm on the GPU, continuum tables from the converted model beside it; the
    .spec columns equal the reference's to its printed precision."""
    from kurucz_py_joss_submission_gb300 import cli

    name = "tiny_500_501"
    g = golden(name)
    w0, w1 = window(name)
    atm = tmp_path / "model.atm"
    atm.write_text((GOLDEN / "atm_t5800g444.atm").read_text())
    (tmp_path / "model.npz").write_bytes((GOLDEN / "atm_t5800g444.npz").read_bytes())
    spec = tmp_path / "out.spec"
    rc = cli.main([str(atm), str(gfall_path(name)), "--spec", str(spec), "--wl-start", str(w0),
                   "--wl-end", str(w1), "--precision", "fp64", "--populations", "gpu"])
    assert rc == 0
    ours = np.loadtxt(spec)
    ref = g["spec"]
    assert ours.shape == ref.shape
    assert np.array_equal(ours[:, 0], ref[:, 0])
    assert np.allclose(ours[:, 1:], ref[:, 1:], rtol=1e-6, atol=0.0)
