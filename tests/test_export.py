"""Row a13: F_nu -> F_lambda (synthe_py/engine/opacity.py:3855-3861) and the
``.spec`` writer (synthe_py/io/export.py:12), against the reference's own
``.spec`` output stored in the golden cases (CPU only)."""

from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from kurucz_py_joss_submission_gb300.engine.opacity import flux_nu_to_lambda
from kurucz_py_joss_submission_gb300.io.export import write_spec_file

GOLDEN = Path(__file__).parent / "golden"
CASES = sorted(p.name for p in GOLDEN.glob("case_*.npz"))


@pytest.mark.parametrize("case", CASES)
def test_spec_text_equals_reference(case, tmp_path):
    c = np.load(GOLDEN / case)
    wl = c["wavelength"]
    result = SimpleNamespace(wavelength=wl, intensity=flux_nu_to_lambda(wl, c["flux_total_hz"]),
                             continuum=flux_nu_to_lambda(wl, c["flux_cont_hz"]))
    ours = tmp_path / "ours.spec"
    write_spec_file(result, ours)
    # the reference's file, re-emitted from its parsed columns (formatting is idempotent)
    ref = tmp_path / "ref.spec"
    np.savetxt(ref, c["spec"], fmt="%15.8f %11.6E %11.6E")
    assert ours.read_text() == ref.read_text()
