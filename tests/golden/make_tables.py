"""Write ``synthe_tables.npz``: the numeric tables the synthesis path needs.

These are data of Kurucz's SYNTHE/ATLAS codes that results must match
exactly, so they are carried over as numbers, not re-derived:

* ``xtau`` (51), ``ch`` (51), ``coefj`` (51 x 51): the JOSH optical-depth
  grid, surface-flux weights and mean-intensity operator
  (``synthe_py/physics/josh_tables.py:6,120,177``).
* ``tabvi``/``tabh1`` (81): the H1 Voigt-function table from which the
  2001-point H0/H1/H2 tables are built (``synthe_py/physics/tables.py:249``).
* ``potion`` (999): ionisation potentials used for the gfall Stark and
  van der Waals damping defaults (``synthe_py/io/lines/atomic.py:22``,
  ``synthe_py/data/fortran_data.npz``).

Run once where the reference checkout exists (``--reference DIR`` or
``$SYNTHE_PY_REFERENCE``, default ``/root/reference``):
``python tests/golden/make_tables.py [--reference DIR]``.  Writes the package's
``data/synthe_tables.npz`` and the test fixture ``tests/golden/tables_ref.npz``.
"""

from __future__ import annotations

import importlib.util
import os
import sys
from pathlib import Path

import numpy as np

REFERENCE = Path(os.environ.get("SYNTHE_PY_REFERENCE", "/root/reference"))
HERE = Path(__file__).resolve().parent
OUT = HERE.parents[1] / "kurucz_py_joss_submission_gb300" / "data" / "synthe_tables.npz"


def _load_module(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.dont_write_bytecode = True
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def main(argv: list) -> int:
    global REFERENCE
    if argv[:1] == ["--reference"]:
        REFERENCE = Path(argv[1])
    josh = _load_module(REFERENCE / "synthe_py/physics/josh_tables.py", "_josh_tables")
    # tables.py imports nothing from the package, so it loads standalone
    tables = _load_module(REFERENCE / "synthe_py/physics/tables.py", "_synthe_tables")
    tabvi, tabh1 = tables._voigt_reference_tables()
    with np.load(REFERENCE / "synthe_py/data/fortran_data.npz") as d:
        potion = np.asarray(d["potion"], dtype=np.float64)
    np.savez_compressed(
        OUT,
        xtau=np.asarray(josh.XTAU_GRID, dtype=np.float64),
        ch=np.asarray(josh.CH_WEIGHTS, dtype=np.float64),
        coefj=np.asarray(josh.COEFJ_MATRIX, dtype=np.float64),
        tabvi=np.asarray(tabvi, dtype=np.float64),
        tabh1=np.asarray(tabh1, dtype=np.float64),
        potion=potion,
    )
    # reference-built 2001-point Voigt and FASTEX tables, kept as a test fixture
    vt = tables.VoigtTables.build()
    et = tables.ExpTables.build()
    np.savez_compressed(
        HERE / "tables_ref.npz",
        h0tab=vt.h0tab, h1tab=vt.h1tab, h2tab=vt.h2tab,
        extab=et.extab, extabf=et.extabf,
    )
    print(f"wrote {OUT}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main(sys.argv[1:]))
