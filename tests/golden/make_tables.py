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
import math
import os
import re
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
    write_pops_tables()
    write_hydrogen_tables()
    return 0


def write_hydrogen_tables() -> None:
    """Write ``hydrogen_tables.npz``: the data of the hydrogen line profiles
    (HPROF4, ``synthe_py/physics/profiles/hydrogen.py:23-1405``: Stark
    correction tables PROPBM/C/D/PP/BETA, fine-structure components
    STALPH/STWTAL/ISTAL/LNGHAL/STCOMP/STCPWT/LNCOMP, the Lyman cutoff tables,
    ASUM/ASUMLYMAN, Y1WTM, XKNMTB), the hydrogen level energies EHYD
    (``synthe_py/engine/opacity.py:49``) and the continuum edges CONTH of the
    wing tables (``synthe_py/physics/tables.py:152``)."""
    sys.path.insert(0, str(Path(__file__).resolve().parent / "numba_shim"))
    sys.path.insert(0, str(REFERENCE))
    from synthe_py.physics.profiles.hydrogen import hydrogen_tables
    from synthe_py.physics.tables import metal_wing_tables
    import synthe_py.engine.opacity as eo

    t = hydrogen_tables()
    out = {k: np.asarray(v) for k, v in t.__dict__.items() if k not in ("tabvi", "tabh1")}
    for k in ("istal", "lnghal", "lncomp"):
        out[k] = out[k].astype(np.int32)
    out["ehyd"] = np.asarray(eo._EHYD_CM, dtype=np.float64)
    out["conth"] = np.asarray(metal_wing_tables().conth, dtype=np.float64)
    # continuum edges of the fort.19 merge limits (tables.py:173, CONTX [25, 17])
    out["contx"] = np.asarray(metal_wing_tables().contx, dtype=np.float64)
    path = OUT.parent / "hydrogen_tables.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


# Level tables of the explicit partition-function sums of PFSAHA
# (synthe_py/tools/pops_exact.py:520-741): energy (cm^-1) and weight per level.
_LEVEL_TABLES = ("HYD", "HE1", "HE2", "C1", "C2", "O1", "MG1", "MG2", "AL1", "SI1", "SI2",
                 "NA1", "B1", "K1")

_TERM = re.compile(r"([+-]?)(?:([0-9.]+(?:[eE][+-]?[0-9]+)?)\*)?math\.exp\(-_HCK/T\*"
                   r"([0-9.]+(?:[eE][+-]?[0-9]+)?)\)")


def _parse_pfground(expr: str):
    """Split one PFGROUND expression into its constant and (weight, energy) terms.

    Every expression is ``g0 + g1*exp(-HCK/T*E1) + ...`` (a missing weight is 1);
    the split is checked against the reference's own evaluation by the caller.
    """
    expr = expr.replace(" ", "")
    m = re.match(r"^([0-9.]+(?:[eE][+-]?[0-9]+)?)", expr)
    g0 = float(m.group(1))
    rest = expr[m.end():]
    terms = []
    pos = 0
    for t in _TERM.finditer(rest):
        if t.start() != pos or t.group(1) != "+":
            raise ValueError(f"unexpected PFGROUND form: {expr}")
        terms.append((float(t.group(2)) if t.group(2) else 1.0, float(t.group(3))))
        pos = t.end()
    if pos != len(rest):
        raise ValueError(f"unexpected PFGROUND form: {expr}")
    return g0, terms


def write_pops_tables() -> None:
    """Write ``pops_tables.npz``: the data of the FP64 population stage.

    * ``potion`` (999), ``nnn`` (6 x 374), ``atmass`` (99): ionisation
      potentials, packed partition-function table and atomic masses
      (``synthe_py/data/fortran_data.npz``);
    * ``pftab`` (7 x 56 x 10 x 9), ``pf_potlo``/``pf_potlolog`` (7): the
      iron-group partition-function table (``synthe_py/data/pfiron_data.npz``);
    * ``lev_<name>_e``/``lev_<name>_g``: level energies and weights of the
      explicit sums (``synthe_py/tools/pops_exact.py:520-741``);
    * ``pfg_first`` (114), ``pfg_second`` (168): PFGROUND labels per NELION,
      and per label its constant and (weight, energy) terms as a CSR table
      ``pfg_label``, ``pfg_g0``, ``pfg_off``, ``pfg_g``, ``pfg_e``
      (``synthe_py/tools/_pfground_table.py``);
    * ``mol_code`` (nummol), ``mol_equil`` (7 x nummol): the molecular
      equilibrium table ``lines/molecules.dat`` as READMOL reads it
      (``synthe_py/tools/readmol_exact.py:20``).
    """
    sys.path.insert(0, str(Path(__file__).resolve().parent / "numba_shim"))
    sys.path.insert(0, str(REFERENCE))
    import synthe_py.tools.pops_exact as pe
    import synthe_py.tools._pfground_table as pg
    from synthe_py.tools.readmol_exact import readmol_exact

    out = {}
    with np.load(REFERENCE / "synthe_py/data/fortran_data.npz") as d:
        out["potion"] = np.asarray(d["potion"], dtype=np.float64)
        out["nnn"] = np.asarray(d["nnn"], dtype=np.int32)
        out["atmass"] = np.asarray(d["atmass"], dtype=np.float64)
    with np.load(REFERENCE / "synthe_py/data/pfiron_data.npz") as d:
        out["pftab"] = np.asarray(d["pftab"], dtype=np.float64)
        out["pf_potlo"] = np.asarray(d["potlo"], dtype=np.float64)
        out["pf_potlolog"] = np.asarray(d["potlolog"], dtype=np.float64)
    for name in _LEVEL_TABLES:
        out[f"lev_{name.lower()}_e"] = np.asarray(getattr(pe, "E" + name), dtype=np.float64)
        out[f"lev_{name.lower()}_g"] = np.asarray(getattr(pe, "G" + name), dtype=np.float64)
    labels = sorted(pg.PFGROUND_EXPRESSIONS)
    g0s, offs, gs, es = [], [0], [], []
    hck = 6.6256e-27 * 2.99792458e10 / 1.38054e-16
    for lab in labels:
        g0, terms = _parse_pfground(pg.PFGROUND_EXPRESSIONS[lab])
        g0s.append(g0)
        gs += [g for g, _ in terms]
        es += [e for _, e in terms]
        offs.append(len(gs))
        ref = pe._PFGROUND_FUNCS[lab]
        for t in (1500.0, 3000.0, 5000.0, 8000.0, 20000.0):
            v = g0
            for g, e in terms:
                v = v + g * math.exp(-hck / t * e)
            if v != float(ref(t)):
                raise ValueError(f"PFGROUND label {lab}: split form differs at T={t}")
    out["pfg_first"] = np.asarray(pg.FIRST_RANGE_LABELS, dtype=np.int32)
    out["pfg_second"] = np.asarray(pg.SECOND_RANGE_LABELS, dtype=np.int32)
    out["pfg_label"] = np.asarray(labels, dtype=np.int32)
    out["pfg_g0"] = np.asarray(g0s, dtype=np.float64)
    out["pfg_off"] = np.asarray(offs, dtype=np.int32)
    out["pfg_g"] = np.asarray(gs, dtype=np.float64)
    out["pfg_e"] = np.asarray(es, dtype=np.float64)
    nummol, code_mol, equil, *_ = readmol_exact(REFERENCE / "lines" / "molecules.dat")
    out["mol_code"] = np.asarray(code_mol[:nummol], dtype=np.float64)
    out["mol_equil"] = np.asarray(equil[:, :nummol], dtype=np.float64)
    path = OUT.parent / "pops_tables.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    raise SystemExit(main(sys.argv[1:]))
