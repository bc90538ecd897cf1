"""ctypes binding of ``libkurucz_gb300.so`` (the C ABI in ``include/kurucz_gb300.h``).

Loading fails loudly when the library has not been built: there is no CPU
fallback for the synthesis path.  On load the constant SYNTHE tables
(``data/synthe_tables.npz``) are handed to ``ks_init_tables``.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Optional

import numpy as np

from . import _build

_lib: Optional[C.CDLL] = None
_lock = threading.Lock()
TABLES_NPZ = Path(__file__).resolve().parent / "data" / "synthe_tables.npz"
POPS_TABLES_NPZ = Path(__file__).resolve().parent / "data" / "pops_tables.npz"
HYDROGEN_TABLES_NPZ = Path(__file__).resolve().parent / "data" / "hydrogen_tables.npz"
# level tables of the explicit partition-function sums, in the library's order
POPS_LEVEL_TABLES = ("hyd", "he1", "he2", "c1", "c2", "o1", "mg1", "mg2", "al1", "si1", "si2", "na1",
                     "b1", "k1")

KS_OK = 0
KS_ERR_INVALID = 1
KS_ERR_UNSUPPORTED = 6
KS_PREC_MIXED = 0
KS_PREC_FP64 = 1

P = C.c_void_p
PD = C.POINTER(C.c_double)


class KsError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"kurucz_gb300 error {code}: {msg}")
        self.code = code


class KsAtmos(C.Structure):
    _fields_ = [
        ("n_layers", C.c_int32),
        ("rhox", P), ("temperature", P), ("electron_density", P), ("mass_density", P),
        ("hckt", P), ("xnf_h", P), ("xnf_he1", P), ("xnf_h2", P),
        ("population", P), ("doppler", P),
        ("n_ion", C.c_int32), ("n_elem", C.c_int32),
        ("wledge", P), ("half_edge", P), ("delta_edge", P),
        ("n_edge", C.c_int32),
        ("cont_abs_coeff", P), ("cont_scat_coeff", P),
        ("coeff_log10", C.c_int32),
        ("turbulent_velocity", P),
    ]


class KsGrid(C.Structure):
    _fields_ = [("n", C.c_int64), ("wavelength", P), ("grid_origin", C.c_double)]


class KsLines(C.Structure):
    _fields_ = [
        ("n_lines", C.c_int64),
        ("wavelength", P), ("gf", P), ("cgf", P), ("gamma_rad", P), ("gamma_stark", P),
        ("gamma_vdw", P), ("elo_cm", P),
        ("element_idx", P), ("ion_stage", P), ("line_type", P),
        ("process_mask", P), ("asynth_mask", P),
        ("sorted_by_wavelength", C.c_int32),
        ("n_hydrogen", C.c_int32),
        ("hydrogen_rows", P), ("hydrogen_n_lower", P), ("hydrogen_n_upper", P),
        ("n_helium", C.c_int32), ("helium_rows", P),
        ("n_f19", C.c_int32), ("f19_rows", P), ("f19_cgf", P), ("f19_gamma_rad", P),
        ("f19_gamma_stark", P), ("f19_gamma_vdw", P), ("f19_kind", P),
        ("f19_nlast", P), ("f19_nelion", P),
        ("helium_ncon", P), ("helium_nelionx", P), ("f19_ncon", P), ("f19_nelionx", P),
    ]


class KsOptions(C.Structure):
    _fields_ = [
        ("cutoff", C.c_double), ("microturb_kms", C.c_double), ("rhoxj", C.c_double),
        ("precision", C.c_int32), ("tile_bins", C.c_int32), ("warps_per_tile", C.c_int32),
        ("profile", C.c_int32), ("short_class", C.c_int32), ("transfer_path", C.c_int32),
        ("long_class", C.c_int32), ("exact_sweeps", C.c_int32),
    ]


class KsJob(C.Structure):
    """One job of a batch (ks_job): host pointers to its atmosphere and grid
    records, its rows of the shared line list, device outputs."""

    _fields_ = [
        ("atm", C.POINTER(KsAtmos)), ("grid", C.POINTER(KsGrid)),
        ("line_first", C.c_int64), ("line_count", C.c_int64),
        ("flux_total", P), ("flux_cont", P),
    ]


class KsStats(C.Structure):
    _fields_ = [
        ("valid_pairs", C.c_int64), ("evaluations", C.c_int64),
        ("maxj_wavelengths", C.c_int64), ("iterations", C.c_int64),
        ("device_flags", C.c_int32), ("kernel_launches", C.c_int32),
        ("stage_ms", C.c_float * 8),
    ]

    STAGES = ("bins_prep", "continuum", "pair_setup", "partition", "accumulate", "transfer",
              "special", "total")

    def as_dict(self) -> dict:
        d = {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "stage_ms"}
        d["stage_ms"] = {n: float(v) for n, v in zip(self.STAGES, self.stage_ms)}
        return d


class KsHydrogenTables(C.Structure):
    """ks_hydrogen_tables: host pointers to the hydrogen line profile tables."""

    _fields_ = [(k, P) for k in (
        "propbm", "c", "d", "pp", "beta", "stalph", "stwtal", "stcomp", "stcpwt",
        "istal", "lnghal", "lncomp",
        "cutoff_h2_plus", "cutoff_h2", "asum_lyman", "asum", "y1wtm", "xknmtb", "ehyd", "conth", "contx")]


HYDROGEN_INT_TABLES = ("istal", "lnghal", "lncomp")


class KsPopsTables(C.Structure):
    """ks_pops_tables: host pointers to the population-stage data tables."""

    _fields_ = [
        ("potion", P), ("nnn", P), ("atmass", P), ("pftab", P), ("pf_potlo", P), ("pf_potlolog", P),
        ("level_e", P), ("level_g", P), ("level_n", P),
        ("pfg_first", P), ("n_pfg_first", C.c_int32), ("pfg_second", P), ("n_pfg_second", C.c_int32),
        ("pfg_label", P), ("pfg_g0", P), ("pfg_off", P), ("n_pfg_label", C.c_int32),
        ("pfg_g", P), ("pfg_e", P),
        ("mol_code", P), ("mol_equil", P), ("n_mol", C.c_int32),
    ]


class KsPopsModel(C.Structure):
    """ks_pops_model: one atmosphere's .atm columns and the population outputs (device)."""

    _fields_ = [
        ("n_layers", C.c_int32),
        ("temperature", P), ("gas_pressure", P), ("vturb", P), ("xabund", P),
        ("electron_density", P), ("mass_density", P), ("hckt", P), ("xnf_h", P), ("xnf_he1", P),
        ("xnf_h2", P), ("population", P), ("doppler", P), ("xnatom", P), ("nmolec_iterations", P),
    ]


class KsPopsTangent(C.Structure):
    """ks_pops_tangent: a model and the derivative outputs for one element's log10 abundance."""

    _fields_ = [
        ("model", KsPopsModel), ("element", C.c_int32),
        ("d_electron_density", P), ("d_mass_density", P), ("d_xnf_h", P), ("d_xnf_he1", P),
        ("d_xnf_h2", P), ("d_population", P),
    ]


class KsAtmGrad(C.Structure):
    """ks_atm_grad: line groups by species and the atmosphere-term outputs of the adjoint."""

    _fields_ = [
        ("line_order", P), ("group_first", P), ("group_species", P), ("n_groups", C.c_int32),
        ("d_ln_population", P), ("d_ln_mass_density", P), ("d_electron_density", P), ("d_txnxn", P),
    ]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "ks_version": (C.c_int32, [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ks_last_error": (C.c_char_p, []),
    "ks_init_tables": (C.c_int32, [PD, PD, C.c_int32, PD, PD, PD]),
    "ks_get_tables": (C.c_int32, [PD, PD, PD, PD, PD]),
    "ks_wavelength_grid": (C.c_int64, [C.c_double, C.c_double, C.c_double, PD, C.c_int64]),
    "ks_line_bins": (C.c_int32, [C.POINTER(KsGrid), P, C.c_int64, P, P, P]),
    "ks_continuum": (C.c_int32, [C.POINTER(KsAtmos), C.POINTER(KsGrid), C.c_int32, P, P, P]),
    "ks_transp": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                              C.POINTER(KsOptions), P, P, P, P, P]),
    "ks_workspace_size": (C.c_int32, [C.c_int64, C.c_int32, C.c_int64, C.POINTER(KsOptions),
                                      C.POINTER(C.c_size_t)]),
    "ks_asynth": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                              C.POINTER(KsOptions), P, P, P, P, C.c_size_t, P,
                              C.POINTER(KsStats), P]),
    "ks_formal_solution": (C.c_int32, [C.POINTER(KsAtmos), C.POINTER(KsGrid), C.c_int32, P, P, P,
                                       P, P, P, P, C.POINTER(KsStats), P]),
    "ks_synthesize": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                                  C.POINTER(KsOptions), P, C.c_size_t, P, P, P,
                                  C.POINTER(KsStats), P]),
    "ks_opacity": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                               C.POINTER(KsOptions), P, C.c_size_t, P, P, P, C.POINTER(KsStats), P]),
    "ks_transfer_opacity": (C.c_int32, [C.POINTER(KsAtmos), C.POINTER(KsGrid), C.POINTER(KsOptions),
                                        P, P, P, P, P, C.POINTER(KsStats), P]),
    "ks_synthesize_adjoint": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                                          C.POINTER(KsOptions), P, C.c_size_t, P, P, P, P, P, P, P,
                                          C.POINTER(KsStats), P]),
    "ks_synthesize_adjoint_atmos": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                                                C.POINTER(KsOptions), P, C.c_size_t, P, P, P, P, P, P, P,
                                                C.POINTER(KsAtmGrad), C.POINTER(KsStats), P]),
    "ks_synthesize_noalloc": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsAtmos), C.POINTER(KsGrid),
                                          C.POINTER(KsOptions), P, P, P, P]),
    "ks_check_flags": (C.c_int32, [P, C.POINTER(C.c_int32)]),
    "ks_batch_workspace_size": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsJob), C.c_int32,
                                            C.POINTER(KsOptions), C.POINTER(C.c_size_t)]),
    "ks_batch_create": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsJob), C.c_int32, C.POINTER(KsOptions),
                                    P, C.c_size_t, C.POINTER(P)]),
    "ks_batch_run": (C.c_int32, [P, C.POINTER(KsStats), P]),
    "ks_batch_free": (None, [P]),
    "ks_synthesize_batch": (C.c_int32, [C.POINTER(KsLines), C.POINTER(KsJob), C.c_int32,
                                        C.POINTER(KsOptions), P, C.c_size_t, C.POINTER(KsStats), P]),
    "ks_init_pops_tables": (C.c_int32, [C.POINTER(KsPopsTables)]),
    "ks_init_hydrogen_tables": (C.c_int32, [C.POINTER(KsHydrogenTables)]),
    "ks_pops_system": (C.c_int32, [P, P, P, P]),
    "ks_populations_workspace_size": (C.c_int32, [C.POINTER(KsPopsModel), C.c_int32, C.POINTER(C.c_size_t)]),
    "ks_populations": (C.c_int32, [C.POINTER(KsPopsModel), C.c_int32, P, C.c_size_t, P]),
    "ks_populations_tangent_workspace_size": (C.c_int32, [C.POINTER(KsPopsTangent), C.c_int32,
                                                          C.POINTER(C.c_size_t)]),
    "ks_populations_tangent": (C.c_int32, [C.POINTER(KsPopsTangent), C.c_int32, P, C.c_size_t, P]),
    "ks_gfall_read": (C.c_int32, [C.c_char_p, C.c_double, C.c_double, PD, C.c_int32,
                                  C.POINTER(P)]),
    "ks_gfall_sort": (C.c_int32, [P]),
    "ks_gfall_count": (C.c_int64, [P]),
    "ks_gfall_fetch": (C.c_int32, [P] + [P] * 15),
    "ks_gfall_fetch_levels": (C.c_int32, [P, P, P]),
    "ks_gfall_fetch_iso": (C.c_int32, [P, P, P]),
    "ks_gfall_fetch_gamma_logs": (C.c_int32, [P, P, P, P]),
    "ks_gfall_fetch_j": (C.c_int32, [P, P, P, P]),
    "ks_gfall_free": (None, [P]),
}


def lib_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load the library (and initialise its tables) once per process."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not path.exists():
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(
                    f"native library {path} is missing: run "
                    "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)"
                )
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        with np.load(TABLES_NPZ) as t:
            tabvi = np.ascontiguousarray(t["tabvi"], dtype=np.float64)
            tabh1 = np.ascontiguousarray(t["tabh1"], dtype=np.float64)
            xtau = np.ascontiguousarray(t["xtau"], dtype=np.float64)
            ch = np.ascontiguousarray(t["ch"], dtype=np.float64)
            coefj = np.ascontiguousarray(t["coefj"], dtype=np.float64)
        st = L.ks_init_tables(_pd(tabvi), _pd(tabh1), tabvi.size, _pd(xtau), _pd(ch), _pd(coefj))
        if st != KS_OK:
            raise KsError(st, L.ks_last_error().decode())
        _init_pops_tables(L)
        _init_hydrogen_tables(L)
        _lib = L
        return _lib


def _init_pops_tables(L: C.CDLL) -> None:
    """Hand the population-stage tables (``data/pops_tables.npz``) to ``ks_init_pops_tables``."""
    with np.load(POPS_TABLES_NPZ) as t:
        a = {k: np.asarray(t[k]) for k in t.files}
    f64 = lambda x: np.ascontiguousarray(x, dtype=np.float64)  # noqa: E731
    i32 = lambda x: np.ascontiguousarray(x, dtype=np.int32)  # noqa: E731
    keep = {
        "potion": f64(a["potion"]), "nnn": i32(a["nnn"]), "atmass": f64(a["atmass"]),
        "pftab": f64(a["pftab"]), "pf_potlo": f64(a["pf_potlo"]), "pf_potlolog": f64(a["pf_potlolog"]),
        "level_e": f64(np.concatenate([a[f"lev_{n}_e"] for n in POPS_LEVEL_TABLES])),
        "level_g": f64(np.concatenate([a[f"lev_{n}_g"] for n in POPS_LEVEL_TABLES])),
        "level_n": i32([a[f"lev_{n}_e"].size for n in POPS_LEVEL_TABLES]),
        "pfg_first": i32(a["pfg_first"]), "pfg_second": i32(a["pfg_second"]),
        "pfg_label": i32(a["pfg_label"]), "pfg_g0": f64(a["pfg_g0"]), "pfg_off": i32(a["pfg_off"]),
        "pfg_g": f64(a["pfg_g"]), "pfg_e": f64(a["pfg_e"]),
        "mol_code": f64(a["mol_code"]), "mol_equil": f64(a["mol_equil"]),
    }
    t = KsPopsTables()
    for k, v in keep.items():
        setattr(t, k, v.ctypes.data)
    t.n_pfg_first = keep["pfg_first"].size
    t.n_pfg_second = keep["pfg_second"].size
    t.n_pfg_label = keep["pfg_label"].size
    t.n_mol = keep["mol_code"].size
    st = L.ks_init_pops_tables(C.byref(t))
    if st != KS_OK:
        raise KsError(st, L.ks_last_error().decode())


def _init_hydrogen_tables(L: C.CDLL) -> None:
    """Hand the hydrogen profile tables (``data/hydrogen_tables.npz``) to ``ks_init_hydrogen_tables``."""
    with np.load(HYDROGEN_TABLES_NPZ) as t:
        keep = {k: np.ascontiguousarray(t[k], dtype=np.int32 if k in HYDROGEN_INT_TABLES else np.float64)
                for k, _ in KsHydrogenTables._fields_}
    t = KsHydrogenTables()
    for k, v in keep.items():
        setattr(t, k, v.ctypes.data)
    st = L.ks_init_hydrogen_tables(C.byref(t))
    if st != KS_OK:
        raise KsError(st, L.ks_last_error().decode())


def _pd(a: np.ndarray):
    return a.ctypes.data_as(PD)


def check(status: int) -> None:
    if status != KS_OK:
        raise KsError(status, load().ks_last_error().decode())


def exported_symbols() -> list:
    return sorted(SIGNATURES)


def check_device_flags(stream: Optional[int] = None) -> int:
    """Synchronise ``stream`` (a cudaStream_t as an int; None = the legacy
    default stream) and raise :class:`KsError` when any call on the current
    device has flagged an internal limit since the last check
    (``ks_check_flags``: the flags are sticky per device and cleared here)."""
    L = load()
    f = C.c_int32(0)
    st = L.ks_check_flags(C.c_void_p(stream) if stream else None, C.byref(f))
    if st != KS_OK:
        raise KsError(st, L.ks_last_error().decode())
    return int(f.value)
