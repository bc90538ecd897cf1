"""CPU restatement of the reference's fort.19 NORMAL-line and autoionizing-line
profiles -- test infrastructure.

Only ``tests/`` use this module, to check the GPU kernels for these lines.

Lines with NBLO/NBUP set (and none of the hydrogen, helium, autoionizing,
coronal or PRD types) leave the TRANSP/ASYNTH route (line_opacity.py:
746-757) for fort.19 (io/lines/fort19.py:343-347) and get their profile in
``_add_fort19_asynth`` (synthe_py/engine/opacity.py:1335-1488), added to
ASYNTH as TMP x STIM per layer:

* the fort.19 record keeps CGF and the damping constants in single
  precision (fort19.py:368-402);
* per (line, layer): population of the line's ion, the line's Doppler width
  from the depth state (physics/populations.py:158-195: thermal velocity of
  mass 56 -- the state is built without element masses, opacity.py:2204 --
  and the model's plus the synthesis microturbulence), XNFDOP, the two
  KAPMIN gates, KAPCEN at the clamped centre bin (opacity.py:1404-1447);
* the wing of ``_accumulate_metal_profile_kernel`` (opacity.py:74-262):
  N10DOP = int(10 DOPPLE RESOLU), the near profile with the incremental
  TABI (ADAMP < 0.2) or the Voigt function, stopping at the first value below
  KAPMIN, else far wings X / n^2 to MAXSTEP; then every step from 1 to NSTEP
  added, red and blue, without a cutoff test.

Autoionizing lines (TYPE 1, the gfall AUT tag) take the Fano-type profile of
``_accumulate_autoionizing_profile`` (opacity.py:901-963) with KAPPA0 =
BSHORE GF XNFPEL BOLT (:1522-1541) in the same per-layer buffer, in fort.19
order, and so do the merged-continuum records (LABELP CONTINUU: fort.19 type
NLAST = XJP, gf x (2 XJ + 1); the ramp of ``_accumulate_merged_continuum``,
opacity.py:863-898, between the merge and tail wavelengths of
``_compute_merged_continuum_limits``, :723-758).  Lines whose fort.19
continuum index is set (NCON > 0 with an element of the CONTX table) taper
their wings at WCON/WTAIL; they are not restated here.
"""

from __future__ import annotations

import math
from typing import Dict

import numpy as np

from . import hydrogen, oracle

C_LIGHT_NM = 2.99792458e17
C_LIGHT_CM = 2.99792458e10
C_LIGHT_KMS = 299792.458
KBOLTZ = 1.380649e-16
AMU = 1.66054e-24
CGF_FACTOR = 0.026538 / 1.77245
MAX_PROFILE_STEPS = 1000000
DEFAULT_ATOMIC_MASS = 56.0


def normal_rows(cat: Dict[str, np.ndarray]) -> np.ndarray:
    """Catalog rows taken as fort.19 NORMAL lines, in catalog (fort.19) order."""
    lt = np.asarray(cat["line_type"])
    nb = np.abs(np.asarray(cat["n_lower"])) + np.abs(np.asarray(cat["n_upper"]))
    known = (np.asarray(cat["nelem"]) >= 1) & (np.asarray(cat["nelem"]) <= 99)
    clab = np.asarray(cat.get("continuum_label", np.zeros(lt.size))) != 0
    return np.flatnonzero((lt == 0) & (nb != 0) & known & (np.asarray(cat["ion_stage"]) >= 1) & ~clab)


def _nlast(cat: Dict[str, np.ndarray]) -> np.ndarray:
    """fort.19 type of a CONTINUU record: XJP, else NBUP (fort19.py:304-306)."""
    xjp = np.asarray(cat["xjp"])
    return np.where(xjp > 0.0, xjp.astype(np.int64), np.asarray(cat["n_upper"]).astype(np.int64))


def cont_rows(cat: Dict[str, np.ndarray]) -> np.ndarray:
    """Catalog rows of merged-continuum records (LABELP CONTINUU, NLAST > 3)."""
    if "continuum_label" not in cat:
        return np.zeros(0, np.int64)
    known = (np.asarray(cat["nelem"]) >= 1) & (np.asarray(cat["nelem"]) <= 99)
    clab = np.asarray(cat["continuum_label"]) != 0
    return np.flatnonzero(clab & (_nlast(cat) > 3) & known & (np.asarray(cat["ion_stage"]) >= 1))


def aut_rows(cat: Dict[str, np.ndarray]) -> np.ndarray:
    """Catalog rows of autoionizing lines (TYPE 1: the gfall AUT tag)."""
    known = (np.asarray(cat["nelem"]) >= 1) & (np.asarray(cat["nelem"]) <= 99)
    clab = np.asarray(cat.get("continuum_label", np.zeros(len(cat["line_type"])))) != 0
    return np.flatnonzero((np.asarray(cat["line_type"]) == 1) & known & (np.asarray(cat["ion_stage"]) >= 1)
                          & ~clab)


CODEX = np.array([1.0, 2.0, 2.01, 6.0, 6.01, 12.0, 12.01, 13.0, 13.01, 14.0, 14.01, 20.0, 20.01, 8.0, 11.0,
                  5.0, 19.0])


def merge_index(cat: Dict[str, np.ndarray], i: int):
    """NCON and NELIONX of record i (fort19.py:330-338); (0, 0) without
    ISO fields."""
    if "iso1" not in cat:
        return 0, 0
    iso1, iso2 = int(cat["iso1"][i]), int(cat["iso2"][i])
    ncon = iso2 if iso1 == 0 and iso2 > 0 else 0
    m = np.nonzero(np.isclose(CODEX, float(cat["code"][i]), rtol=0.0, atol=1e-3))[0]
    return ncon, (int(m[0]) + 1 if m.size else 0)


def continuum_limits(ncon, nelion, nelionx, emerge, emerge_h, contx):
    """_compute_continuum_limits_jit (opacity.py:657-702), vacuum grid:
    (WCON, WTAIL), None where absent."""
    if ncon <= 0 or nelionx <= 0 or nelionx > contx.shape[1] or ncon > contx.shape[0]:
        return None, None
    cv = float(contx[ncon - 1, nelionx - 1])
    if cv <= 0.0:
        return None, None
    em = emerge_h if nelion == 1 else emerge
    denom = cv - em
    if abs(denom) <= 1e-8:
        return None, None
    wcon = 1.0e7 / denom
    wtail = -1.0
    dt = cv - em - 500.0
    if abs(dt) > 1e-8:
        wtail = 1.0e7 / dt
        if wtail < 0.0:
            wtail = 2.0 * wcon
        wtail = min(2.0 * wcon, wtail)
    if wtail > 0.0 and wtail <= wcon:
        wtail = -1.0
    return (wcon if wcon > 0.0 else None), (wtail if wtail > 0.0 else None)


def contx_table() -> np.ndarray:
    from pathlib import Path
    p = Path(__file__).resolve().parent.parent / "kurucz_py_joss_submission_gb300" / "data" / "hydrogen_tables.npz"
    with np.load(p) as t:
        return np.asarray(t["contx"])


def _nelion(code: float) -> int:
    """The fort.19 ion index (fort19.py:323-328)."""
    nelem = int(code + 1.0e-6) if code > 0.0 else 0
    icharge = int((code - nelem) * 100.0 + 0.1) if code > 0.0 else 0
    nelion = nelem * 6 - 6 + int(icharge + 1)
    if 19 < nelem < 29 and icharge > 5:
        nelion = 6 * (nelem + icharge * 10 - 30) - 1
    return nelion


def _merged_limits(wl, nlast, emerge, emerge_h, ion_index):
    """_compute_merged_continuum_limits (opacity.py:723-758), vacuum grid."""
    if wl <= 0.0 or nlast <= 0:
        return None, None
    ryd = 109677.576 if ion_index == 1 else 109737.312
    dshift = 1.0e7 / wl - ryd / float(nlast * nlast)
    if abs(dshift) <= 1e-12:
        return None, None
    wshift = 1.0e7 / dshift
    em = emerge_h if ion_index == 1 else emerge
    dmerge = 1.0e7 / wl - em
    if abs(dmerge) <= 1e-12:
        return None, None
    wmerge = 1.0e7 / dmerge
    if wmerge < 0.0:
        wmerge = wshift + wshift
    wmerge = max(wmerge, wshift)
    wmerge = min(wshift + wshift, wmerge)
    dtail = 1.0e7 / wmerge - 500.0
    if abs(dtail) <= 1e-12:
        return wmerge, None
    wtail = 1.0e7 / dtail
    if wtail < 0.0:
        wtail = wmerge + wmerge
    return wmerge, min(wmerge + wmerge, wtail)


def _merged_continuum(tmp, cont, grid, ci, wl, kappa, cutoff, merge_wl, tail_wl):
    """_accumulate_merged_continuum (opacity.py:863-898)."""
    if kappa <= 0.0:
        return
    n = grid.size
    i0 = max(ci, 0)
    im = int(np.searchsorted(grid, merge_wl, side="left"))
    it = min(int(np.searchsorted(grid, tail_wl, side="right")), n)
    if it <= i0:
        return
    denom = max(it - max(im, i0), 1)
    for b in range(i0, it):
        if grid[b] < wl:
            continue
        v = kappa
        if b >= im:
            v *= max(it - b, 0) / denom
        if v < cont[b] * cutoff:
            break
        tmp[b] += v


def aut_record_values(cat: Dict[str, np.ndarray], rows: np.ndarray) -> Dict[str, np.ndarray]:
    """fort.19 fields of autoionizing lines (fort19.py:352-373, :387): gf and
    the unnormalised damping constants from the gfall logs (GS > 0 encodes a
    negative ASHORE), single precision."""
    wl = np.asarray(cat["wavelength"])[rows]
    denom = 12.5664 * (C_LIGHT_NM / np.maximum(wl, 1.0e-30))
    grl = np.asarray(cat["gamma_rad_log"])[rows]
    gsl = np.asarray(cat["gamma_stark_log"])[rows]
    gwl = np.asarray(cat["gamma_vdw_log"])[rows]
    gr = np.where(grl != 0.0, 10.0 ** grl, np.asarray(cat["gamma_rad"])[rows] * denom)
    gs = np.where(gsl > 0.0, -(10.0 ** (-gsl)),
                  np.where(gsl < 0.0, 10.0 ** gsl, np.asarray(cat["gamma_stark"])[rows] * denom))
    gw = np.where(gwl != 0.0, 10.0 ** gwl, np.asarray(cat["gamma_vdw"])[rows] * denom)
    f32 = lambda x: np.asarray(x, dtype=np.float32).astype(np.float64)  # noqa: E731
    return dict(gf=f32(10.0 ** np.asarray(cat["log_gf"])[rows]), gamma_rad=f32(gr), gamma_stark=f32(gs),
                gamma_vdw=f32(gw))


def _autoionizing(tmp, cont, grid, ci, wl, kappa0, gr, gs, gw, cutoff):
    """_accumulate_autoionizing_profile (opacity.py:901-963), including its
    Python indexing of a centre bin -1 (a line below the grid): the centre
    value and its cutoff go to the last bin."""
    n = grid.size
    cc = ci if ci >= 0 else n + ci
    if kappa0 < cont[cc] * cutoff or kappa0 <= 0.0:
        return
    fc = C_LIGHT_CM / (wl * 1e-7)
    gamma = max(abs(gr), 1e-30)
    ashore = gs
    bshore = gw if abs(gw) >= 1e-30 else 1e-30
    tmp[cc] += kappa0
    for sgn in (1, -1):
        for o in range(1, max(ci, n - ci - 1) + 1):
            b = ci + sgn * o
            if b >= n or b < 0:
                break
            eps = 2.0 * (C_LIGHT_CM / (grid[b] * 1e-7) - fc) / gamma
            v = kappa0 * (ashore * eps + bshore) / (eps * eps + 1.0) / bshore
            if v <= 0.0 or v < cont[b] * cutoff:
                break
            tmp[b] += v


def record_values(cat: Dict[str, np.ndarray], rows: np.ndarray) -> Dict[str, np.ndarray]:
    """The fort.19 record fields of those lines, rounded to single precision
    as the record stores them (fort19.py:379-387, :394-402)."""
    wl = np.asarray(cat["wavelength"])[rows]
    gf = 10.0 ** np.asarray(cat["log_gf"])[rows]
    freq = C_LIGHT_NM / np.maximum(wl, 1.0e-30)
    return dict(
        cgf=np.asarray(CGF_FACTOR * gf / freq, dtype=np.float32).astype(np.float64),
        gamma_rad=np.asarray(cat["gamma_rad"], dtype=np.float32)[rows].astype(np.float64),
        gamma_stark=np.asarray(cat["gamma_stark"], dtype=np.float32)[rows].astype(np.float64),
        gamma_vdw=np.asarray(cat["gamma_vdw"], dtype=np.float32)[rows].astype(np.float64),
    )


def line_doppler(atm: Dict[str, np.ndarray], d: int, wl: float, microturb_kms: float) -> float:
    """Doppler width (nm) of a line in layer d, physics/populations.py:158-195."""
    temp = max(float(atm["temperature"][d]), 1.0)
    thermal = math.sqrt(2.0 * KBOLTZ * temp / (DEFAULT_ATOMIC_MASS * AMU)) / C_LIGHT_CM
    vt = (float(atm["turbulent_velocity"][d]) / 1e5) / C_LIGHT_KMS
    micro = microturb_kms / C_LIGHT_KMS if microturb_kms > 0 else 0.0
    total = math.sqrt(vt * vt + micro * micro)
    return wl * math.sqrt(total * total + thermal * thermal)


def _metal_wing(tmp, cont, grid, ci, wl, kappa0, adamp, dw, cutoff, tb, wcon=None, wtail=None):
    """_accumulate_metal_profile_kernel (opacity.py:74-262)."""
    if dw <= 0.0 or kappa0 <= 0.0:
        return
    n = grid.size
    a = max(adamp, 1e-12)
    cc = max(0, min(ci, n - 1))
    kapmin = cutoff * cont[cc]
    if cc < n - 1:
        resolu = 1.0 / (grid[cc + 1] / grid[cc] - 1.0)
    elif cc > 0:
        resolu = 1.0 / (grid[cc] / grid[cc - 1] - 1.0)
    else:
        resolu = 300000.0
    dopple = dw / wl if wl > 0 else 1e-6
    n10 = min(int(10.0 * dopple * resolu), MAX_PROFILE_STEPS)
    prof = {}
    early = False
    nstep = 0
    if a < 0.2:
        tabstep = 200.0 / (dopple * resolu) if (dopple * resolu) > 0 else 200.0
        tabi = 0.5
        for k in range(1, n10 + 1):
            tabi = tabi + tabstep
            it = min(max(int(tabi), 0), tb["h0tab"].size - 1)
            prof[k] = kappa0 * (tb["h0tab"][it] + a * tb["h1tab"][it])
            if prof[k] < kapmin:
                nstep, early = k, True
                break
    else:
        dv = 1.0 / dopple / resolu if (dopple * resolu) > 0 else 1e-6
        for k in range(1, n10 + 1):
            prof[k] = kappa0 * oracle.voigt(float(k) * dv, a, tb)
            if prof[k] < kapmin:
                nstep, early = k, True
                break
    x_far = 0.0
    if not early:
        x_far = prof[n10] * float(n10) ** 2 if (n10 > 0 and prof.get(n10, 0.0) > 0) else 0.0
        if x_far > 0 and kapmin > 0:
            maxstep = min(int(np.sqrt(x_far / kapmin) + 1.0), MAX_PROFILE_STEPS)
        else:
            maxstep = n10
        nstep = maxstep

    def value(k):
        if k in prof:
            return prof[k]
        return x_far / float(k) ** 2 if (not early and k > n10) else 0.0

    if ci + nstep < 0 or ci - nstep >= n:
        return
    def taper(v, w):
        if wtail is not None and w < wtail:
            base = wcon if wcon is not None else wl
            v = v * (w - base) / max(wtail - base, 1e-12)
        return v

    if ci < n - 1:
        maxred = min(n - 1 - ci, nstep) if ci >= 0 else min(n - 1, nstep)
        for k in range(max(1, -ci), maxred + 1):
            b = ci + k
            if 0 <= b < n:
                if wcon is not None and grid[b] <= wcon:
                    continue
                tmp[b] += taper(value(k), grid[b])
    if ci <= 0:
        return
    for k in range(max(1, ci + 1 - n), min(ci, nstep) + 1):
        b = ci - k
        if 0 <= b < n:
            if wcon is not None and grid[b] <= wcon:
                break
            tmp[b] += taper(value(k), grid[b])


def asynth_term(cat: Dict[str, np.ndarray], atm: Dict[str, np.ndarray], grid: np.ndarray,
                continuum: np.ndarray, cutoff: float = 1e-3, microturb_kms: float = 0.0) -> np.ndarray:
    """TMP x STIM [L, N]: what the fort.19 NORMAL lines add to ASYNTH.  ``cat``
    (gfall.parse_gfall keys) with the centre bins in ``center``."""
    tb = oracle.tables()
    L, N = continuum.shape
    rows = normal_rows(cat)
    rec = record_values(cat, rows)
    arows = aut_rows(cat)
    arec = aut_record_values(cat, arows)
    crows = cont_rows(cat) if "continuum_label" in cat else np.zeros(0, np.int64)
    # fort.19 order = catalog order, the kinds interleaved
    kind = {int(i): ("n", j) for j, i in enumerate(rows)}
    kind.update({int(i): ("a", j) for j, i in enumerate(arows)})
    kind.update({int(i): ("c", j) for j, i in enumerate(crows)})
    order = sorted(kind)
    pop = np.asarray(atm["population_per_ion"])
    rho = np.asarray(atm["mass_density"])
    xne = np.asarray(atm["electron_density"])
    hckt = np.asarray(atm["hckt"])
    txn = oracle.txnxn(atm)
    contx = contx_table()
    nmerge = np.maximum(1600.0 / np.power(np.maximum(xne, 1e-40), 2.0 / 15.0) - 1.5, 1.0)
    emerge = 109737.312 / np.maximum(nmerge ** 2, 1e-12)
    emerge_h = 109677.576 / np.maximum(nmerge ** 2, 1e-12)
    stim = 1.0 - np.exp(-(C_LIGHT_CM / (grid * 1e-7))[None, :]
                        * (6.62607015e-27 / (KBOLTZ * np.asarray(atm["temperature"])))[:, None])
    out = np.zeros((L, N))
    for d in range(L):
        tmp = np.zeros(N)
        for i in order:
            k, j = kind[i]
            z = int(cat["nelem"][i]) - 1
            ion = int(cat["ion_stage"][i])
            pv = float(pop[d, ion - 1, z]) if ion <= pop.shape[1] else 0.0
            if pv <= 0.0:
                continue
            boltz = hydrogen.fast_ex(float(cat["excitation_energy"][i]) * float(hckt[d]))
            wl = float(cat["wavelength"][i])
            ci = int(cat["center"][i])
            if ci >= N:
                continue
            r = float(rho[d])
            if r <= 0.0:
                continue
            if k == "c":
                # merged continuum (opacity.py:1489-1520): KAPPA = GF XNFPEL BOLT
                gfc = float(np.float32(10.0 ** float(cat["log_gf"][i]) * (2.0 * float(cat["xj"][i]) + 1.0)))
                kappa = gfc * (pv / r) * boltz
                nl = int(_nlast(cat)[i])
                wm, wt = _merged_limits(wl, nl, float(emerge[d]), float(emerge_h[d]),
                                        _nelion(float(cat["code"][i])))
                _merged_continuum(tmp, continuum[d], grid, ci, wl, kappa, cutoff,
                                  wm if wm is not None else wl, wt if wt is not None else wl)
                continue
            if k == "a":
                # XLINOP label 700: KAPPA0 = BSHORE * GF * XNFPEL * BOLT (opacity.py:1522-1541)
                k0 = arec["gamma_vdw"][j] * arec["gf"][j] * (pv / r) * boltz
                _autoionizing(tmp, continuum[d], grid, ci, wl, k0, arec["gamma_rad"][j],
                              arec["gamma_stark"][j], arec["gamma_vdw"][j], cutoff)
                continue
            dw = line_doppler(atm, d, wl, microturb_kms)
            if wl <= 0.0 or dw <= 0.0:
                continue
            dopple = dw / wl
            if dopple <= 0.0:
                continue
            xnfdop = pv / (r * dopple)
            k0pre = rec["cgf"][j] * xnfdop
            cc = max(0, min(ci, N - 1))
            kapmin = float(continuum[d, cc]) * cutoff
            if k0pre < kapmin:
                continue
            k0 = k0pre * boltz
            if k0 < kapmin:
                continue
            gt = rec["gamma_rad"][j] + rec["gamma_stark"][j] * float(xne[d]) + rec["gamma_vdw"][j] * float(txn[d])
            adamp = gt / dopple if dopple > 0.0 else 0.0
            kapcen = k0 * (1.0 - 1.128 * adamp) if adamp < 0.2 else k0 * oracle.voigt(0.0, adamp, tb)
            if kapcen >= kapmin:
                tmp[cc] += kapcen
            nc, nx = merge_index(cat, i)
            wcon, wtail = (None, None)
            if nc > 0 and nx > 0:
                wcon, wtail = continuum_limits(nc, _nelion(float(cat["code"][i])), nx, float(emerge[d]),
                                               float(emerge_h[d]), contx)
            _metal_wing(tmp, continuum[d], grid, ci, wl, k0, adamp, dw, cutoff, tb, wcon, wtail)
        if np.any(tmp > 0.0):
            out[d] = tmp * stim[d]
    return out
