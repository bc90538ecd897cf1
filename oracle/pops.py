"""FP64 restatement of the reference's population stage -- test infrastructure.

Only ``tests/`` (and the GPU parity checks) use this module, to check the CUDA
population kernels; it is never part of the product.

It restates, step by step, what the reference's atmosphere converter computes
from an ATLAS ``.atm`` model before synthesis (the secondary hot-path row "P"):

* ``.atm`` parsing and the derived per-layer quantities
  (``synthe_py/tools/convert_atm_to_npz.py:190-372, 374-655``) and the
  abundance vector (``:1775-1800``), WTMOLE (``:1708``);
* PFSAHA -- partition functions, lowered ionisation potentials and Saha
  fractions (``synthe_py/tools/pops_exact.py:987-1636``), with PFGROUND
  (``:220-240``) and PFIRON (``:831-925``);
* READMOL (``synthe_py/tools/readmol_exact.py:20``);
* NMOLEC -- molecular equilibrium by Newton iteration on the element
  densities (``synthe_py/tools/nmolec_exact.py:1742-3575``) with the EQ/DEQ
  assembly (``:760-926``) and SOLVIT (``:3671-3765``);
* XNFPMOL (``synthe_py/tools/pops_exact.py:28-153``) and POPS with its molecular
  branch (``:1639-2025``);
* Doppler widths (``synthe_py/tools/pops_exact.py:2027-2096``);
* the converter's sequence of POPS calls and the fields it stores
  (``convert_atm_to_npz.py:1860-2230, 2470-2650, 2755-2790``).

Arithmetic is FP64 in the reference's operation order.  Three places differ
from the reference by design and only at rounding level: products of
molecular terms are plain products (the reference forms them in log space),
EQ sums are plain sums (the reference adds in signed log space) and the
reference's power-of-two scaled divisions are plain divisions (identical for
normal numbers).  Pinned against the converter's own outputs on the golden
atmospheres (``tests/test_pops_oracle.py``).
"""

from __future__ import annotations

import math
import re
from functools import lru_cache
from pathlib import Path
from typing import Dict, Tuple

import numpy as np

TABLES = Path(__file__).resolve().parents[1] / "kurucz_py_joss_submission_gb300" / "data" / "pops_tables.npz"

# constants of the reference (convert_atm_to_npz.py:68-79, pops_exact.py:156-170)
C_CMS = 2.99792458e10
H_PLANCK = 6.62607015e-27
K_BOLTZ = 1.380649e-16
K_BOLTZ_FORTRAN = 1.38054e-16
KBOLTZ_EV = 1.0 / 8.6171e-5
EV_TO_CM = 8065.479
HCK_PFG = 6.6256e-27 * 2.99792458e10 / 1.38054e-16
LOCZ = (1, 3, 6, 10, 14, 18, 22, 27, 33, 39, 45, 51, 57, 63, 69, 75, 81, 86, 91, 96, 101, 106,
        111, 116, 121, 126, 131, 136, 141)
SCALE = (0.001, 0.01, 0.1, 1.0)
MAXEQ = 30


@lru_cache(maxsize=1)
def tables() -> Dict[str, np.ndarray]:
    with np.load(TABLES) as d:
        return {k: np.asarray(d[k]) for k in d.files}


# ---------------------------------------------------------------------------
# .atm input (convert_atm_to_npz.py:190-372)
# ---------------------------------------------------------------------------

def parse_atm(path: Path) -> dict:
    data = {"teff": None, "glog": None, "abundance_scale": 1.0, "abundances": {}, "layers": []}
    lines = Path(path).read_text(encoding="latin-1", errors="ignore").splitlines()
    i = 0
    while i < len(lines):
        line = lines[i].strip()
        if line.startswith("TEFF"):
            m = re.search(r"TEFF\s+([\d.]+)", line)
            if m:
                data["teff"] = float(m.group(1))
            m = re.search(r"(?:GRAVITY|LOG G)\s+([-\d.]+)", line)
            data["glog"] = float(m.group(1))
        elif line.startswith("ABUNDANCE SCALE"):
            m = re.search(r"ABUNDANCE SCALE\s+([\d.]+)", line)
            if m:
                data["abundance_scale"] = float(m.group(1))
            parts = line.split("ABUNDANCE CHANGE")
            if len(parts) > 1:
                for z, a in re.findall(r"(\d+)\s+([+-]?\d+\.?\d*)", parts[1].strip()):
                    data["abundances"][int(z)] = float(a)
        elif line.startswith("ABUNDANCE CHANGE"):
            for z, a in re.findall(r"(\d+)\s+([+-]?\d+\.?\d*)", line):
                data["abundances"][int(z)] = float(a)
        elif line.startswith("READ DECK6"):
            i += 1
            break
        i += 1
    rows = []
    while i < len(lines):
        parts = lines[i].split()
        if len(parts) >= 7:
            rows.append([float(x) for x in parts[:7]])
        i += 1
    data["layers"] = np.asarray(rows, dtype=np.float64)  # RHOX, T, P, XNE, ABROSS, ACCRAD, VTURB
    return data


def abundances(atm: dict) -> np.ndarray:
    """XABUND (convert_atm_to_npz.py:1775-1800)."""
    out = np.zeros(99)
    sc = atm["abundance_scale"]
    for z in range(1, 100):
        a = atm["abundances"].get(z, -20.0)
        if z <= 2:
            out[z - 1] = 10.0 ** a if a < 0.0 else a
        else:
            la = math.log10(a) if a > 0.0 else a
            out[z - 1] = sc * (10.0 ** la)
    return out


def derived(atm: dict, abundance_offsets: dict = None) -> dict:
    """Per-layer state (convert_atm_to_npz.py:374-655, 1700-1730).
    ``abundance_offsets`` {Z: dex} scales XABUND (used to difference the stage)."""
    L = atm["layers"]
    rhox, T, P, xne, vturb = L[:, 0], L[:, 1].copy(), L[:, 2].copy(), L[:, 3].copy(), L[:, 6].copy()
    if rhox[0] < 0:
        rhox = 10.0 ** rhox
    if rhox.size > 1 and rhox[0] > rhox[-1]:
        raise ValueError("layers must be in order of increasing RHOX")
    tk = K_BOLTZ_FORTRAN * T
    p_ratio = (10.0 ** atm["glog"]) * rhox[0] / P[0] if P[0] > 0 else 0.0
    if p_ratio > 1e5 and not (0.9 < p_ratio < 1.1):
        P = P * 1e6
    xabund = abundances(atm)
    for z, dx in (abundance_offsets or {}).items():
        xabund[int(z) - 1] *= 10.0 ** dx
    wtmole = float(np.sum(xabund * tables()["atmass"][:99]))
    xnatm = np.maximum(P / tk - xne, 1e-30)
    return dict(
        rhox=rhox, temperature=T, tkev=T / KBOLTZ_EV, tk=tk, hkt=H_PLANCK / (K_BOLTZ * T),
        tlog=np.log(T), hckt=H_PLANCK * C_CMS / (K_BOLTZ * T), gas_pressure=P, xne=xne,
        xnatm=xnatm, turbulent_velocity=vturb, xabund=xabund, wtmole=wtmole,
    )


# ---------------------------------------------------------------------------
# PFSAHA (pops_exact.py:987-1636)
# ---------------------------------------------------------------------------

# Explicit partition-function sums keyed by the NNN column of the species:
# (level table, number of levels summed from the 2nd, base terms (g, E),
#  extra terms (g, E), minimum T for the level sum, D1 numerator and n*
#  of the high-T correction, G override).
_SPECIAL = {
    1: ("hyd", 5, [(2.0, None)], [], 9000.0, (109677.576, 6.5), None),
    3: ("he1", 28, [(1.0, None)], [], 15000.0, (109677.576, 5.5), None),
    4: ("he2", 5, [(2.0, None)], [], 30000.0, (4.0 * 109722.267, 6.5), None),
    354: ("c1", 13, [(1.0, None), (3.0, 16.42), (5.0, 43.42)],
          [(108.0, 80000.0), (189.0, 84000.0), (247.0, 87000.0), (231.0, 88000.0),
           (190.0, 89000.0), (300.0, 90000.0)], None, None, None),
    355: ("c2", 5, [(2.0, None), (4.0, 63.42)],
          [(6.0, 131731.80), (4.0, 142027.1), (10.0, 145550.13), (10.0, 150463.62),
           (2.0, 157234.07), (6.0, 162500.0), (42.0, 168000.0), (56.0, 178000.0),
           (102.0, 183000.0), (400.0, 188000.0)], None, None, None),
    51: ("mg1", 10, [(1.0, None)],
         [(5.0, 53134.0), (15.0, 54192.0), (28.0, 54676.0), (9.0, 57853.0)], None,
         (109734.83, 4.5), 4.0),
    52: ("mg2", 5, [(2.0, None)],
         [(10.0, 93310.80), (14.0, 93799.70), (6.0, 97464.32), (10.0, 103419.82),
          (14.0, 103689.89), (18.0, 103705.66)], None, (4.0 * 109734.83, 5.5), 2.0),
    57: ("al1", 8, [(2.0, None), (4.0, 112.061)], [(10.0, 42235.0), (14.0, 43831.0)], None,
         (109735.08, 5.5), 2.0),
    63: ("si1", 10, [(1.0, None), (3.0, 77.115), (5.0, 223.157)],
         [(76.0, 53000.0), (71.0, 57000.0), (191.0, 60000.0), (240.0, 62000.0),
          (251.0, 63000.0), (300.0, 65000.0)], None, None, None),
    64: ("si2", 5, [(2.0, None), (4.0, 287.32)],
         [(6.0, 81231.59), (6.0, 83937.08), (10.0, 101024.09), (14.0, 103556.35),
          (10.0, 108800.0), (42.0, 115000.0), (6.0, 121000.0), (38.0, 125000.0),
          (34.0, 132000.0)], None, (4.0 * 109734.83, 4.5), 2.0),
    367: ("o1", 12, [(5.0, None), (3.0, 158.265), (1.0, 226.977)],
          [(15.0, 101140.0), (131.0, 103000.0), (128.0, 105000.0), (600.0, 107000.0)],
          None, None, None),
    45: ("na1", 7, [(2.0, None)], [(10.0, 34548.745), (14.0, 34586.96)], None,
         (109734.83, 4.5), 2.0),
    14: ("b1", 6, [(2.0, None), (4.0, 15.25)],
         [(6.0, 57786.80), (10.0, 59989.0), (14.0, 60031.03), (2.0, 63561.0)], None,
         (109734.83, 4.5), 2.0),
    91: ("k1", 7, [(2.0, None)], [(10.0, 27397.077), (14.0, 28127.85)], None,
         (109734.83, 5.5), 2.0),
}


def _sum_terms(terms, hckt):
    v = None
    for g, e in terms:
        t = g if e is None else g * math.exp(-e * hckt)
        v = t if v is None else v + t
    return v


def _special_part(col: int, T: float, hckt: float):
    """PART, D1 and G override of the explicitly summed species (pops_exact.py:1130-1430)."""
    name, nlev, base, extra, tmin, d1, g_over = _SPECIAL[col]
    tb = tables()
    part = _sum_terms(base, hckt)
    if tmin is None or T >= tmin:
        ge, gg = tb[f"lev_{name}_e"], tb[f"lev_{name}_g"]
        for i in range(1, nlev + 1):
            part += gg[i] * math.exp(-ge[i] * hckt)
    if extra:
        part += _sum_terms(extra, hckt)
    D1 = d1[0] / d1[1] / d1[1] * hckt if d1 is not None else 0.0
    return part, D1, g_over


def pfground(nelion: int, T: float) -> float:
    """PFGROUND (pops_exact.py:220-240, _pfground_table.py)."""
    tb = tables()
    if T <= 0.0 or nelion <= 0:
        return 1.0
    first, second = tb["pfg_first"], tb["pfg_second"]
    if nelion <= len(first):
        label = int(first[nelion - 1])
    elif nelion < 169:
        return 1.0
    elif nelion - 169 < len(second):
        label = int(second[nelion - 169])
    else:
        label = 666
    idx = np.searchsorted(tb["pfg_label"], label)
    if idx >= len(tb["pfg_label"]) or tb["pfg_label"][idx] != label:
        return 1.0
    v = float(tb["pfg_g0"][idx])
    for k in range(int(tb["pfg_off"][idx]), int(tb["pfg_off"][idx + 1])):
        v = v + float(tb["pfg_g"][k]) * math.exp(-HCK_PFG / T * float(tb["pfg_e"][k]))
    return v


def pfiron(iz: int, ion: int, tlog10: float, potlow_cm: float) -> float:
    """PFIRON for Ca..Ni (pops_exact.py:831-925)."""
    tb = tables()
    pftab, potlo, potlolog = tb["pftab"], tb["pf_potlo"], tb["pf_potlolog"]
    e, i = iz - 20, ion - 1
    if tlog10 > 4.0:
        it = max(1, min(56, int((tlog10 - 4.0) / 0.05 + 31.0)))
        f = (tlog10 - (it - 31) * 0.05 - 4.0) / 0.05
    elif tlog10 < 3.7:
        it = max(2, int((tlog10 - 3.32) / 0.02 + 2.0))
        f = (tlog10 - (it - 2) * 0.02 - 3.32) / 0.02
    else:
        it = int((tlog10 - 3.7) / 0.03 + 21.0)
        f = (tlog10 - (it - 21) * 0.03 - 3.7) / 0.03
    it = max(1, min(56, it))
    a, b = it - 1, max(0, it - 2)
    if potlow_cm < potlo[0]:
        return float(f * pftab[0, a, i, e] + (1.0 - f) * pftab[0, b, i, e])
    low = len(potlo) - 1
    for k in range(1, len(potlo)):
        if potlow_cm < potlo[k]:
            low = k
            break
    p = (math.log10(potlow_cm) - potlolog[low - 1]) / 0.30103
    return float(p * (f * pftab[low, a, i, e] + (1.0 - f) * pftab[low, b, i, e])
                 + (1.0 - p) * (f * pftab[low - 1, a, i, e] + (1.0 - f) * pftab[low - 1, b, i, e]))


def potion_index(iz: int, ion: int) -> int:
    """1-based POTION index (pops_exact.py:928-938)."""
    return iz * (iz + 1) // 2 + ion - 1 if iz <= 30 else iz * 5 + 341 + ion - 1


def pfsaha(iz: int, nion: int, T: float, tv: float, tk: float, hckt: float, tlog: float,
           P: float, xne: float) -> Tuple[np.ndarray, np.ndarray, int]:
    """Saha fractions F and partition functions PART of ions 1..NION2 of one layer.

    Returns ``(F, PART, nion2)``; the modes of the reference map to
    ``F/PART`` (1), ``F`` (2), ``PART`` (3) and ``sum (i-1) F_i`` (4).
    """
    tb = tables()
    potion, nnn = tb["potion"], tb["nnn"]
    charge = xne * 2.0
    excess = 2.0 * xne - P / tk
    if excess > 0.0:
        charge = charge + 2.0 * excess
    if charge == 0.0:
        charge = 1.0
    debye = math.sqrt(tk / 2.8965e-18 / charge)
    potlow = min(1.0, 1.44e-7 / debye)
    if iz <= 28:
        n = LOCZ[iz - 1]
        nions = LOCZ[iz] - LOCZ[iz - 1]
    else:
        n = 3 * iz + 54
        nions = 3
    if iz == 6:
        n, nions = 354, 6
    elif iz == 7:
        n, nions = 360, 7
    elif iz == 8:
        n, nions = 367, 8
    if 20 <= iz < 29:
        nions = 10
    nion2 = min(nion + 2, nions)
    IP = np.zeros(nion2)
    PART = np.ones(nion2)
    POTLO = np.zeros(nion2)
    for ion in range(1, nion2 + 1):
        z = float(ion)
        POTLO[ion - 1] = potlow * z
        pi = potion_index(iz, ion) - 1
        if 0 <= pi < len(potion):
            IP[ion - 1] = potion[pi] / EV_TO_CM
            if IP[ion - 1] == 0.0 and pi > 0:
                IP[ion - 1] = potion[pi - 1] / EV_TO_CM
        if 20 <= iz < 29:
            PART[ion - 1] = pfiron(iz, ion, tlog / 2.30258509299405, POTLO[ion - 1] * EV_TO_CM)
            continue
        col = n - 1 + ion          # 1-based NNN column
        c0 = col - 1
        G = 0.0
        D1 = 0.0
        if c0 < 374:
            G = float(nnn[5, c0] - (nnn[5, c0] // 100) * 100)
        handled = False
        if col == 2:
            PART[ion - 1] = 1.0
            handled = True
        if col in _SPECIAL:
            part, D1, g_over = _special_part(col, T, hckt)
            PART[ion - 1] = part
            if g_over is not None:
                G = g_over
            handled = True
        if not handled and c0 < nnn.shape[1] and IP[ion - 1] > 0.0:
            t2000 = IP[ion - 1] * 2000.0 / 11.0
            it = max(1, min(9, int(T / t2000 - 0.5)))
            dt = T / t2000 - float(it) - 0.5
            pmin = 1.0
            i_idx = max(0, min(5, (it + 1) // 2 - 1))
            v = int(nnn[i_idx, c0])
            k1 = v // 100000
            k2 = v - k1 * 100000
            k3 = k2 // 10
            ks = max(0, min(3, k2 - k3 * 10 - 1))
            if it % 2 == 1:
                p1 = float(k1) * SCALE[ks]
                p2 = float(k3) * SCALE[ks]
                if dt < 0.0 and ks <= 0 and p1 == float(int(p2 + 0.5)):
                    pmin = p1
            else:
                p1 = float(k3) * SCALE[ks]
                v1 = int(nnn[min(i_idx + 1, 5), c0])
                ks1 = max(0, min(3, v1 % 10 - 1))
                p2 = float(v1 // 100000) * SCALE[ks1]
            PART[ion - 1] = max(pmin, p1 + (p2 - p1) * dt)
        elif not handled:
            PART[ion - 1] = 1.0
        skip_high_t = False
        if IP[ion - 1] > 0.0:
            t2000 = IP[ion - 1] * 2000.0 / 11.0
            if T < t2000 * 2.0:
                pg = pfground((iz - 1) * 6 + ion, T)
                if pg > 0.0:
                    PART[ion - 1] = max(PART[ion - 1], pg)
                skip_high_t = True
        bypass = D1 > 0.0
        if (not skip_high_t and (G > 0.0 or D1 > 0.0) and (bypass or POTLO[ion - 1] >= 0.1)
                and IP[ion - 1] > 0.0):
            t2000 = IP[ion - 1] * 2000.0 / 11.0
            if bypass or T >= t2000 * 4.0:
                tvu = tv
                if T > t2000 * 11.0:
                    tvu = (t2000 * 11.0) * 8.6171e-5
                d1v = 0.1 / tvu if D1 <= 0.0 else D1
                d2 = POTLO[ion - 1] / tvu
                term1 = math.sqrt(13.595 * z * z / tvu / d2) ** 3
                term1 *= 1.0 / 3.0 + (1.0 - (0.5 + (1.0 / 18.0 + d2 / 120.0) * d2) * d2) * d2
                term2 = math.sqrt(13.595 * z * z / tvu / d1v) ** 3
                term2 *= 1.0 / 3.0 + (1.0 - (0.5 + (1.0 / 18.0 + d1v / 120.0) * d1v) * d1v) * d1v
                if G > 0.0:
                    PART[ion - 1] += G * math.exp(-IP[ion - 1] / tvu) * (term1 - term2)
    cf = 2.0 * 2.4148e15 * T * math.sqrt(T) / xne
    F = np.zeros(nion2)
    F[0] = 1.0
    for ion in range(2, nion2 + 1):
        if PART[ion - 2] > 0:
            F[ion - 1] = cf * PART[ion - 1] / PART[ion - 2] * math.exp(-(IP[ion - 2] - POTLO[ion - 2]) / tv)
        else:
            F[ion - 1] = 0.0
    Lx = nion2 + 1
    for _ in range(2, nion2 + 1):
        Lx -= 1
        F[0] = 1.0 + F[Lx - 1] * F[0]
    F[0] = 1.0 / F[0]
    for ion in range(2, nion2 + 1):
        F[ion - 1] = F[ion - 2] * F[ion - 1]
    return F, PART, nion2


def _layer(st: dict, j: int, xne: float):
    return (st["temperature"][j], st["tkev"][j], st["tk"][j], st["hckt"][j], st["tlog"][j],
            st["gas_pressure"][j], xne)


# ---------------------------------------------------------------------------
# READMOL (readmol_exact.py:20) and NMOLEC (nmolec_exact.py:1742)
# ---------------------------------------------------------------------------

@lru_cache(maxsize=1)
def readmol():
    """Components of every molecule as equation numbers (0-based; NEQUA = inverse electron)."""
    tb = tables()
    codes, equil = tb["mol_code"], tb["mol_equil"]
    xcode = (1e14, 1e12, 1e10, 1e8, 1e6, 1e4, 1e2, 1e0)
    ifequa = np.zeros(102, dtype=np.int64)
    comps, locj = [], [0]
    for c in codes:
        ii = next(i for i in range(8) if c >= xcode[i])
        x = float(c)
        for i in range(ii, 8):
            idz = int(x / xcode[i])
            x = x - float(idz) * xcode[i]
            if idz == 0:
                idz = 100
            ifequa[idz] = 1
            comps.append(idz)
        ion = int(x * 100.0 + 0.5)
        if ion >= 1:
            ifequa[100] = 1
            ifequa[101] = 1
            comps += [101] * ion
        locj.append(len(comps))
    iequa = 1
    idequa = np.zeros(MAXEQ, dtype=np.int64)
    for i in range(1, 101):
        if ifequa[i] == 1:
            iequa += 1
            ifequa[i] = iequa
            idequa[iequa - 1] = i
    nequa = iequa
    ifequa[101] = nequa + 1
    kcomps = np.array([ifequa[c] - 1 for c in comps], dtype=np.int64)
    return codes, equil, np.array(locj, dtype=np.int64), kcomps, idequa, nequa


def _solvit(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Gauss-Jordan elimination with full pivot search (nmolec_exact.py:3671-3765)."""
    a = a.copy()
    b = b.copy()
    n = len(b)
    done = np.zeros(n, dtype=bool)
    for _ in range(n):
        sub = np.abs(a)
        sub[done, :] = -1.0
        sub[:, done] = -1.0
        flat = int(np.argmax(sub))
        amax = sub.flat[flat]
        irow, icol = (flat // n, flat % n) if amax > 0.0 else (0, 0)
        done[icol] = True
        if irow != icol:
            a[[irow, icol], :] = a[[icol, irow], :]
            b[irow], b[icol] = b[icol], b[irow]
        pivot = a[icol, icol]
        a[icol, icol] = 1.0
        a[icol, :] = a[icol, :] / pivot
        b[icol] = b[icol] / pivot
        t = a[:, icol].copy()
        t[icol] = 0.0
        rows = np.nonzero(t != 0.0)[0]
        a[rows, icol] = 0.0
        a[rows, :] = a[rows, :] - a[icol, :][None, :] * t[rows, None]
        b[rows] = b[rows] - b[icol] * t[rows]
    return b


def _equilj(st: dict, j: int, xne_j: float) -> np.ndarray:
    """Equilibrium constants of every molecule in layer j (nmolec_exact.py:2268-2531)."""
    codes, equil, locj, kcomps, idequa, nequa = readmol()
    T, tkev, tlog = st["temperature"][j], st["tkev"][j], st["tlog"][j]
    out = np.zeros(len(codes))
    for m in range(len(codes)):
        ncomp = int(locj[m + 1] - locj[m])
        if equil[0, m] == 0.0:
            if ncomp > 1:
                F, _, _ = pfsaha(int(codes[m]), ncomp, *_layer(st, j, xne_j))
                ion = ncomp - 1
                out[m] = F[ncomp - 1] / F[0] * xne_j ** ion
            else:
                out[m] = 1.0
            continue
        ion = int((codes[m] - float(int(codes[m]))) * 100.0 + 0.5)
        if T > 10000.0:
            continue
        if abs(codes[m] - 101.0) < 1e-9:
            arg = (4.478 / tkev - 46.4584
                   + (1.63660e-3 + (-4.93992e-7 + (1.11822e-10 + (-1.49567e-14
                      + (1.06206e-18 - 3.08720e-23 * T) * T) * T) * T) * T) * T - 1.5 * tlog)
        else:
            e = equil[:, m]
            arg = (e[0] / tkev - e[1] + (e[2] + (-e[3] + (e[4] + (-e[5] + e[6] * T) * T) * T) * T) * T
                   - 1.5 * float(ncomp - ion - ion - 1) * tlog)
        out[m] = math.exp(arg)
    return out


def nmolec(st: dict, xabund: np.ndarray) -> dict:
    """Molecular equilibrium of every layer, surface first (nmolec_exact.py:1742-3575).

    Returns XN per layer (element densities, XN[0] = XNATOM, last = XNE), the
    molecule densities XNMOL and the Newton iteration counts.
    """
    codes, equil, locj, kcomps, idequa, nequa = readmol()
    nl = len(st["temperature"])
    nmol = len(codes)
    e_idx = nequa - 1
    has_e = idequa[e_idx] == 100
    xab = np.zeros(nequa)
    for k in range(1, nequa):
        if idequa[k] < 100:
            xab[k] = max(xabund[idequa[k] - 1], 1e-20)
    if has_e:
        xab[e_idx] = 0.0
    xnz = np.zeros((nl, nequa))
    xnmol = np.zeros((nl, nmol))
    xne_out = np.zeros(nl)
    iters = np.zeros(nl, dtype=np.int64)
    xn = np.zeros(nequa)
    prev = np.zeros(nequa)
    xne_prev = 0.0
    P, tk = st["gas_pressure"], st["tk"]
    for j in range(nl):
        xntot = P[j] / tk[j]
        if j == 0:
            xn[0] = xntot / 2.0
            x = xn[0] / 10.0
            xn[1:] = x * xab[1:]
            if has_e:
                xn[e_idx] = x
            xne_j = x
        else:
            ratio = P[j] / P[j - 1]
            xn[:] = prev * ratio
            xne_j = xne_prev * ratio
        eqj = _equilj(st, j, xne_j)
        eqold = np.zeros(nequa)
        it = 0
        for it in range(1, 201):
            eq = np.zeros(nequa)
            deq = np.zeros((nequa, nequa))      # deq[row, col]
            eq[0] = -xntot
            for k in range(1, nequa):
                eq[0] = eq[0] + xn[k]
                deq[0, k] = 1.0
                eq[k] = xn[k] - xab[k] * xn[0]
                deq[k, k] = 1.0
                deq[k, 0] = -xab[k]
            if has_e:
                eq[e_idx] = -xn[e_idx]
                deq[e_idx, e_idx] = -1.0
            for m in range(nmol):
                l1, l2 = int(locj[m]), int(locj[m + 1])
                if l2 - l1 <= 1:
                    continue
                term = eqj[m]
                if not (math.isfinite(term) and term > 0.0):
                    continue
                for lk in range(l1, l2):
                    k = int(kcomps[lk])
                    term = term / xn[e_idx] if k >= nequa else term * xn[k]
                eq[0] = eq[0] + term
                for lk in range(l1, l2):
                    k = int(kcomps[lk])
                    if k >= nequa:
                        k = e_idx
                        d = -term / xn[k]
                    else:
                        d = term / xn[k]
                    eq[k] = eq[k] + term
                    deq[0, k] = deq[0, k] + d
                    for lm in range(l1, l2):
                        mm = int(kcomps[lm])
                        mm = e_idx if mm >= nequa else mm
                        deq[mm, k] = deq[mm, k] + d
                if has_e and int(kcomps[l2 - 1]) == e_idx:
                    for lk in range(l1, l2):
                        k = int(kcomps[lk])
                        k = e_idx if k >= nequa else k
                        d = term / xn[k]
                        if k == e_idx:
                            eq[k] = eq[k] - term - term
                        deq[e_idx, k] = deq[e_idx, k] - d - d
            delta = _solvit(deq, eq)
            iferr = 0
            scale = 100.0
            for k in range(nequa):
                if abs(delta[k] / xn[k]) > 0.001:
                    iferr = 1
                flip = (eqold[k] > 0 and delta[k] < 0) or (eqold[k] < 0 and delta[k] > 0)
                if flip:
                    delta[k] = delta[k] * 0.69
                xneq = xn[k] * (1.0 - delta[k] / xn[k]) if abs(xn[k]) > 2.2250738585072014e-308 \
                    else xn[k] - delta[k]
                if xneq < xn[k] / 100.0:
                    xn[k] = xn[k] / scale
                    if flip:
                        scale = math.sqrt(scale)
                else:
                    xn[k] = xneq
                eqold[k] = delta[k]
            if iferr == 0:
                break
        iters[j] = it
        xnz[j] = xn
        prev = xn.copy()
        if has_e:
            xne_j = xn[e_idx]
        xne_prev = xne_j
        xne_out[j] = xne_j
        for m in range(nmol):
            v = eqj[m]
            for lk in range(int(locj[m]), int(locj[m + 1])):
                k = int(kcomps[lk])
                v = v / xn[e_idx] if k >= nequa else v * xn[k]
            xnmol[j, m] = v
    return dict(xnz=xnz, xnmol=xnmol, xne=xne_out, xnatom=xnz[:, 0].copy(), iters=iters)


def xnfpmol(st: dict, xne: np.ndarray, nm: dict) -> np.ndarray:
    """Number densities over partition functions of the molecule-table species (pops_exact.py:28-153)."""
    codes, equil, locj, kcomps, idequa, nequa = readmol()
    atmass = tables()["atmass"]
    nl = len(st["temperature"])
    T = st["temperature"]
    xz = nm["xnz"].copy()
    for k in range(1, nequa):
        idv = int(idequa[k])
        if idv == 100:
            xz[:, k] = xz[:, k] / (2.0 * 2.4148e15 * T * np.sqrt(T))
            continue
        if idv <= 0 or idv > 99:
            continue
        pf = np.array([pfsaha(idv, 1, *_layer(st, j, xne[j]))[1][0] for j in range(nl)])
        xz[:, k] = xz[:, k] / (pf * 1.8786e20 * np.sqrt((atmass[idv - 1] * T) ** 3))
    out = np.zeros((nl, len(codes)))
    for m in range(len(codes)):
        l1, l2 = int(locj[m]), int(locj[m + 1])
        if equil[0, m] != 0.0:
            xnf = np.exp(equil[0, m] / st["tkev"])
            amass = 0.0
            for lk in range(l1, l2):
                k = int(kcomps[lk])
                if k == nequa:
                    xnf = xnf / xz[:, nequa - 1]
                    continue
                idv = int(idequa[k])
                if idv <= 0 or idv > 99:
                    continue
                amass += atmass[idv - 1]
                xnf = xnf * xz[:, k]
            out[:, m] = xnf * 1.8786e20 * np.sqrt((amass * T) ** 3)
        else:
            idv = int(codes[m])
            if idv <= 0 or idv > 99:
                continue
            ncomp = l2 - l1
            pf = np.array([pfsaha(idv, ncomp, *_layer(st, j, xne[j]))[1][ncomp - 1] for j in range(nl)])
            out[:, m] = nm["xnmol"][:, m] / pf
    return out


# ---------------------------------------------------------------------------
# POPS (pops_exact.py:1639-2025), Doppler widths (:2027) and the converter's sequence
# ---------------------------------------------------------------------------

def element_code(z: int) -> float:
    """CODE of the all-ion POPS call of element z (convert_atm_to_npz.py:2496-2532)."""
    if z == 1:
        return 1.01
    if z == 2:
        return 2.02
    if z <= 5:
        return float(z) + 0.03
    if z <= 16:
        return float(z) + 0.05
    if z <= 19:
        return float(z) + 0.04
    if z <= 28:
        return float(z) + 0.09
    return float(z) + 0.02


def pops(code: float, mode: int, st: dict, xne: np.ndarray, xnatom: np.ndarray, xabund: np.ndarray,
         nm: dict, xfp: np.ndarray) -> np.ndarray:
    """NUMBER[layer, ion] of one POPS call after NMOLEC has run (pops_exact.py:1855-2025)."""
    codes = readmol()[0]
    nl = len(st["temperature"])
    number = np.zeros((nl, 10))
    iz = int(code)
    nion = int((code - float(iz)) * 100.0 + 1.5)
    if mode > 10:
        nn = max(1, int((code - float(int(code))) * 100.0 + 1.5))
        has_int = bool(np.any(np.abs(codes - float(iz)) < 1e-3))
        c = code
        matched = False
        for i in range(1, nn + 1):
            ion = nn - i + 1
            hit = np.nonzero(np.abs(codes - c) < 0.001)[0]
            if hit.size:
                m = int(hit[0])
                if mode % 10 == 1:
                    number[:, ion - 1] = xfp[:, m]
                elif mode % 10 == 2:
                    number[:, ion - 1] = nm["xnmol"][:, m]
                matched = True
            elif has_int:
                number[:, ion - 1] = 0.0
            c -= 0.01
        if matched or has_int:
            return number
    mode1 = mode - 10 if mode > 10 else mode
    for j in range(nl):
        F, PART, nion2 = pfsaha(iz, nion, *_layer(st, j, xne[j]))
        for i in range(min(nion, nion2)):
            ans = F[i] / PART[i] if mode1 == 1 else F[i]
            number[j, i] = ans * xnatom[j] * xabund[iz - 1]
    return number


def doppler(st: dict, momass: np.ndarray) -> np.ndarray:
    """DOPPLE[layer, ion, species] (pops_exact.py:2027-2096)."""
    atmass = tables()["atmass"]
    tk, vt = st["tk"], st["turbulent_velocity"]
    nl = len(tk)
    out = np.zeros((nl, 6, 139))
    for z in range(99):
        if atmass[z] > 0:
            out[:, :, z] = (np.sqrt(2.0 * tk / atmass[z] / 1.660e-24 + vt ** 2) / C_CMS)[:, None]
    for z in range(20, 29):
        base = out[:, 0, z - 1].copy()
        for off in (30, 40, 50, 60):
            if off + z - 1 < 139:
                out[:, 4, off + z - 1] = base
    for mi in range(40, 139):
        mm = momass[mi - 39] if mi - 39 < len(momass) else 0.0
        if mm > 0:
            out[:, 5, mi] = np.sqrt(2.0 * tk / mm / 1.660e-24 + vt ** 2) / C_CMS
    return out


def molecule_masses() -> np.ndarray:
    """MOMASS of the first 100 molecule-table entries (convert_atm_to_npz.py:122-187)."""
    codes = readmol()[0]
    atmass = tables()["atmass"]
    fac = (1e14, 1e12, 1e10, 1e8, 1e6, 1e4, 1e2, 1.0)
    out = np.zeros(100)
    for i in range(min(100, len(codes))):
        c = float(codes[i])
        start = next((k for k, f in enumerate(fac) if c >= f), 0)
        rem = c
        tot = 0.0
        for f in fac[start:]:
            el = int(rem / f + 1e-9)
            rem -= el * f
            if el == 0:
                continue
            if 1 <= el <= len(atmass):
                tot += atmass[el - 1]
        out[i] = tot
    return out


def convert(atm_path: Path, abundance_offsets: dict = None) -> dict:
    """The fields the synthesis path reads, as the converter computes them from
    ``atm_path`` (``abundance_offsets`` {Z: dex}: abundances scaled first)."""
    atm = parse_atm(atm_path)
    st = derived(atm, abundance_offsets)
    xabund = st["xabund"]
    nm = nmolec(st, xabund)
    xne = nm["xne"]
    xnatom = nm["xnatom"]
    xfp = xnfpmol(st, xne, nm)
    nl = len(st["temperature"])
    population = np.zeros((nl, 6, 139))
    for z in range(1, 100):
        num = pops(element_code(z), 11, st, xne, xnatom, xabund, nm, xfp)
        population[:, :, z - 1] = num[:, :6]
    xnfh = np.maximum(pops(1.00, 12, st, xne, xnatom, xabund, nm, xfp)[:, 0], 1e-40)
    xnfhe = pops(2.01, 12, st, xne, xnatom, xabund, nm, xfp)
    T, tkev, tlog = st["temperature"], st["tkev"], st["tlog"]
    xnf_h2 = np.zeros(nl)
    for j in range(nl):
        if T[j] > 9000.0:
            continue
        t = T[j]
        eqk = math.exp(4.478 / tkev[j] - 4.64584e1
                       + (1.63660e-3 + (-4.93992e-7 + (1.11822e-10 + (-1.49567e-14
                          + (1.06206e-18 - 3.08720e-23 * t) * t) * t) * t) * t) * t - 1.5 * tlog[j])
        xnf_h2[j] = xnfh[j] ** 2 * eqk
    return dict(
        depth=st["rhox"], temperature=T, gas_pressure=st["gas_pressure"], electron_density=xne,
        xnatm=xnatom, mass_density=xnatom * st["wtmole"] * 1.660e-24,
        turbulent_velocity=st["turbulent_velocity"], hckt=st["hckt"], xnf_h=xnfh,
        xnf_he1=np.maximum(xnfhe[:, 0], 1e-40), xnf_h2=xnf_h2, population_per_ion=population,
        doppler_per_ion=doppler(st, molecule_masses()), nmolec_iterations=nm["iters"],
    )
