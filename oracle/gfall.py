"""Pure-Python restatement of the reference gfall reader (oracle side).

Test infrastructure only.  Follows ``synthe_py/io/lines/atomic.py:299-611``
(``load_catalog``, fixed-width branch) and ``:762-816`` (``filter_by_range``,
DELLIM window), and the routing of ``synthe_py/physics/line_opacity.py:740-784``
that decides which records TRANSP processes.  It returns plain NumPy arrays
in catalog order.
"""

from __future__ import annotations

import math
from pathlib import Path
from typing import Dict, Optional

import numpy as np

# synthe_py/io/lines/tfort.py:14 _ELEMENT_SYMBOLS (Z = 1..92)
ELEMENT_SYMBOLS = [
    "", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al",
    "Si", "P", "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe",
    "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",
    "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te",
    "I", "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb",
    "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt",
    "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa",
    "U",
]

DELLIM = np.array([100.0, 30.0, 10.0, 3.0, 1.0, 0.3, 0.1])


def _stark_default(code, e_lo, e_up, potion):  # atomic.py:59-106
    if code >= 100.0:
        return -5.0
    nelem = int(code + 1e-6)
    icharge = int((code - nelem) * 100.0 + 0.1)
    zeff = icharge + 1
    eup = max(abs(e_lo), abs(e_up))
    effnsq = 25.0
    index = (nelem * (nelem + 1) // 2 + icharge if nelem <= 30 else nelem * 5 + 341 + icharge) - 1
    if 0 <= index < len(potion):
        deleup = potion[index] - eup
        if deleup > 0:
            effnsq = 109737.31 * zeff * zeff / deleup
    return math.log10(1.0e-8 * effnsq * effnsq * math.sqrt(effnsq))


def _vdw_default(code, e_lo, e_up, potion):  # atomic.py:109-199
    nelem = int(code + 1e-6)
    icharge = int((code - nelem) * 100.0 + 0.1)
    zeff = icharge + 1
    if code >= 100.0:
        return math.log10(1.0e-7 / zeff)
    elo = min(abs(e_lo), abs(e_up))
    eup = max(abs(e_lo), abs(e_up))
    index = (nelem * (nelem + 1) // 2 + icharge if nelem <= 30 else nelem * 5 + 341 + icharge) - 1
    ip = potion[index] if 0 <= index < len(potion) else 0.0
    eu = 25.0
    if ip > 0 and ip - eup > 0:
        eu = 109737.31 * zeff * zeff / (ip - eup)
    eu = min(eu, 1000.0)
    rsqup = 2.5 * (eu / zeff) ** 2
    el = 25.0
    if ip > 0 and ip - elo > 0:
        el = 109737.31 * zeff * zeff / (ip - elo)
    el = min(el, 1000.0)
    rsqlo = 2.5 * (el / zeff) ** 2
    nseq = nelem - zeff + 1
    if 20 < nseq < 29:
        rsqup = (45.0 - nseq) / zeff
        rsqlo = 0.0
    if rsqup < rsqlo:
        rsqup = 2.0 * rsqlo
    diff = rsqup - rsqlo
    gammaw = 4.5e-9 * (diff ** 0.4) if diff > 0 else 1.0e-9
    return math.log10(gammaw)


def parse_gfall(path: Path, potion: np.ndarray) -> Dict[str, np.ndarray]:
    """Parse fixed-width gfall records; whitespace-format lines are ignored."""
    rows = []
    text = Path(path).read_text(encoding="ascii", errors="ignore").splitlines()
    for line in text:
        s = line.strip()
        if not s or s.startswith("#") or len(line) < 98:
            continue
        try:
            wl = float(line[0:11].strip())
            loggf_raw = float(line[11:18].strip())
            code = float(line[18:24].strip())
            e_val = float(line[24:36].strip())
            eps = line[52:64].strip()
            ep_val = float(eps) if eps else 0.0
            grs, gss, gws = line[80:86].strip(), line[86:92].strip(), line[92:98].strip()
            xjs, xjps = line[36:41].strip(), line[64:69].strip()
            xj = float(xjs) if xjs else 0.0
            xjp = float(xjps) if xjps else 0.0
        except ValueError:
            continue
        labelp = line[70:78].strip() if len(line) >= 78 else ""
        cont_label = 1 if labelp.upper().startswith("CONTINUU") else 0
        x1 = x2 = 0.0
        if len(line) >= 115 and line[109:115].strip():
            try:
                x1 = float(line[109:115].strip())
            except ValueError:
                pass
        if len(line) >= 124 and line[118:124].strip():
            try:
                x2 = float(line[118:124].strip())
            except ValueError:
                pass
        log_gf = loggf_raw + (x1 + x2)
        elo = min(abs(e_val), abs(ep_val))
        eup = max(abs(e_val), abs(ep_val))
        grl = float(grs) if grs else 0.0
        gsl = float(gss) if gss else 0.0
        gwl = float(gws) if gws else 0.0
        gr = 0.0 if grl == 0.0 else 10.0 ** grl
        gs = 0.0 if gsl == 0.0 else 10.0 ** gsl
        gw = 0.0 if gwl == 0.0 else 10.0 ** gwl
        wavelength = wl
        cother1 = line[124:134] if len(line) >= 134 else ""
        eshift = eshiftp = 0.0
        if cother1.strip():
            try:
                eshift = int(cother1[0:5]) * 1.0e-3
                eshiftp = int(cother1[5:10]) * 1.0e-3
            except ValueError:
                eshift = eshiftp = 0.0
        ediff = abs((abs(ep_val) + eshiftp) - (abs(e_val) + eshift))
        if ediff > 0.0:
            iso = line[154:160].strip() if len(line) >= 160 else ""
            dwliso = 0.0
            if iso:
                try:
                    dwliso = int(iso) * 1.0e-4
                except ValueError:
                    dwliso = 0.0
            wavelength = 1.0e7 / ediff + dwliso
        if gr == 0.0:
            gr = 2.223e13 / (wavelength ** 2)
        if gs == 0.0:
            v = _stark_default(code, elo, eup, potion)
            gs = 10.0 ** v if v != 0.0 else 0.0
        if gw == 0.0:
            v = _vdw_default(code, elo, eup, potion)
            gw = 10.0 ** v if v != 0.0 else 0.0
        frelin = 2.99792458e17 / max(wavelength, 1e-12)
        gr = gr / (12.5664 * frelin)
        gs = gs / (12.5664 * frelin)
        gw = gw / (12.5664 * frelin)
        nelem = int(code + 1e-6)
        frac = code - nelem
        ion = int(round(frac * 100.0)) + 1 if frac > 1e-6 else 1
        nblo = nbup = 0
        if len(line) >= 106:
            try:
                a, b = line[102:104].strip(), line[104:106].strip()
                nblo = int(a) if a else 0
                nbup = int(b) if b else 0
            except ValueError:
                pass
        iso1 = 0
        i1 = line[106:109].strip() if len(line) >= 109 else ""
        if i1:
            try:
                iso1 = int(i1)
            except ValueError:
                iso1 = 0
        iso2 = 0
        i2 = line[116:119].strip() if len(line) >= 119 else ""
        if i2:
            try:
                iso2 = int(i2)
            except ValueError:
                iso2 = 0
        line_size = 0
        tag = ""
        c2 = line[134:144] if len(line) >= 144 else ""
        if c2.strip():
            ls = c2[6:7]
            tag = c2[7:10].strip()
            if ls.strip().isdigit():
                line_size = int(ls)
        lt = 0
        if tag == "AUT":
            lt = 1
        elif tag == "COR":
            lt = 2
        elif tag == "PRD":
            lt = 3
        elif nelem == 1 and ion == 1 and iso1 == 2:
            lt = -2
        elif nelem == 1 and ion == 1:
            lt = -1
        elif nelem == 2 and ion == 1 and iso1 == 3:
            lt = -4
        elif nelem == 2 and ion == 1:
            lt = -3
        elif nelem == 2 and ion == 2:
            lt = -6
        rows.append((wavelength, log_gf, code, elo, gr, gs, gw, nelem, ion, lt, nblo, nbup, line_size,
                     grl, gsl, gwl, xj, xjp, cont_label, iso1, iso2))
    if not rows:
        arr = np.zeros((0, 21))
    else:
        arr = np.array(rows, dtype=np.float64)
    return {
        "wavelength": arr[:, 0].copy(),
        "log_gf": arr[:, 1].copy(),
        "code": arr[:, 2].copy(),
        "excitation_energy": arr[:, 3].copy(),
        "gamma_rad": arr[:, 4].copy(),
        "gamma_stark": arr[:, 5].copy(),
        "gamma_vdw": arr[:, 6].copy(),
        "nelem": arr[:, 7].astype(np.int32),
        "ion_stage": arr[:, 8].astype(np.int32),
        "line_type": arr[:, 9].astype(np.int32),
        "n_lower": arr[:, 10].astype(np.int32),
        "n_upper": arr[:, 11].astype(np.int32),
        "line_size": arr[:, 12].astype(np.int32),
        "gamma_rad_log": arr[:, 13].copy(),
        "gamma_stark_log": arr[:, 14].copy(),
        "gamma_vdw_log": arr[:, 15].copy(),
        "xj": arr[:, 16].copy(),
        "xjp": arr[:, 17].copy(),
        "continuum_label": arr[:, 18].astype(np.int32),
        "iso1": arr[:, 19].astype(np.int32),
        "iso2": arr[:, 20].astype(np.int32),
    }


def filter_window(cat: Dict[str, np.ndarray], wl_min: float, wl_max: float) -> Dict[str, np.ndarray]:
    """atomic.py:718-816 DELLIM window (parsed_cache.py:200-229 vectorised form)."""
    delfactor = 1.0 if wl_min <= 500.0 else wl_min / 500.0
    ls = np.where(cat["line_size"] > 0, cat["line_size"], 0)
    lim = np.minimum(8 - ls, 7)
    hmask = (np.abs(cat["code"] - 1.0) <= 1e-6) | np.isin(cat["line_type"], [-1, -2]) | (cat["nelem"] == 1)
    lim = np.clip(np.where(hmask, 1, lim), 1, 7)
    margin = DELLIM[lim - 1] * delfactor
    w = cat["wavelength"]
    keep = (w >= wl_min - margin) & (w <= wl_max + margin)
    return {k: v[keep] for k, v in cat.items()}


def routing(cat: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
    """line_opacity.py:740-784: which records TRANSP processes, element index
    (Z-1 for symbols known to the reference, Z <= 92), gf and CGF."""
    nelem = cat["nelem"]
    lt = cat["line_type"]
    nb = np.abs(cat["n_lower"]) + np.abs(cat["n_upper"])
    fort12 = (lt != 2) & (lt != 1) & (lt <= 3) & (nb == 0)
    is_h = (nelem == 1) & (cat["ion_stage"] == 1)
    known = (nelem >= 1) & (nelem <= 92)
    process = fort12 & ~((lt == -1) | is_h) & known
    element_idx = np.where(known, nelem - 1, -1).astype(np.int32)
    gf = np.power(10.0, cat["log_gf"])
    freq = 2.99792458e17 / cat["wavelength"]
    cgf = (0.026538 / 1.77245) * gf / freq
    # centre adds skip the dedicated non-Voigt classes (line_opacity.py:1094)
    asynth_mask = ~np.isin(lt, [-2, -1, 1, 2, 3, 4])
    return {
        "process_mask": process.astype(np.uint8),
        "element_idx": element_idx,
        "gf": gf,
        "cgf": cgf,
        "asynth_mask": asynth_mask.astype(np.uint8),
    }
