"""Hydrogen line opacity, restated in Python -- test infrastructure.

Only ``tests/`` use this module, to check the CUDA hydrogen-line kernels; it is
never part of the product.  It restates, step by step:

* the hydrogen depth state (``synthe_py/physics/populations.py:93-125`` and the
  H Doppler width of ``:183-216``);
* the HPROF4 profile ``hydrogen_line_profile``
  (``synthe_py/physics/profiles/hydrogen.py:1541-1710``) with SOFBETA
  (``:1451``), VCSE1F (``:1408``), the fine-structure components (``:1516``),
  HFNM (``:1499``), the Lyman-alpha Lorentz wing (``:1731``) and the
  quasi-static cutoff (``:1800``);
* the wing march ``_accumulate_hydrogen_profile``
  (``synthe_py/engine/opacity.py:1547-1703``) and its driver
  ``_compute_hydrogen_line_opacity`` (``:1706-1884``).

FP64, in the reference's operation order; the tables come from
``data/hydrogen_tables.npz`` (extracted from the reference by
``tests/golden/make_tables.py``).
"""

from __future__ import annotations

import math
from functools import lru_cache
from pathlib import Path

import numpy as np

TABLES = Path(__file__).resolve().parents[1] / "kurucz_py_joss_submission_gb300" / "data" / "hydrogen_tables.npz"

RYDH = 3.2880515e15
C_LIGHT = 2.99792458e18
C_LIGHT_CM = 2.99792458e10
C_LIGHT_NM = 2.99792458e17
C_LIGHT_KMS = 299_792.458
LYMAN_ALPHA_CENTER_WN = 82259.10
HYD_RYD_CM = 109677.576
HYD_EINF_CM = 109678.764
CGF_CONSTANT = 0.026538 / 1.77245
KBOLTZ = 1.380649e-16
AMU = 1.66054e-24
H_PLANCK = 6.62607015e-27
NM_TO_CM = 1e-7


@lru_cache(maxsize=1)
def tables():
    with np.load(TABLES) as d:
        return {k: np.asarray(d[k]) for k in d.files}


@lru_cache(maxsize=1)
def _exp_tables():
    idx = np.arange(1001, dtype=np.float64)
    return np.exp(-idx), np.exp(-idx * 0.001)


def fast_ex(x: float) -> float:
    """FASTEX (synthe_py/physics/tables.py:30-44)."""
    if x <= 0.0:
        return 1.0 if x == 0.0 else math.exp(-x)
    i = int(math.floor(x))
    extab, extabf = _exp_tables()
    if i >= extab.size:
        return math.exp(-x)
    j = int((x - i) * 1000.0 + 0.5)
    j = max(0, min(j, extabf.size - 1))
    return float(extab[i] * extabf[j])


def hydrogen_state(temperature: float, xne_raw: float, xnf_he1: float, xnf_h2: float, xnfph0: float,
                   xnfph1: float, dopph: float) -> dict:
    """populations.py:93-125 (temperature already clamped at 1 K)."""
    xne = max(xne_raw, 1e-40)
    xne16 = xne ** (1.0 / 6.0)
    pp = xne16 * 0.08989 / math.sqrt(max(temperature, 1.0))
    fo = (xne16 ** 4) * 1.25e-9
    y1b = 2.0 / (1.0 + 0.012 / max(temperature, 1.0) * math.sqrt(xne / max(temperature, 1.0)))
    t4 = temperature / 10000.0
    t43 = t4 ** 0.3
    return dict(pp=pp, fo=fo, y1b=y1b, y1s=t43 / xne16, t3nhe=t43 * xnf_he1, t3nh2=t43 * xnf_h2,
                c1d=fo * 78940.0 / max(temperature, 1.0), c2d=(fo ** 2) / 5.96e-23 / xne,
                gcon1=0.2 + 0.09 * math.sqrt(max(t4, 1e-12)) / (1.0 + xne / 1.0e13),
                gcon2=0.2 / (1.0 + xne / 1.0e15), xnfph=(xnfph0, xnfph1), dopph=dopph, xne=xne_raw)


def dopph(temperature: float, vturb_cms: float, microturb_kms: float) -> float:
    """H Doppler width over c (populations.py:183-216), temperature clamped at 1 K."""
    vturb = (vturb_cms / 1e5) / C_LIGHT_KMS
    micro = microturb_kms / C_LIGHT_KMS if microturb_kms > 0 else 0.0
    total = math.sqrt(vturb * vturb + micro * micro)
    thermal = math.sqrt(2.0 * KBOLTZ * temperature / (1.008 * AMU)) / C_LIGHT_CM
    return math.sqrt(thermal * thermal + total * total)


def vcse1f(x: float) -> float:
    if x <= 0:
        return 0.0
    if x <= 0.01:
        return -math.log(x) - 0.577215 + x
    if x <= 1.0:
        return (-math.log(x) - 0.57721566
                + x * (0.99999193 + x * (-0.24991055 + x * (0.05519968 + x * (-0.00976004 + x * 0.00107857)))))
    if x > 30.0:
        return 0.0
    return (x * (x + 2.334733) + 0.25062) / ((x * (x + 3.330657) + 1.681534) * x) * fast_ex(x)


def sofbeta(beta: float, p: float, n: int, m: int) -> float:
    t = tables()
    corr = 1.0
    b2 = beta * beta
    sb = math.sqrt(beta)
    if beta <= 500.0:
        indx = 7
        mmn = m - n
        if n <= 3 and mmn <= 2:
            indx = 2 * (n - 1) + mmn
        indx = max(1, min(indx, 7))
        im = max(min(int(5.0 * p) + 1, 4), 1)
        ip = im + 1
        wtp = max(0.0, min(1.0, 5.0 * (p - t["pp"][im - 1])))
        wtm = 1.0 - wtp
        if beta <= 25.12:
            bg = t["beta"]
            j = int(np.searchsorted(bg, beta, side="right"))
            j = max(1, min(j, bg.size - 1))
            jm, jp = j - 1, j
            denom = bg[jp] - bg[jm]
            wtb = 0.0 if denom <= 0 else (beta - bg[jm]) / denom
            wtbm = 1.0 - wtb
            prop = t["propbm"][indx - 1]
            cbp = prop[ip - 1, jp] * wtp + prop[im - 1, jp] * wtm
            cbm = prop[ip - 1, jm] * wtp + prop[im - 1, jm] * wtm
            corr = 1.0 + cbp * wtb + cbm * wtbm
            pr1 = pr2 = 0.0
            wt = max(min(0.5 * (10.0 - beta), 1.0), 0.0)
            if beta <= 10.0:
                pr1 = 8.0 / (83.0 + (2.0 + 0.95 * b2) * beta)
            if beta >= 8.0:
                pr2 = (1.5 / sb + 27.0 / b2) / b2
            return (pr1 * wt + pr2 * (1.0 - wt)) * corr
        cc = t["c"][im - 1, indx - 1] * wtp + t["c"][ip - 1, indx - 1] * wtm
        dd = t["d"][im - 1, indx - 1] * wtp + t["d"][ip - 1, indx - 1] * wtm
        corr = 1.0 + dd / (cc + beta * sb)
    return (1.5 / sb + 27.0 / b2) / b2 * corr


def hf_nm(n: int, m: int) -> float:
    if m <= n:
        return 0.0
    xn = float(n)
    ginf = 0.2027 / xn ** 0.71
    gca = 0.124 / xn
    fkn = xn * 1.9603
    wtc = 0.45 - 2.4 / xn ** 3 * (xn - 1.0)
    xm = float(m)
    xmn = xm - xn
    fk = fkn * (xm / (xmn * (xm + xn))) ** 3
    xmn12 = xmn ** 1.2
    wt = (xmn12 - 1.0) / (xmn12 + wtc)
    return fk * (1.0 - wt * ginf - (0.222 + gca / xm) * (1.0 - wt))


def fine_structure(n: int, m: int):
    t = tables()
    mmn = m - n
    xn2 = float(n) * float(n)
    if n > 4 or m > 10:
        return [0.0], [1.0]
    if mmn != 1:
        k = int(t["lncomp"][n - 1])
        return list(t["stcomp"][:k, n - 1] * 1.0e7), list(t["stcpwt"][:k, n - 1] / xn2)
    k = int(t["lnghal"][n - 1])
    i0 = int(t["istal"][n - 1])
    return list(t["stalph"][i0:i0 + k] * 1.0e7), list(t["stwtal"][i0:i0 + k] / xn2 / 3.0)


def _interp_cutoff(dwn: float, table: np.ndarray, start: float, step: float):
    if dwn > start + step * (table.size - 1):
        return None
    if dwn <= start:
        return table[0] + (table[1] - table[0]) * ((dwn - start) / step)
    pos = (dwn - start) / step
    i = int(math.floor(pos))
    frac = pos - i
    if i >= table.size - 1:
        return float(table[-1])
    return float(table[i] + (table[i + 1] - table[i]) * frac)


def _lyman_alpha_lorentz(freq, freqnm, del_freq, dop, hwres, hwvdw, hwrad, hyd):
    if dop <= 0.0:
        return 0.0
    hwres_near = hwres * 4.0
    hwlor_near = hwres_near + hwvdw + hwrad
    hhw_near = freqnm * max(hwlor_near, 0.0)
    wn = freq / C_LIGHT_CM
    dwn = wn - LYMAN_ALPHA_CENTER_WN
    if freq > (LYMAN_ALPHA_CENTER_WN - 4000.0) * C_LIGHT_CM and hhw_near > 0.0:
        hres = hwres_near * freqnm / math.pi / (del_freq * del_freq + hhw_near * hhw_near) * 1.77245 * dop
        hhw = hhw_near
    else:
        cut = 0.0
        lg = _interp_cutoff(dwn, tables()["cutoff_h2"], -22000.0, 200.0)
        if lg is not None:
            cut = (10.0 ** (lg - 14.0)) * hyd["xnfph"][0] * 2.0 / C_LIGHT_CM
        hres = cut * 1.77245 * dop
        hhw = freqnm * max(hwres + hwvdw + hwrad, 0.0)
    hrad = 0.0
    if hwrad > 0.0 and hhw > 0.0 and 2.4190611e15 < freq < 0.77 * RYDH:
        hrad = hwrad * freqnm / math.pi / (del_freq * del_freq + hhw * hhw) * 1.77245 * dop
    hvdw = 0.0
    if hwvdw > 0.0 and hhw > 0.0 and freq >= 1.8e15:
        hvdw = hwvdw * freqnm / math.pi / (del_freq * del_freq + hhw * hhw) * 1.77245 * dop
    return hres + hrad + hvdw


def _lyman_qs_cutoff(freq, prqs, hyd, dbeta, dop, n, m):
    if hyd["fo"] <= 0.0:
        return 0.0
    dwn = freq / C_LIGHT_CM - LYMAN_ALPHA_CENTER_WN
    if dwn < -20000.0:
        return 0.0
    extra = 0.0
    if dwn <= -4000.0:
        lg = _interp_cutoff(dwn, tables()["cutoff_h2_plus"], -15000.0, 100.0)
        if lg is not None:
            extra += (10.0 ** (lg - 14.0)) * hyd["xnfph"][1] / C_LIGHT_CM * 1.77245 * dop
    else:
        beta4000 = 4000.0 * C_LIGHT_CM / max(hyd["fo"], 1e-30) * dbeta
        prqs4000 = sofbeta(beta4000, hyd["pp"], n, m) * 0.5
        norm = prqs4000 / max(hyd["fo"], 1e-30) * dbeta
        cut4000 = (10.0 ** (-11.07 - 14.0)) * hyd["xnfph"][1] / C_LIGHT_CM
        if norm > 0.0:
            extra += cut4000 / norm * (prqs / max(hyd["fo"], 1e-30) * dbeta) * 1.77245 * dop
    return extra


def profile(n: int, m: int, hyd: dict, dlam_nm: float) -> float:
    """HPROF4 (profiles/hydrogen.py:1541-1710)."""
    t = tables()
    mmn = m - n
    xn, xm = float(n), float(m)
    xn2, xm2 = xn * xn, xm * xm
    xm2mn2 = xm2 - xn2
    xmn2 = xm2 * xn2
    gnm = xm2mn2 / xmn2
    if mmn <= 0:
        return 0.0
    if mmn <= 3 and n <= 4:
        xknm = t["xknmtb"][n - 1, mmn - 1]
    else:
        xknm = 5.5e-5 / gnm * xmn2 / (1.0 + 0.13 / mmn)
    freqnm = RYDH * gnm
    wavenm = C_LIGHT / freqnm
    dbeta = C_LIGHT / (freqnm * freqnm * xknm)
    c1con = xknm / wavenm * gnm * xm2mn2
    c2con = (xknm / wavenm) ** 2
    radamp = t["asum"][n - 1] + t["asum"][m - 1]
    if n == 1:
        radamp = t["asum_lyman"][m - 1]
    radamp /= 12.5664
    radamp /= freqnm
    resont = hf_nm(1, m) / xm / (1.0 - 1.0 / xm2)
    if n != 1:
        resont += hf_nm(1, n) / xn / (1.0 - 1.0 / xn2)
    resont *= 3.579e-24 / gnm
    vdw = 4.45e-26 / gnm * (xm2 * (7.0 * xm2 + 5.0)) ** 0.4
    hwvdw = vdw * hyd["t3nhe"] + 2.0 * vdw * hyd["t3nh2"]
    hwrad = radamp
    stark = 1.6678e-18 * freqnm * xknm
    hwres = resont * hyd["xnfph"][0] * 2.0
    hwstk = stark * hyd["fo"]
    hwlor = hwres + hwvdw + hwrad
    finest, finswt = fine_structure(n, m)
    wl = wavenm + dlam_nm * 10.0
    freq = C_LIGHT / wl
    del_freq = abs(freq - freqnm)
    dph = max(hyd["dopph"], 1e-40)
    dop = freqnm * dph
    hfwidth = freqnm * max(dph, hwlor, hwstk)
    ifcore = del_freq <= hfwidth
    nwid = 1
    if not (dph >= hwstk and dph >= hwlor):
        nwid = 2
        if hwlor < hwstk:
            nwid = 3
    core = 0.0
    for off, w in zip(finest, finswt):
        d = abs(freq - (freqnm + off)) / max(dop, 1e-30)
        if d <= 7.0:
            core += fast_ex(d * d) * w
    lorentz = 0.0
    hhw = freqnm * hwlor
    if n == 1 and m == 2:
        lorentz = _lyman_alpha_lorentz(freq, freqnm, del_freq, dop, hwres, hwvdw, hwrad, hyd)
    else:
        top = hhw
        if n == 1 and m in (3, 4, 5):
            fr = freq / RYDH
            if (m == 3 and 0.885 <= fr <= 0.890) or (m == 4 and 0.936 <= fr <= 0.938) or \
                    (m == 5 and 0.959 <= fr <= 0.961):
                top = max(hhw - freqnm * hwrad, 0.0)
        if hhw > 0.0:
            lorentz = top / math.pi / (del_freq * del_freq + hhw * hhw) * 1.77245 * dop
    y1num = 550.0 if m == 2 else (380.0 if m == 3 else 320.0)
    y1wht = 1.0e14 if mmn <= 3 else 1.0e13
    if mmn <= 2 and n <= 2:
        y1wht = t["y1wtm"][n - 1, mmn - 1]
    wty1 = 1.0 / (1.0 + max(hyd["xne"], 0.0) / max(y1wht, 1e-30))
    y1_scal = y1num * hyd["y1s"] * wty1 + hyd["y1b"] * (1.0 - wty1)
    c1 = hyd["c1d"] * c1con * y1_scal
    c2 = hyd["c2d"] * c2con
    beta = del_freq / max(hyd["fo"], 1e-30) * dbeta
    y1 = c1 * beta
    y2 = c2 * beta * beta
    g1 = 6.77 * math.sqrt(max(c1, 1e-30))
    ratio = math.sqrt(c2) / max(c1, 1e-30) if (c1 > 0.0 and c2 > 0.0) else 0.0
    log_term = math.log(max(ratio, 1e-30)) if ratio > 0.0 else 0.0
    gamma = g1 * max(0.0, 0.2114 + log_term) * (1.0 - hyd["gcon1"] - hyd["gcon2"])
    if y2 > 1e-4 and y1 > 1e-5:
        gamma = (g1 * (0.5 * fast_ex(min(80.0, y1)) + vcse1f(y1) - 0.5 * vcse1f(y2))
                 * (1.0 - hyd["gcon1"] / (1.0 + (90.0 * y1) ** 3) - hyd["gcon2"] / (1.0 + 2000.0 * y1)))
    f = gamma / math.pi / (gamma * gamma + beta * beta) if gamma > 0 else 0.0
    prqs = sofbeta(beta, hyd["pp"], n, m)
    extra = 0.0
    if m <= 2:
        prqs *= 0.5
        extra = _lyman_qs_cutoff(freq, prqs, hyd, dbeta, dop, n, m)
    p1 = (0.9 * y1) ** 2
    fns = (p1 + 0.03 * math.sqrt(max(y1, 0.0))) / (p1 + 1.0)
    stark_core = (prqs * (1.0 + fns) + f) / max(hyd["fo"], 1e-30) * dbeta * 1.77245 * dop
    if ifcore:
        if nwid == 1:
            return max(core, 0.0)
        if nwid == 2:
            return max(lorentz, 0.0)
        return max(stark_core + extra, 0.0)
    return max(core + lorentz + stark_core + extra, 0.0)


def _ehyd(n: int) -> float:
    e = tables()["ehyd"]
    return float(e[n - 1]) if 1 <= n <= e.size else HYD_EINF_CM - HYD_RYD_CM / float(n * n)


def _march(buf, cont_row, stim_row, grid, ci, wl0, kappa0, hyd, nl, nu, wcon, wtail, wlm1, wlm2, wlp1,
           wlp2, redcut, bluecut, cutoff):
    """_accumulate_hydrogen_profile (engine/opacity.py:1547-1703)."""
    npt = buf.size
    simple = nu <= nl + 2
    taper = (not simple) and (wtail > wcon)
    um2 = max(nu - 2, nl + 1)
    up2 = nu + 2
    red = blue = True
    offset = 1
    max_steps = max(ci, npt - ci - 1)
    if 0 <= ci < npt:
        wc = grid[ci]
        if simple or not (wc < wcon):
            v = kappa0 * profile(nl, nu, hyd, wc - wl0) * stim_row[ci]
            if taper and wc < wtail:
                v *= (wc - wcon) / (wtail - wcon)
            if v >= cont_row[ci] * cutoff:
                buf[ci] += v
    elif ci >= npt:
        red = False
        offset = max(1, ci - (npt - 1))
    else:
        blue = False
        offset = max(1, -ci)
    while offset <= max_steps and (red or blue):
        if red:
            idx = ci + offset
            if idx >= npt:
                red = False
            else:
                w = grid[idx]
                if not simple:
                    if w > wlm1:
                        red = False
                    elif w < wcon:
                        pass
                    else:
                        v = kappa0 * profile(nl, nu, hyd, w - wl0) * stim_row[idx]
                        if taper and w < wtail:
                            v *= (w - wcon) / (wtail - wcon)
                        if w > redcut:
                            v2 = kappa0 * profile(nl, um2, hyd, w - wlm2) * stim_row[idx]
                            if taper and w < wtail:
                                v2 *= (w - wcon) / (wtail - wcon)
                            if v2 >= v:
                                red = False
                                v = 0.0
                        if v <= 0.0 or v < cont_row[idx] * cutoff:
                            red = False
                        else:
                            buf[idx] += v
                else:
                    v = kappa0 * profile(nl, nu, hyd, w - wl0) * stim_row[idx]
                    if v <= 0.0 or v < cont_row[idx] * cutoff:
                        red = False
                    else:
                        buf[idx] += v
        if blue:
            idx = ci - offset
            if idx < 0:
                blue = False
            else:
                w = grid[idx]
                if not simple and (w < wcon or w < wlp1):
                    blue = False
                else:
                    v = kappa0 * profile(nl, nu, hyd, w - wl0) * stim_row[idx]
                    if not simple:
                        if taper and w < wtail:
                            v *= (w - wcon) / (wtail - wcon)
                        if w < bluecut:
                            v2 = kappa0 * profile(nl, up2, hyd, w - wlp2) * stim_row[idx]
                            if taper and w < wtail:
                                v2 *= (w - wcon) / (wtail - wcon)
                            if v2 >= v:
                                blue = False
                                v = 0.0
                    if v <= 0.0 or v < cont_row[idx] * cutoff:
                        blue = False
                    else:
                        buf[idx] += v
        offset += 1


def line_opacity(cat: dict, atm: dict, grid: np.ndarray, continuum: np.ndarray, cutoff: float = 1e-3,
                 microturb_kms: float = 0.0) -> np.ndarray:
    """AHLINE [L, N] of the catalog's hydrogen lines (engine/opacity.py:1706-1884).

    ``cat``: wavelength, gf, elo (cm^-1), n_lower, n_upper, line_type, ion_stage,
    centre bins (``center``); ``continuum``: ABTOT = ACONT + SIGMAC [L, N]."""
    t = tables()
    conth = t["conth"]
    L, N = continuum.shape
    out = np.zeros((L, N))
    T = atm["temperature"]
    pop = atm["population_per_ion"][:, 0, 0]
    dopv = atm["doppler_per_ion"][:, 0, 0]
    rho = atm["mass_density"]
    xne = np.maximum(atm["electron_density"], 1e-40)
    inglis = 1600.0 / np.power(xne, 2.0 / 15.0)
    nmerge = np.maximum(inglis - 1.5, 1.0)
    emerge = HYD_RYD_CM / np.maximum(nmerge * nmerge, 1e-12)
    micro = microturb_kms / C_LIGHT_KMS if microturb_kms > 0.0 else 0.0
    freq = C_LIGHT_CM / (grid * NM_TO_CM)
    hkt = H_PLANCK / (KBOLTZ * T)
    stim = 1.0 - np.exp(-freq[None, :] * hkt[:, None])
    states = []
    for d in range(L):
        temp = max(float(T[d]), 1.0)
        states.append(hydrogen_state(temp, float(atm["electron_density"][d]), float(atm["xnf_he1"][d]),
                                     float(atm["xnf_h2"][d]), float(atm["population_per_ion"][d, 0, 0]),
                                     float(atm["population_per_ion"][d, 1, 0]),
                                     dopph(temp, float(atm["turbulent_velocity"][d]), microturb_kms)))
    extab, extabf = _exp_tables()
    for i in range(len(cat["wavelength"])):
        if int(cat["line_type"][i]) not in (-1, -2) or int(cat["ion_stage"][i]) != 1:
            continue
        wl0 = float(cat["wavelength"][i])
        ci = int(cat["center"][i])
        cgf = CGF_CONSTANT * float(cat["gf"][i]) / (C_LIGHT_NM / wl0)
        nl = int(cat["n_lower"][i])
        nu = int(cat["n_upper"][i])
        conth_val = float(conth[max(1, min(nl, conth.size)) - 1])
        nl_e = max(nl, 1)
        nu_e = max(nu, nl + 1)
        elo = _ehyd(nl)
        wlm1 = 1.0e7 / (_ehyd(nu - 1) - elo) if nu - 1 > nl else wl0
        wlm2 = 1.0e7 / (_ehyd(nu - 2) - elo) if nu - 2 > nl else wl0
        wlp1 = 1.0e7 / (_ehyd(nu + 1) - elo)
        wlp2 = 1.0e7 / (_ehyd(nu + 2) - elo)
        redcut = 1.0e7 / (conth[0] - HYD_RYD_CM / (float(nu) - 0.8) ** 2 - elo)
        bluecut = 1.0e7 / (conth[0] - HYD_RYD_CM / (float(nu) + 0.8) ** 2 - elo)
        cc = max(0, min(ci, N - 1))
        wshift = 1.0e7 / (conth_val - HYD_RYD_CM / 81.0 ** 2)
        for d in range(L):
            pv, dv = float(pop[d]), float(dopv[d])
            if micro > 0.0:
                dv = math.sqrt(dv * dv + micro * micro)
            r = float(rho[d])
            if pv <= 0.0 or dv <= 0.0 or r <= 0.0:
                continue
            k0pre = cgf * (pv / (r * dv))
            kapmin = continuum[d, cc] * cutoff
            if k0pre < kapmin:
                continue
            x = float(cat["elo"][i]) * float(atm["hckt"][d])
            k0 = k0pre * fast_ex(x)
            if k0 < kapmin:
                continue
            wmerge = 1.0e7 / (conth_val - emerge[d])
            if wmerge < 0.0:
                wmerge = wshift + wshift
            wcon = max(wshift, wmerge)
            wtail = 1.0e7 / (1.0e7 / wcon - 500.0) if wcon > 0.0 else wcon + wcon
            wcon = min(wshift + wshift, wcon)
            if wtail < 0.0:
                wtail = wcon + wcon
            wtail = min(wcon + wcon, wtail)
            _march(out[d], continuum[d], stim[d], grid, ci, wl0, k0, states[d], nl_e, nu_e, wcon, wtail,
                   wlm1, wlm2, wlp1, wlp2, redcut, bluecut, cutoff)
    return out
