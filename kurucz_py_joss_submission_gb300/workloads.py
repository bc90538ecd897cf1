"""Seeded synthetic inputs in the reference's own file formats.

Two generators:

* :func:`grey_atmosphere_atm` writes an ATLAS-format ``.atm`` model (header
  ``TEFF … GRAVITY …``, ``ABUNDANCE SCALE/CHANGE`` cards and a
  ``READ DECK6 n RHOX,T,P,XNE,ABROSS,ACCRAD,VTURB`` block) for a grey
  atmosphere, T^4 = 3/4 Teff^4 (tau + 2/3), in hydrostatic equilibrium.
  The reader it must satisfy is ``synthe_py/tools/convert_atm_to_npz.py:190``
  (``parse_atm_file``).
* :func:`random_atomic_lines` draws a line list and :func:`format_gfall`
  writes it in the fixed-width gfall layout parsed by
  ``synthe_py/io/lines/atomic.py:299`` (``load_catalog``, columns at
  ``:332-348``).  The parser re-derives the wavelength from the two level
  energies (``atomic.py:444-457``), so the upper energy is written as
  ``EP = E + 1e7/lambda``; the effective vacuum wavelength is then
  ``1e7/(EP-E)`` after the F12.3 rounding of both energies.

All randomness comes from ``numpy.random.default_rng(seed)``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from pathlib import Path
from typing import Dict, Optional, Sequence

import numpy as np

# ATLAS12 solar abundance scale: log10(N_el / N_total) for Z = 3..99 (the
# H and He number fractions are written separately).  This is the
# composition the reference's sample models use.
_SOLAR_LOG_ABUND = {
    3: -13.24, 4: -12.91, 5: -11.59, 6: -5.86, 7: -6.46, 8: -5.80, 9: -9.73,
    10: -6.56, 11: -8.05, 12: -6.89, 13: -7.84, 14: -6.98, 15: -8.88,
    16: -7.37, 17: -8.79, 18: -7.89, 19: -9.26, 20: -8.15, 21: -11.14,
    22: -9.54, 23: -10.36, 24: -8.65, 25: -8.86, 26: -6.79, 27: -9.30,
    28: -8.07, 29: -10.10, 30: -9.73, 31: -11.25, 32: -10.64, 33: -11.99,
    34: -10.95, 35: -11.75, 36: -11.04, 37: -11.77, 38: -11.42, 39: -12.08,
    40: -11.71, 41: -12.83, 42: -12.41, 43: -22.25, 44: -12.54, 45: -13.38,
    46: -12.72, 47: -13.35, 48: -12.58, 49: -13.49, 50: -12.25, 51: -13.28,
    52: -12.11, 53: -12.74, 54: -12.05, 55: -13.21, 56: -12.11, 57: -13.19,
    58: -12.71, 59: -13.57, 60: -12.87, 61: -22.25, 62: -13.33, 63: -13.77,
    64: -13.22, 65: -13.99, 66: -13.19, 67: -13.81, 68: -13.37, 69: -14.19,
    70: -13.45, 71: -14.19, 72: -13.44, 73: -14.41, 74: -13.44, 75: -14.03,
    76: -12.89, 77: -12.91, 78: -12.67, 79: -13.37, 80: -13.12, 81: -13.39,
    82: -12.54, 83: -13.64, 84: -22.25, 85: -22.25, 86: -22.25, 87: -22.25,
    88: -22.25, 89: -22.25, 90: -14.27, 91: -22.25, 92: -14.83, 93: -22.25,
    94: -22.25, 95: -22.25, 96: -22.25, 97: -22.25, 98: -22.25, 99: -22.25,
}
_H_FRACTION = 0.92163
_HE_FRACTION = 0.07837

_K_BOLTZ = 1.380649e-16
_M_H = 1.6735575e-24


@dataclass(frozen=True)
class GreyAtmosphere:
    """Depth structure of a grey model, surface first."""

    teff: float
    logg: float
    log_tau: np.ndarray
    rhox: np.ndarray
    temperature: np.ndarray
    pressure: np.ndarray
    xne: np.ndarray
    abross: np.ndarray
    vturb_cms: float


def _grey_opacity(p: float, t: float, metal_scale: float) -> float:
    """Rosseland-mean stand-in: H- bound-free/free-free plus e- scattering.

    kappa_H- ~ 2.5e-31 (Z/0.02) rho^0.5 T^9 cm^2/g (3000-6000 K fit), with
    a floor so cool layers stay finite, plus Thomson scattering scaled by
    the hydrogen ionisation fraction.
    """
    mu = 1.3
    rho = p * mu * _M_H / (_K_BOLTZ * t)
    t_eff = min(t, 12000.0)
    kh = 2.5e-31 * metal_scale * math.sqrt(max(rho, 1e-30)) * t_eff ** 9
    x_ion = _hydrogen_ion_fraction(p, t)
    kes = 0.34 * x_ion
    return max(kh + kes, 1e-4)


def _hydrogen_ion_fraction(p: float, t: float) -> float:
    n_tot = p / (_K_BOLTZ * t)
    n_h = n_tot * _H_FRACTION
    s = 2.4147e15 * t ** 1.5 * math.exp(-157807.0 / t)
    # x^2/(1-x) = s/n_h
    r = s / max(n_h, 1e-30)
    return (-r + math.sqrt(r * r + 4.0 * r)) / 2.0


def grey_atmosphere(
    teff: float,
    logg: float,
    log_tau_min: float = -6.875,
    log_tau_max: float = 2.0,
    step: float = 0.125,
    vturb_kms: float = 2.0,
    metallicity: float = 0.0,
) -> GreyAtmosphere:
    """Integrate dP/dtau = g/kappa on the grey T(tau) law."""
    n = int(round((log_tau_max - log_tau_min) / step)) + 1
    log_tau = log_tau_min + step * np.arange(n, dtype=np.float64)
    tau = 10.0 ** log_tau
    temp = (0.75 * teff ** 4 * (tau + 2.0 / 3.0)) ** 0.25
    g = 10.0 ** logg
    metal_scale = 10.0 ** metallicity
    pres = np.zeros(n)
    kap = np.zeros(n)
    # top layer: P = g tau / kappa(P), solved by fixed point
    p = g * tau[0] / 1.0
    for _ in range(200):
        k = _grey_opacity(p, temp[0], metal_scale)
        p_new = g * tau[0] / k
        if abs(p_new - p) <= 1e-12 * p_new:
            p = p_new
            break
        p = math.sqrt(p * p_new)
    pres[0] = p
    kap[0] = _grey_opacity(p, temp[0], metal_scale)
    # march in ln(tau) with a two-stage (Heun) step on dP/dln(tau) = g tau/kappa
    nsub = 8
    for i in range(1, n):
        p = pres[i - 1]
        lt0 = math.log(tau[i - 1])
        lt1 = math.log(tau[i])
        h = (lt1 - lt0) / nsub
        for s in range(nsub):
            lt = lt0 + s * h
            ta = math.exp(lt)
            tb = math.exp(lt + h)
            t_a = (0.75 * teff ** 4 * (ta + 2.0 / 3.0)) ** 0.25
            t_b = (0.75 * teff ** 4 * (tb + 2.0 / 3.0)) ** 0.25
            f_a = g * ta / _grey_opacity(p, t_a, metal_scale)
            p_pred = p + h * f_a
            f_b = g * tb / _grey_opacity(p_pred, t_b, metal_scale)
            p = p + 0.5 * h * (f_a + f_b)
        pres[i] = p
        kap[i] = _grey_opacity(p, temp[i], metal_scale)
    rhox = pres / g
    xne = np.zeros(n)
    metal_donor = 1.0e-4 * metal_scale
    for i in range(n):
        n_tot = pres[i] / (_K_BOLTZ * temp[i])
        x = _hydrogen_ion_fraction(pres[i], temp[i])
        # electrons from hydrogen plus fully ionised low-potential metals
        ne = n_tot * _H_FRACTION * x + n_tot * metal_donor
        xne[i] = ne / (1.0 + ne / n_tot)
    return GreyAtmosphere(
        teff=float(teff), logg=float(logg), log_tau=log_tau, rhox=rhox,
        temperature=temp, pressure=pres, xne=xne, abross=kap,
        vturb_cms=vturb_kms * 1.0e5,
    )


def format_atm(atm: GreyAtmosphere, metallicity: float = 0.0) -> str:
    """Render a :class:`GreyAtmosphere` as ATLAS ``.atm`` text."""
    out = []
    out.append(f"TEFF {atm.teff:7.0f}.  GRAVITY {atm.logg:7.4f} LTE \n")
    out.append("TITLE grey T(tau) model, hydrostatic, synthetic\n")
    out.append(" OPACITY IFOP 1 1 1 1 1 1 1 1 1 1 1 1 1 0 1 0 1 0 0 0\n")
    out.append(" CONVECTION OFF  0.00 TURBULENCE OFF  0.00  0.00  0.00  0.00\n")
    scale = 10.0 ** metallicity
    out.append(
        f"ABUNDANCE SCALE {scale:9.5f} ABUNDANCE CHANGE 1 {_H_FRACTION:.5f} 2 {_HE_FRACTION:.5f}\n"
    )
    zs = sorted(_SOLAR_LOG_ABUND)
    for k in range(0, len(zs), 6):
        chunk = zs[k:k + 6]
        body = "".join(f" {z:2d} {_SOLAR_LOG_ABUND[z]:6.2f}" for z in chunk)
        out.append(" ABUNDANCE CHANGE" + body + "\n")
    n = atm.rhox.size
    out.append(f"READ DECK6 {n} RHOX,T,P,XNE,ABROSS,ACCRAD,VTURB\n")
    for i in range(n):
        out.append(
            f" {atm.rhox[i]:.8E} {atm.temperature[i]:8.1f} {atm.pressure[i]:.3E}"
            f" {atm.xne[i]:.3E} {atm.abross[i]:.3E} {0.0:.3E} {atm.vturb_cms:.3E}\n"
        )
    out.append("PRADK 0.0000E+00\n")
    out.append("BEGIN                    ITERATION   1 COMPLETED\n")
    return "".join(out)


def grey_atmosphere_atm(path: Path, teff: float, logg: float, metallicity: float = 0.0,
                        vturb_kms: float = 2.0, n_layers: int = 72) -> GreyAtmosphere:
    """Write the ``.atm`` of a grey model with ``n_layers`` layers spread evenly
    in log tau over [-6.875, 2.0] (72 layers: the 0.125 step)."""
    step = (2.0 - (-6.875)) / (n_layers - 1)
    atm = grey_atmosphere(teff, logg, step=step, vturb_kms=vturb_kms, metallicity=metallicity)
    Path(path).write_text(format_atm(atm, metallicity))
    return atm


# Species drawn for the atomic line lists: gfall CODE and solar-like weight.
SPECIES_CODES = np.array(
    [26.00, 26.01, 22.00, 22.01, 24.00, 20.00, 20.01, 28.00, 12.00, 14.00]
)
SPECIES_WEIGHTS = np.array(
    [0.40, 0.10, 0.10, 0.05, 0.08, 0.05, 0.02, 0.10, 0.05, 0.05]
)


@dataclass
class LineDraw:
    """Raw draws of a synthetic atomic line list (before gfall rounding)."""

    wavelength_nm: np.ndarray
    log_gf: np.ndarray
    code: np.ndarray
    e_lower_cm: np.ndarray
    log_gamma_rad: np.ndarray
    log_gamma_stark: np.ndarray
    log_gamma_vdw: np.ndarray
    n_lower: Optional[np.ndarray] = None   # NBLO / NBUP of hydrogen lines (None: blank)
    n_upper: Optional[np.ndarray] = None
    tag: Optional[np.ndarray] = None       # columns 142-144 ("AUT": autoionizing; None: blank)
    labelp: Optional[np.ndarray] = None    # upper-level label (None: "SYNTH"; "CONTINUU": merged continuum)
    xjp: Optional[np.ndarray] = None       # upper-level J (None: 2.0)
    iso2: Optional[np.ndarray] = None      # ISO2 (columns 117-119; with ISO1 blank, fort.19's NCON)

    def __len__(self) -> int:
        return int(self.wavelength_nm.size)

    def levels(self):
        n = len(self)
        lo = self.n_lower if self.n_lower is not None else np.zeros(n, np.int32)
        up = self.n_upper if self.n_upper is not None else np.zeros(n, np.int32)
        return np.asarray(lo, np.int32), np.asarray(up, np.int32)


# Hydrogen level energies (cm^-1) of SYNTHE's table (n = 1..8) and log gf of
# the Balmer lines (Kurucz's gfall values for H I 2 -> m).
_EHYD = (0.0, 82259.105, 97492.302, 102823.893, 105291.651, 106632.160, 107440.444, 107965.051)
_BALMER_LOG_GF = {3: 0.710, 4: -0.020, 5: -0.447, 6: -0.753, 7: -0.993, 8: -1.190}


def balmer_lines(upper) -> LineDraw:
    """Hydrogen Balmer lines 2 -> m (m in ``upper``, 3..8) as gfall records with
    NBLO = 2, NBUP = m; the wavelength is the one the level energies give."""
    m = np.asarray(sorted(upper), dtype=np.int32)
    e_lo = np.full(m.size, _EHYD[1])
    e_up = np.array([_EHYD[k - 1] for k in m])
    wl = 1.0e7 / (e_up - e_lo)
    z = np.zeros(m.size)
    return LineDraw(wavelength_nm=wl, log_gf=np.array([_BALMER_LOG_GF[k] for k in m]),
                    code=np.full(m.size, 1.00), e_lower_cm=e_lo, log_gamma_rad=z + 8.76,
                    log_gamma_stark=z - 4.5, log_gamma_vdw=z - 7.5,
                    n_lower=np.full(m.size, 2, np.int32), n_upper=m)


# Helium lines (vacuum wavelength nm, log gf, lower level cm^-1, gfall CODE):
# He I 2p 3P - 4d 3D (447.1 nm air), 2p 1P - 5d 1D (438.8), 2p 3P - 5d 3D
# (402.6), 2p 1P - 4d 1D (492.2), 2s 1S - 3p 1P (501.6) and He II n = 3 - 4
# (468.6 nm air).
_HELIUM_LINES = (
    (447.2735, 0.052, 169086.8, 2.00),
    (438.9166, -0.883, 171134.9, 2.00),
    (402.7328, -0.370, 169086.8, 2.00),
    (492.3304, -0.435, 171134.9, 2.00),
    (501.7077, -0.820, 166277.4, 2.00),
    (468.7087, 1.180, 390140.0, 2.01),
)


def helium_lines(w0: float, w1: float) -> LineDraw:
    """The He I / He II lines of a small table that lie in [w0, w1] nm, as gfall
    records (CODE 2.00 / 2.01, NBLO = NBUP = 0: line types -3 and -6)."""
    rows = [r for r in _HELIUM_LINES if w0 <= r[0] <= w1]
    wl = np.array([r[0] for r in rows], dtype=np.float64)
    z = np.zeros(wl.size)
    return LineDraw(wavelength_nm=wl, log_gf=np.array([r[1] for r in rows], dtype=np.float64),
                    code=np.array([r[3] for r in rows], dtype=np.float64),
                    e_lower_cm=np.array([r[2] for r in rows], dtype=np.float64),
                    log_gamma_rad=z + 8.5, log_gamma_stark=z - 4.2, log_gamma_vdw=z - 7.6)


def random_atomic_lines(
    n_lines: int,
    wl_min: float,
    wl_max: float,
    seed: int,
    log_uniform: bool = False,
) -> LineDraw:
    """Draw ``n_lines`` atomic lines with the distributions of the workloads.

    lambda ~ U(wl_min, wl_max) (or log-uniform), log gf ~ N(-2, 1.5) clipped
    to [-8, 1], E_low ~ U(0, 60000) cm^-1, species from :data:`SPECIES_CODES`,
    log gamma_rad ~ N(8, 0.5), log gamma_Stark ~ N(-5.5, 0.5),
    log gamma_vdW ~ N(-7.5, 0.3).  Lines are returned sorted by wavelength,
    as gfall files are.
    """
    rng = np.random.default_rng(seed)
    if log_uniform:
        wl = np.exp(rng.uniform(math.log(wl_min), math.log(wl_max), n_lines))
    else:
        wl = rng.uniform(wl_min, wl_max, n_lines)
    loggf = np.clip(rng.normal(-2.0, 1.5, n_lines), -8.0, 1.0)
    code = rng.choice(SPECIES_CODES, size=n_lines, p=SPECIES_WEIGHTS / SPECIES_WEIGHTS.sum())
    elo = rng.uniform(0.0, 60000.0, n_lines)
    gr = rng.normal(8.0, 0.5, n_lines)
    gs = rng.normal(-5.5, 0.5, n_lines)
    gw = rng.normal(-7.5, 0.3, n_lines)
    order = np.argsort(wl, kind="stable")
    return LineDraw(
        wavelength_nm=wl[order], log_gf=loggf[order], code=code[order],
        e_lower_cm=elo[order], log_gamma_rad=gr[order],
        log_gamma_stark=gs[order], log_gamma_vdw=gw[order],
    )


# Band lines carry an atomic species code: the synthesis path takes
# populations for Z <= 99 only (line_opacity.py:758-763 maps a record's
# element to its atomic number; records with a molecular code are dropped),
# so molecular-band-like lines are written as Ti I (22.00).
BAND_CODE = 22.00


# sigma_J = sigma_head - BAND_SPACING * B * J^3 (cm^-1): the gap between
# lines J and J + 1 is BAND_SPACING * B * (3 J^2 + 3 J + 1), growing
# quadratically with J (about 0.6 B cm^-1 at J = 30, 13.5 B at J = 150).
BAND_SPACING = 2.0e-4


def band_wavenumbers(sigma_head, b, j):
    """Wavenumbers (cm^-1) of lines J of bands with head ``sigma_head`` and
    rotational constant ``b`` (broadcasting): line spacing quadratic in J."""
    return sigma_head - BAND_SPACING * b * j ** 3


def random_band_lines(n_lines: int, wl_min: float, wl_max: float, seed: int,
                      j_max: int = 150) -> LineDraw:
    """Draw ``n_lines`` lines in molecular-band-like sequences.

    Each band has a head wavelength ~ U(wl_min, wl_max) nm, a rotational
    constant B ~ U(0.3, 2) cm^-1 and lines J = 0..j_max at the wavenumbers
    of :func:`band_wavenumbers` (spacing growing as J^2), lower-level energy
    E = B J (J + 1), log gf ~ N(-4, 1), damping drawn as for the atomic
    lines, species code :data:`BAND_CODE`.  Lines outside [wl_min, wl_max]
    are dropped; bands are drawn until ``n_lines`` lines are kept.  Returned
    sorted by wavelength.
    """
    rng = np.random.default_rng(seed)
    j = np.arange(j_max + 1, dtype=np.float64)
    parts, kept = [], 0
    while kept < n_lines:
        nb = max(64, int(1.3 * (n_lines - kept) / (j_max + 1)) + 1)
        head = rng.uniform(wl_min, wl_max, nb)
        b = rng.uniform(0.3, 2.0, nb)
        sigma = band_wavenumbers((1.0e7 / head)[:, None], b[:, None], j[None, :])
        with np.errstate(divide="ignore"):
            wl = np.where(sigma > 0, 1.0e7 / np.where(sigma > 0, sigma, 1.0), np.inf)
        e = b[:, None] * j[None, :] * (j[None, :] + 1.0)
        ok = (wl >= wl_min) & (wl <= wl_max)
        wl, e = wl[ok], e[ok]
        parts.append((wl, e))
        kept += wl.size
    wl = np.concatenate([p[0] for p in parts])[:n_lines]
    elo = np.concatenate([p[1] for p in parts])[:n_lines]
    n = wl.size
    loggf = np.clip(rng.normal(-4.0, 1.0, n), -8.0, 1.0)
    gr = rng.normal(8.0, 0.5, n)
    gs = rng.normal(-5.5, 0.5, n)
    gw = rng.normal(-7.5, 0.3, n)
    order = np.argsort(wl, kind="stable")
    return LineDraw(
        wavelength_nm=wl[order], log_gf=loggf[order], code=np.full(n, BAND_CODE)[order],
        e_lower_cm=elo[order], log_gamma_rad=gr[order], log_gamma_stark=gs[order],
        log_gamma_vdw=gw[order],
    )


def merge_lines(*draws: LineDraw) -> LineDraw:
    """Concatenate line draws, sorted by wavelength (stable)."""
    tags = None
    if any(d.tag is not None for d in draws):
        tags = np.concatenate([d.tag if d.tag is not None else np.array([""] * len(d), dtype=object)
                               for d in draws]).astype(object)
    cat = {f: np.concatenate([getattr(d, f) for d in draws]) for f in
           ("wavelength_nm", "log_gf", "code", "e_lower_cm", "log_gamma_rad", "log_gamma_stark",
            "log_gamma_vdw")}
    if any(d.n_lower is not None for d in draws):
        cat["n_lower"] = np.concatenate([d.levels()[0] for d in draws])
        cat["n_upper"] = np.concatenate([d.levels()[1] for d in draws])
    if tags is not None:
        cat["tag"] = tags
    if any(d.labelp is not None for d in draws):
        cat["labelp"] = np.concatenate([d.labelp if d.labelp is not None else np.array(["SYNTH"] * len(d), dtype=object)
                                        for d in draws]).astype(object)
    if any(d.iso2 is not None for d in draws):
        cat["iso2"] = np.concatenate([d.iso2 if d.iso2 is not None else np.zeros(len(d), np.int32) for d in draws])
    if any(d.xjp is not None for d in draws):
        cat["xjp"] = np.concatenate([d.xjp if d.xjp is not None else np.full(len(d), 2.0) for d in draws])
    order = np.argsort(cat["wavelength_nm"], kind="stable")
    return LineDraw(**{k: v[order] for k, v in cat.items()})


def _nonzero_f62(x: np.ndarray) -> np.ndarray:
    """Keep damping logs away from the F6.2 value 0.00, which gfall reads as 'absent'."""
    r = np.round(x, 2)
    return np.where(r == 0.0, np.where(x >= 0, 0.01, -0.01), x)


def format_gfall(lines: LineDraw) -> str:
    """Render lines as fixed-width gfall records (160 columns each)."""
    wl = lines.wavelength_nm
    e = np.round(lines.e_lower_cm, 3)
    ep = np.round(e + 1.0e7 / wl, 3)
    gr = _nonzero_f62(lines.log_gamma_rad)
    gs = _nonzero_f62(lines.log_gamma_stark)
    gw = _nonzero_f62(lines.log_gamma_vdw)
    rows = []
    blank_tail = " " * (160 - 98)
    nlo, nup = lines.levels()
    for i in range(len(lines)):
        tail = blank_tail
        if nlo[i] > 0 or nup[i] > 0:
            # REF (4 columns) blank, then NBLO and NBUP (I2 each, columns 103-106)
            tail = f"{'':4s}{nlo[i]:2d}{nup[i]:2d}" + " " * (160 - 106)
        if lines.iso2 is not None and int(lines.iso2[i]) > 0:
            # ISO1 (columns 107-109) blank, ISO2 (I3, columns 117-119)
            tail = tail[:116 - 98] + f"{int(lines.iso2[i]):3d}" + tail[119 - 98:]
        if lines.tag is not None and str(lines.tag[i]).strip():
            # the 3-character tag of columns 142-144 (AUT, COR, PRD)
            tail = tail[:141 - 98] + f"{str(lines.tag[i]):3.3s}" + tail[144 - 98:]
        lp = str(lines.labelp[i]) if lines.labelp is not None and str(lines.labelp[i]) else "SYNTH"
        xjp = float(lines.xjp[i]) if lines.xjp is not None else 2.0
        rows.append(
            f"{wl[i]:11.4f}{lines.log_gf[i]:7.3f}{lines.code[i]:6.2f}{e[i]:12.3f}"
            f"{1.0:5.1f} {'SYNTH   '}{'  '}{ep[i]:12.3f}{xjp:5.1f} {lp:8.8s}{'  '}"
            f"{gr[i]:6.2f}{gs[i]:6.2f}{gw[i]:6.2f}{tail}\n"
        )
    return "".join(rows)


def write_gfall(path: Path, lines: LineDraw) -> None:
    Path(path).write_text(format_gfall(lines))


# The workloads the bench and the tests use, by name.
WORKLOADS: Dict[str, Dict[str, object]] = {
    # 500-510 nm, 20k lines, Teff 5800 log g 4.44 (CPU-runnable reference case)
    "window_500_510": dict(teff=5800.0, logg=4.44, wl_start=500.0, wl_end=510.0,
                           n_lines=20_000, log_uniform=False, seed=20240),
    # full 300-1800 nm, 1.5M lines, same atmosphere (single-GPU headline case)
    "full_300_1800": dict(teff=5800.0, logg=4.44, wl_start=300.0, wl_end=1800.0,
                          n_lines=1_500_000, log_uniform=True, seed=20241),
    # dense stress: Teff 2500 log g -1.0, 300-1800 nm, 1.5M atomic + 8.5M band lines
    "dense_10m": dict(teff=2500.0, logg=-1.0, wl_start=300.0, wl_end=1800.0,
                      n_lines=1_500_000, log_uniform=True, seed=20242,
                      n_band_lines=8_500_000, band_seed=20243),
}
