"""CPU restatement of the reference's helium wing pass -- test infrastructure.

Only ``tests/`` use this module, to check the GPU helium-line kernels.

The reference adds, for every helium line of the catalog (line types -3, -4
and -6: He I, 3He I, He II), a Voigt wing computed apart from ASYNTH to the
line opacity:

* the helium-only pass of ``run_synthesis`` (synthe_py/engine/opacity.py:
  3550-3590) calls ``process_depth`` (:2640) per layer for the helium lines
  (:2531-2544, catalog order);
* per (line, layer) the gates of :2705-2910 -- centre bin inside the grid,
  population and Doppler velocity of the line's ion (:2815-2850), XNFDOP,
  the two KAPMIN tests on CGF*XNFDOP and on it times the Boltzmann factor
  (:2885-2905); no continuum-merge limits for lines without fort.19 metadata
  (:2760-2770, :657-702 with NCON = 0);
* the wing itself, ``_apply_fort19_profile`` (:966-1061) for TYPE < -2: a
  Voigt profile H(|lambda - lambda0| / DOPPLER, a) walked red from the centre
  bin (cutoff tested before adding) and blue from the bin below it (added,
  then tested), 3He with kappa / 1.155 and DOPPLER x 1.155;
* the layer's sum AHE (:3586) enters the line opacity as AHE x STIM
  (:3650-3660), STIM = 1 - exp(-nu h / kT) (:2215-2224).
"""

from __future__ import annotations

from typing import Dict

import numpy as np

from . import hydrogen, oracle

C_LIGHT_NM = 2.99792458e17
C_LIGHT_CM = 2.99792458e10
CGF_CONSTANT = 0.026538 / 1.77245
H_PLANCK = 6.62607015e-27
K_BOLTZ = 1.380649e-16
HELIUM_TYPES = (-3, -4, -6)


def helium_rows(cat: Dict[str, np.ndarray]) -> np.ndarray:
    """Catalog rows the helium pass takes (engine/opacity.py:2531-2544)."""
    return np.flatnonzero(np.isin(np.asarray(cat["line_type"]), HELIUM_TYPES))


def wings(cat: Dict[str, np.ndarray], atm: Dict[str, np.ndarray], grid: np.ndarray,
          continuum: np.ndarray, cutoff: float = 1e-3) -> np.ndarray:
    """AHE [L, N] before STIM.  ``cat``: wavelength, gf, elo, gamma_rad,
    gamma_stark, gamma_vdw, ion_stage, line_type and the centre bins
    (``center``); ``continuum``: ABTOT = ACONT + SIGMAC [L, N]."""
    tb = oracle.tables()
    L, N = continuum.shape
    out = np.zeros((L, N))
    pop = np.asarray(atm["population_per_ion"])
    dop = np.asarray(atm["doppler_per_ion"])
    rho = np.asarray(atm["mass_density"])
    xne = np.asarray(atm["electron_density"])
    hckt = np.asarray(atm["hckt"])
    txn = oracle.txnxn(atm)
    rows = helium_rows(cat)
    from . import fort19
    contx = fort19.contx_table()
    nmerge = np.maximum(1600.0 / np.power(np.maximum(xne, 1e-40), 2.0 / 15.0) - 1.5, 1.0)
    emerge = 109737.312 / np.maximum(nmerge ** 2, 1e-12)
    emerge_h = 109677.576 / np.maximum(nmerge ** 2, 1e-12)
    for d in range(L):
        local = np.zeros(N)
        for i in rows:
            ci = int(cat["center"][i])
            if ci < 0 or ci >= N:
                continue
            nelion = int(cat["ion_stage"][i])
            if nelion > pop.shape[1] or nelion < 1:
                continue
            pv = float(pop[d, nelion - 1, 1])
            dv = float(dop[d, nelion - 1, 1])
            if pv <= 0.0 or dv <= 0.0:
                continue
            r = float(rho[d])
            if not r > 0.0:
                continue
            xnfdop = pv / (r * dv)
            wl = float(cat["wavelength"][i])
            dw = dv * wl
            boltz = hydrogen.fast_ex(float(cat["elo"][i]) * float(hckt[d]))
            cgf = CGF_CONSTANT * float(cat["gf"][i]) / (C_LIGHT_NM / wl)
            kmin = float(continuum[d, max(0, min(ci, N - 1))]) * cutoff
            k0pre = cgf * xnfdop
            if k0pre < kmin or dw <= 0.0:
                continue
            k0 = k0pre * boltz
            if k0 < kmin:
                continue
            doppler = max(dw, 1e-12)
            keff = k0
            if int(cat["line_type"][i]) == -4:
                keff /= 1.155
                doppler *= 1.155
            dn = (float(cat["gamma_rad"][i]) + float(cat["gamma_stark"][i]) * float(xne[d])
                  + float(cat["gamma_vdw"][i]) * float(txn[d])) / max(doppler / wl, 1e-40)
            a = max(dn, 1e-12)
            # continuum-merge limits: only fort.19 records (NBLO/NBUP set) carry them
            wcon = wtail = None
            if "n_lower" in cat and (abs(int(cat["n_lower"][i])) + abs(int(cat["n_upper"][i]))) != 0:
                nc, nx = fort19.merge_index(cat, i)
                if nc > 0 and nx > 0:
                    wcon, wtail = fort19.continuum_limits(nc, nelion, nx, float(emerge[d]), float(emerge_h[d]),
                                                          contx)
            base = wcon if wcon is not None else wl

            def val(b):
                v = keff * oracle.voigt(abs(grid[b] - wl) / doppler, a, tb)
                if wtail is not None and grid[b] < wtail:
                    v = v * (grid[b] - base) / max(wtail - base, 1e-12)
                return v

            tmp = np.zeros(N)
            if wl <= grid[N - 1]:
                for b in range(ci, N):
                    if wcon is not None and grid[b] <= wcon:
                        continue
                    v = val(b)
                    if v < continuum[d, b] * cutoff:
                        break
                    tmp[b] += v
            if ci > 0 and wl >= grid[0]:
                for b in range(ci - 1, -1, -1):
                    if wcon is not None and grid[b] <= wcon:
                        break
                    v = val(b)
                    tmp[b] += v
                    if v < continuum[d, b] * cutoff:
                        break
            local += tmp
        out[d] += local
    return out


def stim(atm: Dict[str, np.ndarray], grid: np.ndarray) -> np.ndarray:
    """STIM [L, N] of engine/opacity.py:2215-2224."""
    freq = C_LIGHT_CM / (grid * 1e-7)
    hkt = H_PLANCK / (K_BOLTZ * np.asarray(atm["temperature"]))
    return 1.0 - np.exp(-freq[None, :] * hkt[:, None])


def line_opacity(cat: Dict[str, np.ndarray], atm: Dict[str, np.ndarray], grid: np.ndarray,
                 continuum: np.ndarray, cutoff: float = 1e-3) -> np.ndarray:
    """AHE x STIM [L, N], the term the helium lines add to the line opacity."""
    return wings(cat, atm, grid, continuum, cutoff) * stim(atm, grid)


__all__ = ["helium_rows", "wings", "stim", "line_opacity"]
