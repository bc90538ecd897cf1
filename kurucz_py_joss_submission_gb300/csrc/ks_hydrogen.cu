// ks_hydrogen.cu -- the special line classes: hydrogen, helium and fort.19
// line opacity (FP64), added to the line opacity after the accumulation of
// the plain lines.
//
// The reference computes the opacity of the catalog's hydrogen lines (line
// types -1/-2, neutral H) apart from ASYNTH, with Kurucz's HPROF4 profile
// (synthe_py/physics/profiles/hydrogen.py:1541), and adds it to the line
// opacity before the transfer (synthe_py/engine/opacity.py:1706-1884,
// :2465-2503).  Per (line, depth) it walks the grid outward from the line
// centre, red and blue, until the profile falls below the continuum cutoff or
// a cut of the neighbouring series members ends the wing (:1547-1703).
//
// Three kernels, all FP64 with every product and sum rounded separately:
//   hyd_setup_kernel   one thread per (line, depth): the TRANSP-style gates,
//                      kappa0, the merge and tail wavelengths, the line's
//                      series-neighbour wavelengths, the hydrogen depth
//                      state (synthe_py/physics/populations.py:93-125) and
//                      the wavelength-independent part of the line's three
//                      HPROF4 profiles (the line and its two neighbours);
//   hyd_walk_*_kernel  where each (line, depth, side) walk ends: every offset
//                      tested at once, one thread per (walk, offset), the
//                      smallest stopping offset kept by atomicMin, offset
//                      blocks visited in order across all walks so that
//                      ends already found cut the later blocks;
//   hyd_gather_kernel  one thread per (depth, grid point): the contributions
//                      of the lines whose walks cover the point, recomputed
//                      and summed in catalog order (the order of the
//                      reference's buffer), then added to the line opacity.
//
// The helium lines (line types -3/-4/-6) get the reference's helium wing pass
// (synthe_py/engine/opacity.py:2515-3590: per layer and line the TRANSP-style
// gates, then ``_apply_fort19_profile``'s Voigt walk for TYPE < -2, :966-1061)
// and enter the line opacity as AHE x STIM (:3650-3660), with the same three
// kernel shapes (he_setup_kernel, he_walk_*_kernel, he_gather_kernel).
//
// The fort.19 records (NORMAL, autoionizing and merged-continuum lines) enter
// ASYNTH (synthe_py/engine/opacity.py:1388-1486): f19_setup_kernel takes the
// gates, KAPCEN and the continuum-merge limits per (line, depth);
// f19_walk_*_kernel finds where the autoionizing walks and continuum ramps
// end (32 walks per block, only those still running evaluated); and
// f19_gather_kernel sums KAPCEN and the wing steps per (depth, grid point) in
// fort.19 order, with the limits as integer grid bounds.
#include <cuda_runtime.h>

#include <cmath>

#include "ks_common.cuh"
#include "ks_launch.h"

namespace ks {
namespace {

constexpr double kRydH = 3.2880515e15;
constexpr double kClightA = 2.99792458e18;   // Angstrom/s
constexpr double kClightCm = 2.99792458e10;
constexpr double kClightNm = 2.99792458e17;
constexpr double kClightKms = 299792.458;
constexpr double kLyAlphaWn = 82259.10;
constexpr double kHydRyd = 109677.576;
constexpr double kHydEinf = 109678.764;
constexpr double kCgf = 0.026538 / 1.77245;
constexpr double kKboltz = 1.380649e-16;
constexpr double kAmu = 1.66054e-24;
constexpr double kHPlanck = 6.62607015e-27;
constexpr double kPi = 3.141592653589793;

__device__ __forceinline__ double fastex(double x, const double* extab, const double* extabf) {
    if (x <= 0.0) return x == 0.0 ? 1.0 : exp(-x);
    const double fl = floor(x);
    if (fl >= (double)EXP_N) return exp(-x);
    const int i = (int)fl;
    int j = (int)((x - (double)i) * 1000.0 + 0.5);
    j = j < 0 ? 0 : (j > EXP_N - 1 ? EXP_N - 1 : j);
    return extab[i] * extabf[j];
}

__device__ double vcse1f(double x, const double* extab, const double* extabf) {
    if (x <= 0) return 0.0;
    if (x <= 0.01) return -log(x) - 0.577215 + x;
    if (x <= 1.0)
        return -log(x) - 0.57721566 +
               x * (0.99999193 + x * (-0.24991055 + x * (0.05519968 + x * (-0.00976004 + x * 0.00107857))));
    if (x > 30.0) return 0.0;
    return (x * (x + 2.334733) + 0.25062) / ((x * (x + 3.330657) + 1.681534) * x) * fastex(x, extab, extabf);
}

__device__ double sofbeta(double beta, double p, int n, int m, const HydTables& T) {
    double corr = 1.0;
    const double b2 = beta * beta;
    const double sb = sqrt(beta);
    if (beta <= 500.0) {
        int indx = 7;
        const int mmn = m - n;
        if (n <= 3 && mmn <= 2) indx = 2 * (n - 1) + mmn;
        indx = indx < 1 ? 1 : (indx > 7 ? 7 : indx);
        int im = (int)(5.0 * p) + 1;
        im = im > 4 ? 4 : im;
        im = im < 1 ? 1 : im;
        const int ip = im + 1;
        double wtp = 5.0 * (p - T.pp[im - 1]);
        wtp = wtp < 0.0 ? 0.0 : (wtp > 1.0 ? 1.0 : wtp);
        const double wtm = 1.0 - wtp;
        if (beta <= 25.12) {
            // searchsorted(beta grid, beta, side="right")
            int j = 0;
            while (j < 15 && T.beta[j] <= beta) j++;
            j = j < 1 ? 1 : (j > 14 ? 14 : j);
            const int jm = j - 1, jp = j;
            const double denom = T.beta[jp] - T.beta[jm];
            const double wtb = denom <= 0 ? 0.0 : (beta - T.beta[jm]) / denom;
            const double wtbm = 1.0 - wtb;
            const double* prop = T.propbm + (indx - 1) * 5 * 15;
            const double cbp = prop[(ip - 1) * 15 + jp] * wtp + prop[(im - 1) * 15 + jp] * wtm;
            const double cbm = prop[(ip - 1) * 15 + jm] * wtp + prop[(im - 1) * 15 + jm] * wtm;
            corr = 1.0 + cbp * wtb + cbm * wtbm;
            double pr1 = 0.0, pr2 = 0.0;
            double wt = 0.5 * (10.0 - beta);
            wt = wt > 1.0 ? 1.0 : wt;
            wt = wt < 0.0 ? 0.0 : wt;
            if (beta <= 10.0) pr1 = 8.0 / (83.0 + (2.0 + 0.95 * b2) * beta);
            if (beta >= 8.0) pr2 = (1.5 / sb + 27.0 / b2) / b2;
            return (pr1 * wt + pr2 * (1.0 - wt)) * corr;
        }
        const double cc = T.c[(im - 1) * 7 + indx - 1] * wtp + T.c[(ip - 1) * 7 + indx - 1] * wtm;
        const double dd = T.d[(im - 1) * 7 + indx - 1] * wtp + T.d[(ip - 1) * 7 + indx - 1] * wtm;
        corr = 1.0 + dd / (cc + beta * sb);
    }
    return (1.5 / sb + 27.0 / b2) / b2 * corr;
}

__device__ double hf_nm(int n, int m) {
    if (m <= n) return 0.0;
    const double xn = (double)n;
    const double ginf = 0.2027 / pow(xn, 0.71);
    const double gca = 0.124 / xn;
    const double fkn = xn * 1.9603;
    const double wtc = 0.45 - 2.4 / pow(xn, 3.0) * (xn - 1.0);
    const double xm = (double)m;
    const double xmn = xm - xn;
    const double fk = fkn * pow(xm / (xmn * (xm + xn)), 3.0);
    const double xmn12 = pow(xmn, 1.2);
    const double wt = (xmn12 - 1.0) / (xmn12 + wtc);
    return fk * (1.0 - wt * ginf - (0.222 + gca / xm) * (1.0 - wt));
}

__device__ double interp_cutoff(double dwn, const double* tab, int n, double start, double step, bool* ok) {
    *ok = true;
    if (dwn > start + step * (double)(n - 1)) {
        *ok = false;
        return 0.0;
    }
    if (dwn <= start) return tab[0] + (tab[1] - tab[0]) * ((dwn - start) / step);
    const double pos = (dwn - start) / step;
    const int i = (int)floor(pos);
    const double frac = pos - (double)i;
    if (i >= n - 1) return tab[n - 1];
    return tab[i] + (tab[i + 1] - tab[i]) * frac;
}

// HPROF4 (profiles/hydrogen.py:1541-1710) for the transition n -> m at
// wavelength offset dlam_nm from the line centre, in the depth state q.
// The wavelength-independent part of HPROF4 (profiles/hydrogen.py:1430-1515,
// :1842-1870) for the (n, m) profile of a line at one layer, computed once
// per (line, layer) by the setup kernel.
__device__ HprofConst hprof4_const(int n, int m, const HydPar& q, const HydTables& T) {
    HprofConst K{};
    const int mmn = m - n;
    K.mmn = mmn;
    if (mmn <= 0) return K;
    const double xn = (double)n, xm = (double)m;
    const double xn2 = xn * xn, xm2 = xm * xm;
    const double xm2mn2 = xm2 - xn2;
    const double xmn2 = xm2 * xn2;
    const double gnm = xm2mn2 / xmn2;
    double xknm;
    if (mmn <= 3 && n <= 4) xknm = T.xknmtb[(n - 1) * 3 + mmn - 1];
    else xknm = 5.5e-5 / gnm * xmn2 / (1.0 + 0.13 / (double)mmn);
    const double freqnm = kRydH * gnm;
    const double wavenm = kClightA / freqnm;
    const double c1con = xknm / wavenm * gnm * xm2mn2;
    const double c2con = pow(xknm / wavenm, 2.0);
    double radamp = T.asum[n - 1] + T.asum[m - 1];
    if (n == 1) radamp = T.asum_lyman[m - 1];
    radamp /= 12.5664;
    radamp /= freqnm;
    double resont = hf_nm(1, m) / xm / (1.0 - 1.0 / xm2);
    if (n != 1) resont += hf_nm(1, n) / xn / (1.0 - 1.0 / xn2);
    resont *= 3.579e-24 / gnm;
    const double vdw = 4.45e-26 / gnm * pow(xm2 * (7.0 * xm2 + 5.0), 0.4);
    const double hwvdw = vdw * q.t3nhe + 2.0 * vdw * q.t3nh2;
    const double hwrad = radamp;
    const double stark = 1.6678e-18 * freqnm * xknm;
    const double hwres = resont * q.xnfph0 * 2.0;
    const double hwstk = stark * q.fo;
    const double hwlor = hwres + hwvdw + hwrad;
    const double dph = fmax(q.dopph, 1e-40);
    K.freqnm = freqnm;
    K.wavenm = wavenm;
    K.dbeta = kClightA / (freqnm * freqnm * xknm);
    K.dop = freqnm * dph;
    K.hfwidth = freqnm * fmax(fmax(dph, hwlor), hwstk);
    K.hhw = freqnm * hwlor;
    K.hwres = hwres;
    K.hwvdw = hwvdw;
    K.hwrad = hwrad;
    K.nwid = 1;
    if (!(dph >= hwstk && dph >= hwlor)) {
        K.nwid = 2;
        if (hwlor < hwstk) K.nwid = 3;
    }
    const double y1num = m == 2 ? 550.0 : (m == 3 ? 380.0 : 320.0);
    double y1wht = mmn <= 3 ? 1.0e14 : 1.0e13;
    if (mmn <= 2 && n <= 2) y1wht = T.y1wtm[(n - 1) * 2 + mmn - 1];
    const double wty1 = 1.0 / (1.0 + fmax(q.xne, 0.0) / fmax(y1wht, 1e-30));
    const double y1_scal = y1num * q.y1s * wty1 + q.y1b * (1.0 - wty1);
    K.c1 = q.c1d * c1con * y1_scal;
    K.c2 = q.c2d * c2con;
    K.g1 = 6.77 * sqrt(fmax(K.c1, 1e-30));
    const double ratio = (K.c1 > 0.0 && K.c2 > 0.0) ? sqrt(K.c2) / fmax(K.c1, 1e-30) : 0.0;
    const double log_term = ratio > 0.0 ? log(fmax(ratio, 1e-30)) : 0.0;
    K.gamma0 = K.g1 * fmax(0.0, 0.2114 + log_term) * (1.0 - q.gcon1 - q.gcon2);
    return K;
}

// HPROF4 at dlam_nm from the line centre (profiles/hydrogen.py:1430-1870):
// Doppler core over the fine-structure components, Lorentz (resonance, van
// der Waals, radiation) wings, the Stark profile with its quasi-static
// cutoffs; K holds the (n, m) profile's wavelength-independent part.
__device__ double hprof4(int n, int m, const HprofConst& K, const HydPar& q, double dlam_nm, const HydTables& T,
                         const double* extab, const double* extabf) {
    const int mmn = K.mmn;
    if (mmn <= 0) return 0.0;
    const double xn = (double)n;
    const double xn2 = xn * xn;
    const double freqnm = K.freqnm, dbeta = K.dbeta, dop = K.dop, hhw = K.hhw;
    const double hwres = K.hwres, hwvdw = K.hwvdw, hwrad = K.hwrad;
    const double wl = K.wavenm + dlam_nm * 10.0;
    const double freq = kClightA / wl;
    const double del_freq = fabs(freq - freqnm);
    const bool ifcore = del_freq <= K.hfwidth;
    const int nwid = K.nwid;
    // Doppler core over the fine-structure components (profiles/hydrogen.py:1516)
    double core = 0.0;
    {
        const double dopc = fmax(dop, 1e-30);
        if (n > 4 || m > 10) {
            const double d = fabs(freq - (freqnm + 0.0)) / dopc;
            if (d <= 7.0) core += fastex(d * d, extab, extabf) * 1.0;
        } else if (mmn != 1) {
            const int k = T.lncomp[n - 1];
            for (int i = 0; i < k; i++) {
                const double off = T.stcomp[i * 4 + n - 1] * 1.0e7;
                const double w = T.stcpwt[i * 4 + n - 1] / xn2;
                const double d = fabs(freq - (freqnm + off)) / dopc;
                if (d <= 7.0) core += fastex(d * d, extab, extabf) * w;
            }
        } else {
            const int k = T.lnghal[n - 1], i0 = T.istal[n - 1];
            for (int i = 0; i < k; i++) {
                const double off = T.stalph[i0 + i] * 1.0e7;
                const double w = T.stwtal[i0 + i] / xn2 / 3.0;
                const double d = fabs(freq - (freqnm + off)) / dopc;
                if (d <= 7.0) core += fastex(d * d, extab, extabf) * w;
            }
        }
    }
    double lorentz = 0.0;
    if (n == 1 && m == 2) {
        // Lyman alpha (profiles/hydrogen.py:1731-1797)
        if (dop > 0.0) {
            const double hwres_near = hwres * 4.0;
            const double hwlor_near = hwres_near + hwvdw + hwrad;
            const double hhw_near = freqnm * fmax(hwlor_near, 0.0);
            const double dwn = freq / kClightCm - kLyAlphaWn;
            double hres, hhw_use;
            if (freq > (kLyAlphaWn - 4000.0) * kClightCm && hhw_near > 0.0) {
                hres = hwres_near * freqnm / kPi / (del_freq * del_freq + hhw_near * hhw_near) * 1.77245 * dop;
                hhw_use = hhw_near;
            } else {
                double cut = 0.0;
                bool ok;
                const double lg = interp_cutoff(dwn, T.cutoff_h2, 91, -22000.0, 200.0, &ok);
                if (ok) cut = pow(10.0, lg - 14.0) * q.xnfph0 * 2.0 / kClightCm;
                hres = cut * 1.77245 * dop;
                hhw_use = freqnm * fmax(hwres + hwvdw + hwrad, 0.0);
            }
            double hrad = 0.0, hvdw = 0.0;
            if (hwrad > 0.0 && hhw_use > 0.0 && freq > 2.4190611e15 && freq < 0.77 * kRydH)
                hrad = hwrad * freqnm / kPi / (del_freq * del_freq + hhw_use * hhw_use) * 1.77245 * dop;
            if (hwvdw > 0.0 && hhw_use > 0.0 && freq >= 1.8e15)
                hvdw = hwvdw * freqnm / kPi / (del_freq * del_freq + hhw_use * hhw_use) * 1.77245 * dop;
            lorentz = hres + hrad + hvdw;
        }
    } else {
        double top = hhw;
        if (n == 1 && (m == 3 || m == 4 || m == 5)) {
            const double fr = freq / kRydH;
            if ((m == 3 && 0.885 <= fr && fr <= 0.890) || (m == 4 && 0.936 <= fr && fr <= 0.938) ||
                (m == 5 && 0.959 <= fr && fr <= 0.961))
                top = fmax(hhw - freqnm * hwrad, 0.0);
        }
        if (hhw > 0.0) lorentz = top / kPi / (del_freq * del_freq + hhw * hhw) * 1.77245 * dop;
    }
    const double beta = del_freq / fmax(q.fo, 1e-30) * dbeta;
    const double y1 = K.c1 * beta;
    const double y2 = K.c2 * beta * beta;
    double gamma = K.gamma0;
    if (y2 > 1e-4 && y1 > 1e-5)
        gamma = K.g1 *
                (0.5 * fastex(fmin(80.0, y1), extab, extabf) + vcse1f(y1, extab, extabf) -
                 0.5 * vcse1f(y2, extab, extabf)) *
                (1.0 - q.gcon1 / (1.0 + pow(90.0 * y1, 3.0)) - q.gcon2 / (1.0 + 2000.0 * y1));
    const double f = gamma > 0 ? gamma / kPi / (gamma * gamma + beta * beta) : 0.0;
    double prqs = sofbeta(beta, q.pp, n, m, T);
    double extra = 0.0;
    if (m <= 2) {
        prqs *= 0.5;
        // quasi-static cutoff (profiles/hydrogen.py:1800-1841)
        if (q.fo > 0.0) {
            const double dwn = freq / kClightCm - kLyAlphaWn;
            if (!(dwn < -20000.0)) {
                if (dwn <= -4000.0) {
                    bool ok;
                    const double lg = interp_cutoff(dwn, T.cutoff_h2_plus, 111, -15000.0, 100.0, &ok);
                    if (ok) extra += pow(10.0, lg - 14.0) * q.xnfph1 / kClightCm * 1.77245 * dop;
                } else {
                    const double beta4000 = 4000.0 * kClightCm / fmax(q.fo, 1e-30) * dbeta;
                    const double prqs4000 = sofbeta(beta4000, q.pp, n, m, T) * 0.5;
                    const double norm = prqs4000 / fmax(q.fo, 1e-30) * dbeta;
                    const double cut4000 = pow(10.0, -11.07 - 14.0) * q.xnfph1 / kClightCm;
                    if (norm > 0.0) extra += cut4000 / norm * (prqs / fmax(q.fo, 1e-30) * dbeta) * 1.77245 * dop;
                }
            }
        }
    }
    const double p1 = pow(0.9 * y1, 2.0);
    const double fns = (p1 + 0.03 * sqrt(fmax(y1, 0.0))) / (p1 + 1.0);
    const double stark_core = (prqs * (1.0 + fns) + f) / fmax(q.fo, 1e-30) * dbeta * 1.77245 * dop;
    if (ifcore) {
        if (nwid == 1) return fmax(core, 0.0);
        if (nwid == 2) return fmax(lorentz, 0.0);
        return fmax(stark_core + extra, 0.0);
    }
    return fmax(core + lorentz + stark_core + extra, 0.0);
}

__device__ __forceinline__ double ehyd(int n, const HydTables& T) {
    return (n >= 1 && n <= 8) ? T.ehyd[n - 1] : kHydEinf - kHydRyd / (double)(n * n);
}

template <typename R>
__device__ __forceinline__ double abtot(const HydArgs& a, int d, int64_t b) {
    const int64_t i = (int64_t)d * a.n_wl + b;
    return (double)((const R*)a.cabs)[i] + (double)((const R*)a.cscat)[i];
}

// WCON / WTAIL of a fort.19 line (opacity.py:657-702, vacuum grid):
// the CONTX edge of (NCON, NELIONX) less the merge energy of the layer (the
// hydrogen one for NELION 1); <= 0 where a limit is absent.
__device__ __forceinline__ void continuum_limits(int ncon, int nelion, int nelionx, double xne,
                                                 const HydTables& T, double* wcon, double* wtail) {
    *wcon = -1.0;
    *wtail = -1.0;
    if (ncon <= 0 || nelionx <= 0 || nelionx > 17 || ncon > 26) return;
    const double cv = T.contx[(ncon - 1) * 17 + (nelionx - 1)];
    if (cv <= 0.0) return;
    const double nmerge = fmax(1600.0 / pow(fmax(xne, 1e-40), 2.0 / 15.0) - 1.5, 1.0);
    const double nm2 = fmax(nmerge * nmerge, 1e-12);
    const double em = nelion == 1 ? 109677.576 / nm2 : 109737.312 / nm2;
    const double denom = cv - em;
    if (fabs(denom) <= 1e-8) return;
    const double wc = 1.0e7 / denom;
    double wt = -1.0;
    const double dt = cv - em - 500.0;
    if (fabs(dt) > 1e-8) {
        wt = 1.0e7 / dt;
        if (wt < 0.0) wt = 2.0 * wc;
        wt = (2.0 * wc) < wt ? 2.0 * wc : wt;
    }
    if (wt > 0.0 && wt <= wc) wt = -1.0;
    *wcon = wc;
    *wtail = wt;
}

// The WTAIL taper of a wing value at wavelength w (opacity.py:1031-1032,
// :236-240): (w - base) / (WTAIL - base) below WTAIL, base = WCON or the line.
__device__ __forceinline__ double wing_taper(double v, double w, double wcon, double wtail, double wl0) {
    if (wtail > 0.0 && w < wtail) {
        const double base = wcon > 0.0 ? wcon : wl0;
        v = v * (w - base) / fmax(wtail - base, 1e-12);
    }
    return v;
}

template <typename R>
__device__ __forceinline__ double abtot_he(const HeArgs& a, int d, int64_t b) {
    const int64_t i = (int64_t)d * a.n_wl + b;
    return (double)((const R*)a.cabs)[i] + (double)((const R*)a.cscat)[i];
}

__device__ __forceinline__ double stim_at(const HydArgs& a, const HydPar& q, int64_t b) {
    const double freq = kClightCm / (a.grid[b] * 1e-7);
    return 1.0 - exp(-freq * q.hkt);
}

// Value the walk adds at grid point b on `side` (+1 red, -1 blue) or at the
// centre (side 0); *stop = true where the reference's walk ends there,
// *add = false where it passes the point without adding (red, below WCON).
template <typename R>
__device__ double walk_value(const HydArgs& a, const HydPar& q, int64_t b, int side, bool* stop, bool* add) {
    const HydTables& T = *a.tab;
    const double w = a.grid[b];
    const bool simple = q.nu <= q.nl + 2;
    const bool taper = !simple && (q.wtail > q.wcon);
    const double stim = stim_at(a, q, b);
    const double cut = abtot<R>(a, q.d, b) * a.cutoff;
    *stop = false;
    *add = true;
    if (side == 0) {
        if (!simple && w < q.wcon) {
            *add = false;
            return 0.0;
        }
        double v = q.kappa0 * hprof4(q.nl, q.nu, q.k_line, q, w - q.wl0, T, a.extab, a.extabf) * stim;
        if (taper && w < q.wtail) v *= (w - q.wcon) / (q.wtail - q.wcon);
        if (!(v >= cut)) *add = false;
        return v;
    }
    if (side > 0) {
        if (!simple) {
            if (w > q.wlm1) {
                *stop = true;
                return 0.0;
            }
            if (w < q.wcon) {
                *add = false;
                return 0.0;
            }
            double v = q.kappa0 * hprof4(q.nl, q.nu, q.k_line, q, w - q.wl0, T, a.extab, a.extabf) * stim;
            if (taper && w < q.wtail) v *= (w - q.wcon) / (q.wtail - q.wcon);
            if (w > q.redcut) {
                const int um2 = q.nu - 2 > q.nl + 1 ? q.nu - 2 : q.nl + 1;
                double v2 = q.kappa0 * hprof4(q.nl, um2, q.k_red, q, w - q.wlm2, T, a.extab, a.extabf) * stim;
                if (taper && w < q.wtail) v2 *= (w - q.wcon) / (q.wtail - q.wcon);
                if (v2 >= v) {
                    *stop = true;
                    return 0.0;
                }
            }
            if (v <= 0.0 || v < cut) *stop = true;
            return v;
        }
        const double v = q.kappa0 * hprof4(q.nl, q.nu, q.k_line, q, w - q.wl0, T, a.extab, a.extabf) * stim;
        if (v <= 0.0 || v < cut) *stop = true;
        return v;
    }
    if (!simple && (w < q.wcon || w < q.wlp1)) {
        *stop = true;
        return 0.0;
    }
    double v = q.kappa0 * hprof4(q.nl, q.nu, q.k_line, q, w - q.wl0, T, a.extab, a.extabf) * stim;
    if (!simple) {
        if (taper && w < q.wtail) v *= (w - q.wcon) / (q.wtail - q.wcon);
        if (w < q.bluecut) {
            double v2 = q.kappa0 * hprof4(q.nl, q.nu + 2, q.k_blue, q, w - q.wlp2, T, a.extab, a.extabf) * stim;
            if (taper && w < q.wtail) v2 *= (w - q.wcon) / (q.wtail - q.wcon);
            if (v2 >= v) {
                *stop = true;
                return 0.0;
            }
        }
    }
    if (v <= 0.0 || v < cut) *stop = true;
    return v;
}

template <typename R>
__global__ void __launch_bounds__(128) hyd_setup_kernel(HydArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_h * a.n_layers) return;
    const int h = (int)(i / a.n_layers), d = (int)(i - (int64_t)h * a.n_layers);
    const HydTables& T = *a.tab;
    HydPar q;
    q.active = 0;
    q.d = d;
    const int row = a.rows[h];
    const int nl = a.n_lower[h], nu = a.n_upper[h];
    q.nl = nl > 1 ? nl : 1;
    q.nu = nu > nl + 1 ? nu : nl + 1;
    // the profile reads ASUM at the upper level and at two levels above it
    // (96 entries): a line outside those, or a row outside the catalog, is
    // flagged and left out
    if (row < 0 || (int64_t)row >= a.n_lines || q.nu + 2 > 96) {
        if (d == 0) atomicOr(a.flags, FLAG_HYDROGEN_LINE);
        q.nl = 1;
        q.nu = 2;
        q.ci = 0;
        a.par[i] = q;
        return;
    }
    q.wl0 = a.wavelength[row];
    q.ci = a.center[row];
    // depth state (populations.py:93-125, :183-216)
    const double temp = fmax(a.temperature[d], 1.0);
    const double xne_raw = a.xne[d];
    const double xne = fmax(xne_raw, 1e-40);
    const double xne16 = pow(xne, 1.0 / 6.0);
    q.pp = xne16 * 0.08989 / sqrt(fmax(temp, 1.0));
    q.fo = pow(xne16, 4.0) * 1.25e-9;
    q.y1b = 2.0 / (1.0 + 0.012 / fmax(temp, 1.0) * sqrt(xne / fmax(temp, 1.0)));
    const double t4 = temp / 10000.0;
    const double t43 = pow(t4, 0.3);
    q.y1s = t43 / xne16;
    const double he1 = a.xnf_he1 ? a.xnf_he1[d] : 0.0;
    const double h2 = a.xnf_h2 ? a.xnf_h2[d] : 0.0;
    q.t3nhe = t43 * he1;
    q.t3nh2 = t43 * h2;
    q.c1d = q.fo * 78940.0 / fmax(temp, 1.0);
    q.c2d = pow(q.fo, 2.0) / 5.96e-23 / xne;
    q.gcon1 = 0.2 + 0.09 * sqrt(fmax(t4, 1e-12)) / (1.0 + xne / 1.0e13);
    q.gcon2 = 0.2 / (1.0 + xne / 1.0e15);
    const int64_t per = (int64_t)a.n_ion * a.n_elem;
    q.xnfph0 = a.population[(int64_t)d * per + 0 * a.n_elem + 0];
    q.xnfph1 = a.population[(int64_t)d * per + 1 * a.n_elem + 0];
    {
        const double vt = (a.vturb[d] / 1e5) / kClightKms;
        const double micro = a.microturb_kms > 0 ? a.microturb_kms / kClightKms : 0.0;
        const double total = sqrt(vt * vt + micro * micro);
        const double thermal = sqrt(2.0 * kKboltz * temp / (1.008 * kAmu)) / kClightCm;
        q.dopph = sqrt(thermal * thermal + total * total);
    }
    q.xne = xne_raw;
    q.hkt = kHPlanck / (kKboltz * a.temperature[d]);
    // the line's series neighbours and cuts (engine/opacity.py:1780-1815)
    const int ncon = nl < 1 ? 1 : (nl > 15 ? 15 : nl);
    const double conth = T.conth[ncon - 1];
    const double elo = ehyd(nl, T);
    q.wlm1 = nu - 1 > nl ? 1.0e7 / (ehyd(nu - 1, T) - elo) : q.wl0;
    q.wlm2 = nu - 2 > nl ? 1.0e7 / (ehyd(nu - 2, T) - elo) : q.wl0;
    q.wlp1 = 1.0e7 / (ehyd(nu + 1, T) - elo);
    q.wlp2 = 1.0e7 / (ehyd(nu + 2, T) - elo);
    q.redcut = 1.0e7 / (T.conth[0] - kHydRyd / pow((double)nu - 0.8, 2.0) - elo);
    q.bluecut = 1.0e7 / (T.conth[0] - kHydRyd / pow((double)nu + 0.8, 2.0) - elo);
    // gates (engine/opacity.py:1817-1845)
    const double pv = q.xnfph0;
    double dv = a.doppler[(int64_t)d * per + 0 * a.n_elem + 0];
    const double micro = a.microturb_kms > 0.0 ? a.microturb_kms / kClightKms : 0.0;
    if (micro > 0.0) dv = sqrt(dv * dv + micro * micro);
    const double rho = a.rho[d];
    q.kappa0 = 0.0;
    if (pv > 0.0 && dv > 0.0 && rho > 0.0) {
        const double cgf = kCgf * a.gf[row] / (kClightNm / q.wl0);
        const double k0pre = cgf * (pv / (rho * dv));
        const int64_t cc = q.ci < 0 ? 0 : (q.ci > a.n_wl - 1 ? a.n_wl - 1 : q.ci);
        const double kapmin = abtot<R>(a, d, cc) * a.cutoff;
        if (k0pre >= kapmin) {
            const double k0 = k0pre * fastex(a.elo[row] * a.hckt[d], a.extab, a.extabf);
            if (k0 >= kapmin) {
                q.kappa0 = k0;
                q.active = 1;
            }
        }
    }
    // merge and tail wavelengths (engine/opacity.py:1755-1757, :1846-1858)
    double inglis = 1600.0 / pow(xne, 2.0 / 15.0);
    double nmerge = fmax(inglis - 1.5, 1.0);
    const double emerge = kHydRyd / fmax(nmerge * nmerge, 1e-12);
    const double wshift = 1.0e7 / (conth - kHydRyd / (81.0 * 81.0));
    double wmerge = 1.0e7 / (conth - emerge);
    if (wmerge < 0.0) wmerge = wshift + wshift;
    double wcon = fmax(wshift, wmerge);
    double wtail = wcon > 0.0 ? 1.0e7 / (1.0e7 / wcon - 500.0) : wcon + wcon;
    wcon = fmin(wshift + wshift, wcon);
    if (wtail < 0.0) wtail = wcon + wcon;
    wtail = fmin(wcon + wcon, wtail);
    q.wcon = wcon;
    q.wtail = wtail;
    q.k_line = hprof4_const(q.nl, q.nu, q, T);
    q.k_red = hprof4_const(q.nl, q.nu - 2 > q.nl + 1 ? q.nu - 2 : q.nl + 1, q, T);
    q.k_blue = hprof4_const(q.nl, q.nu + 2, q, T);
    a.par[i] = q;
}

// The walks' first offsets and, as a start, their last possible end (one
// thread per (line, depth, side)): offsets [x, y) with y = MAX_STEPS + 1.
template <typename R>
__global__ void __launch_bounds__(128) hyd_walk_init_kernel(HydArgs a) {
    const int64_t gw = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gw >= (int64_t)a.n_h * a.n_layers * 2) return;
    const HydPar& q = a.par[gw >> 1];
    const int side = (gw & 1) ? -1 : 1;
    int2 out = make_int2(1, 1);
    if (q.active) {
        const int64_t n = a.n_wl, ci = q.ci;
        int64_t first = 1;
        bool alive = true;
        if (ci >= n) {
            if (side > 0) alive = false;
            first = ci - (n - 1) > 1 ? ci - (n - 1) : 1;
        } else if (ci < 0) {
            if (side < 0) alive = false;
            first = -ci > 1 ? -ci : 1;
        }
        const int64_t max_steps = ci > n - ci - 1 ? ci : n - ci - 1;
        out = make_int2((int)first, (int)(alive ? max_steps + 1 : first));
    }
    a.walk[gw] = out;
}

// Where each walk ends: the reference steps outward until the first offset
// whose value stops it.  Here every offset is tested at once, one thread per
// (walk, offset) in blocks of 256 consecutive offsets, and the smallest
// stopping offset is kept with atomicMin (order-free, so the same on every
// run); a block whose offsets all lie past the end found so far returns.
template <typename R>
__global__ void __launch_bounds__(256) hyd_walk_stop_kernel(HydArgs a, int64_t n_oblocks) {
    const int64_t n_walks = (int64_t)a.n_h * a.n_layers * 2;
    for (int64_t blk = blockIdx.x; blk < n_walks * n_oblocks; blk += gridDim.x) {
        const int64_t ob = blk / n_walks, gw = blk - ob * n_walks;  // offset blocks in order: ends found early cut later blocks
        int* end = &a.walk[gw].y;
        const int first = a.walk[gw].x;
        const int64_t o = (int64_t)first + ob * 256 + threadIdx.x;
        if ((int64_t)first + ob * 256 >= (int64_t)*(volatile int*)end) continue;  // block-uniform
        if (o >= (int64_t)*(volatile int*)end) continue;
        const HydPar& q = a.par[gw >> 1];
        const int side = (gw & 1) ? -1 : 1;
        const int64_t b = (int64_t)q.ci + side * o;
        bool stop = true;
        if (b >= 0 && b < a.n_wl) {
            bool add;
            walk_value<R>(a, q, b, side, &stop, &add);
        }
        if (stop) atomicMin(end, (int)o);
    }
}

// One thread per (depth, grid point): every line whose walk covers the point
// adds its value, in catalog order; the sum goes onto the line opacity.
template <typename R>
__global__ void __launch_bounds__(256) hyd_gather_kernel(HydArgs a, R* __restrict__ cube) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_layers * a.n_wl) return;
    const int d = (int)(i / a.n_wl);
    const int64_t b = i - (int64_t)d * a.n_wl;
    double acc = 0.0;
    bool any = false;
    for (int h = 0; h < a.n_h; h++) {
        const int64_t pd = (int64_t)h * a.n_layers + d;
        if (!a.par[pd].active) continue;
        const int64_t ci = a.par[pd].ci;
        int side;
        int64_t o;
        if (b == ci) {
            side = 0;
            o = 0;
        } else if (b > ci) {
            side = 1;
            o = b - ci;
        } else {
            side = -1;
            o = ci - b;
        }
        if (side != 0) {
            const int2 wk = a.walk[pd * 2 + (side > 0 ? 0 : 1)];
            if (o < wk.x || o >= wk.y) continue;
        }
        const HydPar& q = a.par[pd];
        bool stop, add;
        const double v = walk_value<R>(a, q, b, side, &stop, &add);
        if (!add) continue;
        acc += v;
        any = true;
    }
    if (any) cube[i] = (R)((double)cube[i] + acc);
}

// ---------------------------------------------------------------------------
// helium lines
// ---------------------------------------------------------------------------

// One thread per (helium line, depth): the gates and wing parameters of
// process_depth (engine/opacity.py:2686-2910) and _apply_fort19_profile
// (:996-1016) for a line without fort.19 continuum limits (NCON = 0).
template <typename R>
__global__ void __launch_bounds__(128) he_setup_kernel(HeArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_he * a.n_layers) return;
    const int h = (int)(i / a.n_layers), d = (int)(i - (int64_t)h * a.n_layers);
    HePar q;
    q.active = 0;
    q.d = d;
    q.ci = 0;
    q.pad = 0;
    q.wl0 = q.keff = q.dop = q.adamp = 0.0;
    q.wcon = q.wtail = -1.0;
    const int row = a.rows[h];
    if (row < 0 || (int64_t)row >= a.n_lines) {
        if (d == 0) atomicOr(a.flags, FLAG_HELIUM_LINE);
        a.par[i] = q;
        return;
    }
    const int ci = a.center[row];
    const int nelion = a.ion_stage[row];
    // centre outside the grid (:2690-2696); ion stage beyond the table (:2838)
    if (ci < 0 || (int64_t)ci >= a.n_wl || nelion < 1 || nelion > a.n_ion) {
        a.par[i] = q;
        return;
    }
    q.ci = ci;
    const DepthPar& dp = a.depth[d];
    const int64_t k = ((int64_t)d * a.n_ion + (nelion - 1)) * a.n_elem + 1;  // element He
    const double pv = a.population[k], dv = a.doppler[k];
    if (pv <= 0.0 || dv <= 0.0 || !(dp.rho > 0.0)) {
        a.par[i] = q;
        return;
    }
    const double xnfdop = pv / (dp.rho * dv);
    const double wl = a.wavelength[row];
    const double dw = dv * wl;
    const double boltz = fastex(a.elo[row] * dp.hckt, a.extab, a.extabf);
    const double cgf = kCgf * a.gf[row] / (kClightNm / wl);
    const double kmin = abtot_he<R>(a, d, ci) * a.cutoff;
    const double k0pre = cgf * xnfdop;
    if (k0pre < kmin || dw <= 0.0) {
        a.par[i] = q;
        return;
    }
    const double k0 = k0pre * boltz;
    if (k0 < kmin) {
        a.par[i] = q;
        return;
    }
    double dop = fmax(dw, 1e-12), keff = k0;
    if (a.line_type[row] == -4) {  // 3He
        keff /= 1.155;
        dop *= 1.155;
    }
    const double dn = (a.gamma_rad[row] + a.gamma_stark[row] * dp.xne + a.gamma_vdw[row] * dp.txnxn) /
                      fmax(dop / wl, 1e-40);
    q.wl0 = wl;
    q.keff = keff;
    q.dop = dop;
    q.adamp = fmax(dn, 1e-12);
    // fort.19 continuum-merge limits (process_depth, opacity.py:2760-2770, :2909)
    continuum_limits(a.ncon[h], nelion, a.nelionx[h], dp.xne, *a.tab, &q.wcon, &q.wtail);
    q.active = 1;
    a.par[i] = q;
}

template <typename R>
__device__ __forceinline__ double he_value(const HeArgs& a, const HePar& q, int64_t b) {
    const double w = a.grid[b];
    const double v = q.keff * voigt_hv<double>(fabs(w - q.wl0) / q.dop, q.adamp, a.h0, a.h1, a.h2);
    return wing_taper(v, w, q.wcon, q.wtail, q.wl0);
}

// A red step at or below WCON is passed over; a blue one ends the walk
// (opacity.py:1026-1028, :1043-1045).
__device__ __forceinline__ bool he_below_wcon(const HeArgs& a, const HePar& q, int64_t b) {
    return q.wcon > 0.0 && a.grid[b] <= q.wcon;
}

// The helium walks: first offsets and their last possible ends (one thread
// per (line, depth, side)).
template <typename R>
__global__ void __launch_bounds__(128) he_walk_init_kernel(HeArgs a) {
    const int64_t gw = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gw >= (int64_t)a.n_he * a.n_layers * 2) return;
    const HePar& q = a.par[gw >> 1];
    const bool red = (gw & 1) == 0;
    const int64_t n = a.n_wl;
    bool alive = q.active != 0;
    if (alive) alive = red ? q.wl0 <= a.grid[n - 1] : (q.ci > 0 && q.wl0 >= a.grid[0]);
    const int first = red ? 0 : 1;
    const int64_t last = red ? n - 1 - q.ci : q.ci;  // largest offset inside the grid
    a.walk[gw] = make_int2(first, alive ? (int)(last + 1) : first);
}

// Where each helium walk ends (one thread per (walk, offset), smallest end by
// atomicMin): the red walk ends before the first step under the cutoff (steps
// at or below WCON are passed over), the blue walk after it, or before the
// first step at or below WCON (opacity.py:1019-1046).
template <typename R>
__global__ void __launch_bounds__(256) he_walk_stop_kernel(HeArgs a, int64_t n_oblocks) {
    const int64_t n_walks = (int64_t)a.n_he * a.n_layers * 2;
    for (int64_t blk = blockIdx.x; blk < n_walks * n_oblocks; blk += gridDim.x) {
        const int64_t ob = blk / n_walks, gw = blk - ob * n_walks;  // offset blocks in order: ends found early cut later blocks
        int* end = &a.walk[gw].y;
        const int first = a.walk[gw].x;
        const int64_t o = (int64_t)first + ob * 256 + threadIdx.x;
        if ((int64_t)first + ob * 256 >= (int64_t)*(volatile int*)end) continue;  // block-uniform
        if (o >= (int64_t)*(volatile int*)end) continue;
        const HePar q = a.par[gw >> 1];
        const bool red = (gw & 1) == 0;
        const int64_t b = red ? q.ci + o : q.ci - o;
        if (he_below_wcon(a, q, b)) {
            if (!red) atomicMin(end, (int)o);
            continue;
        }
        if (he_value<R>(a, q, b) < abtot_he<R>(a, q.d, b) * a.cutoff) atomicMin(end, (int)(red ? o : o + 1));
    }
}

// One thread per (depth, grid point): the wing values of the helium lines
// whose walks cover the point, summed in catalog order (AHE), times STIM,
// added to the cube.
template <typename R>
__global__ void __launch_bounds__(256) he_gather_kernel(HeArgs a, R* __restrict__ cube) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_layers * a.n_wl) return;
    const int d = (int)(i / a.n_wl);
    const int64_t b = i - (int64_t)d * a.n_wl;
    double acc = 0.0;
    bool any = false;
    for (int h = 0; h < a.n_he; h++) {
        const int64_t pd = (int64_t)h * a.n_layers + d;
        if (!a.par[pd].active) continue;
        const int64_t ci = a.par[pd].ci;
        const bool red = b >= ci;
        const int64_t o = red ? b - ci : ci - b;
        const int2 wk = a.walk[pd * 2 + (red ? 0 : 1)];
        if (o < wk.x || o >= wk.y) continue;
        const HePar q = a.par[pd];
        if (he_below_wcon(a, q, b)) continue;   // red steps at or below WCON add nothing
        acc += he_value<R>(a, q, b);
        any = true;
    }
    if (any) {
        const double freq = kClightCm / (a.grid[b] * 1e-7);
        const double stim = 1.0 - exp(-freq * (kHPlanck / (kKboltz * a.temperature[d])));
        cube[i] = (R)((double)cube[i] + acc * stim);
    }
}

// ---------------------------------------------------------------------------
// fort.19 NORMAL lines (NBLO/NBUP set, not H/He/autoionizing/coronal/PRD)
// ---------------------------------------------------------------------------

template <typename R>
__device__ __forceinline__ double abtot_f19(const F19Args& a, int d, int64_t b) {
    const int64_t i = (int64_t)d * a.n_wl + b;
    return (double)((const R*)a.cabs)[i] + (double)((const R*)a.cscat)[i];
}

// Near-wing profile value at step k (k <= N10DOP): the incremental TABI of
// opacity.py:151-162 (k additions of TABSTEP to 0.5) or the Voigt function.
// Number of grid points at or below x (le) or below x; the grid ascends.
__device__ __forceinline__ int grid_count(const double* g, int64_t n, double x, bool le) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (le ? g[mid] <= x : g[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return (int)lo;
}

// The truncated TABI after k additions: each addition of a positive TABSTEP
// rounds by at most half an ulp of a partial sum no larger than the last, so
// the sequential sum lies within (k + 1) |s| 2^-53 of s = fma(k, TABSTEP, 0.5);
// where s is farther than twice that from an integer both truncate alike, and
// only the other points replay the k additions.
__device__ __forceinline__ int tabi_index(double tabstep, int k) {
    if (tabstep > 0.0) {
        const double s = fma((double)k, tabstep, 0.5);
        const double f = floor(s);
        const double bound = (double)(k + 1) * (s + 1.0) * 2.220446049250313e-16;
        if (s - f > bound && (f + 1.0) - s > bound && s < 2.0e9) return (int)f;
    }
    double tabi = 0.5;
    for (int j = 0; j < k; j++) tabi = tabi + tabstep;
    return (int)tabi;
}

__device__ __forceinline__ double f19_near(const F19Args& a, const F19Par& q, int k) {
    if (q.adamp < 0.2) {
        int it = tabi_index(q.tabstep, k);
        it = it < 0 ? 0 : (it > VOIGT_N - 1 ? VOIGT_N - 1 : it);
        return q.kappa0 * (a.h0[it] + q.adamp * a.h1[it]);
    }
    return q.kappa0 * voigt_hv<double>((double)k * q.dvoigt, q.adamp, a.h0, a.h1, a.h2);
}

// One thread per (line, depth): _add_fort19_asynth's gates and KAPCEN
// (opacity.py:1388-1447) and the near-wing scan of
// _accumulate_metal_profile_kernel (:117-196), sequential like the reference.
template <typename R>
__global__ void __launch_bounds__(128) f19_setup_kernel(F19Args a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_f19 * a.n_layers) return;
    const int h = (int)(i / a.n_layers), d = (int)(i - (int64_t)h * a.n_layers);
    F19Par q;
    q.kappa0 = q.adamp = q.tabstep = q.dvoigt = q.x_far = q.kapcen = 0.0;
    q.wcon = q.wtail = -1.0;
    q.ci = q.cc = q.n10 = q.nstep = q.early = q.active = q.kc_ok = q.kind = q.bw_tail = 0;
    q.bw_con = -1;
    q.d = d;
    const int row = a.rows[h];
    const int e = (row >= 0 && (int64_t)row < a.n_lines) ? a.element_idx[row] : -1;
    const int ion = (row >= 0 && (int64_t)row < a.n_lines) ? a.ion_stage[row] : 0;
    if (e < 0 || e >= a.n_elem || ion < 1 || ion > a.n_ion) {
        if (d == 0) atomicOr(a.flags, FLAG_F19_LINE);
        a.par[i] = q;
        return;
    }
    const DepthPar& dp = a.depth[d];
    const double pv = a.population[((int64_t)d * a.n_ion + (ion - 1)) * a.n_elem + e];
    const int64_t n = a.n_wl;
    const int ci = a.center[row];
    const double wl = a.wavelength[row];
    if (!(pv > 0.0) || (int64_t)ci >= n || !(dp.rho > 0.0)) {
        a.par[i] = q;
        return;
    }
    const double boltz = fastex(a.elo[row] * dp.hckt, a.extab, a.extabf);
    if (a.kind[h] == 2) {
        // merged continuum: KAPPA = GF XNFPEL BOLT (opacity.py:1489-1497), the
        // merge and tail wavelengths of _compute_merged_continuum_limits
        // (:723-758) and the ramp of _accumulate_merged_continuum (:863-898)
        q.kind = 2;
        const double kappa = a.cgf[h] * (pv / dp.rho) * boltz;
        if (!(kappa > 0.0)) {
            a.par[i] = q;
            return;
        }
        const double xne = fmax(dp.xne, 1e-40);
        const double nmerge = fmax(1600.0 / pow(xne, 2.0 / 15.0) - 1.5, 1.0);
        const double nm2 = fmax(nmerge * nmerge, 1e-12);
        const int ionx = a.nelion[h], nlast = a.nlast[h];
        double wmerge = wl, wtail = wl;
        if (wl > 0.0 && nlast > 0) {
            const double ryd = ionx == 1 ? 109677.576 : 109737.312;
            const double dshift = 1.0e7 / wl - ryd / (double)(nlast * nlast);
            if (fabs(dshift) > 1e-12) {
                const double wshift = 1.0e7 / dshift;
                const double em = ionx == 1 ? 109677.576 / nm2 : 109737.312 / nm2;
                const double dmerge = 1.0e7 / wl - em;
                if (fabs(dmerge) > 1e-12) {
                    double wm = 1.0e7 / dmerge;
                    if (wm < 0.0) wm = wshift + wshift;
                    wm = wshift > wm ? wshift : wm;
                    wm = (wshift + wshift) < wm ? wshift + wshift : wm;
                    wmerge = wm;
                    const double dtail = 1.0e7 / wm - 500.0;
                    if (fabs(dtail) > 1e-12) {
                        double wt = 1.0e7 / dtail;
                        if (wt < 0.0) wt = wm + wm;
                        wtail = (wm + wm) < wt ? wm + wm : wt;
                    }
                }
            }
        }
        // searchsorted left / right on the grid
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (a.grid[mid] < wmerge) lo = mid + 1;
            else hi = mid;
        }
        const int64_t i_merge = lo;
        lo = 0;
        hi = n;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (a.grid[mid] <= wtail) lo = mid + 1;
            else hi = mid;
        }
        const int64_t i_tail = lo < n ? lo : n;
        const int64_t i_start = ci > 0 ? ci : 0;
        if (i_tail <= i_start) {
            a.par[i] = q;
            return;
        }
        const int64_t denom = i_tail - (i_merge > i_start ? i_merge : i_start);
        q.kappa0 = kappa;
        q.tabstep = wl;
        q.ci = ci;
        q.cc = (int)i_start;
        q.n10 = (int)i_merge;
        q.nstep = (int)i_tail;
        q.early = (int)(denom > 1 ? denom : 1);
        q.active = 1;
        a.par[i] = q;
        return;
    }
    if (a.kind[h] == 1) {
        // autoionizing: KAPPA0 = BSHORE GF XNFPEL BOLT (opacity.py:1522-1541), then
        // _accumulate_autoionizing_profile (:901-963); a centre bin -1 (line
        // below the grid) is Python's index -1 there: the last bin
        q.kind = 1;
        const double k0 = a.gamma_vdw[h] * a.cgf[h] * (pv / dp.rho) * boltz;
        const int cc = ci >= 0 ? ci : (int)n + ci;
        if (cc < 0 || k0 < abtot_f19<R>(a, d, cc) * a.cutoff || k0 <= 0.0) {
            a.par[i] = q;
            return;
        }
        q.kappa0 = k0;
        q.kapcen = k0;
        q.kc_ok = 1;
        q.ci = ci;
        q.cc = cc;
        q.tabstep = kClightCm / (wl * 1e-7);           // line frequency
        q.dvoigt = fmax(fabs(a.gamma_rad[h]), 1e-30);  // width
        q.x_far = a.gamma_stark[h];                    // ASHORE
        q.adamp = fabs(a.gamma_vdw[h]) < 1e-30 ? 1e-30 : a.gamma_vdw[h];  // BSHORE
        q.active = 1;
        a.par[i] = q;
        return;
    }
    // the line's Doppler width in the depth state (populations.py:158-195):
    // thermal velocity of mass 56, model and synthesis microturbulence
    const double temp = fmax(a.temperature[d], 1.0);
    const double thermal = sqrt(2.0 * kKboltz * temp / (56.0 * kAmu)) / kClightCm;
    const double vt = (a.vturb[d] / 1e5) / kClightKms;
    const double micro = a.microturb_kms > 0 ? a.microturb_kms / kClightKms : 0.0;
    const double total = sqrt(vt * vt + micro * micro);
    const double dw = wl * sqrt(total * total + thermal * thermal);
    if (wl <= 0.0 || dw <= 0.0) {
        a.par[i] = q;
        return;
    }
    const double dopple = dw / wl;
    if (dopple <= 0.0) {
        a.par[i] = q;
        return;
    }
    const double xnfdop = pv / (dp.rho * dopple);
    const double k0pre = a.cgf[h] * xnfdop;
    const int cc = ci < 0 ? 0 : (ci > (int)n - 1 ? (int)n - 1 : ci);
    const double kapmin = abtot_f19<R>(a, d, cc) * a.cutoff;
    if (k0pre < kapmin) {
        a.par[i] = q;
        return;
    }
    const double k0 = k0pre * boltz;
    if (k0 < kapmin) {
        a.par[i] = q;
        return;
    }
    const double gt = a.gamma_rad[h] + a.gamma_stark[h] * dp.xne + a.gamma_vdw[h] * dp.txnxn;
    const double adamp = dopple > 0.0 ? gt / dopple : 0.0;
    q.kapcen = adamp < 0.2 ? k0 * (1.0 - 1.128 * adamp) : k0 * voigt_hv<double>(0.0, adamp, a.h0, a.h1, a.h2);
    q.kc_ok = q.kapcen >= kapmin;
    q.ci = ci;
    q.cc = cc;
    q.active = 1;
    // continuum-merge limits of the record (opacity.py:1449-1461), with the
    // fort.19 ion index as NELION
    continuum_limits(a.ncon[h], a.nelion[h], a.nelionx[h], dp.xne, *a.tab, &q.wcon, &q.wtail);
    // the limits as grid indices, so that the gather's per-line tests are integer ones
    q.bw_con = q.wcon > 0.0 ? grid_count(a.grid, a.n_wl, q.wcon, true) - 1 : -1;
    q.bw_tail = q.wtail > 0.0 ? grid_count(a.grid, a.n_wl, q.wtail, false) : 0;
    // wing (_accumulate_metal_profile_kernel, no WCON/WTAIL)
    if (k0 <= 0.0) {
        q.nstep = 0;
        q.early = 1;
        a.par[i] = q;
        return;
    }
    q.kappa0 = k0;
    q.adamp = fmax(adamp, 1e-12);
    const double kmin = a.cutoff * abtot_f19<R>(a, d, cc);
    double resolu;
    if (cc < (int)n - 1) resolu = 1.0 / (a.grid[cc + 1] / a.grid[cc] - 1.0);
    else if (cc > 0) resolu = 1.0 / (a.grid[cc] / a.grid[cc - 1] - 1.0);
    else resolu = 300000.0;
    int n10 = (int)(10.0 * dopple * resolu);
    n10 = n10 > MAX_PROFILE_STEPS ? MAX_PROFILE_STEPS : n10;
    q.n10 = n10;
    q.tabstep = (dopple * resolu) > 0 ? 200.0 / (dopple * resolu) : 200.0;
    q.dvoigt = (dopple * resolu) > 0 ? 1.0 / dopple / resolu : 1e-6;
    double p_n10 = 0.0;
    if (q.adamp < 0.2) {
        double tabi = 0.5;
        for (int k = 1; k <= n10; k++) {
            tabi = tabi + q.tabstep;
            int it = (int)tabi;
            it = it < 0 ? 0 : (it > VOIGT_N - 1 ? VOIGT_N - 1 : it);
            const double p = k0 * (a.h0[it] + q.adamp * a.h1[it]);
            if (k == n10) p_n10 = p;
            if (p < kmin) {
                q.nstep = k;
                q.early = 1;
                break;
            }
        }
    } else {
        for (int k = 1; k <= n10; k++) {
            const double p = k0 * voigt_hv<double>((double)k * q.dvoigt, q.adamp, a.h0, a.h1, a.h2);
            if (k == n10) p_n10 = p;
            if (p < kmin) {
                q.nstep = k;
                q.early = 1;
                break;
            }
        }
    }
    if (!q.early) {
        q.x_far = (n10 > 0 && p_n10 > 0) ? p_n10 * ((double)n10 * (double)n10) : 0.0;
        int maxstep = n10;
        if (q.x_far > 0 && kmin > 0) {
            const double ms = sqrt(q.x_far / kmin) + 1.0;
            maxstep = ms >= (double)MAX_PROFILE_STEPS ? MAX_PROFILE_STEPS : (int)ms;
        }
        q.nstep = maxstep;
    }
    a.par[i] = q;
}

// Autoionizing profile at grid point b (opacity.py:934-960).
__device__ __forceinline__ double f19_aut_value(const F19Args& a, const F19Par& q, int64_t b) {
    const double freq = kClightCm / (a.grid[b] * 1e-7);
    const double eps = 2.0 * (freq - q.tabstep) / q.dvoigt;
    return q.kappa0 * (q.x_far * eps + q.adamp) / (eps * eps + 1.0) / q.adamp;
}

// Merged-continuum ramp value at grid point b (opacity.py:889-894).
__device__ __forceinline__ double f19_cont_value(const F19Par& q, int64_t b) {
    double v = q.kappa0;
    if (b >= q.n10) {
        const int64_t r = (int64_t)q.nstep - b;
        v *= (double)(r > 0 ? r : 0) / (double)q.early;
    }
    return v;
}

// The autoionizing walks (offsets 1, 2, ... on each side) and the merged-
// continuum ramps (red slot only, absolute bins from the first bin of the
// ramp): first positions and their last possible ends, one thread per
// (line, depth, side).
template <typename R>
__global__ void __launch_bounds__(128) f19_walk_init_kernel(F19Args a) {
    const int64_t gw = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gw >= (int64_t)a.n_f19 * a.n_layers * 2) return;
    const F19Par& q = a.par[gw >> 1];
    const bool red = (gw & 1) == 0;
    const int64_t n = a.n_wl;
    int2 out = make_int2(1, 1);
    if (q.active && q.kind == 2 && red) {
        out = make_int2(q.cc, q.nstep);                   // bins [first, tail)
    } else if (q.active && q.kind == 1) {
        const int64_t last = red ? n - 1 - q.ci : q.ci;  // offsets that stay inside the grid
        out = make_int2(1, (int)(last >= 1 ? last + 1 : 1));
    }
    a.walk[gw] = out;
}

// Where each autoionizing walk and merged-continuum ramp ends: one thread per
// (walk, position), the smallest stopping position kept with atomicMin.  An
// autoionizing step stops at a value <= 0 or under the cutoff
// (opacity.py:944-958); a ramp point stops under the cutoff, points blueward
// of the line being passed over (:885-897).  Most fort.19 walks are empty
// (NORMAL lines have none) or end early, so a block takes 32 walks at one
// block of 256 positions: one warp's ballot keeps those still running and the
// block evaluates only them.  Blocks run position blocks in order across all
// walks, so ends found by earlier blocks cut the later ones.
template <typename R>
__global__ void __launch_bounds__(256) f19_walk_stop_kernel(F19Args a, int64_t n_oblocks) {
    __shared__ int live[32];
    __shared__ int n_live;
    const int64_t n_walks = (int64_t)a.n_f19 * a.n_layers * 2;
    const int64_t n_chunks = (n_walks + 31) / 32;
    for (int64_t blk = blockIdx.x; blk < n_chunks * n_oblocks; blk += gridDim.x) {
        const int64_t ob = blk / n_chunks, c0 = (blk - ob * n_chunks) * 32;
        if (threadIdx.x < 32) {
            const int64_t gw = c0 + threadIdx.x;
            bool alive = false;
            if (gw < n_walks)
                alive = (int64_t)a.walk[gw].x + ob * 256 < (int64_t)*(volatile int*)&a.walk[gw].y;
            const unsigned m = __ballot_sync(0xffffffffu, alive);
            if (alive) live[__popc(m & ((1u << threadIdx.x) - 1u))] = (int)threadIdx.x;
            if (threadIdx.x == 0) n_live = __popc(m);
        }
        __syncthreads();
        const int nl = n_live;
        for (int k = 0; k < nl; ++k) {
            const int64_t gw = c0 + live[k];
            int* end = &a.walk[gw].y;
            const int64_t o = (int64_t)a.walk[gw].x + ob * 256 + threadIdx.x;
            if (o >= (int64_t)*(volatile int*)end) continue;
            const F19Par q = a.par[gw >> 1];
            if (q.kind == 2) {
                if (a.grid[o] < q.tabstep) continue;
                if (f19_cont_value(q, o) < abtot_f19<R>(a, q.d, o) * a.cutoff) atomicMin(end, (int)o);
                continue;
            }
            const bool red = (gw & 1) == 0;
            const int64_t b = red ? (int64_t)q.ci + o : (int64_t)q.ci - o;
            const double v = f19_aut_value(a, q, b);
            if (v <= 0.0 || v < abtot_f19<R>(a, q.d, b) * a.cutoff) atomicMin(end, (int)o);
        }
        __syncthreads();  // live[] and n_live are rewritten for the next chunk
    }
}

// Wing value at step k.  The far wing X / k^2 is an FP64 division in the FP64
// path; the mixed path, whose cube holds FP32, divides in FP32.
template <typename R>
__device__ __forceinline__ double f19_value(const F19Args& a, const F19Par& q, int k) {
    const int near_end = q.early ? q.nstep : q.n10;
    if (k <= near_end) return f19_near(a, q, k);
    if (sizeof(R) == sizeof(float)) return (double)((float)q.x_far / ((float)k * (float)k));
    return q.x_far / ((double)k * (double)k);
}

// One thread per (depth, grid point): the fort.19 lines' KAPCEN and wing
// steps at the point, in catalog (fort.19) order, times STIM, onto the cube
// (opacity.py:1485-1486).
template <typename R>
__global__ void __launch_bounds__(256) f19_gather_kernel(F19Args a, R* __restrict__ cube) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)a.n_layers * a.n_wl) return;
    const int d = (int)(i / a.n_wl);
    const int b = (int)(i - (int64_t)d * a.n_wl);
    const int n = (int)a.n_wl;
    double acc = 0.0;
    bool any = false;
    for (int h = 0; h < a.n_f19; h++) {
        const F19Par& q = a.par[(int64_t)h * a.n_layers + d];
        if (!q.active) continue;
        if (q.kc_ok && b == q.cc) {
            acc += q.kapcen;
            any = true;
        }
        if (q.kind == 2) {
            const int2 wk = a.walk[((int64_t)h * a.n_layers + d) * 2];
            if (b >= wk.x && b < wk.y && !(a.grid[b] < q.tabstep)) {
                acc += f19_cont_value(q, b);
                any = true;
            }
            continue;
        }
        if (q.kind == 1) {
            if (b == q.ci) continue;
            const int64_t pd = (int64_t)h * a.n_layers + d;
            const bool red = b > q.ci;
            const int64_t o = red ? (int64_t)b - q.ci : (int64_t)q.ci - b;
            const int2 wk = a.walk[pd * 2 + (red ? 0 : 1)];
            if (o >= wk.x && o < wk.y) {
                acc += f19_aut_value(a, q, b);
                any = true;
            }
            continue;
        }
        const int ci = q.ci, ns = q.nstep;
        if (ns <= 0 || ci + ns < 0 || ci - ns >= n) continue;
        // at or below WCON nothing is added: the red loop passes over such
        // steps, the blue one ends there (opacity.py:224-228, :264-267)
        // (grid[b] <= WCON exactly for b <= bw_con; the taper applies below bw_tail)
        if (b <= q.bw_con) continue;
        int k = 0;
        if (b > ci && ci < n - 1) {
            const int kr = b - ci;
            const int maxred = ci >= 0 ? min(n - 1 - ci, ns) : min(n - 1, ns);
            if (kr >= max(1, -ci) && kr <= maxred) k = kr;
        } else if (b < ci && ci > 0) {
            const int kb = ci - b;
            if (kb >= max(1, ci + 1 - n) && kb <= min(ci, ns)) k = kb;
        }
        if (k > 0) {
            const double v = f19_value<R>(a, q, k);
            acc += b < q.bw_tail ? wing_taper(v, a.grid[b], q.wcon, q.wtail, a.wavelength[a.rows[h]]) : v;
            any = true;
        }
    }
    if (any) {
        const double freq = kClightCm / (a.grid[b] * 1e-7);
        const double stim = 1.0 - exp(-freq * (kHPlanck / (kKboltz * a.temperature[d])));
        cube[i] = (R)((double)cube[i] + acc * stim);
    }
}

}  // namespace

template <typename R>
static cudaError_t launch_f19_t(const F19Args& a, R* cube, cudaStream_t s) {
    if (a.n_f19 <= 0) return cudaSuccess;
    const int64_t nhd = (int64_t)a.n_f19 * a.n_layers;
    f19_setup_kernel<R><<<(unsigned)((nhd + 127) / 128), 128, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    f19_walk_init_kernel<R><<<(unsigned)((nhd * 2 + 127) / 128), 128, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    {
        const int64_t n_ob = (a.n_wl + 1 + 255) / 256;
        const int64_t blocks = (nhd * 2 + 31) / 32 * n_ob;
        f19_walk_stop_kernel<R><<<(unsigned)(blocks < (1LL << 30) ? blocks : (1LL << 30)), 256, 0, s>>>(a, n_ob);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t cells = (int64_t)a.n_layers * a.n_wl;
    if (cells > 0) f19_gather_kernel<R><<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(a, cube);
    return cudaGetLastError();
}

cudaError_t launch_f19_f32(const F19Args& a, float* cube, cudaStream_t s) { return launch_f19_t<float>(a, cube, s); }
cudaError_t launch_f19_f64(const F19Args& a, double* cube, cudaStream_t s) { return launch_f19_t<double>(a, cube, s); }

template <typename R>
static cudaError_t launch_helium_t(const HeArgs& a, R* cube, cudaStream_t s) {
    if (a.n_he <= 0) return cudaSuccess;
    const int64_t nhd = (int64_t)a.n_he * a.n_layers;
    he_setup_kernel<R><<<(unsigned)((nhd + 127) / 128), 128, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    he_walk_init_kernel<R><<<(unsigned)((nhd * 2 + 127) / 128), 128, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    {
        const int64_t n_ob = (a.n_wl + 1 + 255) / 256;
        const int64_t blocks = nhd * 2 * n_ob;
        he_walk_stop_kernel<R><<<(unsigned)(blocks < (1LL << 30) ? blocks : (1LL << 30)), 256, 0, s>>>(a, n_ob);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t cells = (int64_t)a.n_layers * a.n_wl;
    if (cells > 0) he_gather_kernel<R><<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(a, cube);
    return cudaGetLastError();
}

cudaError_t launch_helium_f32(const HeArgs& a, float* cube, cudaStream_t s) {
    return launch_helium_t<float>(a, cube, s);
}
cudaError_t launch_helium_f64(const HeArgs& a, double* cube, cudaStream_t s) {
    return launch_helium_t<double>(a, cube, s);
}

template <typename R>
static cudaError_t launch_hydrogen_t(const HydArgs& a, R* cube, cudaStream_t s) {
    if (a.n_h <= 0) return cudaSuccess;
    const int64_t nhd = (int64_t)a.n_h * a.n_layers;
    hyd_setup_kernel<R><<<(unsigned)((nhd + 127) / 128), 128, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hyd_walk_init_kernel<R><<<(unsigned)((nhd * 2 + 127) / 128), 128, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    {
        const int64_t n_ob = (a.n_wl + 1 + 255) / 256;
        const int64_t blocks = nhd * 2 * n_ob;
        hyd_walk_stop_kernel<R><<<(unsigned)(blocks < (1LL << 30) ? blocks : (1LL << 30)), 256, 0, s>>>(a, n_ob);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t cells = (int64_t)a.n_layers * a.n_wl;
    if (cells > 0) hyd_gather_kernel<R><<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(a, cube);
    return cudaGetLastError();
}

cudaError_t launch_hydrogen_f32(const HydArgs& a, float* cube, cudaStream_t s) {
    return launch_hydrogen_t<float>(a, cube, s);
}
cudaError_t launch_hydrogen_f64(const HydArgs& a, double* cube, cudaStream_t s) {
    return launch_hydrogen_t<double>(a, cube, s);
}

}  // namespace ks

// ---------------------------------------------------------------------------
// tables: host copy (ks_init_hydrogen_tables), device copy per device
// ---------------------------------------------------------------------------

#include <cstring>
#include <mutex>
#include <string>

namespace {
__device__ ks::HydTables g_hyd;
ks::HydTables g_hyd_host;
bool g_hyd_ready = false;
bool g_hyd_dev[64];
std::mutex g_hyd_mu;

template <typename T>
void copy_n(T* dst, const T* src, size_t n) {
    std::memcpy(dst, src, sizeof(T) * n);
}
}  // namespace

extern "C" ks_status ks_init_hydrogen_tables(const ks_hydrogen_tables* t) {
    if (!t || !t->propbm || !t->c || !t->d || !t->pp || !t->beta || !t->stalph || !t->stwtal || !t->stcomp ||
        !t->stcpwt || !t->istal || !t->lnghal || !t->lncomp || !t->cutoff_h2_plus || !t->cutoff_h2 ||
        !t->asum_lyman || !t->asum || !t->y1wtm || !t->xknmtb || !t->ehyd || !t->conth || !t->contx)
        return ks::set_error(KS_ERR_INVALID, "ks_init_hydrogen_tables: null table pointer");
    ks::HydTables h;
    copy_n(h.propbm, t->propbm, 7 * 5 * 15);
    copy_n(h.c, t->c, 5 * 7);
    copy_n(h.d, t->d, 5 * 7);
    copy_n(h.pp, t->pp, 5);
    copy_n(h.beta, t->beta, 15);
    copy_n(h.stalph, t->stalph, 34);
    copy_n(h.stwtal, t->stwtal, 34);
    copy_n(h.stcomp, t->stcomp, 5 * 4);
    copy_n(h.stcpwt, t->stcpwt, 5 * 4);
    for (int i = 0; i < 4; i++) {
        h.istal[i] = t->istal[i];
        h.lnghal[i] = t->lnghal[i];
        h.lncomp[i] = t->lncomp[i];
        if (h.lncomp[i] < 0 || h.lncomp[i] > 5 || h.lnghal[i] < 0 || h.istal[i] < 0 || h.istal[i] > 34)
            return ks::set_error(KS_ERR_INVALID, "ks_init_hydrogen_tables: fine-structure table out of range");
        // the reference slices STALPH[ISTAL : ISTAL + LNGHAL] with its 1-based
        // ISTAL as a 0-based start (profiles/hydrogen.py:1529-1532); a slice
        // past the 34 entries ends at the last one
        if (h.istal[i] + h.lnghal[i] > 34) h.lnghal[i] = 34 - h.istal[i];
    }
    copy_n(h.cutoff_h2_plus, t->cutoff_h2_plus, 111);
    copy_n(h.cutoff_h2, t->cutoff_h2, 91);
    copy_n(h.asum_lyman, t->asum_lyman, 100);
    copy_n(h.asum, t->asum, 96);
    copy_n(h.y1wtm, t->y1wtm, 4);
    copy_n(h.xknmtb, t->xknmtb, 12);
    copy_n(h.ehyd, t->ehyd, 8);
    copy_n(h.conth, t->conth, 15);
    copy_n(h.contx, t->contx, 26 * 17);
    std::lock_guard<std::mutex> lk(g_hyd_mu);
    g_hyd_host = h;
    g_hyd_ready = true;
    for (bool& r : g_hyd_dev) r = false;
    return KS_OK;
}

ks_status ks::hydrogen_device_tables(const ks::HydTables** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ks::set_error(KS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return ks::set_error(KS_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_hyd_mu);
    if (!g_hyd_ready)
        return ks::set_error(KS_ERR_INVALID, "hydrogen lines given but the hydrogen tables are not initialised "
                                             "(ks_init_hydrogen_tables)");
    if (!g_hyd_dev[dev]) {
        e = cudaMemcpyToSymbol(g_hyd, &g_hyd_host, sizeof(ks::HydTables));
        if (e != cudaSuccess)
            return ks::set_error(KS_ERR_CUDA, std::string("hydrogen tables: ") + cudaGetErrorString(e));
        g_hyd_dev[dev] = true;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_hyd);
    if (e != cudaSuccess) return ks::set_error(KS_ERR_CUDA, std::string("hydrogen tables: ") + cudaGetErrorString(e));
    *out = (const ks::HydTables*)p;
    return KS_OK;
}
