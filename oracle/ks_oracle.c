/*
 * ks_oracle.c -- CPU restatement of the synthe_py line-opacity and transfer
 * path, used ONLY as test infrastructure: the parity reference for the CUDA
 * library and the timed CPU baseline ("port") in bench.py.  Nothing in the
 * product links or calls this file.
 *
 * Every routine follows the reference's arithmetic in the reference's order
 * (file:line cited per function).  All physics is IEEE double; the JOSH
 * scattering iteration runs in single precision exactly as the reference
 * runs it (josh_solver.py:670-687 casts to float32).  Build with
 * -ffp-contract=off so no multiply-add is fused behind the reference's back.
 *
 * Parallelism: OpenMP over lines (TRANSP, like the Numba prange at
 * line_opacity.py:101), over depths (ASYNTH: every depth row is written only
 * by pairs of that depth, so rows are independent and each row keeps the
 * reference's line order of accumulation) and over wavelengths (transfer,
 * like the ThreadPoolExecutor at radiative.py:394).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define C_LIGHT_NM 2.99792458e17
#define C_LIGHT_CM 2.99792458e10
#define C_LIGHT_KM 299792.458
#define H_PLANCK 6.62607015e-27
#define K_BOLTZ 1.380649e-16
#define CGF_CONSTANT (0.026538 / 1.77245)
#define MAX_PROFILE_STEPS 1000000
#define VOIGT_N 2001
#define EXP_N 1001
#define NXTAU 51
#define EPS 1.0e-38
#define MAX_OPACITY_REAL4 3.4e38

int kso_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void kso_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------- grid --- */

/* opacity.py:526-547 _build_wavelength_grid: start snapped up to
 * exp(k*ln r) >= start, then sequential multiplication by r. */
int64_t kso_wavelength_grid(double start, double end, double resolution,
                            double *out, int64_t cap) {
    double ratio = 1.0 + 1.0 / resolution;
    double rlog = log(ratio);
    double ix_start = log(start) / rlog;
    double ix_floor = floor(ix_start);
    if (exp(ix_floor * rlog) < start) ix_floor += 1.0;
    double wl = exp(ix_floor * rlog);
    int64_t n = 0;
    while (wl <= end * (1.0 + 1e-9)) {
        if (out && n < cap) out[n] = wl;
        n++;
        wl *= ratio;
    }
    return n;
}

/* opacity.py:550-592 _nearest_grid_indices: IXWL = int(ln(wl)/ratiolg + .5)
 * minus the same for the first grid point; -1 below, n above the grid. */
void kso_center_indices(const double *grid, int64_t n, const double *wl,
                        int64_t nl, int64_t *out) {
    if (n < 2) {
        for (int64_t i = 0; i < nl; i++) out[i] = 0;
        return;
    }
    double ratio = grid[1] / grid[0];
    double ratiolg = log(ratio);
    int64_t ix_start = (int64_t)(log(grid[0]) / ratiolg + 0.5);
    for (int64_t i = 0; i < nl; i++) {
        int64_t ix = (int64_t)(log(wl[i]) / ratiolg + 0.5);
        int64_t idx = ix - ix_start;
        if (wl[i] < grid[0]) idx = -1;
        if (wl[i] > grid[n - 1]) idx = n;
        out[i] = idx;
    }
}

/* line_opacity.py:1030-1059 _nearest_grid_indices_raw + grid_origin shift:
 * rint(ln(wl/wbegin)/ratiolg) - rint(ln(grid0/wbegin)/ratiolg). */
void kso_wing_indices(const double *grid, int64_t n, const double *wl,
                      int64_t nl, double grid_origin, int64_t *out) {
    if (n < 2) {
        for (int64_t i = 0; i < nl; i++) out[i] = 0;
        return;
    }
    double ratio = grid[1] / grid[0];
    double ratiolg = log(ratio);
    double start_val = grid_origin;
    double ix_floor = floor(log(start_val) / ratiolg);
    double wbegin = exp(ix_floor * ratiolg);
    if (wbegin < start_val) {
        ix_floor += 1.0;
        wbegin = exp(ix_floor * ratiolg);
    }
    int64_t grid_offset = (int64_t)nearbyint(log(grid[0] / wbegin) / ratiolg);
    for (int64_t i = 0; i < nl; i++)
        out[i] = (int64_t)nearbyint(log(wl[i] / wbegin) / ratiolg) - grid_offset;
}

/* -------------------------------------------------------------- tables --- */

/* tables.py:21-27 ExpTables.build */
void kso_exp_tables(double *extab, double *extabf) {
    for (int i = 0; i < EXP_N; i++) {
        extab[i] = exp(-((double)i));
        extabf[i] = exp(-((double)i) * 0.001);
    }
}

/* tables.py:29-42 fast_ex */
static double fast_ex(double x, const double *extab, const double *extabf) {
    if (x <= 0.0) return x == 0.0 ? 1.0 : exp(-x);
    double fl = floor(x);
    if (fl >= (double)EXP_N) return exp(-x);
    int i = (int)fl;
    double frac = x - (double)i;
    int j = (int)(frac * 1000.0 + 0.5);
    if (j < 0) j = 0;
    if (j > EXP_N - 1) j = EXP_N - 1;
    return extab[i] * extabf[j];
}

/* tables.py:275-391 _map1_interpolate (the TABVOIGT variant of MAP1). */
static void map1_tables(const double *xold, const double *fold, int nold,
                        const double *xnew, double *fnew, int nnew) {
    double x1[128], f1[128];
    for (int i = 0; i < nold; i++) {
        x1[i + 1] = xold[i];
        f1[i + 1] = fold[i];
    }
    int l = 2, ll = 0;
    double a = 0, b = 0, c = 0, abac = 0, bbac = 0, cbac = 0;
    double afor = 0, bfor = 0, cfor = 0;
    for (int k = 1; k <= nnew; k++) {
        double x = xnew[k - 1];
        for (;;) {
            if (x < x1[l]) break;
            l++;
            if (l > nold) break;
        }
        if (l > nold) {
            if (l != ll) {
                l = l < nold ? l : nold;
                c = 0.0;
                b = (f1[l] - f1[l - 1]) / (x1[l] - x1[l - 1]);
                a = f1[l] - x1[l] * b;
                ll = l;
            }
            fnew[k - 1] = a + (b + c * x) * x;
            continue;
        }
        if (l == ll) {
            fnew[k - 1] = a + (b + c * x) * x;
            continue;
        }
        if (l == 2) {
            c = 0.0;
            b = (f1[l] - f1[l - 1]) / (x1[l] - x1[l - 1]);
            a = f1[l] - x1[l] * b;
            ll = l;
            fnew[k - 1] = a + (b + c * x) * x;
            continue;
        }
        int l1 = l - 1;
        if (l > ll + 1 || l == 3) {
            int l2 = l - 2;
            double d = (f1[l1] - f1[l2]) / (x1[l1] - x1[l2]);
            cbac = f1[l] / ((x1[l] - x1[l1]) * (x1[l] - x1[l2])) +
                   (f1[l2] / (x1[l] - x1[l2]) - f1[l1] / (x1[l] - x1[l1])) /
                       (x1[l1] - x1[l2]);
            bbac = d - (x1[l1] + x1[l2]) * cbac;
            abac = f1[l2] - x1[l2] * d + x1[l1] * x1[l2] * cbac;
            if (l == nold) {
                c = cbac; b = bbac; a = abac; ll = l;
                fnew[k - 1] = a + (b + c * x) * x;
                continue;
            }
        } else {
            cbac = cfor; bbac = bfor; abac = afor;
            if (l == nold) {
                c = cbac; b = bbac; a = abac; ll = l;
                fnew[k - 1] = a + (b + c * x) * x;
                continue;
            }
        }
        double d = (f1[l] - f1[l1]) / (x1[l] - x1[l1]);
        cfor = f1[l + 1] / ((x1[l + 1] - x1[l]) * (x1[l + 1] - x1[l1])) +
               (f1[l1] / (x1[l + 1] - x1[l1]) - f1[l] / (x1[l + 1] - x1[l])) /
                   (x1[l] - x1[l1]);
        bfor = d - (x1[l] + x1[l1]) * cfor;
        afor = f1[l1] - x1[l1] * d + x1[l] * x1[l1] * cfor;
        double wt = 0.0;
        if (fabs(cfor) != 0.0) wt = fabs(cfor) / (fabs(cfor) + fabs(cbac));
        a = afor + wt * (abac - afor);
        b = bfor + wt * (bbac - bfor);
        c = cfor + wt * (cbac - cfor);
        ll = l;
        fnew[k - 1] = a + (b + c * x) * x;
    }
}

/* tables.py:224-241 VoigtTables.build from the 81-point H1 table
 * (tabvi/tabh1 passed in: the numeric SYNTHE table). */
void kso_voigt_tables(const double *tabvi, const double *tabh1, int ntab,
                      double *h0, double *h1, double *h2) {
    double *grid = (double *)malloc(sizeof(double) * VOIGT_N);
    for (int i = 0; i < VOIGT_N; i++) grid[i] = (double)i / 200.0;
    map1_tables(tabvi, tabh1, ntab, grid, h1, VOIGT_N);
    for (int i = 0; i < VOIGT_N; i++) {
        double v = (double)i / 200.0;
        double vv = v * v;
        h0[i] = exp(-vv);
        h2[i] = h0[i] - (vv + vv) * h0[i];
    }
    free(grid);
}

/* voigt_jit.py:17-69 voigt_profile_jit */
double kso_voigt(double v, double a, const double *h0tab, const double *h1tab,
                 const double *h2tab) {
    double av = fabs(v);
    long iv = (long)(av * 200.0 + 0.5);
    if (iv < 0) iv = 0;
    if (iv > VOIGT_N - 1) iv = VOIGT_N - 1;
    if (a < 0.2) {
        if (av > 10.0) return 0.5642 * a / (v * v);
        return (h2tab[iv] * a + h1tab[iv]) * a + h0tab[iv];
    } else if (a > 1.4 || (a + av) > 3.2) {
        double aa = a * a;
        double vv = v * v;
        double u = (aa + vv) * 1.4142;
        double voigt_val = a * 0.79788 / u;
        if (a <= 100.0) {
            double aau = aa / u;
            double vvu = vv / u;
            double uu = u * u;
            voigt_val = ((((aau - 10.0 * vvu) * aau * 3.0 + 15.0 * vvu * vvu) +
                          3.0 * vv - aa) / uu + 1.0) * voigt_val;
        }
        return voigt_val;
    } else {
        double vv = v * v;
        double hh0 = h0tab[iv];
        double hh1 = h1tab[iv] + hh0 * 1.12838;
        double hh2 = h2tab[iv] + hh1 * 1.12838 - hh0;
        double hh3 = (1.0 - h2tab[iv]) * 0.37613 - hh1 * 0.66667 * vv + hh2 * 1.12838;
        double hh4 = (3.0 * hh3 - hh1) * 0.37613 + hh0 * 0.66667 * vv * vv;
        double poly_a = (((hh4 * a + hh3) * a + hh2) * a + hh1) * a + hh0;
        double poly_b = ((-0.122727278 * a + 0.532770573) * a - 0.96284325) * a + 0.979895032;
        return poly_a * poly_b;
    }
}

/* ----------------------------------------------------------- continuum --- */

/* continuum.py:73-303 build_depth_continuum (coefficient path, log10). */
void kso_continuum(int64_t L, const double *wl, int64_t n, const double *wledge,
                   const double *half_edge, const double *delta_edge, int64_t nedge,
                   const double *abs_coeff, const double *scat_coeff, int coeff_log10,
                   double *cont_abs, double *cont_scat) {
    int64_t nseg = nedge - 1;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double w = wl[j];
        double aw = fabs(w);
        /* searchsorted(|wledge|, |w|, side=right) - 1, clipped */
        int64_t lo = 0, hi = nedge;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (fabs(wledge[mid]) <= aw) lo = mid + 1; else hi = mid;
        }
        int64_t e = lo - 1;
        if (e < 0) e = 0;
        if (e > nedge - 2) e = nedge - 2;
        double left = fabs(wledge[e]);
        double right = fabs(wledge[e + 1]);
        double half = half_edge ? half_edge[e] : 0.5 * (left + right);
        double delta = delta_edge ? delta_edge[e] : 0.5 * (right - left) * (right - left);
        if (delta == 0.0) delta = 1e-20;
        double c1 = (w - half) * (w - right) / delta;
        double c2 = (left - w) * (w - right) * 2.0 / delta;
        double c3 = (w - left) * (w - half) / delta;
        for (int64_t d = 0; d < L; d++) {
            const double *a = abs_coeff + (d * nseg + e) * 3;
            const double *s = scat_coeff + (d * nseg + e) * 3;
            double la = a[0] * c1 + a[1] * c2 + a[2] * c3;
            double ls = s[0] * c1 + s[1] * c2 + s[2] * c3;
            if (coeff_log10) {
                if (la > 38.0) la = 38.0;
                if (ls > 38.0) ls = 38.0;
                la = pow(10.0, la);
                ls = pow(10.0, ls);
                if (la < 0.0) la = 0.0;
                if (la > MAX_OPACITY_REAL4) la = MAX_OPACITY_REAL4;
                if (ls < 0.0) ls = 0.0;
                if (ls > MAX_OPACITY_REAL4) ls = MAX_OPACITY_REAL4;
                if (!isfinite(la)) la = MAX_OPACITY_REAL4;
                if (!isfinite(ls)) ls = MAX_OPACITY_REAL4;
            }
            cont_abs[d * n + j] = la;
            cont_scat[d * n + j] = ls;
        }
    }
}

/* -------------------------------------------------------------- TRANSP --- */

/* Per-depth state used by TRANSP/ASYNTH: populations.py:196-204 TXNXN
 * (npz has no txnxn: (xnf_h + .42 xnf_he1 + .85 xnf_h2) (T/1e4)^.3 with
 * T = max(T, 1)). */
void kso_txnxn(int64_t L, const double *temperature, const double *xnf_h,
               const double *xnf_he1, const double *xnf_h2, double *txnxn) {
    for (int64_t d = 0; d < L; d++) {
        double temp = temperature[d] > 1.0 ? temperature[d] : 1.0;
        double h = xnf_h ? xnf_h[d] : 0.0;
        double he = xnf_he1 ? xnf_he1[d] : 0.0;
        double h2 = xnf_h2 ? xnf_h2[d] : 0.0;
        txnxn[d] = (h + 0.42 * he + 0.85 * h2) * pow(temp / 10000.0, 0.3);
    }
}

/* line_opacity.py:56-184 _compute_transp_numba_kernel, with the Boltzmann
 * factor of populations.py:172 (FASTEX(ELO * HCKT)) computed in place.
 * Lines with process_mask == 0 are skipped (the routing rules of
 * line_opacity.py:740-784 are applied by the caller).  pop/dop are
 * [L, nion, nelem] C-order. */
void kso_transp(int64_t nl, int64_t L, const uint8_t *process_mask,
                const int32_t *element_idx, const int32_t *ion_stage,
                const int32_t *line_type, const double *wavelength,
                const double *gf, const double *cgf, const double *gamma_rad,
                const double *gamma_stark, const double *gamma_vdw,
                const double *elo_cm, const int64_t *center_idx,
                const double *hckt, const double *pop, const double *dop,
                int64_t nion, int64_t nelem, const double *rho, const double *xne,
                const double *txnxn, const double *cont_kapmin, int64_t n_wl,
                double cutoff, double microturb_kms, const double *h0tab,
                const double *h1tab, const double *h2tab, const double *extab,
                const double *extabf, double *transp, uint8_t *valid) {
    double micro = microturb_kms > 0.0 ? microturb_kms / C_LIGHT_KM : 0.0;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t li = 0; li < nl; li++) {
        for (int64_t d = 0; d < L; d++) {
            transp[li * L + d] = 0.0;
            valid[li * L + d] = 0;
        }
        if (!process_mask[li]) continue;
        int64_t e = element_idx[li];
        if (e < 0 || e >= nelem) continue;
        int64_t ion = ion_stage[li];
        if (ion <= 0 || ion > nion) continue;
        double lw = wavelength[li];
        int64_t c = center_idx[li];
        int64_t cc = c < 0 ? 0 : (c > n_wl - 1 ? n_wl - 1 : c);
        for (int64_t d = 0; d < L; d++) {
            double pop_val = pop[(d * nion + (ion - 1)) * nelem + e];
            double dop_val = dop[(d * nion + (ion - 1)) * nelem + e];
            if (micro > 0.0) dop_val = sqrt(dop_val * dop_val + micro * micro);
            if (pop_val <= 0.0 || dop_val <= 0.0) continue;
            double r = rho[d];
            if (r <= 0.0) continue;
            double xnfdop = pop_val / (r * dop_val);
            double doppler_width = dop_val * lw;
            double boltz = fast_ex(elo_cm[li] * hckt[d], extab, extabf);
            double k0pre;
            if (line_type[li] == 1) k0pre = gamma_vdw[li] * gf[li] * (pop_val / r);
            else k0pre = cgf[li] * xnfdop;
            double kapmin = cont_kapmin[d * n_wl + cc] * cutoff;
            if (k0pre < kapmin) continue;
            double post = k0pre * boltz;
            if (post < kapmin) continue;
            double kappa0 = post;
            if (kappa0 <= 0.0) continue;
            double dopple = lw > 0 ? doppler_width / lw : 1e-6;
            double adamp;
            if (doppler_width > 0 && dopple > 0) {
                double gt = gamma_rad[li] + gamma_stark[li] * xne[d] + gamma_vdw[li] * txnxn[d];
                adamp = gt / dopple;
            } else {
                adamp = 0.0;
            }
            if (adamp >= 0.0 && kappa0 > 0.0) {
                double kapcen;
                if (line_type[li] == 1) kapcen = kappa0;
                else if (adamp < 0.2) kapcen = kappa0 * (1.0 - 1.128 * adamp);
                else kapcen = kappa0 * kso_voigt(0.0, adamp, h0tab, h1tab, h2tab);
                transp[li * L + d] = kapcen;
                valid[li * L + d] = 1;
            }
        }
    }
}

/* -------------------------------------------------------------- ASYNTH --- */

/* Profile value at an offset in the near zone (line_opacity.py:474-491 and
 * :546-565), with the reference's incremental TABI carried by the caller. */
static inline double near_profile(int64_t off, double *tabi, double tabstep,
                                  double dvoigt, double adamp, double kappa0,
                                  const double *h0, const double *h1, const double *h2) {
    if (adamp < 0.2) {
        *tabi += tabstep;
        int64_t idx = (int64_t)(*tabi);
        if (idx < 0) idx = 0;
        double x = (double)off * dvoigt;
        if (x > 10.0) return kappa0 * (0.5642 * adamp / (x * x));
        if (idx >= VOIGT_N) idx = VOIGT_N - 1;
        return kappa0 * (h0[idx] + adamp * h1[idx]);
    }
    double x = (double)off * dvoigt;
    return kappa0 * kso_voigt(x, adamp, h0, h1, h2);
}

/* line_opacity.py:946-1340 compute_asynth_from_transp with its wing kernel
 * (:187-617), for plain lines (line_type 0).  Per depth: centre adds in line
 * order (:1091-1102), then wings in line order (:241-617), then x STIM
 * (:1338).  evals_per_depth receives the number of grid points written per
 * depth (centre + wings, the unit of work); maxstep_out (optional, [nl, L])
 * the wing reach of each pair, negated when the near-wing cutoff ended it
 * (no far wing). */
void kso_asynth(int64_t nl, int64_t L, const uint8_t *valid, const double *transp,
                const int32_t *line_type, const uint8_t *asynth_mask,
                const int32_t *ion_stage, const int32_t *element_idx,
                const double *wavelength, const int64_t *center_idx,
                const int64_t *wing_idx, const double *gamma_rad,
                const double *gamma_stark, const double *gamma_vdw,
                const double *dop, int64_t nion, int64_t nelem, const double *xne,
                const double *txnxn, const double *temperature,
                const double *cont_kapmin, const double *grid, int64_t n_wl,
                double cutoff, const double *h0, const double *h1, const double *h2,
                double *asynth, int64_t *evals_per_depth, int32_t *maxstep_out) {
    double resolu = 300000.0;
    if (n_wl > 1) {
        double ratio = grid[1] / grid[0];
        if (ratio > 1.0) resolu = 1.0 / (ratio - 1.0);
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t d = 0; d < L; d++) {
        double *row = asynth + d * n_wl;
        int64_t evals = 0;
        for (int64_t j = 0; j < n_wl; j++) row[j] = 0.0;
        /* centre contributions first (line_opacity.py:1091-1102) */
        for (int64_t li = 0; li < nl; li++) {
            if (!asynth_mask[li]) continue;
            int64_t c = center_idx[li];
            if (c >= 0 && c < n_wl && valid[li * L + d]) {
                row[c] += transp[li * L + d];
                evals++;
            }
        }
        /* wings (line_opacity.py:1141-1294 precompute + :241-617 kernel) */
        for (int64_t li = 0; li < nl; li++) {
            if (line_type[li] != 0) continue;
            int64_t e = element_idx[li];
            if (e < 0 || e >= nelem) continue;
            int64_t c = wing_idx[li];
            if (c < -MAX_PROFILE_STEPS || c > n_wl - 1 + MAX_PROFILE_STEPS) continue;
            if (!valid[li * L + d]) continue;
            double tv = transp[li * L + d];
            if (tv <= 0.0) continue;
            int64_t ion = ion_stage[li];
            if (ion > nion) continue;
            double pop_ok = 1.0; /* pop > 0 is implied by a valid TRANSP pair */
            (void)pop_ok;
            double dop_val = dop[(d * nion + (ion - 1)) * nelem + e];
            if (dop_val <= 0.0) continue;
            double lw = wavelength[li];
            double doppler_width = dop_val * lw;
            double dopple = lw > 0 ? doppler_width / lw : 1e-6;
            double adamp;
            if (dopple > 0 && lw > 0) {
                double gt = gamma_rad[li] + gamma_stark[li] * xne[d] + gamma_vdw[li] * txnxn[d];
                adamp = gt / dopple;
            } else {
                adamp = 0.0;
            }
            if (adamp < 1e-12) adamp = 1e-12;
            int64_t cc = c < 0 ? 0 : (c > n_wl - 1 ? n_wl - 1 : c);
            double kapmin_ref = cont_kapmin[d * n_wl + cc] * cutoff;
            double vc = adamp < 0.2 ? 1.0 - 1.128 * adamp : kso_voigt(0.0, adamp, h0, h1, h2);
            double kappa0 = vc > 0 ? tv / vc : tv;
            if (doppler_width <= 0.0) continue;
            /* kernel body (:416-617) */
            double dopple_k = lw > 0.0 ? doppler_width / lw : 1e-10;
            int64_t n10dop = (int64_t)(10.0 * dopple_k * resolu);
            double dvoigt = dopple_k > 0 ? 1.0 / (dopple_k * resolu) : 1.0;
            double tabstep = 200.0 * dvoigt;
            double tabi = 0.5;
            int64_t nstep_cutoff = -1;
            double prof_n10 = 0.0;
            for (int64_t ns = 1; ns <= n10dop; ns++) {
                double p = near_profile(ns, &tabi, tabstep, dvoigt, adamp, kappa0, h0, h1, h2);
                if (ns == n10dop) prof_n10 = p;
                if (p < kapmin_ref) {
                    nstep_cutoff = ns;
                    break;
                }
            }
            int64_t maxstep;
            int use_far = 0;
            double x_far = 0.0;
            if (nstep_cutoff != -1) {
                maxstep = nstep_cutoff;
            } else {
                use_far = 1;
                if (n10dop > 0 && prof_n10 > 0.0 && kapmin_ref > 0.0) {
                    x_far = prof_n10 * (double)n10dop * (double)n10dop;
                    maxstep = (int64_t)(sqrt(x_far / kapmin_ref) + 1.0);
                } else {
                    maxstep = 0;
                }
                if (maxstep > MAX_PROFILE_STEPS) maxstep = MAX_PROFILE_STEPS;
            }
            if (maxstep_out) maxstep_out[li * L + d] = (int32_t)(use_far ? maxstep : -maxstep);
            int red = 1, blue = 1;
            double tabo = 0.5;
            for (int64_t off = 1; off <= maxstep && (red || blue); off++) {
                double p;
                if (use_far && off > n10dop) p = x_far / ((double)off * (double)off);
                else p = near_profile(off, &tabo, tabstep, dvoigt, adamp, kappa0, h0, h1, h2);
                if (red) {
                    int64_t idx = c + off;
                    if (idx >= n_wl) red = 0;
                    else if (idx >= 0) { row[idx] += p; evals++; }
                }
                if (blue) {
                    int64_t idx = c - off;
                    if (idx < 0) blue = 0;
                    else if (idx < n_wl) { row[idx] += p; evals++; }
                }
            }
        }
        /* stim after accumulation (:1006-1016, :1067, :1338) */
        double t = temperature[d] > 1.0 ? temperature[d] : 1.0;
        double hkt = H_PLANCK / (K_BOLTZ * t);
        for (int64_t j = 0; j < n_wl; j++) {
            double freq = C_LIGHT_NM / grid[j];
            row[j] *= 1.0 - exp(-freq * hkt);
        }
        if (evals_per_depth) evals_per_depth[d] = evals;
    }
}

/* ------------------------------------------------------------- transfer -- */

/* josh_solver.py:96-167 _parcoe */
static void parcoe(const double *f, const double *x, int n, double *a, double *b, double *c) {
    for (int i = 0; i < n; i++) a[i] = b[i] = c[i] = 0.0;
    if (n == 0) return;
    if (n == 1) { a[0] = f[0]; return; }
    c[0] = 0.0;
    double den = x[1] - x[0];
    b[0] = den != 0.0 ? (f[1] - f[0]) / den : 0.0;
    a[0] = f[0] - x[0] * b[0];
    int n1 = n - 1;
    c[n - 1] = 0.0;
    den = x[n - 1] - x[n1 - 1];
    b[n - 1] = den != 0.0 ? (f[n - 1] - f[n1 - 1]) / den : 0.0;
    a[n - 1] = f[n - 1] - x[n - 1] * b[n - 1];
    if (n == 2) return;
    for (int j = 1; j < n1; j++) {
        int j1 = j - 1;
        den = x[j] - x[j1];
        double d = den != 0.0 ? (f[j] - f[j1]) / den : 0.0;
        double den1 = (x[j + 1] - x[j]) * (x[j + 1] - x[j1]);
        double term1 = den1 != 0.0 ? f[j + 1] / den1 : 0.0;
        double den2 = x[j + 1] - x[j1];
        double den3 = x[j + 1] - x[j];
        double den4 = x[j] - x[j1];
        double part = 0.0;
        if (den4 != 0.0) {
            double t1 = den2 != 0.0 ? f[j1] / den2 : 0.0;
            double t2 = den3 != 0.0 ? f[j] / den3 : 0.0;
            part = (t1 - t2) / den4;
        }
        c[j] = term1 + part;
        b[j] = d - (x[j] + x[j1]) * c[j];
        a[j] = f[j1] - x[j1] * d + x[j] * x[j1] * c[j];
    }
    c[1] = 0.0;
    den = x[2] - x[1];
    b[1] = den != 0.0 ? (f[2] - f[1]) / den : 0.0;
    a[1] = f[1] - x[1] * b[1];
    if (n > 3) {
        c[2] = 0.0;
        den = x[3] - x[2];
        b[2] = den != 0.0 ? (f[3] - f[2]) / den : 0.0;
        a[2] = f[2] - x[2] * b[2];
    }
    for (int j = 1; j < n1; j++) {
        if (c[j] == 0.0) continue;
        int j1 = j + 1 < n - 1 ? j + 1 : n - 1;
        double den5 = fabs(c[j1]) + fabs(c[j]);
        double wt = den5 > 0.0 ? fabs(c[j1]) / den5 : 0.0;
        a[j] = a[j1] + wt * (a[j] - a[j1]);
        b[j] = b[j1] + wt * (b[j] - b[j1]);
        c[j] = c[j1] + wt * (c[j] - c[j1]);
    }
    a[n1 - 1] = a[n - 1];
    b[n1 - 1] = b[n - 1];
    c[n1 - 1] = c[n - 1];
}

/* josh_solver.py:171-189 _integ */
static void integ(const double *x, const double *f, int n, double start, double *fint) {
    double a[256], b[256], c[256];
    if (n == 0) return;
    parcoe(f, x, n, a, b, c);
    fint[0] = start;
    for (int i = 0; i < n - 1; i++) {
        double dx = x[i + 1] - x[i];
        double term = a[i] + 0.5 * b[i] * (x[i + 1] + x[i]);
        term += (c[i] / 3.0) * ((x[i + 1] + x[i]) * x[i + 1] + x[i] * x[i]);
        fint[i + 1] = fint[i] + term * dx;
    }
}

/* josh_solver.py:193-217 _deriv */
static void deriv(const double *x, const double *f, int n, double *dfdx) {
    for (int i = 0; i < n; i++) dfdx[i] = 0.0;
    if (n < 2) return;
    dfdx[0] = (f[1] - f[0]) / (x[1] - x[0]);
    dfdx[n - 1] = (f[n - 1] - f[n - 2]) / (x[n - 1] - x[n - 2]);
    if (n == 2) return;
    double s = x[1] != x[0] ? fabs(x[1] - x[0]) / (x[1] - x[0]) : 1.0;
    for (int j = 1; j < n - 1; j++) {
        double scale = fabs(f[j - 1]);
        if (fabs(f[j]) > scale) scale = fabs(f[j]);
        if (fabs(f[j + 1]) > scale) scale = fabs(f[j + 1]);
        scale = x[j] != 0.0 ? scale / fabs(x[j]) : scale;
        if (scale == 0.0) scale = 1.0;
        double d1 = (f[j + 1] - f[j]) / (x[j + 1] - x[j]) / scale;
        double d0 = (f[j] - f[j - 1]) / (x[j] - x[j - 1]) / scale;
        double tan1 = d1 / (s * sqrt(1.0 + d1 * d1) + 1.0);
        double tan0 = d0 / (s * sqrt(1.0 + d0 * d0) + 1.0);
        dfdx[j] = (tan1 + tan0) / (1.0 - tan1 * tan0) * scale;
    }
}

/* josh_solver.py:220-353 _map1_kernel (the JOSH variant of MAP1).
 * Returns MAXJ (= ll - 1). */
static int map1_josh(const double *xold, const double *fold, int nold,
                     const double *xnew, int nnew, double *fnew) {
    double x1[257], f1[257];
    for (int i = 0; i < nnew; i++) fnew[i] = 0.0;
    if (nold == 0 || nnew == 0) return 0;
    for (int i = 0; i < nold; i++) {
        x1[i + 1] = xold[i];
        f1[i + 1] = fold[i];
    }
    int l = 2, ll = 0;
    double cfor = 0, bfor = 0, afor = 0, cbac = 0, bbac = 0, abac = 0;
    double a = 0, b = 0, c = 0;
    for (int k = 1; k <= nnew; k++) {
        double xk = xnew[k - 1];
        for (;;) {
            if (xk < x1[l]) {
                if (l == ll) break;
                if (l == 2 || l == 3) {
                    l = l < nold ? l : nold;
                    c = 0.0;
                    b = (f1[l] - f1[l - 1]) / (x1[l] - x1[l - 1]);
                    a = f1[l] - x1[l] * b;
                    ll = l;
                    break;
                }
                int l1 = l - 1;
                if (l > ll + 1 || l == 4) {
                    int l2 = l - 2;
                    double d = (f1[l1] - f1[l2]) / (x1[l1] - x1[l2]);
                    cbac = f1[l] / ((x1[l] - x1[l1]) * (x1[l] - x1[l2])) +
                           (f1[l2] / (x1[l] - x1[l2]) - f1[l1] / (x1[l] - x1[l1])) /
                               (x1[l1] - x1[l2]);
                    bbac = d - (x1[l1] + x1[l2]) * cbac;
                    abac = f1[l2] - x1[l2] * d + x1[l1] * x1[l2] * cbac;
                    if (!(l < nold)) {
                        c = cbac; b = bbac; a = abac; ll = l;
                        break;
                    }
                } else {
                    cbac = cfor; bbac = bfor; abac = afor;
                    if (l == nold) {
                        c = cbac; b = bbac; a = abac; ll = l;
                        break;
                    }
                }
                double d = (f1[l] - f1[l1]) / (x1[l] - x1[l1]);
                cfor = f1[l + 1] / ((x1[l + 1] - x1[l]) * (x1[l + 1] - x1[l1])) +
                       (f1[l1] / (x1[l + 1] - x1[l1]) - f1[l] / (x1[l + 1] - x1[l])) /
                           (x1[l] - x1[l1]);
                bfor = d - (x1[l] + x1[l1]) * cfor;
                afor = f1[l1] - x1[l1] * d + x1[l] * x1[l1] * cfor;
                double wt = 0.0;
                if (fabs(cfor) != 0.0) wt = fabs(cfor) / (fabs(cfor) + fabs(cbac));
                a = afor + wt * (abac - afor);
                b = bfor + wt * (bbac - bfor);
                c = cfor + wt * (cbac - cfor);
                ll = l;
                break;
            }
            l += 1;
            if (l > nold) {
                l = nold;
                c = 0.0;
                b = (f1[l] - f1[l - 1]) / (x1[l] - x1[l - 1]);
                a = f1[l] - x1[l] * b;
                ll = l;
                break;
            }
        }
        fnew[k - 1] = a + (b + c * xk) * xk;
    }
    return ll - 1;
}

/* josh_solver.py:24-92 _josh_iteration_kernel in float32 (the reference
 * casts every operand to float32 before the call, :670-686). */
static int josh_iterate_f32(const float *coefj, const float *cdiag, float *xs,
                            const float *xalpha, const float *xsbar_mod) {
    float diag[NXTAU];
    const float tol = 1.0e-5f;
    const float eps = 1.0e-38f;
    for (int k = 0; k < NXTAU; k++) diag[k] = 1.0f - xalpha[k] * cdiag[k];
    for (int it = 0; it < NXTAU; it++) {
        int iferr = 0;
        for (int k = NXTAU - 1; k >= 0; k--) {
            float delxs = 0.0f;
            for (int m = 0; m < NXTAU; m++) delxs += coefj[k * NXTAU + m] * xs[m];
            delxs = (delxs * xalpha[k] + xsbar_mod[k] - xs[k]) / diag[k];
            float errorx = xs[k] != 0.0f ? fabsf(delxs / xs[k]) : INFINITY;
            if (errorx > tol) iferr = 1;
            float nv = xs[k] + delxs;
            xs[k] = nv > eps ? nv : eps;
        }
        if (!iferr) return it + 1;
    }
    return NXTAU;
}

typedef struct {
    const double *xtau, *ch, *coefj;
    float coefj32[NXTAU * NXTAU];
    float cdiag32[NXTAU];
} josh_tables_t;

/* Exact-sweep mode (not the reference's arithmetic): the JOSH system
 * (I - diag(xalpha) COEFJ) xs = xsbar (1 - xalpha) solved in FP64 by
 * Gauss-Seidel to 1e-13 instead of the reference's FP32 sweep with its 1e-5
 * stop (josh_solver.py:24-92), so that the fluxes are smooth in the inputs
 * and can be differenced to check gradients. */
static int g_exact_sweeps = 0;
void kso_set_exact_sweeps(int on) { g_exact_sweeps = on ? 1 : 0; }

static int josh_iterate_exact(const double *coefj, double *xs, const double *xalpha, const double *xsbar_mod) {
    for (int it = 0; it < 2000; it++) {
        double dmax = 0.0;
        for (int k = NXTAU - 1; k >= 0; k--) {
            double sum = 0.0;
            for (int m = 0; m < NXTAU; m++) sum += coefj[k * NXTAU + m] * xs[m];
            double nv = sum * xalpha[k] + xsbar_mod[k];
            double d = fabs(nv - xs[k]) / fmax(fabs(nv), 1e-300);
            if (d > dmax) dmax = d;
            xs[k] = nv;
        }
        if (dmax < 1e-13) return it + 1;
    }
    return 2000;
}

/* josh_solver.py:367-767 solve_josh_flux (IFSCAT=1 path, surface flux). */
static double solve_josh(const josh_tables_t *T, int n, const double *acont,
                         const double *scont, const double *aline, const double *sline,
                         const double *sigmac, const double *sigmal, const double *rho,
                         int *iters_out) {
    double abtot[256] = {0}, alpha[256] = {0}, snubar[256] = {0}, taunu[256] = {0};
    if (n <= 0 || n > 256) return 0.0;
    for (int j = 0; j < n; j++) {
        double ab = acont[j] + aline[j] + sigmac[j] + sigmal[j];
        abtot[j] = ab > EPS ? ab : EPS;
        if (isnan(ab)) abtot[j] = ab;
        double sc = sigmac[j] + sigmal[j];
        double al = abtot[j] > 0.0 ? sc / abtot[j] : 0.0;
        alpha[j] = al < 0.0 ? 0.0 : (al > 1.0 ? 1.0 : al);
        double den = acont[j] + aline[j];
        snubar[j] = den > 0 ? (acont[j] * scont[j] + aline[j] * sline[j]) / den : scont[j];
    }
    int rev = n > 1 && rho[0] > rho[n - 1];
    double rhoi[256] = {0}, abi[256] = {0};
    double start;
    for (int j = 0; j < n; j++) {
        rhoi[j] = rev ? rho[n - 1 - j] : rho[j];
        abi[j] = rev ? abtot[n - 1 - j] : abtot[j];
    }
    start = abi[rev ? n - 1 : 0] * rhoi[rev ? n - 1 : 0];
    integ(rhoi, abi, n, start, taunu);
    if (rev) {
        for (int j = 0; j < n / 2; j++) {
            double t = snubar[j]; snubar[j] = snubar[n - 1 - j]; snubar[n - 1 - j] = t;
            t = alpha[j]; alpha[j] = alpha[n - 1 - j]; alpha[n - 1 - j] = t;
        }
    }
    const double *xtau = T->xtau;
    int force401 = taunu[0] > xtau[NXTAU - 1];
    double xsbar[NXTAU], xalpha[NXTAU], xs[NXTAU];
    if (!force401) {
        map1_josh(taunu, snubar, n, xtau, NXTAU, xsbar);
        map1_josh(taunu, alpha, n, xtau, NXTAU, xalpha);
        for (int l = 0; l < NXTAU; l++) {
            if (xsbar[l] < EPS) xsbar[l] = EPS;
            xalpha[l] = xalpha[l] < 0.0 ? 0.0 : (xalpha[l] > 1.0 ? 1.0 : xalpha[l]);
        }
        for (int l = 0; l < NXTAU; l++) {
            if (xtau[l] < taunu[0]) {
                xsbar[l] = snubar[0] > EPS ? snubar[0] : EPS;
                xalpha[l] = alpha[0] < 0.0 ? 0.0 : (alpha[0] > 1.0 ? 1.0 : alpha[0]);
            }
        }
        if (g_exact_sweeps) {
            double xm[NXTAU];
            for (int l = 0; l < NXTAU; l++) {
                xs[l] = xsbar[l];
                xm[l] = xsbar[l] * (1.0 - xalpha[l]);
            }
            int it = josh_iterate_exact(T->coefj, xs, xalpha, xm);
            if (iters_out) *iters_out = it;
            double flux = 0.0;
            for (int l = 0; l < NXTAU; l++) flux += T->ch[l] * xs[l];
            return flux;
        }
        float xs32[NXTAU], xa32[NXTAU], xm32[NXTAU];
        for (int l = 0; l < NXTAU; l++) {
            xs32[l] = (float)xsbar[l];
            xa32[l] = (float)xalpha[l];
            xm32[l] = (float)(xsbar[l] * (1.0 - xalpha[l]));
        }
        int it = josh_iterate_f32(T->coefj32, T->cdiag32, xs32, xa32, xm32);
        if (iters_out) *iters_out = it;
        for (int l = 0; l < NXTAU; l++) xs[l] = (double)xs32[l];
        double flux = 0.0;
        for (int l = 0; l < NXTAU; l++) flux += T->ch[l] * xs[l];
        return flux;
    }
    /* MAXJ = 1 (label 401) path, :700-727 */
    double snu[256], hnu[256], jm[256], jnu[256];
    for (int j = 0; j < n; j++) snu[j] = snubar[j];
    int it_done = 0;
    for (int it = 0; it < NXTAU; it++) {
        deriv(taunu, snu, n, hnu);
        for (int j = 0; j < n; j++) hnu[j] = hnu[j] / 3.0;
        deriv(taunu, hnu, n, jm);
        double err = 0.0;
        double snew[256];
        for (int j = 0; j < n; j++) {
            jnu[j] = jm[j] + snu[j];
            snew[j] = (1.0 - alpha[j]) * snubar[j] + alpha[j] * jnu[j];
            double den = fabs(snew[j]) > EPS ? fabs(snew[j]) : EPS;
            err += fabs(snew[j] - snu[j]) / den;
        }
        for (int j = 0; j < n; j++) snu[j] = snew[j];
        it_done = it + 1;
        if (err < 1.0e-5) break;
    }
    if (iters_out) *iters_out = -it_done;
    return hnu[0];
}

/* radiative.py:20-39 _planck_nu */
static double planck_nu(double freq, double t) {
    double freq15 = freq / 1.0e15;
    double hkt = H_PLANCK / (K_BOLTZ * t);
    double ehvkt = exp(-freq * hkt);
    double stim = 1.0 - ehvkt;
    double bnu = 1.47439e-2 * pow(freq15, 3.0) * ehvkt / stim;
    if (isnan(bnu)) bnu = 0.0;
    return bnu;
}

/* radiative.py:42-218 solve_lte_frequency, driven per wavelength as in
 * solve_lte_spectrum (:282-494).  Field arrays are [L, n] C-order.
 * line_source may be NULL (Planck).  iters (optional, [n, 2]) receives the
 * scattering-iteration counts of the continuum and total solves. */
void kso_transfer(int64_t L, int64_t n, const double *wavelength,
                  const double *temperature, const double *column_mass,
                  const double *cont_abs, const double *cont_scat,
                  const double *line_opacity, const double *line_scattering,
                  const double *line_source, const double *xtau, const double *ch,
                  const double *coefj, double *flux_total, double *flux_cont,
                  int32_t *iters) {
    josh_tables_t T;
    T.xtau = xtau;
    T.ch = ch;
    T.coefj = coefj;
    for (int i = 0; i < NXTAU * NXTAU; i++) T.coefj32[i] = (float)coefj[i];
    for (int i = 0; i < NXTAU; i++) T.cdiag32[i] = (float)coefj[i * NXTAU + i];
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < n; j++) {
        double mass[256], temp[256], ca[256], cs[256], la[256], ls_[256], src[256];
        int m = 0;
        double freq = C_LIGHT_NM / (wavelength[j] > 1e-12 ? wavelength[j] : 1e-12);
        for (int64_t d = 0; d < L; d++) {
            double cm = column_mass[d];
            double a = cont_abs[d * n + j], s = cont_scat[d * n + j];
            double lo = line_opacity[d * n + j], lsg = line_scattering[d * n + j];
            int ok = cm >= 0.0 && isfinite(cm) && isfinite(a) && isfinite(s) &&
                     isfinite(lo) && isfinite(lsg) && a < MAX_OPACITY_REAL4 &&
                     s < MAX_OPACITY_REAL4 && lo < MAX_OPACITY_REAL4 &&
                     lsg < MAX_OPACITY_REAL4;
            if (!ok || !(cm > 0)) continue;
            mass[m] = cm;
            temp[m] = temperature[d];
            ca[m] = a;
            cs[m] = s;
            la[m] = lo;
            ls_[m] = lsg;
            if (line_source) {
                double v = line_source[d * n + j];
                if (!isfinite(v)) v = planck_nu(freq, temperature[d]);
                src[m] = v;
            }
            m++;
        }
        if (m == 0) {
            flux_total[j] = 0.0;
            flux_cont[j] = 0.0;
            continue;
        }
        if (m > 1 && !(mass[0] < mass[m - 1])) {
            for (int q = 0; q < m / 2; q++) {
#define SWP(arr) { double t_ = arr[q]; arr[q] = arr[m - 1 - q]; arr[m - 1 - q] = t_; }
                SWP(mass) SWP(temp) SWP(ca) SWP(cs) SWP(la) SWP(ls_)
                if (line_source) SWP(src)
#undef SWP
            }
        }
        double planck[256], zero[256];
        for (int q = 0; q < m; q++) {
            planck[q] = planck_nu(freq, temp[q]);
            zero[q] = 0.0;
        }
        const double *lsrc = line_source ? src : planck;
        int itc = 0, itt = 0;
        flux_cont[j] = solve_josh(&T, m, ca, planck, zero, planck, cs, zero, mass, &itc);
        flux_total[j] = solve_josh(&T, m, ca, planck, la, lsrc, cs, ls_, mass, &itt);
        if (iters) {
            iters[2 * j] = itc;
            iters[2 * j + 1] = itt;
        }
    }
}

/* opacity.py:2215-2228 + bfudge.py:143-145: SLINEC = BNU*STIM/(1-EHVKT) with
 * BFUDGE = 1 (LTE), the line source used in ASYNTH mode (opacity.py:3678). */
void kso_line_source(int64_t L, int64_t n, const double *wavelength,
                     const double *temperature, double *slinec) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double freq = C_LIGHT_CM / (wavelength[j] * 1.0e-7);
        double freq15 = freq / 1.0e15;
        double f3 = pow(freq15, 3.0);
        for (int64_t d = 0; d < L; d++) {
            double hkt = H_PLANCK / (K_BOLTZ * temperature[d]);
            double ehvkt = exp(-freq * hkt);
            double stim = 1.0 - ehvkt;
            double bnu = 1.47439e-02 * f3 * ehvkt / stim;
            slinec[d * n + j] = (bnu * stim) / (1.0 - ehvkt);
        }
    }
}
