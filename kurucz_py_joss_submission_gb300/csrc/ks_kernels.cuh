// ks_kernels.cuh -- the GB300 kernels of the line-opacity and transfer path,
// templated on the working type R (float: KS_PREC_MIXED, double:
// KS_PREC_FP64).  Included by ks_f32.cu and ks_f64.cu, which instantiate one
// type each (the FP64 unit is compiled without multiply-add contraction so
// its rounding follows the reference's separately rounded operations).
//
// Kernels, in pipeline order:
//   prep_depth_kernel     per-depth state and the (depth, ion, element) table
//   continuum_kernel      ACONT/SIGMAC on the grid        (continuum.py:73)
//   pair_setup_kernel     TRANSP gates + wing descriptor  (line_opacity.py:56,1141,416)
//   accumulate_kernel     ASYNTH on lambda tiles           (line_opacity.py:187,1091,1338)
//   transfer_kernel       JOSH surface flux per lambda     (radiative.py:42, josh_solver.py:367)
#pragma once

#include "ks_common.cuh"
#include "ks_internal.h"
#include "ks_launch.h"

namespace ks {

// ---------------------------------------------------------------------------
// per-depth preparation
// ---------------------------------------------------------------------------

// One thread per (depth, ion, element) entry; entry 0 of each depth also
// fills the per-depth record.  populations.py:196-204 (TXNXN),
// line_opacity.py:124-136 (XNFDOP = pop / (rho dop), microturbulence added to
// DOPPLE for TRANSP only), :416-420 and :465 (N10DOP, DVOIGT from
// DOPPLE = doppler width / wavelength).
template <typename R>
__device__ __forceinline__ void prep_depth_kernel_body(VB vb, const PrepArgs& a) {
    int64_t per_depth = (int64_t)a.n_ion * a.n_elem;
    int64_t i = (int64_t)vb.x * blockDim.x + threadIdx.x;
    if (a.abs_coeff_f) {
        const int64_t stride = (int64_t)vb.gx * blockDim.x;
        for (int64_t k = i; k < a.n_coeff; k += stride) {
            a.abs_coeff_f[k] = (float)a.abs_coeff[k];
            a.scat_coeff_f[k] = (float)a.scat_coeff[k];
        }
    }
    if (i >= (int64_t)a.n_layers * per_depth) return;
    int d = (int)(i / per_depth);
    double temp_raw = a.temperature[d];
    double rho = a.mass_density[d];
    if (i % per_depth == 0) {
        DepthPar p;
        double temp = temp_raw > 1.0 ? temp_raw : 1.0;
        double h = a.xnf_h ? a.xnf_h[d] : 0.0;
        double he = a.xnf_he1 ? a.xnf_he1[d] : 0.0;
        double h2 = a.xnf_h2 ? a.xnf_h2[d] : 0.0;
        p.txnxn = (h + 0.42 * he + 0.85 * h2) * pow(temp / 10000.0, 0.3);
        p.rho = rho;
        p.xne = a.electron_density[d];
        p.hckt = a.hckt[d];
        p.hkt_asynth = H_PLANCK / (K_BOLTZ * temp);
        p.hkt = H_PLANCK / (K_BOLTZ * temp_raw);
        p.temperature = temp_raw;
        p.rhox = a.rhox[d];
        p.fscat = a.rhoxj > 0.0 ? exp(-p.rhox / a.rhoxj) : 0.0;
        p.hckt_hi = (float)p.hckt;
        p.hckt_lo = (float)(p.hckt - (double)p.hckt_hi);
        p.xne_f = (float)p.xne;
        p.txnxn_f = (float)p.txnxn;
        p.hkt_f = (float)p.hkt;
        p.rhox_f = (float)p.rhox;
        p.fscat_f = (float)p.fscat;
        p.pad = 0.f;
        a.depth[d] = p;
    }
    double pop = a.population[i];
    double dop = a.doppler[i];
    double micro = a.microturb_kms > 0.0 ? a.microturb_kms / C_LIGHT_KM : 0.0;
    double dop_t = micro > 0.0 ? sqrt(dop * dop + micro * micro) : dop;
    IonPar q;
    q.pop = pop;
    q.dop = dop;
    q.dop_transp = dop_t;
    q.xnfdop = (pop > 0.0 && dop_t > 0.0 && rho > 0.0) ? pop / (rho * dop_t) : 0.0;
    const double resolu = a.gp->resolu;
    int64_t n10 = dop > 0.0 ? (int64_t)(10.0 * dop * resolu) : 0;
    q.n10dop = (int)(n10 > 0x7fffffff ? 0x7fffffff : n10);
    q.dvoigt = dop > 0.0 ? 1.0 / (dop * resolu) : 1.0;
    q.xnfdop_f = (float)q.xnfdop;
    q.dop_f = (float)dop_t;
    q.dvoigt_f = (float)q.dvoigt;
    q.pop_over_rho_f = rho > 0.0 ? (float)(pop / rho) : 0.0f;
    q.dopw_f = (float)dop;
    q.ok = ((pop > 0.0 && dop_t > 0.0 && rho > 0.0) ? 1 : 0) | ((pop > 0.0 && dop > 0.0) ? 2 : 0);
    a.ion[i] = q;
}
template <typename R>
__global__ void prep_depth_kernel(PrepArgs a) {
    prep_depth_kernel_body<R>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a);
}


// ---------------------------------------------------------------------------
// continuum
// ---------------------------------------------------------------------------

// One thread per wavelength, looping over depths so the edge search and the
// Lagrange weights are computed once per wavelength.  continuum.py:146-256.
template <typename R>
__device__ __forceinline__ void continuum_kernel_body(VB vb, const ContArgs& a, R* __restrict__ cont_abs, R* __restrict__ cont_scat) {
    int64_t j = (int64_t)vb.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    double w = a.grid[j];
    double aw = fabs(w);
    int lo = 0, hi = a.n_edge;
    while (lo < hi) {  // searchsorted(|wledge|, |w|, side="right")
        int mid = (lo + hi) >> 1;
        if (fabs(a.wledge[mid]) <= aw) lo = mid + 1; else hi = mid;
    }
    int e = lo - 1;
    e = e < 0 ? 0 : (e > a.n_edge - 2 ? a.n_edge - 2 : e);
    double left = fabs(a.wledge[e]);
    double right = fabs(a.wledge[e + 1]);
    double half = a.half_edge ? a.half_edge[e] : 0.5 * (left + right);
    double delta = a.delta_edge ? a.delta_edge[e] : 0.5 * (right - left) * (right - left);
    if (delta == 0.0) delta = 1e-20;
    double c1 = (w - half) * (w - right) / delta;
    double c2 = (left - w) * (w - right) * 2.0 / delta;
    double c3 = (w - left) * (w - half) / delta;
    if (a.freq_f) a.freq_f[j] = (float)(C_LIGHT_NM / w);
    const int nseg = a.n_edge - 1;
    for (int d = 0; d < a.n_layers; d++) {
        const double* ca = a.abs_coeff + ((int64_t)d * nseg + e) * 3;
        const double* cs = a.scat_coeff + ((int64_t)d * nseg + e) * 3;
        R la, ls;
        if (sizeof(R) == 8) {
            la = (R)(ca[0] * c1 + ca[1] * c2 + ca[2] * c3);
            ls = (R)(cs[0] * c1 + cs[1] * c2 + cs[2] * c3);
        } else {
            float fc1 = (float)c1, fc2 = (float)c2, fc3 = (float)c3;
            if (a.abs_coeff_f) {  // tables already in single precision
                const float* fa = a.abs_coeff_f + ((int64_t)d * nseg + e) * 3;
                const float* fs = a.scat_coeff_f + ((int64_t)d * nseg + e) * 3;
                la = (R)(fa[0] * fc1 + fa[1] * fc2 + fa[2] * fc3);
                ls = (R)(fs[0] * fc1 + fs[1] * fc2 + fs[2] * fc3);
            } else {
                la = (R)((float)ca[0] * fc1 + (float)ca[1] * fc2 + (float)ca[2] * fc3);
                ls = (R)((float)cs[0] * fc1 + (float)cs[1] * fc2 + (float)cs[2] * fc3);
            }
        }
        if (a.coeff_log10) {
            la = la > R(38) ? R(38) : la;
            ls = ls > R(38) ? R(38) : ls;
            if (sizeof(R) == 8) {
                la = (R)pow(10.0, (double)la);
                ls = (R)pow(10.0, (double)ls);
            } else {
                la = (R)exp10f((float)la);
                ls = (R)exp10f((float)ls);
            }
            const R mx = (R)MAX_OPACITY_REAL4;
            la = la < R(0) ? R(0) : (la > mx ? mx : la);
            ls = ls < R(0) ? R(0) : (ls > mx ? mx : ls);
            if (!isfinite(la)) la = mx;
            if (!isfinite(ls)) ls = mx;
        }
        cont_abs[(int64_t)d * a.n + j] = la;
        cont_scat[(int64_t)d * a.n + j] = ls;
    }
}
template <typename R>
__global__ void continuum_kernel(ContArgs a, R* __restrict__ cont_abs, R* __restrict__ cont_scat) {
    continuum_kernel_body<R>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a, cont_abs, cont_scat);
}


// ---------------------------------------------------------------------------
// pair setup: TRANSP gates + wing descriptor
// ---------------------------------------------------------------------------

// FASTEX (tables.py:29-42): exp(-x) from the EXTAB/EXTABF tables, in FP64.
__device__ __forceinline__ double fast_ex(double x, const double* __restrict__ extab,
                                          const double* __restrict__ extabf) {
    if (x <= 0.0) return x == 0.0 ? 1.0 : exp(-x);
    double fl = floor(x);
    if (fl >= (double)EXP_N) return exp(-x);
    int i = (int)fl;
    double frac = __dadd_rn(x, -(double)i);
    int j = (int)__dadd_rn(__dmul_rn(frac, 1000.0), 0.5);
    j = j < 0 ? 0 : (j > EXP_N - 1 ? EXP_N - 1 : j);
    return __dmul_rn(extab[i], extabf[j]);
}

// FASTEX for the mixed path.  The table cell (i, j) must be the one the
// FP64 reference picks, so x = ELO*HCKT is formed as an unevaluated float
// sum p + lo (error ~1e-14 relative) and j = int(frac*1000 + 0.5) is taken
// from it; only when that value lies within 2e-4 of an integer -- where
// single precision cannot decide -- is the index recomputed in FP64.
__device__ __forceinline__ float fast_ex_mixed(float e_hi, float e_lo, float h_hi, float h_lo,
                                               double elo, double hckt,
                                               const float* __restrict__ extab,
                                               const float* __restrict__ extabf) {
    float p = e_hi * h_hi;
    float perr = fmaf(e_hi, h_hi, -p);
    float lo = perr + (e_hi * h_lo + e_lo * h_hi);
    if (!(p > 0.0f)) {
        double x = elo * hckt;
        if (x <= 0.0) return x == 0.0 ? 1.0f : (float)exp(-x);
    }
    float fi = floorf(p);
    float r = (p - fi) + lo;
    if (r < 0.0f) { fi -= 1.0f; r += 1.0f; }
    else if (r >= 1.0f) { fi += 1.0f; r -= 1.0f; }
    if (fi >= (float)EXP_N) return __expf(-(p + lo));
    float t = r * 1000.0f + 0.5f;
    float tr = rintf(t);
    int i = (int)fi, j;
    if (fabsf(t - tr) < 2.0e-4f || fi < 0.0f) {
        double x = __dmul_rn(elo, hckt);
        double fl = floor(x);
        if (fl >= (double)EXP_N) return (float)exp(-x);
        i = (int)fl;
        double frac = __dadd_rn(x, -(double)i);
        j = (int)__dadd_rn(__dmul_rn(frac, 1000.0), 0.5);
    } else {
        j = (int)t;
    }
    j = j < 0 ? 0 : (j > EXP_N - 1 ? EXP_N - 1 : j);
    return extab[i] * extabf[j];
}

// Voigt table index of near-wing step `off` (ADAMP < 0.2).  The reference
// carries TABI incrementally, TABI = 0.5, then TABI += TABSTEP per step
// (line_opacity.py:474-480, :546-552), and takes int(TABI).  The closed form
// 0.5 + off*TABSTEP has the same integer part unless the sum lies within its
// accumulated rounding of an integer: each of the `off` additions rounds by
// at most half an ulp of a value <= TABI, the closed form by about one ulp.
// FP64: inside that band the incremental sum is replayed, so the index is
// the reference's; outside it (all but ~1e-10 of the steps) the closed form
// is used.  FP32 (mixed path): the closed form; an index one off at a tie is
// within the mixed contract.
template <typename R>
__device__ __forceinline__ int tabi_index(int off, R tabstep) {
    if constexpr (sizeof(R) == 8) {
        const double t = __dadd_rn(0.5, __dmul_rn((double)off, tabstep));
        const double fl = floor(t);
        const double ulp = t >= 1.0 ? ldexp(1.0, ilogb(t) - 52) : 0x1p-53;
        const double band = (0.5 * (double)off + 2.0) * ulp;
        if (t - fl > band && fl + 1.0 - t > band) return (int)t;
        double s = 0.5;
        for (int k = 0; k < off; k++) s = __dadd_rn(s, tabstep);
        return (int)s;
    } else {
        return (int)(R(0.5) + (R)off * tabstep);
    }
}

// Near-zone wing profile at step `off` (line_opacity.py:474-491, :546-565).
template <typename R>
__device__ __forceinline__ R near_profile(int off, R dvoigt, R adamp, R kappa0,
                                          const R* __restrict__ h0, const R* __restrict__ h1,
                                          const R* __restrict__ h2) {
    R x = (R)off * dvoigt;
    if (adamp < R(0.2)) {
        if (x > R(10)) return kappa0 * (R(0.5642) * adamp / (x * x));
        int idx = tabi_index<R>(off, R(200) * dvoigt);
        idx = idx < 0 ? 0 : (idx > VOIGT_N - 1 ? VOIGT_N - 1 : idx);
        return kappa0 * (h0[idx] + adamp * h1[idx]);
    }
    return kappa0 * voigt_hv<R>(x, adamp, h0, h1, h2);
}

// One thread per (line, depth): depth = blockIdx.y, line = x index in the
// catalog's (wavelength-sorted) order.  In the fused mode it evaluates the
// TRANSP gates itself (line_opacity.py:101-184, Boltzmann factor from
// populations.py:172); in the seam mode it takes TRANSP/valid as given
// (compute_asynth_from_transp).  Then it recovers the wing parameters
// (:1141-1272), scans the near wing for the KAPMIN cutoff (:474-537) and
// writes the pair's descriptor and reach class (0xff: no contribution).
// FP64 instantiation: the reference's arithmetic operation by operation.
// FP32 instantiation: single precision after exact FASTEX table indices.
// First half of one (line, depth) pair: the TRANSP gates and the centre
// add.  Returns true when the pair still needs its wings (pair_wings), with
// KAPCEN, the wing kappa0 and the centre code; otherwise the pair is
// finished (no contribution, or a centre-only descriptor written here).
template <typename R, bool FUSED>
__device__ __forceinline__ bool pair_gate(const PairArgs& a, const R* __restrict__ kap_a,
                                          const R* __restrict__ kap_b, PairDesc<R>* __restrict__ desc,
                                          uint8_t* __restrict__ cls, int64_t li, int d, R& kc_out,
                                          R& k0_out, int& code_out, float& num_out, int& qi_out) {
    constexpr bool F32 = sizeof(R) == 4;
    const int L = a.n_layers;
    int64_t slot = (int64_t)d * a.stride + li;
    cls[slot] = 0xff;
    if (FUSED && a.transp_out) {
        a.transp_out[li * L + d] = 0.0;
        a.valid_out[li * L + d] = 0;
    }
    const int e = a.element_idx[li];
    const int ion = a.ion_stage[li];
    const int lt = a.line_type[li];
    if (e < 0 || e >= a.n_elem || ion <= 0 || ion > a.n_ion) return false;
    const DepthPar& dp = a.depth[d];
    const int qi = (d * a.n_ion + (ion - 1)) * a.n_elem + e;
    const IonPar& q = a.ion[qi];
    const int c_ctr = a.center_idx[li];
    const int c_wing = a.wing_idx[li];
    const int64_t nwl = a.n_wl;
    auto kap_at = [&](int c) -> R {
        int cc = c < 0 ? 0 : (c > (int)nwl - 1 ? (int)nwl - 1 : c);
        R v = kap_a[(int64_t)d * nwl + cc];
        if (kap_b) v += kap_b[(int64_t)d * nwl + cc];
        return v;
    };

    // ---------------- TRANSP (line_opacity.py:101-184) ----------------
    float num = 0.0f;  // FP32: GAMRF + GAMSF*XNE + GAMWF*TXNXN, reused by the wings
    R kapcen = R(0);
    R kappa0_w = R(0);  // kappa0 for the wings
    bool valid = false;
    if (FUSED) {
        if (a.process_mask[li] && (q.ok & 1)) {
            if (!F32) {
                const double lw = a.wavelength[li];
                double kapmin = (double)kap_at(c_ctr) * a.cutoff;
                double k0pre = (lt == 1) ? a.gamma_vdw[li] * a.gf[li] * (q.pop / dp.rho)
                                         : a.cgf[li] * q.xnfdop;
                if (k0pre >= kapmin) {
                    double post = k0pre * fast_ex(a.elo_cm[li] * dp.hckt, a.extab, a.extabf);
                    if (post >= kapmin && post > 0.0) {
                        double dw = q.dop_transp * lw;
                        double dopple = lw > 0 ? dw / lw : 1e-6;
                        double adamp = 0.0;
                        if (dw > 0 && dopple > 0)
                            adamp = (a.gamma_rad[li] + a.gamma_stark[li] * dp.xne +
                                     a.gamma_vdw[li] * dp.txnxn) / dopple;
                        if (adamp >= 0.0) {
                            double kc;
                            if (lt == 1) kc = post;
                            else if (adamp < 0.2) kc = post * (1.0 - 1.128 * adamp);
                            else kc = post * voigt_hv<double>(0.0, adamp, a.h0d, a.h1d, a.h2d);
                            kapcen = (R)kc;
                            valid = true;
                        }
                    }
                }
            } else {
                const LineF lf = a.linef[li];
                float kapmin = (float)kap_at(c_ctr) * a.cutoff_f;
                float k0pre = (lt == 1) ? lf.gw * lf.gf * q.pop_over_rho_f : lf.cgf * q.xnfdop_f;
                if (k0pre >= kapmin) {
                    float boltz = fast_ex_mixed(lf.elo_hi, lf.elo_lo, dp.hckt_hi, dp.hckt_lo,
                                                a.elo_cm[li], dp.hckt, a.extab_f, a.extabf_f);
                    float post = k0pre * boltz;
                    if (post >= kapmin && post > 0.0f) {
                        num = lf.gr + lf.gs * dp.xne_f + lf.gw * dp.txnxn_f;
                        float adamp = num / q.dop_f;
                        if (adamp >= 0.0f) {
                            float vc = (lt == 1) ? 1.0f
                                     : (adamp < 0.2f ? 1.0f - 1.128f * adamp
                                                     : voigt_hv<float>(0.0f, adamp, a.h0f, a.h1f, a.h2f));
                            kapcen = (R)(post * vc);
                            kappa0_w = (R)post;
                            valid = true;
                        }
                    }
                }
            }
        }
        if (a.transp_out && valid) {
            a.transp_out[li * L + d] = (double)kapcen;
            a.valid_out[li * L + d] = 1;
        }
    } else {
        valid = a.valid_in[li * L + d] != 0;
        kapcen = (R)a.transp_in[li * L + d];
    }
    if (!valid || !(kapcen > R(0))) return false;

    // ---------------- ASYNTH parameters (line_opacity.py:1161-1272) ----------------
    int ctr_code = 0;  // centre add, line_opacity.py:1091-1102
    if (a.asynth_mask[li] && c_ctr >= 0 && c_ctr < nwl) {
        int dlt = c_ctr - c_wing;
        if (dlt < -7 || dlt > 7) {
            atomicOr(a.flags, FLAG_N10DOP_RANGE);
            return false;
        }
        ctr_code = dlt + 8;
    }
    const bool wl_pos = F32 ? a.linef[li].wl > 0.0f : a.wavelength[li] > 0.0;
    const bool wings = (lt == 0) && (q.ok & 2) && wl_pos &&
                       c_wing >= -MAX_PROFILE_STEPS && c_wing <= nwl - 1 + MAX_PROFILE_STEPS;
    if (wings) {
        if (F32 && !FUSED) {
            const LineF lf = a.linef[li];
            num = lf.gr + lf.gs * dp.xne_f + lf.gw * dp.txnxn_f;
        }
        kc_out = kapcen;
        k0_out = kappa0_w;
        code_out = ctr_code;
        num_out = num;
        qi_out = qi;
        return true;
    }
    if (ctr_code != 0) {
        PairDesc<R> out;
        out.wing_c = c_wing;
        out.kapcen = kapcen;
        out.kappa0 = R(0);
        out.adamp = R(0);
        out.dvoigt = R(0);
        out.xfar = R(0);
        out.maxstep_far = 0;
        out.ctr_n10 = ctr_code;
        desc[slot] = out;
        cls[slot] = 0;
    }
    return false;
}

// Second half: the wing parameters (line_opacity.py:1161-1272), the
// near-wing KAPMIN crossing (:474-537), MAXSTEP and X_far, the descriptor and
// the reach class.
template <typename R>
__device__ __forceinline__ void pair_wings(const PairArgs& a, const R* __restrict__ kap_a,
                                           const R* __restrict__ kap_b, PairDesc<R>* __restrict__ desc,
                                           uint8_t* __restrict__ cls, int64_t li, int d, R kapcen,
                                           R kappa0_w, int ctr_code, float num, int qi) {
    constexpr bool F32 = sizeof(R) == 4;
    const int64_t slot = (int64_t)d * a.stride + li;
    const DepthPar& dp = a.depth[d];
    const IonPar& q = a.ion[qi];
    const int c_wing = a.wing_idx[li];
    const int64_t nwl = a.n_wl;
    auto kap_at = [&](int c) -> R {
        int cc = c < 0 ? 0 : (c > (int)nwl - 1 ? (int)nwl - 1 : c);
        R v = kap_a[(int64_t)d * nwl + cc];
        if (kap_b) v += kap_b[(int64_t)d * nwl + cc];
        return v;
    };
    PairDesc<R> out;
    out.wing_c = c_wing;
    out.kapcen = kapcen;
    out.kappa0 = R(0);
    out.adamp = R(0);
    out.dvoigt = R(0);
    out.xfar = R(0);
    out.maxstep_far = 0;
    int reach = 0;
    int n10dop = 0;
    {
        R adamp, kappa0, dvoigt;
        if (!F32) {
            const double lw = a.wavelength[li];
            double dw = q.dop * lw;
            double dopple = dw / lw;
            double ad = (a.gamma_rad[li] + a.gamma_stark[li] * dp.xne + a.gamma_vdw[li] * dp.txnxn) / dopple;
            ad = ad > 1e-12 ? ad : 1e-12;
            double vc = ad < 0.2 ? 1.0 - 1.128 * ad : voigt_hv<double>(0.0, ad, a.h0d, a.h1d, a.h2d);
            kappa0 = (R)(vc > 0 ? (double)kapcen / vc : (double)kapcen);
            adamp = (R)ad;
            const double resolu = a.gp->resolu;
            n10dop = (int)(int64_t)(10.0 * dopple * resolu);
            dvoigt = (R)(dopple > 0 ? 1.0 / (dopple * resolu) : 1.0);
        } else {
            float ad = __fdividef(num, q.dopw_f);
            ad = ad > 1e-12f ? ad : 1e-12f;
            adamp = (R)ad;
            kappa0 = kappa0_w;
            if (q.dop_f != q.dopw_f) {
                // microturbulence broadens the TRANSP Doppler width only
                // (line_opacity.py:629): KAPCEN carries H(0, a) of the
                // broadened width, and the wing kappa0 is KAPCEN / H(0, a)
                // of the wing's own width (:1161-1190), not the gate's kappa0
                const float vc = ad < 0.2f ? 1.0f - 1.128f * ad : voigt_hv<float>(0.0f, ad, a.h0f, a.h1f, a.h2f);
                kappa0 = vc > 0.0f ? (R)((float)kapcen / vc) : kapcen;
            }
            n10dop = q.n10dop;
            dvoigt = (R)q.dvoigt_f;
        }
        if (n10dop > 0xffffff) {
            atomicOr(a.flags, FLAG_N10DOP_RANGE);
            return;
        }
        const R kapmin_ref = kap_at(c_wing) * (F32 ? (R)a.cutoff_f : (R)a.cutoff);
        const R* h0 = F32 ? (const R*)a.h0f : (const R*)a.h0d;
        const R* h1 = F32 ? (const R*)a.h1f : (const R*)a.h1d;
        const R* h2 = F32 ? (const R*)a.h2f : (const R*)a.h2d;
        // near-wing KAPMIN scan (line_opacity.py:474-537): the first offset
        // whose profile falls below KAPMIN
        int cut = -1;
        R prof_n10 = R(0);
        int ns = 1;
        // FP32 with ADAMP < 0.2: from table index 5 on, H0 + a*H1 does not
        // increase with the offset for any a in [0, 0.2] (the tabulated
        // differences satisfy dH0 + 0.2*dH1 <= 0 there; only the first
        // four steps near v = 0 rise), nor does the x > 10 asymptote, which
        // also lies below the last table value.  Offsets mapping below
        // index 5 are scanned one by one, the rest by a galloping search.
        const bool monotone = F32 && adamp < R(0.2);
        for (; ns <= n10dop; ns++) {
            if (monotone && (int)(R(0.5) + (R)ns * (R(200) * dvoigt)) >= 5) break;
            R p = near_profile<R>(ns, dvoigt, adamp, kappa0, h0, h1, h2);
            if (ns == n10dop) prof_n10 = p;
            if (p < kapmin_ref) {
                cut = ns;
                break;
            }
        }
        if (monotone && cut == -1 && ns <= n10dop) {
            // The search starts at the offset where kappa0 (exp(-v^2) +
            // 0.5642 a / v^2) meets KAPMIN and gallops down or up from it;
            // with the profile non-increasing on [ns, n10dop] it returns the
            // first offset below KAPMIN whatever the start.
            int g = n10dop;
            const float r = (float)kapmin_ref / (float)kappa0;
            if (r > 0.0f && r < 1.0f) {
                const float v = fmaxf(sqrtf(-__logf(r)), sqrtf(0.5642f * (float)adamp / r));
                const float og = v / (float)dvoigt;
                if (og < (float)n10dop) g = max(ns, (int)og);
            } else if (r >= 1.0f) {
                g = ns;
            }
            int lo = ns - 1, hi = -1;
            const R pg = near_profile<R>(g, dvoigt, adamp, kappa0, h0, h1, h2);
            if (pg < kapmin_ref) {
                hi = g;
                int step = 1;
                while (hi - lo > 1) {
                    const int probe = max(hi - step, lo + 1);
                    if (near_profile<R>(probe, dvoigt, adamp, kappa0, h0, h1, h2) < kapmin_ref) {
                        hi = probe;
                        step <<= 1;
                    } else {
                        lo = probe;
                    }
                    if (lo == probe) break;
                }
            } else if (g == n10dop) {
                prof_n10 = pg;
            } else {
                lo = g;
                int probe = g + 1, step = 1;
                for (;;) {
                    const R p = near_profile<R>(probe, dvoigt, adamp, kappa0, h0, h1, h2);
                    if (p < kapmin_ref) {
                        hi = probe;
                        break;
                    }
                    lo = probe;
                    if (probe == n10dop) {
                        prof_n10 = p;
                        break;
                    }
                    probe = min(probe + step, n10dop);
                    step <<= 1;
                }
            }
            if (hi > 0) {
                while (hi - lo > 1) {
                    const int mid = lo + ((hi - lo) >> 1);
                    if (near_profile<R>(mid, dvoigt, adamp, kappa0, h0, h1, h2) < kapmin_ref) hi = mid;
                    else lo = mid;
                }
                cut = hi;
            }
        }
        bool far = false;
        R xfar = R(0);
        if (cut != -1) {
            reach = cut;
        } else {
            far = true;
            if (n10dop > 0 && prof_n10 > R(0) && kapmin_ref > R(0)) {
                xfar = prof_n10 * (R)n10dop * (R)n10dop;
                R ms;
                if constexpr (F32) ms = sqrtf(__fdividef(xfar, kapmin_ref)) + 1.0f;
                else ms = sqrt(xfar / kapmin_ref) + 1.0;
                reach = ms > (R)MAX_PROFILE_STEPS ? MAX_PROFILE_STEPS : (int)ms;
            }
        }
        out.kappa0 = kappa0;
        out.adamp = adamp;
        out.dvoigt = dvoigt;
        out.xfar = xfar;
        out.maxstep_far = reach | (far ? (int)0x80000000 : 0);
    }
    if (ctr_code == 0 && reach == 0) return;
    out.ctr_n10 = ctr_code | (n10dop << 8);
    desc[slot] = out;
    cls[slot] = (uint8_t)reach_class(reach);
}

// One CTA per (128 consecutive lines, depth): every thread runs the gates of
// its pair and queues it in shared memory if it needs wings; the queue is
// then worked by the CTA's first threads, so the wing code and its variable
// scan run on packed lanes instead of on the lanes whose pairs passed the
// gates.  Each pair writes only its own descriptor slot and class byte, so
// the queue order does not change the result.
template <typename R, bool FUSED>
__device__ __forceinline__ void pair_setup_kernel_body(VB vb, const PairArgs& a, const R* __restrict__ kap_a,
                                                         const R* __restrict__ kap_b,
                                                         PairDesc<R>* __restrict__ desc,
                                                         uint8_t* __restrict__ cls) {
    __shared__ int q_n;
    __shared__ int q_li[128], q_code[128], q_qi[128];
    __shared__ float q_num[128];
    __shared__ R q_kc[128], q_k0[128];
    if (threadIdx.x == 0) q_n = 0;
    __syncthreads();
    const int d = vb.y;
    const int64_t li = (int64_t)vb.x * blockDim.x + threadIdx.x;
    if (li < a.n_lines) {
        R kc, k0;
        int code, qi;
        float num;
        if (pair_gate<R, FUSED>(a, kap_a, kap_b, desc, cls, li, d, kc, k0, code, num, qi)) {
            const int i = atomicAdd(&q_n, 1);
            q_li[i] = (int)li;
            q_kc[i] = kc;
            q_k0[i] = k0;
            q_code[i] = code;
            q_num[i] = num;
            q_qi[i] = qi;
        }
    }
    __syncthreads();
    const int i = threadIdx.x;
    if (i < q_n)
        pair_wings<R>(a, kap_a, kap_b, desc, cls, q_li[i], d, q_kc[i], q_k0[i], q_code[i], q_num[i], q_qi[i]);
}
template <typename R, bool FUSED>
__global__ void __launch_bounds__(128) pair_setup_kernel(PairArgs a, const R* __restrict__ kap_a,
                                                         const R* __restrict__ kap_b,
                                                         PairDesc<R>* __restrict__ desc,
                                                         uint8_t* __restrict__ cls) {
    pair_setup_kernel_body<R, FUSED>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a, kap_a,
                                     kap_b, desc, cls);
}


// ---------------------------------------------------------------------------
// accumulation
// ---------------------------------------------------------------------------

// Shared-memory accumulator cell of one bin in one warp's copy of the tile:
// a plain sum in the working precision.  In FP32 each copy holds only the
// share of a bin's contributions that its warp processed, and the copies are
// combined with Kahan compensation, which keeps the summation error far below
// the other single-precision errors of the path (the normalised flux agrees
// with the FP64 path to the same 2e-5 as with compensated copies).
template <typename R> struct Cell;
template <> struct Cell<float> { using T = float; };
template <> struct Cell<double> { using T = double; };

__device__ __forceinline__ void cell_add(float* c, int b, float v) { c[b] += v; }
__device__ __forceinline__ void cell_add(double* c, int b, double v) { c[b] += v; }

// Near-zone profile with the (H0, H1) table interleaved in shared memory.
template <typename R, typename R2>
__device__ __forceinline__ R near_profile_tab(int off, R dv, R tabstep, R ad, R k0,
                                              const R2* __restrict__ h01, const R* __restrict__ h0g,
                                              const R* __restrict__ h1g, const R* __restrict__ h2g) {
    R x = (R)off * dv;
    if (ad < R(0.2)) {
        if (x > R(10)) return k0 * (R(0.5642) * ad / (x * x));
        int idx = tabi_index<R>(off, tabstep);
        idx = idx > VOIGT_N - 1 ? VOIGT_N - 1 : idx;
        R2 h = h01[idx];
        return k0 * (h.x + ad * h.y);
    }
    return k0 * voigt_hv<R>(x, ad, h0g, h1g, h2g);
}

template <typename R> struct Vec2;
template <> struct Vec2<float> { using T = float2; };
template <> struct Vec2<double> { using T = double2; };

// Accumulates profile values for offsets [lo, hi] into bins base + sgn*o of
// the warp's copy (lanes take consecutive offsets).
template <typename R, typename R2, typename CellT, bool FAR>
__device__ __forceinline__ void wing_run(CellT* my, int base, int sgn, int lo, int hi, int lane,
                                         R k0, R ad, R dv, R tabstep, R xf, const R2* h01,
                                         const R* h0g, const R* h1g, const R* h2g) {
    for (int o = lo + lane; o <= hi; o += 32) {
        R v;
        if (FAR) {
            R oo = (R)o * (R)o;
            if constexpr (sizeof(R) == 4) v = __fdividef(xf, oo);
            else v = xf / oo;
        } else {
            v = near_profile_tab<R, R2>(o, dv, tabstep, ad, k0, h01, h0g, h1g, h2g);
        }
        cell_add(my, base + sgn * o, v);
    }
}

// Near wings on both sides at once, offsets [1, m] (both sides inside the
// tile): one profile value per offset, added to bins base + o and base - o.
// Each bin receives the same single addition as with two one-sided runs.
template <typename R, typename R2, typename CellT>
__device__ __forceinline__ void near_both(CellT* my, int base, int m, int lane, R k0, R ad, R dv,
                                          R tabstep, const R2* h01, const R* h0g, const R* h1g,
                                          const R* h2g) {
    for (int o = 1 + lane; o <= m; o += 32) {
        const R v = near_profile_tab<R, R2>(o, dv, tabstep, ad, k0, h01, h0g, h1g, h2g);
        cell_add(my, base + o, v);
        cell_add(my, base - o, v);
    }
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Far wing in FP32 (XFAR / o^2 at offsets [lo, hi]): the run's bins
// [b_lo, b_hi] are taken as aligned pairs (2j, 2j+1), one pair per lane,
// with both values from packed FP32x2 arithmetic and one 8-byte
// read-modify-write; a bin at either end without its partner is added by
// lane 0 / lane 1.  Each bin gets the same additions in the same order as
// with one bin per lane.
// Long far runs (>= 64 bins): aligned quads of bins (4q .. 4q+3), one per
// lane, four values from packed FP32x2 arithmetic and one 16-byte
// read-modify-write; the up to three bins at each end outside whole quads
// are added by lanes 0-2 (low end) and 4-6 (high end).
__device__ __forceinline__ void far_run_x4(float* my, int b_lo, int b_hi, int base, int sgn, int lane,
                                           float xf) {
    const int e_lo = (4 - (b_lo & 3)) & 3;  // bins before the first whole quad
    const int e_hi = (b_hi + 1) & 3;        // bins after the last whole quad
    int eb = -1;
    if (lane < e_lo) eb = b_lo + lane;
    else if (lane >= 4 && lane < 4 + e_hi) eb = b_hi - e_hi + 1 + (lane - 4);
    if (eb >= 0) {
        const float o = (float)(sgn * (eb - base));
        my[eb] += __fdividef(xf, o * o);
    }
    float4* my4 = reinterpret_cast<float4*>(my);
    const int q0 = (b_lo + e_lo) >> 2, q1 = ((b_hi - e_hi + 1) >> 2) - 1;
    const float2 xf2 = make_float2(xf, xf);
    const float2 d2 = make_float2(2.0f * (float)sgn, 2.0f * (float)sgn);
    // offsets as floats, stepped by 128 per iteration (exact: |o| < 2^24)
    const int qs = q0 + lane;
    const int o0s = sgn * (4 * qs - base);
    float2 oa = make_float2((float)o0s, (float)(o0s + sgn));
    const float2 step = make_float2(128.0f * (float)sgn, 128.0f * (float)sgn);
    for (int q = qs; q <= q1; q += 32) {
        const float2 ob = __fadd2_rn(oa, d2);
        const float2 sa = __fmul2_rn(oa, oa), sb = __fmul2_rn(ob, ob);
        const float2 va = __fmul2_rn(xf2, make_float2(rcp_approx(sa.x), rcp_approx(sa.y)));
        const float2 vb = __fmul2_rn(xf2, make_float2(rcp_approx(sb.x), rcp_approx(sb.y)));
        oa = __fadd2_rn(oa, step);
        float4 c = my4[q];
        const float2 ca = __fadd2_rn(make_float2(c.x, c.y), va);
        const float2 cb = __fadd2_rn(make_float2(c.z, c.w), vb);
        my4[q] = make_float4(ca.x, ca.y, cb.x, cb.y);
    }
}

__device__ __forceinline__ void far_run_x2(float* my, int base, int sgn, int lo, int hi, int lane, float xf) {
    if (lo > hi) return;
    if (hi - lo >= 63) {
        far_run_x4(my, sgn > 0 ? base + lo : base - hi, sgn > 0 ? base + hi : base - lo, base, sgn, lane, xf);
        return;
    }
    const int b_lo = sgn > 0 ? base + lo : base - hi;
    const int b_hi = sgn > 0 ? base + hi : base - lo;
    int eb = -1;
    if (lane == 0 && (b_lo & 1)) eb = b_lo;
    if (lane == 1 && !(b_hi & 1)) eb = b_hi;
    if (eb >= 0) {
        const float o = (float)(sgn * (eb - base));
        my[eb] += __fdividef(xf, o * o);
    }
    float2* my2 = reinterpret_cast<float2*>(my);
    const int j1 = (b_hi - 1) >> 1;
    const float2 xf2 = make_float2(xf, xf);
    const int js = ((b_lo + 1) >> 1) + lane;
    const int o0s = sgn * (2 * js - base);
    float2 of = make_float2((float)o0s, (float)(o0s + sgn));
    const float2 step = make_float2(64.0f * (float)sgn, 64.0f * (float)sgn);
    for (int j = js; j <= j1; j += 32) {
        const float2 oo = __fmul2_rn(of, of);
        my2[j] = __fadd2_rn(my2[j], __fmul2_rn(xf2, make_float2(rcp_approx(oo.x), rcp_approx(oo.y))));
        of = __fadd2_rn(of, step);
    }
}

// Adds v to a bin of the warp's own copy with a shared-memory atomic (the
// short pairs, where two lanes may hit one bin).  Only lanes of one warp
// touch a copy, and a warp's atomics to one word are applied in a fixed
// order, so the result does not vary between runs.
__device__ __forceinline__ void cell_atomic(float* c, int b, float v) { atomicAdd(&c[b], v); }
__device__ __forceinline__ void cell_atomic(double* c, int b, double v) { atomicAdd(&c[b], v); }

// One CTA per (lambda tile, depth).  For every reach class k the contributing
// pairs are those whose wing centre lies within 2^k (+1) bins of the tile --
// a contiguous range of that class's centre-sorted list.  The pairs are dealt
// to the warps in batches of 32, round-robin in a fixed order, each lane
// loading one pair's descriptor.
//  * Classes below short_class (reach <= 2^(short_class-1) bins: most pairs,
//    each a few evaluations): every lane walks its own pair, offset by
//    offset in lockstep with the others, and adds the red and blue values
//    with shared-memory atomics -- two lanes may hit the same bin.
//  * Longer classes: each lane works out its pair's in-tile red/blue x
//    near/far offset ranges, a ballot drops pairs that miss the tile, and
//    the warp walks the rest, broadcasting each pair by shuffles, running up
//    to four branch-free loops -- near wings with lanes on consecutive
//    offsets, far wings (FP32) with lanes on consecutive bin pairs -- and
//    adding into the warp's copy (no two lanes write the same word).
// The copies are then summed in warp order (Kahan in FP32), multiplied by STIM
// (line_opacity.py:1338) and stored coalesced.  Every sum has a fixed order,
// so results are bit-identical across runs.
template <typename R>
__device__ __forceinline__ void accumulate_kernel_body(VB vb, const AccArgs& a, const PairDesc<R>* __restrict__ desc,
                                                         R* __restrict__ out) {
    using CellT = typename Cell<R>::T;
    using R2 = typename Vec2<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int W = a.tile_bins;
    const int nwarps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int d = vb.y;
    const int T0 = vb.x * W;
    const int T1 = (int)min((int64_t)T0 + W, a.n_wl);
    const int span = T1 - T0;

    R2* h01 = reinterpret_cast<R2*>(smem_raw);  // interleaved (H0, H1)
    size_t tab_bytes = (VOIGT_N * sizeof(R2) + 15) & ~size_t(15);
    CellT* acc = reinterpret_cast<CellT*>(smem_raw + tab_bytes);  // [nwarps][W]
    __shared__ int64_t cls_lo[N_REACH_CLASSES];        // absolute index of the class's first contributing pair
    __shared__ int64_t cls_n[N_REACH_CLASSES];         // contributing pairs of the class
    __shared__ int64_t bat_base[N_REACH_CLASSES + 1];  // first batch of each class

    const R* gh0 = sizeof(R) == 8 ? (const R*)a.h0d : (const R*)a.h0f;
    const R* gh1 = sizeof(R) == 8 ? (const R*)a.h1d : (const R*)a.h1f;
    const R* gh2 = sizeof(R) == 8 ? (const R*)a.h2d : (const R*)a.h2f;
    if (threadIdx.x < N_REACH_CLASSES) {
        const int k = threadIdx.x;
        const int2 r = a.tile_rng[((int64_t)d * vb.gx + vb.x) * N_REACH_CLASSES + k];
        cls_lo[k] = a.class_off[(int64_t)d * (N_REACH_CLASSES + 1) + k] + r.x;
        cls_n[k] = r.y - r.x;
    }
    for (int i = threadIdx.x; i < VOIGT_N; i += blockDim.x) {
        R2 h;
        h.x = gh0[i];
        h.y = gh1[i];
        h01[i] = h;
    }
    for (int i = threadIdx.x; i < nwarps * W; i += blockDim.x) {
        acc[i] = CellT(0);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t nb = 0;
        for (int k = 0; k < N_REACH_CLASSES; k++) {
            bat_base[k] = nb;
            nb += k < a.long_class ? (cls_n[k] + 31) >> 5 : (cls_n[k] + 7) >> 3;
        }
        bat_base[N_REACH_CLASSES] = nb;
    }
    __syncthreads();

    CellT* my = acc + warp * W;
    const PairDesc<R>* drow = desc + (int64_t)d * a.stride;
    unsigned long long evals = 0;
    const int64_t nbatch = bat_base[N_REACH_CLASSES];
    // Batches are software-pipelined: the descriptors of the warp's next
    // batch and the positions of the one after it are in flight while the
    // current batch is processed.
    int kcur = 0;  // class of the furthest batch looked up (batches ascend)
    auto batch_class = [&](int64_t bt) {
        while (bt >= bat_base[kcur + 1]) kcur++;
        return kcur;
    };
    int64_t bt = warp;
    int kb = 0, cnt = 0, kb_n = 0, cnt_n = 0;
    int32_t pos_n = 0;
    PairDesc<R> pd{};
    if (bt < nbatch) {
        kb = batch_class(bt);
        const int bs = kb < a.long_class ? 32 : 8;
        const int64_t f = (bt - bat_base[kb]) * bs;
        cnt = (int)min((int64_t)bs, cls_n[kb] - f);
        if (lane < cnt) pd = drow[a.class_pos[cls_lo[kb] + f + lane]];
    }
    if (bt + nwarps < nbatch) {
        kb_n = batch_class(bt + nwarps);
        const int bs = kb_n < a.long_class ? 32 : 8;
        const int64_t f = (bt + nwarps - bat_base[kb_n]) * bs;
        cnt_n = (int)min((int64_t)bs, cls_n[kb_n] - f);
        if (lane < cnt_n) pos_n = a.class_pos[cls_lo[kb_n] + f + lane];
    }
    for (; bt < nbatch; bt += nwarps) {
        PairDesc<R> pd_n{};
        if (lane < cnt_n && bt + nwarps < nbatch) pd_n = drow[pos_n];
        int kb_nn = 0, cnt_nn = 0;
        int32_t pos_nn = 0;
        if (bt + 2 * nwarps < nbatch) {
            kb_nn = batch_class(bt + 2 * nwarps);
            const int bs = kb_nn < a.long_class ? 32 : 8;
            const int64_t f = (bt + 2 * nwarps - bat_base[kb_nn]) * bs;
            cnt_nn = (int)min((int64_t)bs, cls_n[kb_nn] - f);
            if (lane < cnt_nn) pos_nn = a.class_pos[cls_lo[kb_nn] + f + lane];
        }
        const bool valid = lane < cnt;
        if (kb < a.short_class) {
            // ---- short pairs: one lane per pair ----
            int cb = 0, reach = 0, nz = 0;
            R k0 = R(0), ad = R(0), dv = R(0), xf = R(0);
            if (valid) {
                cb = pd.wing_c - T0;
                const int ctr = pd.ctr_n10 & 15;
                if (ctr) {
                    const int cc = cb + (ctr - 8);
                    if ((unsigned)cc < (unsigned)span) {
                        cell_atomic(my, cc, pd.kapcen);
                        evals++;
                    }
                }
                reach = pd.maxstep_far & 0x7fffffff;
                nz = pd.maxstep_far < 0 ? (pd.ctr_n10 >> 8) : 0x7fffffff;
                k0 = pd.kappa0;
                ad = pd.adamp;
                dv = pd.dvoigt;
                xf = pd.xfar;
                if (reach > 0) {
                    const int rlo = max(1, -cb), rhi = min(reach, span - 1 - cb);
                    const int blo = max(1, cb - (span - 1)), bhi = min(reach, cb);
                    if (rlo <= rhi) evals += (unsigned long long)(rhi - rlo + 1);
                    if (blo <= bhi) evals += (unsigned long long)(bhi - blo + 1);
                }
            }
            const R ts = R(200) * dv;
            const int maxr = __reduce_max_sync(0xffffffffu, reach);
            for (int o = 1; o <= maxr; o++) {
                if (o <= reach) {
                    R v;
                    if (o <= nz) {
                        v = near_profile_tab<R, R2>(o, dv, ts, ad, k0, h01, gh0, gh1, gh2);
                    } else {
                        const R oo = (R)o * (R)o;
                        if constexpr (sizeof(R) == 4) v = __fdividef(xf, oo);
                        else v = xf / oo;
                    }
                    if ((unsigned)(cb + o) < (unsigned)span) cell_atomic(my, cb + o, v);
                    if ((unsigned)(cb - o) < (unsigned)span) cell_atomic(my, cb - o, v);
                }
            }
            __syncwarp();
        } else {
            // ---- per lane: one pair and its in-tile offset ranges ----
            int c = 0, cb = -1, rlo = 1, rhi = 0, blo = 1, bhi = 0, nz = 0;
            R k0 = R(0), ad = R(0), dv = R(0), xf = R(0), kc = R(0);
            if (valid) {
                c = pd.wing_c;
                const int ctr = pd.ctr_n10 & 15;
                if (ctr) {
                    int cc = c + (ctr - 8);
                    if (cc >= T0 && cc < T1) {
                        cb = cc - T0;
                        kc = pd.kapcen;
                        evals++;
                    }
                }
                const int reach = pd.maxstep_far & 0x7fffffff;
                if (reach > 0) {
                    rlo = max(1, T0 - c);
                    rhi = min(reach, T1 - 1 - c);
                    blo = max(1, c - (T1 - 1));
                    bhi = min(reach, c - T0);
                    if (rlo <= rhi) evals += (unsigned long long)(rhi - rlo + 1);
                    if (blo <= bhi) evals += (unsigned long long)(bhi - blo + 1);
                }
                nz = pd.maxstep_far < 0 ? (pd.ctr_n10 >> 8) : 0x7fffffff;  // last near-zone offset
                k0 = pd.kappa0;
                ad = pd.adamp;
                dv = pd.dvoigt;
                xf = pd.xfar;
            }
            const bool active = cb >= 0 || rlo <= rhi || blo <= bhi;
            unsigned mask = __ballot_sync(0xffffffffu, active);
            while (mask) {
                const int i = __ffs(mask) - 1;
                mask &= mask - 1;
                const int ci = __shfl_sync(0xffffffffu, c, i);
                const int cbi = __shfl_sync(0xffffffffu, cb, i);
                if (cbi >= 0) {
                    const R kci = __shfl_sync(0xffffffffu, kc, i);
                    if (lane == 0) cell_add(my, cbi, kci);
                }
                const int rl = __shfl_sync(0xffffffffu, rlo, i), rh = __shfl_sync(0xffffffffu, rhi, i);
                const int bl = __shfl_sync(0xffffffffu, blo, i), bh = __shfl_sync(0xffffffffu, bhi, i);
                if (rl > rh && bl > bh) continue;
                const int nzi = __shfl_sync(0xffffffffu, nz, i);
                const R adi = __shfl_sync(0xffffffffu, ad, i);
                const R dvi = __shfl_sync(0xffffffffu, dv, i);
                const R k0i = __shfl_sync(0xffffffffu, k0, i);
                const R xfi = __shfl_sync(0xffffffffu, xf, i);
                const R ts = R(200) * dvi;
                const int base = ci - T0;
                // red: bins base + o; blue: bins base - o
                if constexpr (sizeof(R) == 4) {
                    // near wings: both sides together where both are in the tile,
                    // one bin per lane; far wings: bin pairs / quads
                    const int nr = min(rh, nzi), nb = min(bh, nzi);
                    int m = 0;
                    if (rl == 1 && bl == 1) {
                        m = min(nr, nb);
                        near_both<R, R2, CellT>(my, base, m, lane, k0i, adi, dvi, ts, h01, gh0, gh1, gh2);
                    }
                    wing_run<R, R2, CellT, false>(my, base, 1, max(rl, m + 1), nr, lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                    wing_run<R, R2, CellT, false>(my, base, -1, max(bl, m + 1), nb, lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                    if (nzi != 0x7fffffff) {
                        far_run_x2(my, base, 1, max(rl, nzi + 1), rh, lane, xfi);
                        far_run_x2(my, base, -1, max(bl, nzi + 1), bh, lane, xfi);
                    }
                } else {
                    wing_run<R, R2, CellT, false>(my, base, 1, rl, min(rh, nzi), lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                    wing_run<R, R2, CellT, false>(my, base, -1, bl, min(bh, nzi), lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                    if (nzi != 0x7fffffff) {
                        wing_run<R, R2, CellT, true>(my, base, 1, max(rl, nzi + 1), rh, lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                        wing_run<R, R2, CellT, true>(my, base, -1, max(bl, nzi + 1), bh, lane, k0i, adi, dvi, ts, xfi, h01, gh0, gh1, gh2);
                    }
                }
            }
        }
        pd = pd_n;
        kb = kb_n;
        cnt = cnt_n;
        pos_n = pos_nn;
        kb_n = kb_nn;
        cnt_n = cnt_nn;
    }
    __syncthreads();
    // combine the warp copies in warp order, apply STIM and store
    const DepthPar dp = a.depth[d];
    for (int b = threadIdx.x; b < span; b += blockDim.x) {
        R v;
        if constexpr (sizeof(R) == 4) {
            float s = 0.f, cp = 0.f;
            for (int w = 0; w < nwarps; w++) {
                kahan_add(s, cp, acc[w * W + b]);
            }
            const float freq = a.freq_f[T0 + b];
            float stim = -expm1f(-freq * (float)dp.hkt_asynth);
            v = s * stim;
        } else {
            double s = 0.0;
            for (int w = 0; w < nwarps; w++) s += acc[w * W + b];
            double freq = C_LIGHT_NM / a.grid[T0 + b];
            double stim = 1.0 - exp(-freq * dp.hkt_asynth);
            v = (R)(s * stim);
        }
        out[(int64_t)d * a.n_wl + T0 + b] = v;
    }
    // evaluation counter: warp sum, one atomic per warp
    if (a.evals) {
        for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
        if (lane == 0 && evals) atomicAdd(a.evals, evals);
    }
}
template <typename R>
__global__ void __launch_bounds__(512) accumulate_kernel(AccArgs a, const PairDesc<R>* __restrict__ desc,
                                                         R* __restrict__ out) {
    accumulate_kernel_body<R>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a, desc, out);
}


// ---------------------------------------------------------------------------
// transfer (JOSH)
// ---------------------------------------------------------------------------

// Division of the transfer arithmetic: IEEE in FP64 (the reference's
// operations), the fast reciprocal-multiply in FP32 (2 ulp; operands here are
// opacities, optical depths and column masses far below 2^126).
__device__ __forceinline__ float tdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double tdiv(double a, double b) { return a / b; }

// Parabolic coefficients of PARCOE after its boundary overrides
// (josh_solver.py:110-152) at index j, before the smoothing pass.
template <typename R>
__device__ __forceinline__ void parcoe_raw(const R* f, const R* x, int n, int j, R& a, R& b, R& c) {
    if (j == 0 || j == 1 || (j == 2 && n > 3) || j == n - 1) {
        int j0 = (j == n - 1) ? n - 2 : j;
        R den = x[j0 + 1] - x[j0];
        b = den != R(0) ? tdiv(f[j0 + 1] - f[j0], den) : R(0);
        a = f[j] - x[j] * b;
        c = R(0);
        return;
    }
    int j1 = j - 1;
    R den = x[j] - x[j1];
    R dd = den != R(0) ? tdiv(f[j] - f[j1], den) : R(0);
    R den1 = (x[j + 1] - x[j]) * (x[j + 1] - x[j1]);
    R term1 = den1 != R(0) ? tdiv(f[j + 1], den1) : R(0);
    R den2 = x[j + 1] - x[j1];
    R den3 = x[j + 1] - x[j];
    R den4 = x[j] - x[j1];
    R part = R(0);
    if (den4 != R(0)) {
        R t1 = den2 != R(0) ? tdiv(f[j1], den2) : R(0);
        R t2 = den3 != R(0) ? tdiv(f[j], den3) : R(0);
        part = tdiv(t1 - t2, den4);
    }
    c = term1 + part;
    b = dd - (x[j] + x[j1]) * c;
    a = f[j1] - x[j1] * dd + x[j] * x[j1] * c;
}

// INTEG (josh_solver.py:171-189) over PARCOE with its smoothing pass
// (:154-166) folded in, streaming over the layers.
//
// FP64 evaluates each interval's integral from the polynomial's coefficients
// in absolute column mass, a + b x + c x^2, as the reference does.  In FP32
// that form cancels (the coefficients are large against the interval), so
// the FP32 path uses the equivalent local form: every PARCOE polynomial of
// interval i -- the line of the first and last intervals and of the
// overridden second and third, the Newton parabolas through three
// neighbouring points, and the smoothing blend of two parabolas that share
// the interval's end points -- passes through (x_i, f_i) and
// (x_{i+1}, f_{i+1}), so its integral is h (f_i + f_{i+1}) / 2 - c_i h^3 / 6
// with h = x_{i+1} - x_i and c_i the smoothed curvature.  Only c is needed;
// the integral is accumulated with Kahan compensation.
template <typename R>
__device__ void integ_tau(const R* x, const R* f, int n, R start, R* fint) {
    if constexpr (sizeof(R) == 4) {
        fint[0] = start;
        if (n == 1) return;
        float ci = 0.f, cn = 0.f, a_, b_;  // curvature at i and i+1 after the overrides
        if (n > 2) parcoe_raw<R>(f, x, n, 1, a_, b_, cn);
        float s = start, comp = 0.f;
        for (int i = 0; i < n - 1; i++) {
            float c_i = ci;
            if (i >= 1 && i <= n - 2) {
                if (i == n - 2) {
                    c_i = 0.f;
                } else if (ci != 0.f) {
                    const float acn = fabsf(cn);
                    const float den = acn + fabsf(ci);
                    const float wt = den > 0.f ? tdiv(acn, den) : 0.f;
                    c_i = cn + wt * (ci - cn);
                }
            }
            const float dx = x[i + 1] - x[i];
            kahan_add(s, comp, dx * (0.5f * (f[i] + f[i + 1]) - c_i * dx * dx * (1.0f / 6.0f)));
            fint[i + 1] = s;
            ci = cn;
            if (i + 2 <= n - 1) parcoe_raw<R>(f, x, n, i + 2, a_, b_, cn);
        }
        return;
    }
    fint[0] = start;
    if (n == 1) return;
    if (n == 2) {
        R den = x[1] - x[0];
        R b = den != R(0) ? tdiv(f[1] - f[0], den) : R(0);
        R a0 = f[0] - x[0] * b;
        R dx = x[1] - x[0];
        R term = a0 + R(0.5) * b * (x[1] + x[0]);
        fint[1] = fint[0] + term * dx;
        return;
    }
    R an, bn, cn;  // coefficients at i+1 after overrides (before smoothing)
    R ai, bi, ci;
    parcoe_raw<R>(f, x, n, 0, ai, bi, ci);
    parcoe_raw<R>(f, x, n, 1, an, bn, cn);
    R s = start, comp = R(0);
    for (int i = 0; i < n - 1; i++) {
        R a_i = ai, b_i = bi, c_i = ci;
        if (i >= 1 && i <= n - 2) {
            if (i == n - 2) {
                // a[n1-1] = a[-1] (josh_solver.py:164-166)
                R den = x[n - 1] - x[n - 2];
                b_i = den != R(0) ? tdiv(f[n - 1] - f[n - 2], den) : R(0);
                a_i = f[n - 1] - x[n - 1] * b_i;
                c_i = R(0);
            } else if (ci != R(0)) {
                R acn = cn < R(0) ? -cn : cn;
                R den = acn + (ci < R(0) ? -ci : ci);
                R wt = den > R(0) ? tdiv(acn, den) : R(0);
                a_i = an + wt * (ai - an);
                b_i = bn + wt * (bi - bn);
                c_i = cn + wt * (ci - cn);
            }
        }
        R dx = x[i + 1] - x[i];
        R term = a_i + R(0.5) * b_i * (x[i + 1] + x[i]);
        term += (c_i / R(3)) * ((x[i + 1] + x[i]) * x[i + 1] + x[i] * x[i]);
        R inc = term * dx;
        if constexpr (sizeof(R) == 4) {
            kahan_add(s, comp, inc);
        } else {
            s = s + inc;
        }
        fint[i + 1] = s;
        ai = an; bi = bn; ci = cn;
        if (i + 2 <= n - 1) parcoe_raw<R>(f, x, n, i + 2, an, bn, cn);
    }
}

// DERIV (josh_solver.py:193-217)
template <typename R>
__device__ void deriv(const R* x, const R* f, int n, R* dfdx) {
    dfdx[0] = tdiv(f[1] - f[0], x[1] - x[0]);
    dfdx[n - 1] = tdiv(f[n - 1] - f[n - 2], x[n - 1] - x[n - 2]);
    if (n == 2) return;
    R s = x[1] != x[0] ? (R)(((x[1] - x[0]) < R(0)) ? -1 : 1) : R(1);
    for (int j = 1; j < n - 1; j++) {
        R sc = fabs(f[j - 1]);
        R t = fabs(f[j]);
        sc = t > sc ? t : sc;
        t = fabs(f[j + 1]);
        sc = t > sc ? t : sc;
        sc = x[j] != R(0) ? tdiv(sc, (R)fabs(x[j])) : sc;
        if (sc == R(0)) sc = R(1);
        R d1 = tdiv(tdiv(f[j + 1] - f[j], x[j + 1] - x[j]), sc);
        R d0 = tdiv(tdiv(f[j] - f[j - 1], x[j] - x[j - 1]), sc);
        R tan1 = tdiv(d1, s * sqrt(R(1) + d1 * d1) + R(1));
        R tan0 = tdiv(d0, s * sqrt(R(1) + d0 * d0) + R(1));
        dfdx[j] = tdiv(tan1 + tan0, R(1) - tan1 * tan0) * sc;
    }
}

// MAP1 (josh_solver.py:220-353) of fold(xold) onto the JOSH grid.
template <typename R>
__device__ void map1_xtau(const R* xold, const R* fold, int nold, const R* xnew, R* fnew) {
    int l = 2, ll = 0;
    R cfor = 0, bfor = 0, afor = 0, cbac = 0, bbac = 0, abac = 0, A = 0, B = 0, Cc = 0;
    // 1-based views
    const R* x1 = xold - 1;
    const R* f1 = fold - 1;
    for (int k = 1; k <= NXTAU; k++) {
        R xk = xnew[k - 1];
        for (;;) {
            if (xk < x1[l]) {
                if (l == ll) break;
                if (l == 2 || l == 3) {
                    l = l < nold ? l : nold;
                    Cc = R(0);
                    B = tdiv(f1[l] - f1[l - 1], x1[l] - x1[l - 1]);
                    A = f1[l] - x1[l] * B;
                    ll = l;
                    break;
                }
                int l1 = l - 1;
                if (l > ll + 1 || l == 4) {
                    int l2 = l - 2;
                    R dd = tdiv(f1[l1] - f1[l2], x1[l1] - x1[l2]);
                    cbac = tdiv(f1[l], (x1[l] - x1[l1]) * (x1[l] - x1[l2])) +
                           tdiv(tdiv(f1[l2], x1[l] - x1[l2]) - tdiv(f1[l1], x1[l] - x1[l1]),
                                x1[l1] - x1[l2]);
                    bbac = dd - (x1[l1] + x1[l2]) * cbac;
                    abac = f1[l2] - x1[l2] * dd + x1[l1] * x1[l2] * cbac;
                    if (!(l < nold)) {
                        Cc = cbac; B = bbac; A = abac; ll = l;
                        break;
                    }
                } else {
                    cbac = cfor; bbac = bfor; abac = afor;
                    if (l == nold) {
                        Cc = cbac; B = bbac; A = abac; ll = l;
                        break;
                    }
                }
                R dd = tdiv(f1[l] - f1[l1], x1[l] - x1[l1]);
                cfor = tdiv(f1[l + 1], (x1[l + 1] - x1[l]) * (x1[l + 1] - x1[l1])) +
                       tdiv(tdiv(f1[l1], x1[l + 1] - x1[l1]) - tdiv(f1[l], x1[l + 1] - x1[l]),
                            x1[l] - x1[l1]);
                bfor = dd - (x1[l] + x1[l1]) * cfor;
                afor = f1[l1] - x1[l1] * dd + x1[l] * x1[l1] * cfor;
                R acf = cfor < R(0) ? -cfor : cfor;
                R acb = cbac < R(0) ? -cbac : cbac;
                R wt = acf != R(0) ? tdiv(acf, acf + acb) : R(0);
                A = afor + wt * (abac - afor);
                B = bfor + wt * (bbac - bfor);
                Cc = cfor + wt * (cbac - cfor);
                ll = l;
                break;
            }
            l += 1;
            if (l > nold) {
                l = nold;
                Cc = R(0);
                B = tdiv(f1[l] - f1[l - 1], x1[l] - x1[l - 1]);
                A = f1[l] - x1[l] * B;
                ll = l;
                break;
            }
        }
        fnew[k - 1] = A + (B + Cc * xk) * xk;
    }
}

// Gauss-Seidel scattering sweeps of the reference (josh_solver.py:24-92), in
// single precision as the reference runs them, with the reference's
// summation order and no fused multiply-add.
__device__ __forceinline__ int josh_sweeps_ref(const float* __restrict__ coefj, float* xs,
                                               const float* xalpha, const float* xsbar_mod) {
    float diag[NXTAU];
    for (int k = 0; k < NXTAU; k++) diag[k] = __fsub_rn(1.0f, __fmul_rn(xalpha[k], coefj[k * NXTAU + k]));
    for (int it = 0; it < NXTAU; it++) {
        int iferr = 0;
        for (int k = NXTAU - 1; k >= 0; k--) {
            float delxs = 0.0f;
            for (int m = 0; m < NXTAU; m++) delxs = __fadd_rn(delxs, __fmul_rn(coefj[k * NXTAU + m], xs[m]));
            delxs = __fdiv_rn(__fsub_rn(__fadd_rn(__fmul_rn(delxs, xalpha[k]), xsbar_mod[k]), xs[k]), diag[k]);
            float errorx = xs[k] != 0.0f ? fabsf(__fdiv_rn(delxs, xs[k])) : __int_as_float(0x7f800000);
            if (errorx > 1.0e-5f) iferr = 1;
            float nv = __fadd_rn(xs[k], delxs);
            xs[k] = nv > 1.0e-38f ? nv : 1.0e-38f;
        }
        if (!iferr) return it + 1;
    }
    return NXTAU;
}

// Fast sweeps: the same iteration with the 51x51 operator in the kernel's
// constant bank (a __grid_constant__ parameter), XS in registers (fully
// unrolled) and four interleaved partial dot products per row.
__device__ __forceinline__ int josh_sweeps_fast(const CoefJ32& cj, const float* xa, const float* xm,
                                                float* xs_io) {
    float xs[NXTAU];
#pragma unroll
    for (int m = 0; m < NXTAU; m++) xs[m] = xs_io[m];
    int it_done = NXTAU;
    for (int it = 0; it < NXTAU; it++) {
        bool err = false;
#pragma unroll
        for (int k = NXTAU - 1; k >= 0; k--) {
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
            for (int m = 0; m + 3 < NXTAU; m += 4) {
                s0 = fmaf(cj.c[k * NXTAU + m], xs[m], s0);
                s1 = fmaf(cj.c[k * NXTAU + m + 1], xs[m + 1], s1);
                s2 = fmaf(cj.c[k * NXTAU + m + 2], xs[m + 2], s2);
                s3 = fmaf(cj.c[k * NXTAU + m + 3], xs[m + 3], s3);
            }
#pragma unroll
            for (int m = (NXTAU / 4) * 4; m < NXTAU; m++) s0 = fmaf(cj.c[k * NXTAU + m], xs[m], s0);
            float s = (s0 + s1) + (s2 + s3);
            float xak = xa[k];
            float diag = 1.0f - xak * cj.c[k * NXTAU + k];
            float dl = __fdividef(fmaf(s, xak, xm[k]) - xs[k], diag);
            float xk = xs[k];
            err |= (xk == 0.0f) || (fabsf(dl) > 1.0e-5f * fabsf(xk));
            float nv = xk + dl;
            xs[k] = nv > 1.0e-38f ? nv : 1.0e-38f;
        }
        if (!err) {
            it_done = it + 1;
            break;
        }
    }
#pragma unroll
    for (int m = 0; m < NXTAU; m++) xs_io[m] = xs[m];
    return it_done;
}

// JOSH surface flux for one column (josh_solver.py:367-767).  aline, sline
// and sigmal may be NULL (no line opacity / source = scont / no line
// scattering).
template <typename R, bool REF_SWEEP>
__device__ double josh_flux(int n, const R* acont, const R* scont, const R* aline, const R* sline,
                            const R* sigmac, const R* sigmal, const R* rho, const R* xtau,
                            const double* ch, const CoefJ32& cj, const float* coefj_ref,
                            int* iters_out, const double* coefj64 = nullptr) {
    R abtot[MAX_LAYERS], alpha[MAX_LAYERS], snubar[MAX_LAYERS], taunu[MAX_LAYERS];
    const R eps = (R)EPS38;
    for (int j = 0; j < n; j++) {
        const R al_j = aline ? aline[j] : R(0);
        const R sl_j = sigmal ? sigmal[j] : R(0);
        R ab = acont[j] + al_j + sigmac[j] + sl_j;
        abtot[j] = ab > eps ? ab : (ab != ab ? ab : eps);
        R sc = sigmac[j] + sl_j;
        R alp = abtot[j] > R(0) ? tdiv(sc, abtot[j]) : R(0);
        alpha[j] = alp < R(0) ? R(0) : (alp > R(1) ? R(1) : alp);
        R den = acont[j] + al_j;
        const R sline_j = sline ? sline[j] : scont[j];
        snubar[j] = den > R(0) ? tdiv(acont[j] * scont[j] + al_j * sline_j, den) : scont[j];
    }
    // rho ascending after solve_lte_frequency's reversal, so needs_reverse
    // (josh_solver.py:465) is false here.
    integ_tau<R>(rho, abtot, n, abtot[0] * rho[0], taunu);
    if (taunu[0] > xtau[NXTAU - 1]) {
        // MAXJ = 1 path (josh_solver.py:700-727)
        R snu[MAX_LAYERS], hnu[MAX_LAYERS], jm[MAX_LAYERS];
        for (int j = 0; j < n; j++) snu[j] = snubar[j];
        int it_done = 0;
        for (int it = 0; it < NXTAU; it++) {
            deriv<R>(taunu, snu, n, hnu);
            for (int j = 0; j < n; j++) hnu[j] = hnu[j] / R(3);
            deriv<R>(taunu, hnu, n, jm);
            R err = R(0);
            for (int j = 0; j < n; j++) {
                R jnu = jm[j] + snu[j];
                R snew = (R(1) - alpha[j]) * snubar[j] + alpha[j] * jnu;
                R an = snew < R(0) ? -snew : snew;
                R dn = an > eps ? an : eps;
                R df = snew - snu[j];
                err += tdiv(df < R(0) ? -df : df, dn);
                snu[j] = snew;
            }
            it_done = it + 1;
            if (err < R(1.0e-5)) break;
        }
        *iters_out = -it_done;
        return (double)hnu[0];
    }
    R xsbar[NXTAU], xalpha[NXTAU];
    map1_xtau<R>(taunu, snubar, n, xtau, xsbar);
    map1_xtau<R>(taunu, alpha, n, xtau, xalpha);
    float xs32[NXTAU], xa32[NXTAU], xm32[NXTAU];
    R s0 = snubar[0] > eps ? snubar[0] : eps;
    R a0 = alpha[0] < R(0) ? R(0) : (alpha[0] > R(1) ? R(1) : alpha[0]);
    for (int l = 0; l < NXTAU; l++) {
        R xb = xsbar[l] > eps ? xsbar[l] : eps;
        R xa = xalpha[l] < R(0) ? R(0) : (xalpha[l] > R(1) ? R(1) : xalpha[l]);
        if (xtau[l] < taunu[0]) {
            xb = s0;
            xa = a0;
        }
        xs32[l] = (float)xb;
        xa32[l] = (float)xa;
        xm32[l] = (float)(xb * (R(1) - xa));
    }
    if (sizeof(R) == 8 && coefj64) {
        // Gauss-Seidel in FP64 to a tight tolerance: the converged solution of
        // (I - diag(xa) C) xs = xb (1 - xa), smooth in the inputs
        double xs[NXTAU], xa[NXTAU], xm[NXTAU];
        for (int l = 0; l < NXTAU; l++) {
            R xb = xsbar[l] > eps ? xsbar[l] : eps;
            R xl = xalpha[l] < R(0) ? R(0) : (xalpha[l] > R(1) ? R(1) : xalpha[l]);
            if (xtau[l] < taunu[0]) {
                xb = s0;
                xl = a0;
            }
            xs[l] = (double)xb;
            xa[l] = (double)xl;
            xm[l] = (double)(xb * (R(1) - xl));
        }
        int it = 0;
        for (; it < 2000; it++) {
            double dmax = 0.0;
            for (int k = NXTAU - 1; k >= 0; k--) {
                double sum = 0.0;
                for (int q = 0; q < NXTAU; q++) sum += coefj64[k * NXTAU + q] * xs[q];
                const double nv = sum * xa[k] + xm[k];
                const double dl = fabs(nv - xs[k]) / fmax(fabs(nv), 1e-300);
                dmax = dl > dmax ? dl : dmax;
                xs[k] = nv;
            }
            if (dmax < 1e-13) break;
        }
        *iters_out = it + 1;
        double flux = 0.0;
        for (int l = 0; l < NXTAU; l++) flux += ch[l] * xs[l];
        return flux;
    }
    int it;
    if (REF_SWEEP) it = josh_sweeps_ref(coefj_ref, xs32, xa32, xm32);
    else it = josh_sweeps_fast(cj, xa32, xm32, xs32);
    *iters_out = it;
    double flux = 0.0;
    for (int l = 0; l < NXTAU; l++) flux += ch[l] * (double)xs32[l];
    return flux;
}

// Planck function B_nu (radiative.py:20-39).
__device__ __forceinline__ double planck_nu(double freq, double hkt) {
    double freq15 = freq / 1.0e15;
    double ehvkt = exp(-freq * hkt);
    double stim = 1.0 - ehvkt;
    double bnu = 1.47439e-2 * pow(freq15, 3.0) * ehvkt / stim;
    return bnu != bnu ? 0.0 : bnu;
}
__device__ __forceinline__ float planck_nu(float freq15, float freq_hkt_x) {
    // freq15^3 * e^-x / (1 - e^-x), x = h nu / k T
    float bnu = 1.47439e-2f * freq15 * freq15 * freq15 * __fdividef(__expf(-freq_hkt_x), -expm1f(-freq_hkt_x));
    return bnu != bnu ? 0.0f : bnu;
}

// One wavelength's depth column (radiative.py:42-218 and the per-lambda loop
// of :282-494).  Field arrays are [L, n]; in ASYNTH mode the line opacity is
// the stimulated-emission-corrected ASYNTH, split by FSCAT into absorption
// and scattering (opacity.py:2408-2420).
template <typename R, bool REF_SWEEP>
__device__ __forceinline__ void transfer_column(const TransferArgs& a, const CoefJ32& cj,
                                                const R* __restrict__ cont_abs,
                                                const R* __restrict__ cont_scat,
                                                const R* __restrict__ line_op,
                                                const R* __restrict__ line_sc,
                                                const R* __restrict__ line_src, int64_t j) {
    constexpr bool F32 = sizeof(R) == 4;
    const int L = a.n_layers;
    R mass[MAX_LAYERS], ca[MAX_LAYERS], cs[MAX_LAYERS], la[MAX_LAYERS], ls[MAX_LAYERS],
        src[MAX_LAYERS], pl[MAX_LAYERS], hk[MAX_LAYERS];
    const double wl = a.grid[j];
    const double freq = C_LIGHT_NM / (wl > 1e-12 ? wl : 1e-12);
    const float freq15_f = (float)(freq / 1.0e15);
    const float freq_f = (float)freq;
    const bool has_ls = (!a.asynth_mode && line_sc != nullptr) || (a.asynth_mode && a.line_scat);
    const bool own_src = line_src != nullptr || (a.slinec_mode && !F32);
    int m = 0;
    for (int d = 0; d < L; d++) {
        const DepthPar& dp = a.depth[d];
        R cm = F32 ? (R)dp.rhox_f : (R)dp.rhox;
        R aa = cont_abs[(int64_t)d * a.n + j];
        R ss = cont_scat[(int64_t)d * a.n + j];
        R lo, lsg = R(0);
        if (a.asynth_mode) {
            R A = line_op[(int64_t)d * a.n + j];
            if (a.line_scat) {
                R fs = F32 ? (R)dp.fscat_f : (R)dp.fscat;
                lo = A * (R(1) - fs);
                R one_m = R(1) - fs;
                R alinec = tdiv(lo, one_m > R(1e-12) ? one_m : R(1e-12));
                lsg = alinec * fs;
            } else {
                lo = A;
            }
        } else {
            lo = line_op[(int64_t)d * a.n + j];
            lsg = line_sc ? line_sc[(int64_t)d * a.n + j] : R(0);
        }
        const R mx = (R)MAX_OPACITY_REAL4;
        bool ok = cm >= R(0) && isfinite(cm) && isfinite(aa) && isfinite(ss) && isfinite(lo) &&
                  isfinite(lsg) && aa < mx && ss < mx && lo < mx && lsg < mx;
        if (!ok || !(cm > R(0))) continue;
        mass[m] = cm;
        ca[m] = aa;
        cs[m] = ss;
        la[m] = lo;
        if (has_ls) ls[m] = lsg;
        hk[m] = F32 ? (R)dp.hkt_f : (R)dp.hkt;
        if (line_src) {
            R v = line_src[(int64_t)d * a.n + j];
            if (!isfinite(v)) {
                if constexpr (F32) v = planck_nu(freq15_f, freq_f * dp.hkt_f);
                else v = planck_nu(freq, dp.hkt);
            }
            src[m] = v;
        } else if (own_src) {
            // SLINEC = BNU*STIM/(1-EHVKT) with the driver's frequency
            // (opacity.py:2215-2227, bfudge.py:144-145)
            double fr = C_LIGHT_CM / (wl * 1.0e-7);
            double f15 = fr / 1.0e15;
            double eh = exp(-fr * dp.hkt);
            double st = 1.0 - eh;
            double bnu = 1.47439e-02 * pow(f15, 3.0) * eh / st;
            double v = (bnu * st) / (1.0 - eh);
            src[m] = isfinite(v) ? (R)v : (R)planck_nu(freq, dp.hkt);
        }
        m++;
    }
    if (m < 2) {
        // fewer than two usable layers: no tau scale to interpolate on (the
        // reference returns 0 for an empty column and cannot map one layer)
        a.flux_total[j] = 0.0;
        a.flux_cont[j] = 0.0;
        if (a.iters) {
            a.iters[2 * j] = 0;
            a.iters[2 * j + 1] = 0;
        }
        return;
    }
    if (m > 1 && !(mass[0] < mass[m - 1])) {
        for (int q = 0; q < m / 2; q++) {
            int r = m - 1 - q;
            R t;
            t = mass[q]; mass[q] = mass[r]; mass[r] = t;
            t = ca[q]; ca[q] = ca[r]; ca[r] = t;
            t = cs[q]; cs[q] = cs[r]; cs[r] = t;
            t = la[q]; la[q] = la[r]; la[r] = t;
            if (has_ls) { t = ls[q]; ls[q] = ls[r]; ls[r] = t; }
            if (own_src) { t = src[q]; src[q] = src[r]; src[r] = t; }
            t = hk[q]; hk[q] = hk[r]; hk[r] = t;
        }
    }
    for (int q = 0; q < m; q++) {
        if constexpr (F32) pl[q] = planck_nu(freq15_f, freq_f * hk[q]);
        else pl[q] = planck_nu(freq, hk[q]);
    }
    R xtau[NXTAU];
    for (int l = 0; l < NXTAU; l++) xtau[l] = (R)a.xtau[l];
    int itc = 0, itt = 0;
    double fc = josh_flux<R, REF_SWEEP>(m, ca, pl, nullptr, nullptr, cs, nullptr, mass, xtau, a.ch, cj,
                                        a.coefj32, &itc, a.coefj64);
    double ft = josh_flux<R, REF_SWEEP>(m, ca, pl, la, own_src ? src : pl, cs, has_ls ? ls : nullptr, mass,
                                        xtau, a.ch, cj, a.coefj32, &itt, a.coefj64);
    a.flux_cont[j] = fc;
    a.flux_total[j] = ft;
    if (a.iters) {
        a.iters[2 * j] = itc;
        a.iters[2 * j + 1] = itt;
    }
}

template <typename R, bool REF_SWEEP>
__global__ void __launch_bounds__(128) transfer_kernel(TransferArgs a, const __grid_constant__ CoefJ32 cj,
                                                       const R* __restrict__ cont_abs,
                                                       const R* __restrict__ cont_scat,
                                                       const R* __restrict__ line_op,
                                                       const R* __restrict__ line_sc,
                                                       const R* __restrict__ line_src) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    transfer_column<R, REF_SWEEP>(a, cj, cont_abs, cont_scat, line_op, line_sc, line_src, j);
}

// ---------------------------------------------------------------------------
// Streaming single-precision transfer (fused ASYNTH mode)
// ---------------------------------------------------------------------------
//
// The same per-wavelength JOSH solution as transfer_column<float, false>, in
// one pass over the layers with nothing per layer kept in memory: layer i+3
// is read while INTEG (PARCOE with its smoothing) closes tau[i+1], and MAP1
// onto the 51-point JOSH grid consumes each new tau together with S-bar and
// alpha through a four-layer window, writing the mapped (S-bar, alpha) pairs
// to shared memory.  The sweeps then run with XS in registers.  Columns the
// pass does not cover -- a non-finite or out-of-range input, fewer than three
// layers, column masses that do not increase, or the MAXJ = 1 branch -- are
// appended to a list for transfer_column.

constexpr int TS_THREADS = 128;

// Shared-memory load the compiler may not hoist out of the sweep loop (the
// 51 loop-invariant pairs would otherwise be held in registers).
__device__ __forceinline__ float2 ts_ld(const float2* p) {
    float2 v;
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}

// One layer of one solve: total opacity, albedo and S-bar (radiative.py
// solve_lte_frequency, josh_solver.py:367-420); false when an input is not
// usable.
template <bool TOTAL>
__device__ __forceinline__ bool ts_layer(const float* __restrict__ cab, const float* __restrict__ csc,
                                         const float* __restrict__ lop, int line_scat, int64_t off,
                                         float fscat, float hkt, float freq15, float freq, float& ab,
                                         float& al, float& sn) {
    const float mx = (float)MAX_OPACITY_REAL4;
    const float eps = (float)EPS38;
    const float ca = cab[off], cs = csc[off];
    float lo = 0.f, lsg = 0.f;
    bool ok = isfinite(ca) && isfinite(cs) && ca < mx && cs < mx;
    if (TOTAL) {
        const float A = lop[off];
        if (line_scat) {
            lo = A * (1.f - fscat);
            const float one_m = 1.f - fscat;
            lsg = tdiv(lo, one_m > 1e-12f ? one_m : 1e-12f) * fscat;
        } else {
            lo = A;
        }
        ok = ok && isfinite(lo) && isfinite(lsg) && lo < mx && lsg < mx;
    }
    const float pl = planck_nu(freq15, freq * hkt);
    const float t = ((ca + lo) + cs) + lsg;
    ab = t > eps ? t : (t != t ? t : eps);
    const float alp = ab > 0.f ? tdiv(cs + lsg, ab) : 0.f;
    al = alp < 0.f ? 0.f : (alp > 1.f ? 1.f : alp);
    const float den = ca + lo;
    sn = den > 0.f ? tdiv(ca * pl + lo * pl, den) : pl;
    return ok;
}

// Quadratic coefficients through three points, the MAP1 "back"/"forward"
// parabola (josh_solver.py:220-353).
__device__ __forceinline__ void ts_parab(float xa, float xb, float xc, float fa, float fb, float fc,
                                         float& A, float& B, float& C) {
    const float dd = tdiv(fb - fa, xb - xa);
    C = tdiv(fc, (xc - xb) * (xc - xa)) + tdiv(tdiv(fa, xc - xa) - tdiv(fb, xc - xb), xb - xa);
    B = dd - (xb + xa) * C;
    A = fa - xa * dd + xb * xa * C;
}
__device__ __forceinline__ void ts_line(float xa, float xb, float fa, float fb, float& A, float& B, float& C) {
    B = tdiv(fb - fa, xb - xa);
    A = fb - xb * B;
    C = 0.f;
}
__device__ __forceinline__ void ts_blend(float xa, float xb, float xc, float xd, float fa, float fb, float fc,
                                         float fd, float& A, float& B, float& C) {
    float ab, bb, cb, af, bf, cf;
    ts_parab(xa, xb, xc, fa, fb, fc, ab, bb, cb);
    ts_parab(xb, xc, xd, fb, fc, fd, af, bf, cf);
    const float acf = fabsf(cf), acb = fabsf(cb);
    const float wt = acf != 0.f ? tdiv(acf, acf + acb) : 0.f;
    A = af + wt * (ab - af);
    B = bf + wt * (bb - bf);
    C = cf + wt * (cb - cf);
}

// MAP1 of (S-bar, alpha) onto the JOSH grid, fed one layer at a time.
struct TsMap {
    float x0, x1, x2, x3, f0, f1, f2, f3, g0, g1, g2, g3;  // the newest four layers
    int avail, k;
    float tau0, s0, a0;
    float2* out;         // this thread's column of the [NXTAU][TS_THREADS] array
    const float* xtau;   // JOSH grid in shared memory

    __device__ __forceinline__ void emit(float xk, float As, float Bs, float Cs, float Aa, float Ba, float Ca) {
        const float vs = As + (Bs + Cs * xk) * xk;
        const float va = Aa + (Ba + Ca * xk) * xk;
        const float eps = (float)EPS38;
        float xb = vs > eps ? vs : eps;
        float xa = va < 0.f ? 0.f : (va > 1.f ? 1.f : va);
        if (xk < tau0) {
            xb = s0;
            xa = a0;
        }
        out[k * TS_THREADS] = make_float2(xb, xa);
    }
    // Grid points below x1[l] = x2, with l = avail - 1 (1-based) and the
    // window x0..x3 = x1[l-2..l+1].
    __device__ __forceinline__ void step() {
        if (k >= NXTAU) return;
        float xk = xtau[k];
        if (!(xk < x2)) return;
        const int l = avail - 1;
        float As, Bs, Cs, Aa, Ba, Ca;
        if (l <= 3) {
            ts_line(x1, x2, f1, f2, As, Bs, Cs);
            ts_line(x1, x2, g1, g2, Aa, Ba, Ca);
        } else {
            ts_blend(x0, x1, x2, x3, f0, f1, f2, f3, As, Bs, Cs);
            ts_blend(x0, x1, x2, x3, g0, g1, g2, g3, Aa, Ba, Ca);
        }
        do {
            emit(xk, As, Bs, Cs, Aa, Ba, Ca);
            if (++k >= NXTAU) break;
            xk = xtau[k];
        } while (xk < x2);
    }
    __device__ __forceinline__ void push(float x, float f, float g) {
        x0 = x1; x1 = x2; x2 = x3; x3 = x;
        f0 = f1; f1 = f2; f2 = f3; f3 = f;
        g0 = g1; g1 = g2; g2 = g3; g3 = g;
        if (++avail >= 3) step();
    }
    // After the last layer (avail = n, window x1[n-3..n]): the last interval
    // and the linear extrapolation beyond it.
    __device__ __forceinline__ void finish() {
        if (k >= NXTAU) return;
        float xk = xtau[k];
        float As, Bs, Cs, Aa, Ba, Ca;
        if (xk < x3) {
            if (avail <= 3) {
                ts_line(x2, x3, f2, f3, As, Bs, Cs);
                ts_line(x2, x3, g2, g3, Aa, Ba, Ca);
            } else {
                ts_parab(x1, x2, x3, f1, f2, f3, As, Bs, Cs);
                ts_parab(x1, x2, x3, g1, g2, g3, Aa, Ba, Ca);
            }
            do {
                emit(xk, As, Bs, Cs, Aa, Ba, Ca);
                if (++k >= NXTAU) return;
                xk = xtau[k];
            } while (xk < x3);
        }
        ts_line(x2, x3, f2, f3, As, Bs, Cs);
        ts_line(x2, x3, g2, g3, Aa, Ba, Ca);
        for (; k < NXTAU; k++) emit(xtau[k], As, Bs, Cs, Aa, Ba, Ca);
    }
};

// PARCOE curvature at layer j from f[j-1], f[j], f[j+1] (fm, f0, fp), the
// cases of parcoe_raw for j >= 2 (the local-form integral of integ_tau needs
// no other coefficient).
__device__ __forceinline__ float ts_parcoe_c(const float* x, int n, int j, float fm, float f0, float fp) {
    if ((j == 2 && n > 3) || j == n - 1) return 0.f;
    const int j1 = j - 1;
    const float den1 = (x[j + 1] - x[j]) * (x[j + 1] - x[j1]);
    const float term1 = den1 != 0.f ? tdiv(fp, den1) : 0.f;
    const float den2 = x[j + 1] - x[j1];
    const float den3 = x[j + 1] - x[j];
    const float den4 = x[j] - x[j1];
    float part = 0.f;
    if (den4 != 0.f) {
        const float t1 = den2 != 0.f ? tdiv(fm, den2) : 0.f;
        const float t2 = den3 != 0.f ? tdiv(f0, den3) : 0.f;
        part = tdiv(t1 - t2, den4);
    }
    return term1 + part;
}

// One JOSH solve of one column, streamed; returns the sweep count, or 0 when
// the column needs transfer_column.
template <bool TOTAL>
__device__ __forceinline__ int ts_solve(const TransferArgs& a, const CoefJ32& cj, const float* __restrict__ cab,
                                        const float* __restrict__ csc, const float* __restrict__ lop,
                                        int64_t j, int n, const float* s_x, const float* s_hkt,
                                        const float* s_fs, const float* s_xtau, float freq15, float freq,
                                        float2* col, double& flux) {
    const int64_t N = a.n;
    const int ls = a.line_scat;
    // window f[i..i+3] of abtot, S-bar and alpha
    float F0, F1, F2, F3 = 0.f, N0, N1, N2, N3 = 0.f, G0, G1, G2, G3 = 0.f;
    bool ok = ts_layer<TOTAL>(cab, csc, lop, ls, j, s_fs[0], s_hkt[0], freq15, freq, F0, G0, N0);
    ok &= ts_layer<TOTAL>(cab, csc, lop, ls, N + j, s_fs[1], s_hkt[1], freq15, freq, F1, G1, N1);
    ok &= ts_layer<TOTAL>(cab, csc, lop, ls, 2 * N + j, s_fs[2], s_hkt[2], freq15, freq, F2, G2, N2);
    if (n > 3) ok &= ts_layer<TOTAL>(cab, csc, lop, ls, 3 * N + j, s_fs[3], s_hkt[3], freq15, freq, F3, G3, N3);
    const float tau0 = F0 * s_x[0];
    if (!ok || !(tau0 <= s_xtau[NXTAU - 1])) return 0;
    const float eps = (float)EPS38;
    TsMap m;
    m.x0 = m.x1 = m.x2 = m.x3 = 0.f;
    m.f0 = m.f1 = m.f2 = m.f3 = 0.f;
    m.g0 = m.g1 = m.g2 = m.g3 = 0.f;
    m.avail = 0;
    m.k = 0;
    m.tau0 = tau0;
    m.s0 = N0 > eps ? N0 : eps;
    m.a0 = G0;
    m.out = col;
    m.xtau = s_xtau;
    m.push(tau0, N0, G0);
    // INTEG (josh_solver.py:171-189) with PARCOE's smoothing folded in, in
    // the local form of integ_tau (interval integral h (f_i + f_{i+1}) / 2 -
    // c_i h^3 / 6; the curvature of layers 0 and 1 is 0 by PARCOE's overrides)
    const float* x = s_x;
    float ci = 0.f, cn = 0.f;
    float s = tau0, comp = 0.f;
    for (int i = 0; i < n - 1; i++) {
        float c_i = ci;
        if (i >= 1) {
            if (i == n - 2) {
                c_i = 0.f;
            } else if (ci != 0.f) {
                const float acn = fabsf(cn);
                const float den = acn + fabsf(ci);
                const float wt = den > 0.f ? tdiv(acn, den) : 0.f;
                c_i = cn + wt * (ci - cn);
            }
        }
        const float dx = x[i + 1] - x[i];
        kahan_add(s, comp, dx * (0.5f * (F0 + F1) - c_i * dx * dx * (1.0f / 6.0f)));
        m.push(s, N1, G1);
        ci = cn;
        if (i + 2 <= n - 1) cn = ts_parcoe_c(x, n, i + 2, F1, F2, F3);
        F0 = F1; F1 = F2; F2 = F3;
        N0 = N1; N1 = N2; N2 = N3;
        G0 = G1; G1 = G2; G2 = G3;
        if (i + 4 <= n - 1) {
            const int d = i + 4;
            ok &= ts_layer<TOTAL>(cab, csc, lop, ls, (int64_t)d * N + j, s_fs[d], s_hkt[d], freq15, freq, F3, G3, N3);
        } else {
            F3 = G3 = N3 = 0.f;
        }
    }
    if (!ok) return 0;
    m.finish();
    // Gauss-Seidel sweeps (josh_solver.py:24-92), XS in registers, the
    // operator in the constant bank
    float xs[NXTAU];
#pragma unroll
    for (int l = 0; l < NXTAU; l++) xs[l] = col[l * TS_THREADS].x;
    int it_done = NXTAU;
    for (int it = 0; it < NXTAU; it++) {
        bool err = false;
#pragma unroll
        for (int k = NXTAU - 1; k >= 0; k--) {
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
            for (int q = 0; q + 3 < NXTAU; q += 4) {
                s0 = fmaf(cj.c[k * NXTAU + q], xs[q], s0);
                s1 = fmaf(cj.c[k * NXTAU + q + 1], xs[q + 1], s1);
                s2 = fmaf(cj.c[k * NXTAU + q + 2], xs[q + 2], s2);
                s3 = fmaf(cj.c[k * NXTAU + q + 3], xs[q + 3], s3);
            }
#pragma unroll
            for (int q = (NXTAU / 4) * 4; q < NXTAU; q++) s0 = fmaf(cj.c[k * NXTAU + q], xs[q], s0);
            const float sum = (s0 + s1) + (s2 + s3);
            const float2 ba = ts_ld(col + k * TS_THREADS);
            const float xak = ba.y;
            const float xm = ba.x * (1.f - ba.y);
            const float diag = 1.0f - xak * cj.c[k * NXTAU + k];
            const float dl = __fdividef(fmaf(sum, xak, xm) - xs[k], diag);
            const float xk = xs[k];
            err |= (xk == 0.0f) || (fabsf(dl) > 1.0e-5f * fabsf(xk));
            const float nv = xk + dl;
            xs[k] = nv > 1.0e-38f ? nv : 1.0e-38f;
        }
        if (!err) {
            it_done = it + 1;
            break;
        }
    }
    // surface flux, compensated single-precision sum
    float fs = 0.f, fc = 0.f;
#pragma unroll
    for (int l = 0; l < NXTAU; l++) kahan_add(fs, fc, cj.ch[l] * xs[l]);
    flux = (double)fs - (double)fc;
    return it_done;
}

template <typename R>
__device__ __forceinline__ void transfer_stream_kernel_body(VB vb, 
    const TransferArgs& a, const CoefJ32& cj, const float* __restrict__ cab,
    const float* __restrict__ csc, const float* __restrict__ lop, int32_t* __restrict__ list,
    unsigned long long* __restrict__ count) {
    extern __shared__ float2 ts_cols[];  // [NXTAU][TS_THREADS]
    __shared__ float s_x[MAX_LAYERS], s_hkt[MAX_LAYERS], s_fs[MAX_LAYERS], s_xtau[NXTAU];
    __shared__ int s_ok;
    const int L = a.n_layers;
    for (int d = threadIdx.x; d < L; d += blockDim.x) {
        s_x[d] = a.depth[d].rhox_f;
        s_hkt[d] = a.depth[d].hkt_f;
        s_fs[d] = a.depth[d].fscat_f;
    }
    for (int l = threadIdx.x; l < NXTAU; l += blockDim.x) s_xtau[l] = cj.xtau[l];
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = L >= 3 && L <= MAX_LAYERS;
        for (int d = 0; ok && d < L; d++) {
            const float v = s_x[d];
            ok = isfinite(v) && v > 0.f && (d == 0 || v > s_x[d - 1]);
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    const int64_t j = (int64_t)vb.x * TS_THREADS + threadIdx.x;
    if (j >= a.n) return;
    bool done = false;
    if (s_ok) {
        const double wl = a.grid[j];
        const double freq = C_LIGHT_NM / (wl > 1e-12 ? wl : 1e-12);
        const float freq15 = (float)(freq / 1.0e15);
        const float freq_f = (float)freq;
        float2* col = ts_cols + threadIdx.x;
        double ft = 0.0, fc = 0.0;
        const int itt = ts_solve<true>(a, cj, cab, csc, lop, j, L, s_x, s_hkt, s_fs, s_xtau, freq15, freq_f, col, ft);
        if (itt > 0) {
            const int itc = ts_solve<false>(a, cj, cab, csc, lop, j, L, s_x, s_hkt, s_fs, s_xtau, freq15, freq_f, col, fc);
            if (itc > 0) {
                a.flux_total[j] = ft;
                a.flux_cont[j] = fc;
                if (a.iters) {
                    a.iters[2 * j] = itc;
                    a.iters[2 * j + 1] = itt;
                }
                done = true;
            }
        }
    }
    if (!done) list[atomicAdd(count, 1ull)] = (int32_t)j;
}
template <typename R>
__global__ void __launch_bounds__(TS_THREADS, 4) transfer_stream_kernel(
    TransferArgs a, const __grid_constant__ CoefJ32 cj, const float* __restrict__ cab,
    const float* __restrict__ csc, const float* __restrict__ lop, int32_t* __restrict__ list,
    unsigned long long* __restrict__ count) {
    transfer_stream_kernel_body<R>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a, cj, cab, csc, lop, list, count);
}


// transfer_column for the wavelengths the streaming pass listed.
template <typename R>
__device__ __forceinline__ void transfer_list_kernel_body(VB vb, const TransferArgs& a, const CoefJ32& cj,
                                                            const R* __restrict__ cab, const R* __restrict__ csc,
                                                            const R* __restrict__ lop,
                                                            const int32_t* __restrict__ list,
                                                            const unsigned long long* __restrict__ count) {
    const int64_t nl = (int64_t)*count;
    for (int64_t i = (int64_t)vb.x * blockDim.x + threadIdx.x; i < nl; i += (int64_t)vb.gx * blockDim.x)
        transfer_column<R, false>(a, cj, cab, csc, lop, nullptr, nullptr, list[i]);
}
template <typename R>
__global__ void __launch_bounds__(128) transfer_list_kernel(TransferArgs a, const __grid_constant__ CoefJ32 cj,
                                                            const R* __restrict__ cab, const R* __restrict__ csc,
                                                            const R* __restrict__ lop,
                                                            const int32_t* __restrict__ list,
                                                            const unsigned long long* __restrict__ count) {
    transfer_list_kernel_body<R>(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, a, cj, cab, csc, lop, list, count);
}


}  // namespace ks
