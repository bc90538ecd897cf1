// ks_adjoint.cuh -- reverse-mode (adjoint) kernels of the fused FP64 path,
// for gradients of a spectrum loss with respect to the line parameters.
//
// Given g_F[lambda] = dLoss/dF_total[lambda]:
//  * transfer_adjoint_kernel -- one thread per wavelength: recomputes the
//    column and the total-flux JOSH solve of transfer_column (FP64, ASYNTH
//    mode, SLINEC source, no line scattering; radiative.py:42-218,
//    josh_solver.py:367-767), then runs it backwards: the transposed linear
//    solve of the converged Gauss-Seidel system (I - diag(xa) C) xs = xb(1-xa),
//    the XTAU clamps and overrides, MAP1 (node values and node optical depths),
//    INTEG with PARCOE's smoothing, and the ABTOT / ALPHA / SNUBAR split,
//    giving G[d, lambda] = dLoss/dASYNTH[d, lambda] times STIM.  Local
//    derivatives of the rational MAP1 / PARCOE formulas come from forward-mode
//    dual numbers.  Columns that take the MAXJ = 1 branch or need the
//    per-layer masks get zero and are counted.
//  * line_adjoint_kernel -- one warp per (line, depth) pair with a
//    descriptor: recomputes the pair's profile over its wing range as the
//    forward accumulation does and forms sum_b G[d,b] c(b) and
//    sum_b G[d,b] dc/da(b); contributions are proportional to gf
//    (line_opacity.py:101-184, :1161-1272), so the first sum is
//    dLoss/dln(gf) of the pair.
//  * line_grad_kernel -- one thread per line: sums over depths and applies
//    da/dgamma (a = (gamma_rad + gamma_stark XNE + gamma_vdw TXNXN) / DOPPLE)
//    for gradients with respect to log10 gf and the log10 damping constants.
#pragma once

#include "ks_kernels.cuh"

namespace ks {

template <int N>
struct Dual {
    double v;
    double d[N];
};
template <int N>
__device__ __forceinline__ Dual<N> dc(double v) {
    Dual<N> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = 0.0;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dv(double v, int k) {
    Dual<N> r = dc<N>(v);
    r.d[k] = 1.0;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a * b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a * b.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dabs(const Dual<N>& a) {
    return a.v < 0.0 ? (-1.0) * a : a;
}

// MAP1 coefficient formulas (josh_solver.py:220-353).
template <int N>
__device__ __forceinline__ void map_line(const Dual<N>& xa, const Dual<N>& xb, const Dual<N>& fa,
                                         const Dual<N>& fb, Dual<N>& A, Dual<N>& B, Dual<N>& C) {
    B = (fb - fa) / (xb - xa);
    A = fb - xb * B;
    C = dc<N>(0.0);
}
template <int N>
__device__ __forceinline__ void map_parab(const Dual<N>& xa, const Dual<N>& xb, const Dual<N>& xc,
                                          const Dual<N>& fa, const Dual<N>& fb, const Dual<N>& fc, Dual<N>& A,
                                          Dual<N>& B, Dual<N>& C) {
    const Dual<N> dd = (fb - fa) / (xb - xa);
    C = fc / ((xc - xb) * (xc - xa)) + (fa / (xc - xa) - fb / (xc - xb)) / (xb - xa);
    B = dd - (xb + xa) * C;
    A = fa - xa * dd + xb * xa * C;
}

// Coefficients (A, B, C) of the MAP1 interval for 1-based node l (nodes
// x1[l-2..l+1] and f1[..] given as x[0..3] / f[0..3], the 4-point window
// ending at l+1), case: 0 linear (l-1, l), 1 parabola (l-2, l-1, l),
// 2 blend of the two parabolas.
template <int N>
__device__ __forceinline__ void map_coeffs(int kase, const Dual<N>* x, const Dual<N>* f, Dual<N>& A, Dual<N>& B,
                                           Dual<N>& C) {
    if (kase == 0) {
        map_line<N>(x[1], x[2], f[1], f[2], A, B, C);
    } else if (kase == 1) {
        map_parab<N>(x[0], x[1], x[2], f[0], f[1], f[2], A, B, C);
    } else {
        Dual<N> ab, bb, cb, af, bf, cf;
        map_parab<N>(x[0], x[1], x[2], f[0], f[1], f[2], ab, bb, cb);
        map_parab<N>(x[1], x[2], x[3], f[1], f[2], f[3], af, bf, cf);
        const Dual<N> acf = dabs(cf), acb = dabs(cb);
        Dual<N> wt = dc<N>(0.0);
        if (acf.v != 0.0) wt = acf / (acf + acb);
        A = af + wt * (ab - af);
        B = bf + wt * (bb - bf);
        C = cf + wt * (cb - cf);
    }
}

// PARCOE raw coefficients at layer j (josh_solver.py:110-152) from the
// window w = f[j-1], f[j], f[j+1]; x are the layer column masses.
__device__ __forceinline__ void adj_parcoe(const double* x, int n, int j, const Dual<4>* w, Dual<4>& a,
                                           Dual<4>& b, Dual<4>& c) {
    const Dual<4> zero = dc<4>(0.0);
    if (j == 0 || j == 1 || (j == 2 && n > 3) || j == n - 1) {
        const int j0 = (j == n - 1) ? n - 2 : j;
        const double den = x[j0 + 1] - x[j0];
        const Dual<4>& f0 = (j0 == j) ? w[1] : w[0];
        const Dual<4>& f1 = (j0 == j) ? w[2] : w[1];
        b = den != 0.0 ? (1.0 / den) * (f1 - f0) : zero;
        a = w[1] - x[j] * b;
        c = zero;
        return;
    }
    const int j1 = j - 1;
    const double den = x[j] - x[j1];
    const Dual<4> dd = den != 0.0 ? (1.0 / den) * (w[1] - w[0]) : zero;
    const double den1 = (x[j + 1] - x[j]) * (x[j + 1] - x[j1]);
    const Dual<4> term1 = den1 != 0.0 ? (1.0 / den1) * w[2] : zero;
    const double den2 = x[j + 1] - x[j1], den3 = x[j + 1] - x[j], den4 = x[j] - x[j1];
    Dual<4> part = zero;
    if (den4 != 0.0) {
        const Dual<4> t1 = den2 != 0.0 ? (1.0 / den2) * w[0] : zero;
        const Dual<4> t2 = den3 != 0.0 ? (1.0 / den3) * w[1] : zero;
        part = (1.0 / den4) * (t1 - t2);
    }
    c = term1 + part;
    b = dd - (x[j] + x[j1]) * c;
    a = w[0] - x[j1] * dd + (x[j] * x[j1]) * c;
}

// Increment of INTEG (josh_solver.py:171-189) over [x_i, x_{i+1}] with
// PARCOE's smoothing (:154-166), as a function of f[i-1..i+2] = w[0..3].
__device__ __forceinline__ Dual<4> adj_integ_inc(const double* x, int n, int i, const Dual<4>* w) {
    Dual<4> ai, bi, ci, an, bn, cn;
    adj_parcoe(x, n, i, w, ai, bi, ci);
    adj_parcoe(x, n, i + 1, w + 1, an, bn, cn);
    Dual<4> a_i = ai, b_i = bi, c_i = ci;
    if (i >= 1 && i <= n - 2) {
        if (i == n - 2) {
            const double den = x[n - 1] - x[n - 2];
            b_i = den != 0.0 ? (1.0 / den) * (w[2] - w[1]) : dc<4>(0.0);
            a_i = w[2] - x[n - 1] * b_i;
            c_i = dc<4>(0.0);
        } else if (ci.v != 0.0) {
            const Dual<4> acn = dabs(cn);
            const Dual<4> den = acn + dabs(ci);
            Dual<4> wt = dc<4>(0.0);
            if (den.v > 0.0) wt = acn / den;
            a_i = an + wt * (ai - an);
            b_i = bn + wt * (bi - bn);
            c_i = cn + wt * (ci - cn);
        }
    }
    const double xa = x[i], xb = x[i + 1];
    Dual<4> term = a_i + (0.5 * (xb + xa)) * b_i;
    term = term + (((xb + xa) * xb + xa * xa) / 3.0) * c_i;
    return (xb - xa) * term;
}


__global__ void __launch_bounds__(64) transfer_adjoint_kernel(AdjArgs a) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const int L = a.n_layers;
    const double eps = EPS38;
    const double wl = a.grid[j];
    const double freq = C_LIGHT_NM / (wl > 1e-12 ? wl : 1e-12);
    double mass[MAX_LAYERS], ca[MAX_LAYERS], cs[MAX_LAYERS], la[MAX_LAYERS], src[MAX_LAYERS], pl[MAX_LAYERS];
    double ab[MAX_LAYERS], al[MAX_LAYERS], sn[MAX_LAYERS], tau[MAX_LAYERS];
    double gab[MAX_LAYERS], gal[MAX_LAYERS], gsn[MAX_LAYERS], gtau[MAX_LAYERS];
    int dmap[MAX_LAYERS];
    bool ok = L >= 3 && L <= MAX_LAYERS;
    for (int d = 0; ok && d < L; d++) {
        const DepthPar& dp = a.depth[d];
        const double cm = dp.rhox;
        const double aa = a.cont_abs[(int64_t)d * a.n + j], ss = a.cont_scat[(int64_t)d * a.n + j];
        const double lo = a.asynth[(int64_t)d * a.n + j];
        const double mx = MAX_OPACITY_REAL4;
        ok = cm > 0.0 && isfinite(cm) && isfinite(aa) && isfinite(ss) && isfinite(lo) && aa < mx && ss < mx &&
             lo < mx;
        mass[d] = cm;
        ca[d] = aa;
        cs[d] = ss;
        la[d] = lo;
        dmap[d] = d;
        pl[d] = planck_nu(freq, dp.hkt);
        // SLINEC with the driver's frequency (opacity.py:2215-2227, bfudge.py:144-145)
        const double fr = C_LIGHT_CM / (wl * 1.0e-7);
        const double f15 = fr / 1.0e15;
        const double eh = exp(-fr * dp.hkt);
        const double st = 1.0 - eh;
        const double bnu = 1.47439e-02 * pow(f15, 3.0) * eh / st;
        const double v = (bnu * st) / (1.0 - eh);
        src[d] = isfinite(v) ? v : pl[d];
    }
    if (ok && !(mass[0] < mass[L - 1])) {
        for (int q = 0; q < L / 2; q++) {
            const int r = L - 1 - q;
            double t;
            t = mass[q]; mass[q] = mass[r]; mass[r] = t;
            t = ca[q]; ca[q] = ca[r]; ca[r] = t;
            t = cs[q]; cs[q] = cs[r]; cs[r] = t;
            t = la[q]; la[q] = la[r]; la[r] = t;
            t = src[q]; src[q] = src[r]; src[r] = t;
            t = pl[q]; pl[q] = pl[r]; pl[r] = t;
            int ti = dmap[q]; dmap[q] = dmap[r]; dmap[r] = ti;
        }
    }
    for (int q = 1; ok && q < L; q++) ok = mass[q] > mass[q - 1];
    // forward: ABTOT, ALPHA, SNUBAR, TAU (josh_solver.py:367-470)
    bool ab_free[MAX_LAYERS], al_free[MAX_LAYERS];
    if (ok) {
        for (int q = 0; q < L; q++) {
            const double t = ca[q] + la[q] + cs[q];
            ab_free[q] = t > eps;
            ab[q] = t > eps ? t : eps;
            const double alp = ab[q] > 0.0 ? cs[q] / ab[q] : 0.0;
            al_free[q] = alp >= 0.0 && alp <= 1.0 && ab[q] > 0.0;
            al[q] = alp < 0.0 ? 0.0 : (alp > 1.0 ? 1.0 : alp);
            const double den = ca[q] + la[q];
            sn[q] = den > 0.0 ? (ca[q] * pl[q] + la[q] * src[q]) / den : pl[q];
        }
        integ_tau<double>(mass, ab, L, ab[0] * mass[0], tau);
        ok = !(tau[0] > a.xtau[NXTAU - 1]);
    }
    if (!ok) {
        for (int d = 0; d < L; d++) a.g_asy[(int64_t)d * a.n + j] = 0.0;
        atomicAdd(a.skipped, 1ull);
        return;
    }
    // MAP1 onto XTAU with the interval case of every grid point
    double xsb[NXTAU], xal[NXTAU], xb[NXTAU], xa[NXTAU], xm[NXTAU];
    int kl[NXTAU], kcase[NXTAU];
    {
        int l = 2;
        for (int k = 0; k < NXTAU; k++) {
            const double xk = a.xtau[k];
            while (l <= L && !(xk < tau[l - 1])) l++;
            int kase, node;
            if (l > L) {
                kase = 0;
                node = L;  // linear extrapolation on (L-1, L)
            } else if (l <= 3) {
                kase = 0;
                node = l;
            } else {
                kase = (l == L) ? 1 : 2;
                node = l;
            }
            kl[k] = node;
            kcase[k] = kase;
            // window x1[node-2..node+1] -> 0-based node-3..node
            Dual<1> x4[4], f4[4], g4[4];
            for (int q = 0; q < 4; q++) {
                const int idx = node - 3 + q;
                const int ic = idx < 0 ? 0 : (idx > L - 1 ? L - 1 : idx);
                x4[q] = dc<1>(tau[ic]);
                f4[q] = dc<1>(sn[ic]);
                g4[q] = dc<1>(al[ic]);
            }
            Dual<1> A, B, C;
            map_coeffs<1>(kase, x4, f4, A, B, C);
            xsb[k] = A.v + (B.v + C.v * xk) * xk;
            map_coeffs<1>(kase, x4, g4, A, B, C);
            xal[k] = A.v + (B.v + C.v * xk) * xk;
        }
    }
    const double s0 = sn[0] > eps ? sn[0] : eps;
    const double a0 = al[0] < 0.0 ? 0.0 : (al[0] > 1.0 ? 1.0 : al[0]);
    for (int k = 0; k < NXTAU; k++) {
        double b = xsb[k] > eps ? xsb[k] : eps;
        double x = xal[k] < 0.0 ? 0.0 : (xal[k] > 1.0 ? 1.0 : xal[k]);
        if (a.xtau[k] < tau[0]) {
            b = s0;
            x = a0;
        }
        xb[k] = b;
        xa[k] = x;
        xm[k] = b * (1.0 - x);
    }
    // converged solution of (I - diag(xa) C) xs = xm
    double xs[NXTAU], cxs[NXTAU];
    for (int k = 0; k < NXTAU; k++) xs[k] = xb[k];
    for (int it = 0; it < 2000; it++) {
        double dmax = 0.0;
        for (int k = NXTAU - 1; k >= 0; k--) {
            double sum = 0.0;
            for (int q = 0; q < NXTAU; q++) sum += a.coefj64[k * NXTAU + q] * xs[q];
            const double nv = sum * xa[k] + xm[k];
            const double dl = fabs(nv - xs[k]) / fmax(fabs(nv), 1e-300);
            dmax = dl > dmax ? dl : dmax;
            xs[k] = nv;
        }
        if (dmax < 1e-13) break;
    }
    for (int k = 0; k < NXTAU; k++) {
        double sum = 0.0;
        for (int q = 0; q < NXTAU; q++) sum += a.coefj64[k * NXTAU + q] * xs[q];
        cxs[k] = sum;
    }
    // ---- reverse ----
    const double gF = a.g_flux[j];
    // y = xsbar_bar + C^T (xa * y)
    double y[NXTAU], rhs[NXTAU];
    for (int k = 0; k < NXTAU; k++) {
        rhs[k] = gF * a.ch[k];
        y[k] = rhs[k];
    }
    for (int it = 0; it < 2000; it++) {
        double dmax = 0.0;
        for (int k = 0; k < NXTAU; k++) {
            double sum = 0.0;
            for (int q = 0; q < NXTAU; q++) sum += a.coefj64[q * NXTAU + k] * xa[q] * y[q];
            const double nv = rhs[k] + sum;
            const double dl = fabs(nv - y[k]) / fmax(fabs(nv), 1e-300);
            dmax = dl > dmax ? dl : dmax;
            y[k] = nv;
        }
        if (dmax < 1e-13) break;
    }
    for (int q = 0; q < L; q++) {
        gab[q] = 0.0;
        gal[q] = 0.0;
        gsn[q] = 0.0;
        gtau[q] = 0.0;
    }
    double gs0 = 0.0, ga0 = 0.0;
    for (int k = 0; k < NXTAU; k++) {
        const double gxa = y[k] * cxs[k] - y[k] * xb[k];
        const double gxb = y[k] * (1.0 - xa[k]);
        const double xk = a.xtau[k];
        if (xk < tau[0]) {
            gs0 += gxb;
            ga0 += gxa;
            continue;
        }
        const double gxsb = xsb[k] > eps ? gxb : 0.0;
        const double gxal = (xal[k] >= 0.0 && xal[k] <= 1.0) ? gxa : 0.0;
        if (gxsb == 0.0 && gxal == 0.0) continue;
        // d(value)/d(node x, node f) through the interval's coefficients
        const int node = kl[k];
        Dual<8> x8[4], f8[4], g8[4];
        int idx[4];
        for (int q = 0; q < 4; q++) {
            const int id = node - 3 + q;
            idx[q] = id;
            const int ic = id < 0 ? 0 : (id > L - 1 ? L - 1 : id);
            x8[q] = dv<8>(tau[ic], q);
            f8[q] = dv<8>(sn[ic], 4 + q);
            g8[q] = dv<8>(al[ic], 4 + q);
        }
        Dual<8> A, B, C;
        if (gxsb != 0.0) {
            map_coeffs<8>(kcase[k], x8, f8, A, B, C);
            for (int q = 0; q < 4; q++) {
                if (idx[q] < 0 || idx[q] > L - 1) continue;
                gtau[idx[q]] += gxsb * (A.d[q] + (B.d[q] + C.d[q] * xk) * xk);
                gsn[idx[q]] += gxsb * (A.d[4 + q] + (B.d[4 + q] + C.d[4 + q] * xk) * xk);
            }
        }
        if (gxal != 0.0) {
            map_coeffs<8>(kcase[k], x8, g8, A, B, C);
            for (int q = 0; q < 4; q++) {
                if (idx[q] < 0 || idx[q] > L - 1) continue;
                gtau[idx[q]] += gxal * (A.d[q] + (B.d[q] + C.d[q] * xk) * xk);
                gal[idx[q]] += gxal * (A.d[4 + q] + (B.d[4 + q] + C.d[4 + q] * xk) * xk);
            }
        }
    }
    if (sn[0] > eps) gsn[0] += gs0;
    if (al[0] >= 0.0 && al[0] <= 1.0) gal[0] += ga0;
    // INTEG: tau_0 = ab_0 x_0, tau_{i+1} = tau_i + inc_i(ab[i-1..i+2])
    double S = 0.0;
    for (int i = L - 2; i >= 0; i--) {
        S += gtau[i + 1];
        Dual<4> w[4];
        for (int q = 0; q < 4; q++) {
            const int id = i - 1 + q;
            const int ic = id < 0 ? 0 : (id > L - 1 ? L - 1 : id);
            w[q] = dv<4>(ab[ic], q);
        }
        const Dual<4> inc = adj_integ_inc(mass, L, i, w);
        for (int q = 0; q < 4; q++) {
            const int id = i - 1 + q;
            if (id >= 0 && id <= L - 1) gab[id] += S * inc.d[q];
        }
    }
    gab[0] += (S + gtau[0]) * mass[0];
    // ABTOT = ca + A + cs, ALPHA = cs / ABTOT, SNUBAR = (ca B + A S) / (ca + A)
    for (int q = 0; q < L; q++) {
        double g = 0.0;
        if (al_free[q]) gab[q] += gal[q] * (-cs[q] / (ab[q] * ab[q]));
        if (ab_free[q]) g += gab[q];
        const double den = ca[q] + la[q];
        if (den > 0.0) g += gsn[q] * (src[q] - sn[q]) / den;
        const int d = dmap[q];
        const double stim = 1.0 - exp(-freq * a.depth[d].hkt_asynth);
        a.g_asy[(int64_t)d * a.n + j] = g * stim;
    }
}


// d(near profile)/d(adamp) at offset o (a < 0.2: k0 h1; x > 10: k0 0.5642 /x^2;
// otherwise a central difference of H(v, a)).
__device__ __forceinline__ double near_profile_da(int o, double dvg, double ad, double k0, const double* h0,
                                                  const double* h1, const double* h2) {
    const double x = (double)o * dvg;
    if (ad < 0.2) {
        if (x > 10.0) return k0 * (0.5642 / (x * x));
        int idx = tabi_index<double>(o, 200.0 * dvg);
        idx = idx < 0 ? 0 : (idx > VOIGT_N - 1 ? VOIGT_N - 1 : idx);
        return k0 * h1[idx];
    }
    const double h = 1e-6 * (ad > 1.0 ? ad : 1.0);
    return k0 * (voigt_hv<double>(x, ad + h, h0, h1, h2) - voigt_hv<double>(x, ad - h, h0, h1, h2)) / (2.0 * h);
}

__global__ void __launch_bounds__(256) line_adjoint_kernel(LineAdjArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nslot = (int64_t)a.n_layers * a.stride;
    for (int64_t slot = warp; slot < nslot; slot += nwarp) {
        const int d = (int)(slot / a.stride);
        const int64_t li = slot - (int64_t)d * a.stride;
        if (li >= a.n_lines || a.cls[slot] == 0xff) continue;
        const PairDesc<double> pd = a.desc[slot];
        const double* G = a.g_asy + (int64_t)d * a.n_wl;
        const int64_t n = a.n_wl;
        double s_c = 0.0, s_a = 0.0;
        const int c = pd.wing_c;
        const int ctr = pd.ctr_n10 & 15;
        if (ctr && lane == 0) {
            const int64_t cc = (int64_t)c + (ctr - 8);
            if (cc >= 0 && cc < n) {
                s_c += G[cc] * pd.kapcen;
                // KAPCEN = kappa0 (1 - 1.128 a) for a < 0.2, kappa0 H(0, a) above
                const double ad = pd.adamp;
                double dk = 0.0;
                if (pd.kappa0 > 0.0) {
                    if (ad < 0.2) {
                        dk = -1.128 * pd.kappa0;
                    } else {
                        const double h = 1e-6 * (ad > 1.0 ? ad : 1.0);
                        dk = pd.kappa0 * (voigt_hv<double>(0.0, ad + h, a.h0, a.h1, a.h2) -
                                          voigt_hv<double>(0.0, ad - h, a.h0, a.h1, a.h2)) / (2.0 * h);
                    }
                }
                s_a += G[cc] * dk;
            }
        }
        const int reach = pd.maxstep_far & 0x7fffffff;
        if (reach > 0) {
            const int nz = pd.maxstep_far < 0 ? (pd.ctr_n10 >> 8) : 0x7fffffff;
            const double k0 = pd.kappa0, ad = pd.adamp, dvg = pd.dvoigt, xf = pd.xfar;
            // d xfar / d a = n10^2 k0 dH(n10 dv, a)/da
            double dxf = 0.0;
            if (nz != 0x7fffffff) dxf = (double)nz * (double)nz * near_profile_da(nz, dvg, ad, k0, a.h0, a.h1, a.h2);
            for (int o = 1 + lane; o <= reach; o += 32) {
                double v, dvda;
                if (o <= nz) {
                    v = near_profile<double>(o, dvg, ad, k0, a.h0, a.h1, a.h2);
                    dvda = near_profile_da(o, dvg, ad, k0, a.h0, a.h1, a.h2);
                } else {
                    const double oo = (double)o * (double)o;
                    v = xf / oo;
                    dvda = dxf / oo;
                }
                const int64_t br = (int64_t)c + o, bb = (int64_t)c - o;
                if (br >= 0 && br < n) {
                    s_c += G[br] * v;
                    s_a += G[br] * dvda;
                }
                if (bb >= 0 && bb < n) {
                    s_c += G[bb] * v;
                    s_a += G[bb] * dvda;
                }
            }
        }
        for (int off = 16; off > 0; off >>= 1) {
            s_c += __shfl_xor_sync(0xffffffffu, s_c, off);
            s_a += __shfl_xor_sync(0xffffffffu, s_a, off);
        }
        if (lane == 0) {
            a.g_gf[slot] = s_c;
            a.g_a[slot] = s_a;
        }
    }
}


// Per line: dLoss/dlog10 gf = ln10 sum_d (sum G c); dLoss/dlog10 gamma_x =
// ln10 gamma_x sum_d (sum G dc/da) da/dgamma_x, with da/dgamma = (1, XNE,
// TXNXN) / DOPPLE of the wing (line_opacity.py:1161-1272); the clamp of a at
// 1e-12 stops the gradient.
__global__ void line_grad_kernel(LineGradArgs a) {
    const int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= a.n_lines) return;
    const double ln10 = 2.302585092994046;
    double sgf = 0.0, sr = 0.0, ss = 0.0, sw = 0.0;
    const int e = a.element_idx[li], ion = a.ion_stage[li];
    const bool ion_ok = e >= 0 && e < a.n_elem && ion > 0 && ion <= a.n_ion;
    for (int d = 0; d < a.n_layers; d++) {
        const int64_t slot = (int64_t)d * a.stride + li;
        if (a.cls[slot] == 0xff) continue;
        sgf += a.g_gf[slot];
        if (!ion_ok) continue;
        const double ga = a.g_a[slot];
        if (ga == 0.0) continue;
        const DepthPar& dp = a.depth[d];
        const IonPar& q = a.ion[((int64_t)d * a.n_ion + (ion - 1)) * a.n_elem + e];
        const double dopple = q.dop;
        if (!(dopple > 0.0) || !(a.desc[slot].adamp > 1e-12)) continue;
        const double f = ga / dopple;
        sr += f;
        ss += f * dp.xne;
        sw += f * dp.txnxn;
    }
    a.d_loggf[li] = ln10 * sgf;
    a.d_loggr[li] = ln10 * a.gamma_rad[li] * sr;
    a.d_loggs[li] = ln10 * a.gamma_stark[li] * ss;
    a.d_loggw[li] = ln10 * a.gamma_vdw[li] * sw;
}

// Atmosphere terms, stage 1: one block per (species group, depth).  With the
// line's contributions c proportional to kappa0 = CGF * POP / (RHO * DOPPLE)
// * BOLT (line_opacity.py:101-184, :1141-1294), sum G c over a pair is
// dLoss/d ln POP of its species at that depth (and minus dLoss/d ln RHO); with
// a = (GAMRF + GAMSF * XNE + GAMWF * TXNXN) / DOPPLE, sum G dc/da * GAMSF /
// DOPPLE is its dLoss/dXNE and * GAMWF / DOPPLE its dLoss/dTXNXN.  The gates
// and the wing reach are held fixed, as for the line gradients.  Lanes take
// the group's lines in a fixed stride and the block sums in a fixed tree.
__global__ void __launch_bounds__(128) atm_grad_group_kernel(AtmGradArgs a) {
    const int g = blockIdx.x, d = blockIdx.y;
    const int f0 = a.group_first[g], f1 = a.group_first[g + 1];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = f0 + (int)threadIdx.x; k < f1; k += blockDim.x) {
        const int64_t li = a.order[k];
        const int64_t slot = (int64_t)d * a.stride + li;
        if (a.cls[slot] == 0xff) continue;
        s0 += a.g_gf[slot];
        const double ga = a.g_a[slot];
        if (ga == 0.0) continue;
        const int e = a.element_idx[li], ion = a.ion_stage[li];
        if (e < 0 || e >= a.n_elem || ion <= 0 || ion > a.n_ion) continue;
        const IonPar& q = a.ion[((int64_t)d * a.n_ion + (ion - 1)) * a.n_elem + e];
        if (!(q.dop > 0.0) || !(a.desc[slot].adamp > 1e-12)) continue;
        const double f = ga / q.dop;
        s1 += f * a.gamma_stark[li];
        s2 += f * a.gamma_vdw[li];
    }
    __shared__ double r0[128], r1[128], r2[128];
    r0[threadIdx.x] = s0;
    r1[threadIdx.x] = s1;
    r2[threadIdx.x] = s2;
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            r0[threadIdx.x] += r0[threadIdx.x + w];
            r1[threadIdx.x] += r1[threadIdx.x + w];
            r2[threadIdx.x] += r2[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double* p = a.part + ((int64_t)d * a.n_groups + g) * 3;
        p[0] = r0[0];
        p[1] = r1[0];
        p[2] = r2[0];
        a.d_ln_pop[(int64_t)d * a.n_ion * a.n_elem + a.group_species[g]] = r0[0];
    }
}

// Stage 2: per depth, the groups' sums in group order.
__global__ void atm_grad_depth_kernel(AtmGradArgs a) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= a.n_layers) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int g = 0; g < a.n_groups; g++) {
        const double* p = a.part + ((int64_t)d * a.n_groups + g) * 3;
        s0 += p[0];
        s1 += p[1];
        s2 += p[2];
    }
    a.d_ln_rho[d] = -s0;
    a.d_xne[d] = s1;
    a.d_txnxn[d] = s2;
}

}  // namespace ks
