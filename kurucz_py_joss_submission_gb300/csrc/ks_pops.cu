// ks_pops.cu -- FP64 populations of model atmospheres on the GPU.
//
// What the reference's atmosphere converter computes from an ATLAS model
// before synthesis (synthe_py/tools/convert_atm_to_npz.py:1860-2650): the
// molecular equilibrium NMOLEC (synthe_py/tools/nmolec_exact.py:1742), the
// Saha-Boltzmann ion populations of POPS/PFSAHA
// (synthe_py/tools/pops_exact.py:987, :1639) and the Doppler widths
// (:2027), every step in double precision.  Compiled with --fmad=false, so
// every product and sum is rounded separately as in the reference.
//
// Two kernels, each templated on the scalar (double, or a dual number that
// carries d/d log10 XABUND of one element for the forward-mode derivatives):
//   nmolec_block_kernel  one block per model atmosphere: the molecular
//                        equilibrium, layer after layer (see below).
//   pops_kernel          one block per (model, layer): the ion populations of
//                        the 99 elements (one thread per element) and the
//                        Doppler widths of the 6 x 139 species.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kurucz_gb300.h"
#include "ks_launch.h"

namespace {

constexpr int kMaxEq = 32;     // one lane per equation (the reference allows 30)
constexpr int kMaxMol = 200;   // MAXMOL (nmolec_exact.py:26)
constexpr int kMaxLoc = 600;   // MAXLOC
constexpr int kNIon = 6, kNSpec = 139, kNEl = 99;
constexpr int kMaxIter = 200;  // Newton iterations per layer (nmolec_exact.py:2544)
constexpr int kNLevTab = 14;
constexpr int kLevCap = 192;
constexpr int kPfgLabels = 667;  // labels run 1..666
constexpr int kPfgRows = 256, kPfgTerms = 640;

// Constants of the reference (convert_atm_to_npz.py:68-79, pops_exact.py:156-170).
constexpr double kCcms = 2.99792458e10;
constexpr double kHPlanck = 6.62607015e-27;
constexpr double kKBoltz = 1.380649e-16;
constexpr double kKBoltzFortran = 1.38054e-16;
constexpr double kEvToCm = 8065.479;

// Explicitly summed partition functions (pops_exact.py:1130-1430), keyed by
// the NNN column of the species.  Terms are (weight, energy in cm^-1); an
// energy of -1 marks a bare weight.  tmin < 0: the level sum always applies.
struct SpecialPF {
    int col, lev, nlev;
    int nbase;
    double base_g[3], base_e[3];
    int nextra;
    double extra_g[10], extra_e[10];
    double tmin;
    double d1_num, d1_n;  // D1 = d1_num / d1_n / d1_n * HCKT (0: not set)
    double g_over;        // replaces the NNN weight G when > 0
};

// Level tables in the order of the reference's DATA blocks.
enum { LV_HYD, LV_HE1, LV_HE2, LV_C1, LV_C2, LV_O1, LV_MG1, LV_MG2, LV_AL1, LV_SI1, LV_SI2, LV_NA1,
       LV_B1, LV_K1 };

__constant__ SpecialPF c_special[16] = {
    {1, LV_HYD, 5, 1, {2.0}, {-1.0}, 0, {}, {}, 9000.0, 109677.576, 6.5, 0.0},
    {3, LV_HE1, 28, 1, {1.0}, {-1.0}, 0, {}, {}, 15000.0, 109677.576, 5.5, 0.0},
    {4, LV_HE2, 5, 1, {2.0}, {-1.0}, 0, {}, {}, 30000.0, 4.0 * 109722.267, 6.5, 0.0},
    {354, LV_C1, 13, 3, {1.0, 3.0, 5.0}, {-1.0, 16.42, 43.42}, 6,
     {108.0, 189.0, 247.0, 231.0, 190.0, 300.0},
     {80000.0, 84000.0, 87000.0, 88000.0, 89000.0, 90000.0}, -1.0, 0.0, 1.0, 0.0},
    {355, LV_C2, 5, 2, {2.0, 4.0}, {-1.0, 63.42}, 10,
     {6.0, 4.0, 10.0, 10.0, 2.0, 6.0, 42.0, 56.0, 102.0, 400.0},
     {131731.80, 142027.1, 145550.13, 150463.62, 157234.07, 162500.0, 168000.0, 178000.0,
      183000.0, 188000.0}, -1.0, 0.0, 1.0, 0.0},
    {51, LV_MG1, 10, 1, {1.0}, {-1.0}, 4, {5.0, 15.0, 28.0, 9.0},
     {53134.0, 54192.0, 54676.0, 57853.0}, -1.0, 109734.83, 4.5, 4.0},
    {52, LV_MG2, 5, 1, {2.0}, {-1.0}, 6, {10.0, 14.0, 6.0, 10.0, 14.0, 18.0},
     {93310.80, 93799.70, 97464.32, 103419.82, 103689.89, 103705.66}, -1.0, 4.0 * 109734.83, 5.5,
     2.0},
    {57, LV_AL1, 8, 2, {2.0, 4.0}, {-1.0, 112.061}, 2, {10.0, 14.0}, {42235.0, 43831.0}, -1.0,
     109735.08, 5.5, 2.0},
    {63, LV_SI1, 10, 3, {1.0, 3.0, 5.0}, {-1.0, 77.115, 223.157}, 6,
     {76.0, 71.0, 191.0, 240.0, 251.0, 300.0},
     {53000.0, 57000.0, 60000.0, 62000.0, 63000.0, 65000.0}, -1.0, 0.0, 1.0, 0.0},
    {64, LV_SI2, 5, 2, {2.0, 4.0}, {-1.0, 287.32}, 9,
     {6.0, 6.0, 10.0, 14.0, 10.0, 42.0, 6.0, 38.0, 34.0},
     {81231.59, 83937.08, 101024.09, 103556.35, 108800.0, 115000.0, 121000.0, 125000.0, 132000.0},
     -1.0, 4.0 * 109734.83, 4.5, 2.0},
    {367, LV_O1, 12, 3, {5.0, 3.0, 1.0}, {-1.0, 158.265, 226.977}, 4,
     {15.0, 131.0, 128.0, 600.0}, {101140.0, 103000.0, 105000.0, 107000.0}, -1.0, 0.0, 1.0, 0.0},
    {45, LV_NA1, 7, 1, {2.0}, {-1.0}, 2, {10.0, 14.0}, {34548.745, 34586.96}, -1.0, 109734.83, 4.5,
     2.0},
    {14, LV_B1, 6, 2, {2.0, 4.0}, {-1.0, 15.25}, 4, {6.0, 10.0, 14.0, 2.0},
     {57786.80, 59989.0, 60031.03, 63561.0}, -1.0, 109734.83, 4.5, 2.0},
    {91, LV_K1, 7, 1, {2.0}, {-1.0}, 2, {10.0, 14.0}, {27397.077, 28127.85}, -1.0, 109734.83, 5.5,
     2.0},
    {0}, {0}};
constexpr int kNSpecial = 14;

__constant__ int c_locz[29] = {1,  3,  6,  10, 14, 18, 22, 27, 33, 39, 45,  51,  57,  63, 69,
                               75, 81, 86, 91, 96, 101, 106, 111, 116, 121, 126, 131, 136, 141};
__constant__ double c_scale[4] = {0.001, 0.01, 0.1, 1.0};

// Data tables and the molecular system, resident on every device.
struct PopsTables {
    double potion[999];
    int nnn[6 * 374];
    double atmass[kNEl];
    double pftab[7 * 56 * 10 * 9];
    double pf_potlo[7], pf_potlolog[7];
    double lev_e[kLevCap], lev_g[kLevCap];
    int lev_off[kNLevTab + 1];
    int pfg_first[114], pfg_second[168], n_first, n_second;
    int pfg_row[kPfgLabels];  // label -> row, -1 if the label has no expression
    double pfg_g0[kPfgRows];
    int pfg_off[kPfgRows + 1];
    double pfg_g[kPfgTerms], pfg_e[kPfgTerms];
    // molecular system (READMOL, readmol_exact.py:20)
    int nmol, nequa, has_e;
    double mol_code[kMaxMol];
    double mol_equil[7 * kMaxMol];  // [7][kMaxMol]
    int locj[kMaxMol + 1];
    int kcomps[kMaxLoc];            // equation numbers; nequa = inverse electron
    int idequa[kMaxEq];
    int col_off[kMaxEq + 1];        // molecules holding equation k (ascending), CSR
    int col_mol[kMaxLoc];
    int slot_mol[kMaxLoc];          // molecule of each component slot
    // POPS molecular branch (pops_exact.py:1855-1900) per element: 1 when the
    // element's populations come from the molecule table; the table row of
    // each ion (-1: none, the population is zero)
    int elem_mol_branch[kNEl];
    int elem_mol_row[kNEl][10];
    int elem_nion[kNEl];            // NION of the all-ion POPS call
    int row_h1, row_he1;            // rows of "1." and "2."
    double momass[100];
};

__device__ PopsTables g_pops;

struct HostPops {
    bool ready = false;
    PopsTables t;
};
HostPops g_host;
std::mutex g_mu;
constexpr int kMaxDev = 64;
bool g_dev_ready[kMaxDev];

// ---------------------------------------------------------------------------
// scalar types: double, and a forward-mode dual number (value, derivative)
// carrying d/d(log10 XABUND of one element) through the same code
// ---------------------------------------------------------------------------

struct D1 {
    double v, d;
    __host__ __device__ constexpr D1() : v(0.0), d(0.0) {}
    __host__ __device__ constexpr D1(double x) : v(x), d(0.0) {}
    __host__ __device__ constexpr D1(double x, double dx) : v(x), d(dx) {}
};
__device__ __forceinline__ D1 mk(double v, double d = 0.0) { return D1{v, d}; }
__device__ __forceinline__ D1 operator+(D1 a, D1 b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ D1 operator-(D1 a, D1 b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ D1 operator-(D1 a) { return {-a.v, -a.d}; }
__device__ __forceinline__ D1 operator*(D1 a, D1 b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ D1 operator/(D1 a, D1 b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ D1 operator+(D1 a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ D1 operator+(double a, D1 b) { return {a + b.v, b.d}; }
__device__ __forceinline__ D1 operator-(D1 a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ D1 operator-(double a, D1 b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ D1 operator*(D1 a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ D1 operator*(double a, D1 b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ D1 operator/(D1 a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ D1 operator/(double a, D1 b) {
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
__device__ __forceinline__ D1& operator+=(D1& a, D1 b) { return a = a + b; }
__device__ __forceinline__ D1& operator*=(D1& a, D1 b) { return a = a * b; }
// elementary functions of a scalar that may be a dual number
__device__ __forceinline__ double sexp(double x) { return exp(x); }
__device__ __forceinline__ D1 sexp(D1 a) {
    const double e = exp(a.v);
    return {e, e * a.d};
}
__device__ __forceinline__ double ssqrt(double x) { return sqrt(x); }
__device__ __forceinline__ D1 ssqrt(D1 a) {
    const double r = sqrt(a.v);
    return {r, a.d / (2.0 * r)};
}
__device__ __forceinline__ double slog10(double x) { return log10(x); }
__device__ __forceinline__ D1 slog10(D1 a) { return {log10(a.v), a.d / (a.v * 2.302585092994046)}; }
__device__ __forceinline__ double spow(double x, double p) { return pow(x, p); }
__device__ __forceinline__ D1 spow(D1 a, double p) {
    const double r = pow(a.v, p);
    return {r, p * pow(a.v, p - 1.0) * a.d};
}

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(D1 x) { return x.v; }
__device__ __forceinline__ double der(double) { return 0.0; }
__device__ __forceinline__ double der(D1 x) { return x.d; }
template <typename S>
__device__ __forceinline__ S lift(double v);
template <>
__device__ __forceinline__ double lift<double>(double v) { return v; }
template <>
__device__ __forceinline__ D1 lift<D1>(double v) { return D1{v, 0.0}; }
// min / max by value (the choice the reference's arithmetic makes)
template <typename S>
__device__ __forceinline__ S smin(S a, S b) { return val(b) < val(a) ? b : a; }
template <typename S>
__device__ __forceinline__ S smax(S a, S b) { return val(b) > val(a) ? b : a; }

// ---------------------------------------------------------------------------
// PFSAHA (pops_exact.py:987-1636) for one layer
// ---------------------------------------------------------------------------

struct LayerState {
    double t, tkev, tk, hckt, tlog, p, xntot, vturb;
};

__device__ double pfground_dev(int nelion, double t) {
    const PopsTables& P = g_pops;
    if (t <= 0.0 || nelion <= 0) return 1.0;
    int label;
    if (nelion <= P.n_first) label = P.pfg_first[nelion - 1];
    else if (nelion < 169) return 1.0;
    else if (nelion - 169 < P.n_second) label = P.pfg_second[nelion - 169];
    else label = 666;
    if (label < 0 || label >= kPfgLabels) return 1.0;
    const int row = P.pfg_row[label];
    if (row < 0) return 1.0;
    const double hck = 6.6256e-27 * 2.99792458e10 / 1.38054e-16;
    double v = P.pfg_g0[row];
    for (int k = P.pfg_off[row]; k < P.pfg_off[row + 1]; k++) v = v + P.pfg_g[k] * exp(-hck / t * P.pfg_e[k]);
    return v;
}

template <typename S>
__device__ S pfiron_dev(int iz, int ion, double tlog10, S potlow) {
    const PopsTables& P = g_pops;
    const int e = iz - 20, i = ion - 1;
    int it;
    double f;
    if (tlog10 > 4.0) {
        it = (int)((tlog10 - 4.0) / 0.05 + 31.0);
        it = it < 1 ? 1 : (it > 56 ? 56 : it);
        f = (tlog10 - (it - 31) * 0.05 - 4.0) / 0.05;
    } else if (tlog10 < 3.7) {
        it = (int)((tlog10 - 3.32) / 0.02 + 2.0);
        it = it < 2 ? 2 : it;
        f = (tlog10 - (it - 2) * 0.02 - 3.32) / 0.02;
    } else {
        it = (int)((tlog10 - 3.7) / 0.03 + 21.0);
        f = (tlog10 - (it - 21) * 0.03 - 3.7) / 0.03;
    }
    it = it < 1 ? 1 : (it > 56 ? 56 : it);
    const int a = it - 1, b = (it - 2) > 0 ? it - 2 : 0;
    auto tab = [&](int low, int k) { return P.pftab[((low * 56 + k) * 10 + i) * 9 + e]; };
    if (val(potlow) < P.pf_potlo[0]) return lift<S>(f * tab(0, a) + (1.0 - f) * tab(0, b));
    int low = 6;
    for (int k = 1; k < 7; k++)
        if (val(potlow) < P.pf_potlo[k]) {
            low = k;
            break;
        }
    const S p = (slog10(potlow) - P.pf_potlolog[low - 1]) / 0.30103;
    return p * (f * tab(low, a) + (1.0 - f) * tab(low, b)) +
           (1.0 - p) * (f * tab(low - 1, a) + (1.0 - f) * tab(low - 1, b));
}

__device__ __forceinline__ int potion_index(int iz, int ion) {
    return iz <= 30 ? iz * (iz + 1) / 2 + ion - 1 : iz * 5 + 341 + ion - 1;
}

// Saha fractions F[0..nion2) (normalised) and partition functions PART of
// element iz for a layer; returns NION2 = min(nion + 2, number of ions).
// Only the electron density carries a derivative (S = D1); the partition
// functions depend on it through the lowered ionisation potential.
template <typename S>
__device__ int pfsaha_dev(int iz, int nion, const LayerState& s, S xne, S* F, S* PART) {
    const PopsTables& P = g_pops;
    S charge = xne * 2.0;
    const S excess = 2.0 * xne - s.p / s.tk;
    if (val(excess) > 0.0) charge = charge + 2.0 * excess;
    if (val(charge) == 0.0) charge = lift<S>(1.0);
    const S debye = ssqrt(s.tk / 2.8965e-18 / charge);
    const S potlow = smin<S>(lift<S>(1.0), 1.44e-7 / debye);
    int n, nions;
    if (iz <= 28) {
        n = c_locz[iz - 1];
        nions = c_locz[iz] - c_locz[iz - 1];
    } else {
        n = 3 * iz + 54;
        nions = 3;
    }
    if (iz == 6) { n = 354; nions = 6; }
    else if (iz == 7) { n = 360; nions = 7; }
    else if (iz == 8) { n = 367; nions = 8; }
    if (iz >= 20 && iz < 29) nions = 10;
    const int nion2 = (nion + 2) < nions ? nion + 2 : nions;
    double IP[10];
    S POTLO[10];
    const double T = s.t, hckt = s.hckt;
    for (int ion = 1; ion <= nion2; ion++) {
        const double z = (double)ion;
        POTLO[ion - 1] = potlow * z;
        IP[ion - 1] = 0.0;
        PART[ion - 1] = lift<S>(1.0);
        const int pi = potion_index(iz, ion) - 1;
        if (pi >= 0 && pi < 999) {
            IP[ion - 1] = P.potion[pi] / kEvToCm;
            if (IP[ion - 1] == 0.0 && pi > 0) IP[ion - 1] = P.potion[pi - 1] / kEvToCm;
        }
        if (iz >= 20 && iz < 29) {
            PART[ion - 1] = pfiron_dev<S>(iz, ion, s.tlog / 2.30258509299405, POTLO[ion - 1] * kEvToCm);
            continue;
        }
        const int col = n - 1 + ion;  // 1-based NNN column
        const int c0 = col - 1;
        double G = 0.0, D1v = 0.0;
        if (c0 < 374) {
            const int v = P.nnn[5 * 374 + c0];
            G = (double)(v - (v / 100) * 100);
        }
        bool handled = false;
        if (col == 2) {
            PART[ion - 1] = lift<S>(1.0);
            handled = true;
        }
        for (int q = 0; q < kNSpecial; q++) {
            const SpecialPF& sp = c_special[q];
            if (sp.col != col) continue;
            double part = 0.0;
            for (int b = 0; b < sp.nbase; b++) {
                const double term = sp.base_e[b] < 0.0 ? sp.base_g[b] : sp.base_g[b] * exp(-sp.base_e[b] * hckt);
                part = b == 0 ? term : part + term;
            }
            if (sp.tmin < 0.0 || T >= sp.tmin) {
                const int o = P.lev_off[sp.lev];
                for (int i = 1; i <= sp.nlev; i++) part += P.lev_g[o + i] * exp(-P.lev_e[o + i] * hckt);
            }
            if (sp.nextra > 0) {
                double x = 0.0;
                for (int b = 0; b < sp.nextra; b++) {
                    const double term = sp.extra_g[b] * exp(-sp.extra_e[b] * hckt);
                    x = b == 0 ? term : x + term;
                }
                part += x;
            }
            PART[ion - 1] = lift<S>(part);
            if (sp.d1_num > 0.0) D1v = sp.d1_num / sp.d1_n / sp.d1_n * hckt;
            if (sp.g_over > 0.0) G = sp.g_over;
            handled = true;
            break;
        }
        if (!handled && c0 < 374 && IP[ion - 1] > 0.0) {
            const double t2000 = IP[ion - 1] * 2000.0 / 11.0;
            int it = (int)(T / t2000 - 0.5);
            it = it < 1 ? 1 : (it > 9 ? 9 : it);
            const double dt = T / t2000 - (double)it - 0.5;
            double pmin = 1.0;
            int ii = (it + 1) / 2 - 1;
            ii = ii < 0 ? 0 : (ii > 5 ? 5 : ii);
            const int v = P.nnn[ii * 374 + c0];
            const int k1 = v / 100000, k2 = v - k1 * 100000, k3 = k2 / 10;
            int ks = k2 - k3 * 10 - 1;
            ks = ks < 0 ? 0 : (ks > 3 ? 3 : ks);
            double p1, p2;
            if (it % 2 == 1) {
                p1 = (double)k1 * c_scale[ks];
                p2 = (double)k3 * c_scale[ks];
                if (dt < 0.0 && ks <= 0 && p1 == (double)(int)(p2 + 0.5)) pmin = p1;
            } else {
                p1 = (double)k3 * c_scale[ks];
                const int v1 = P.nnn[(ii + 1 < 5 ? ii + 1 : 5) * 374 + c0];
                int ks1 = v1 % 10 - 1;
                ks1 = ks1 < 0 ? 0 : (ks1 > 3 ? 3 : ks1);
                p2 = (double)(v1 / 100000) * c_scale[ks1];
            }
            PART[ion - 1] = lift<S>(fmax(pmin, p1 + (p2 - p1) * dt));
        } else if (!handled) {
            PART[ion - 1] = lift<S>(1.0);
        }
        bool skip_high_t = false;
        if (IP[ion - 1] > 0.0) {
            const double t2000 = IP[ion - 1] * 2000.0 / 11.0;
            if (T < t2000 * 2.0) {
                const double pg = pfground_dev((iz - 1) * 6 + ion, T);
                if (pg > 0.0) PART[ion - 1] = smax<S>(PART[ion - 1], lift<S>(pg));
                skip_high_t = true;
            }
        }
        const bool bypass = D1v > 0.0;
        if (!skip_high_t && (G > 0.0 || D1v > 0.0) && (bypass || val(POTLO[ion - 1]) >= 0.1) && IP[ion - 1] > 0.0) {
            const double t2000 = IP[ion - 1] * 2000.0 / 11.0;
            if (bypass || T >= t2000 * 4.0) {
                double tvu = s.tkev;
                if (T > t2000 * 11.0) tvu = (t2000 * 11.0) * 8.6171e-5;
                const double d1v = D1v <= 0.0 ? 0.1 / tvu : D1v;
                const S d2 = POTLO[ion - 1] / tvu;
                S term1 = spow(ssqrt(13.595 * z * z / tvu / d2), 3.0);
                term1 *= 1.0 / 3.0 + (1.0 - (0.5 + (1.0 / 18.0 + d2 / 120.0) * d2) * d2) * d2;
                double term2 = pow(sqrt(13.595 * z * z / tvu / d1v), 3.0);
                term2 *= 1.0 / 3.0 + (1.0 - (0.5 + (1.0 / 18.0 + d1v / 120.0) * d1v) * d1v) * d1v;
                if (G > 0.0) PART[ion - 1] += G * exp(-IP[ion - 1] / tvu) * (term1 - term2);
            }
        }
    }
    const S cf = 2.0 * 2.4148e15 * T * sqrt(T) / xne;
    F[0] = lift<S>(1.0);
    for (int ion = 2; ion <= nion2; ion++)
        F[ion - 1] = val(PART[ion - 2]) > 0.0
                         ? cf * PART[ion - 1] / PART[ion - 2] * sexp(-(IP[ion - 2] - POTLO[ion - 2]) / s.tkev)
                         : lift<S>(0.0);
    int l = nion2 + 1;
    for (int ion = 2; ion <= nion2; ion++) {
        l -= 1;
        F[0] = 1.0 + F[l - 1] * F[0];
    }
    F[0] = 1.0 / F[0];
    for (int ion = 2; ion <= nion2; ion++) F[ion - 1] = F[ion - 2] * F[ion - 1];
    return nion2;
}

__device__ LayerState layer_state(double t, double p, double vturb) {
    LayerState s;
    s.t = t;
    s.tkev = t / (1.0 / 8.6171e-5);
    s.tk = kKBoltzFortran * t;
    s.hckt = kHPlanck * kCcms / (kKBoltz * t);
    s.tlog = log(t);
    s.p = p;
    s.xntot = p / s.tk;
    s.vturb = vturb;
    return s;
}

// Equilibrium constant of molecule m in a layer (nmolec_exact.py:2268-2531);
// the NLTE partition-function corrections are 1 in LTE.
template <typename S>
__device__ S equilj_dev(int m, const LayerState& s, S xne) {
    const PopsTables& P = g_pops;
    const int ncomp = P.locj[m + 1] - P.locj[m];
    const double code = P.mol_code[m];
    if (P.mol_equil[m] == 0.0) {
        if (ncomp <= 1) return lift<S>(1.0);
        S F[10], PART[10];
        pfsaha_dev<S>((int)code, ncomp, s, xne, F, PART);
        const S f0 = F[0];
        if (val(f0) == 0.0 || fabs(val(f0)) < 1e-300 || !isfinite(val(f0))) return lift<S>(0.0);
        return F[ncomp - 1] / f0 * spow(xne, (double)(ncomp - 1));
    }
    if (s.t > 10000.0) return lift<S>(0.0);
    const int ion = (int)((code - (double)(int)code) * 100.0 + 0.5);
    const double T = s.t;
    double arg;
    if (fabs(code - 101.0) < 1e-9) {
        arg = 4.478 / s.tkev - 46.4584 +
              (1.63660e-3 +
               (-4.93992e-7 + (1.11822e-10 + (-1.49567e-14 + (1.06206e-18 - 3.08720e-23 * T) * T) * T) * T) * T) *
                  T -
              1.5 * s.tlog;
    } else {
        const double* e = P.mol_equil;
        auto E = [&](int k) { return e[k * kMaxMol + m]; };
        arg = E(0) / s.tkev - E(1) + (E(2) + (-E(3) + (E(4) + (-E(5) + E(6) * T) * T) * T) * T) * T -
              1.5 * (double)(ncomp - ion - ion - 1) * s.tlog;
    }
    return lift<S>(exp(arg));
}

// ---------------------------------------------------------------------------
// job records and shared helpers of the molecular equilibrium
// ---------------------------------------------------------------------------

template <typename S>
struct PopsJobT {
    int n_layers;
    int dparam;          // D1: Z-1 of the element whose log10 abundance is differentiated
    const double *t, *p, *vturb, *xabund;
    double *xne, *rho, *xnatom, *hckt, *xnf_h, *xnf_he1, *xnf_h2, *population, *doppler;
    int32_t* iterations;
    // D1: derivatives of the outputs (device) w.r.t. log10 XABUND[dparam]
    double *d_xne, *d_rho, *d_xnf_h, *d_xnf_he1, *d_xnf_h2, *d_population;
    S* xnmol;            // workspace [L, kMaxMol]
    S* xnat;             // workspace [L] XNATOM
    S* xnes;             // workspace [L] XNE
    LayerState* state;   // workspace [L]
};
using PopsJob = PopsJobT<double>;

__device__ __forceinline__ int comp_eq(int kr, int ne) { return kr >= ne ? ne - 1 : kr; }

__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }

// numpy's pairwise sum of 99 values (8 accumulators, then the rest), the
// order np.sum gives WTMOLE in the reference.
template <typename S>
__device__ S wtmole_dev(const S* xabund) {
    const PopsTables& P = g_pops;
    S r[8];
    for (int j = 0; j < 8; j++) r[j] = xabund[j] * P.atmass[j];
    int i = 8;
    for (; i < kNEl - (kNEl % 8); i += 8)
        for (int j = 0; j < 8; j++) r[j] += xabund[i + j] * P.atmass[i + j];
    S res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < kNEl; i++) res += xabund[i] * P.atmass[i];
    return res;
}

template <typename S>
__device__ __forceinline__ S abundance(const PopsJobT<S>& J, int z0) {
    const double x = J.xabund[z0];
    if constexpr (sizeof(S) == sizeof(double)) {
        return x;
    } else {
        return D1{x, z0 == J.dparam ? 2.302585092994046 * x : 0.0};
    }
}

template <typename S>
__device__ __forceinline__ void store(double* v, double* d, size_t i, S x) {
    if (v) v[i] = val(x);
    if constexpr (sizeof(S) != sizeof(double)) {
        if (d) d[i] = der(x);
    }
}

// ---------------------------------------------------------------------------
// nmolec_block_kernel: NMOLEC (nmolec_exact.py:1742-3575), one block of
// kPopThreads per model.  The layers are solved surface first, each Newton
// iteration seeded from the previous layer's solution times the pressure
// ratio, so a model is one sequential chain.  FP64 arithmetic is scarce on
// this part (1/64 of the FP32 rate), so the work of an iteration is spread
// over the block: the molecular terms and every division of the Jacobian
// (term / XN of each component slot) in parallel, then each column of DEQ
// summed by one thread in the reference's molecule and component order
// (:760-926; every DEQ and EQ entry gets the reference's additions in the
// reference's order), SOLVIT (:3671-3765) with one matrix entry per thread
// in the elimination, and the divisions of the update in parallel ahead of
// its sequential SCALE logic.
// ---------------------------------------------------------------------------

constexpr int kPopThreads = 128;

template <typename S>
struct BlockShared {
    S a[kMaxEq * kMaxEq];
    S b[kMaxEq];
    S xn[kMaxEq], xab[kMaxEq], eqold[kMaxEq], dcol[kMaxEq];
    S equilj[kMaxMol], term[kMaxMol];
    S dmain[kMaxLoc];               // term / XN (minus for an inverse electron) per component slot
    S dcorr[kMaxLoc];               // term / XN of the slot's equation (negative-ion correction)
    S xab_all[kNEl];
    S xneq[kMaxEq];
    unsigned char skip[kMaxMol];
    unsigned char ratio_err[kMaxEq], flip[kMaxEq];
    double best[kPopThreads / 32];
    int bidx[kPopThreads / 32];
    int piv_row, piv_col;
    int pcount[kMaxEq];
    int iferr;
};

template <typename S>
__device__ void assemble_column_pre(BlockShared<S>& B, int k, double xntot) {
    const PopsTables& P = g_pops;
    const int ne = P.nequa, e = ne - 1;
    for (int r = 0; r < ne; r++) B.a[r * kMaxEq + k] = lift<S>(0.0);
    S eqk;
    if (k == 0) {
        eqk = lift<S>(-xntot);
        for (int q = 1; q < ne; q++) {
            eqk = eqk + B.xn[q];
            B.a[q * kMaxEq + 0] = -B.xab[q];
        }
        for (int m = 0; m < P.nmol; m++) {
            if (P.locj[m + 1] - P.locj[m] <= 1 || B.skip[m]) continue;
            eqk = eqk + B.term[m];
        }
        B.b[0] = eqk;
        return;
    }
    B.a[0 * kMaxEq + k] = lift<S>(1.0);
    B.a[k * kMaxEq + k] = lift<S>(1.0);
    eqk = B.xn[k] - B.xab[k] * B.xn[0];
    if (P.has_e && k == e) {
        eqk = -B.xn[e];
        B.a[e * kMaxEq + e] = lift<S>(-1.0);
    }
    for (int q = P.col_off[k]; q < P.col_off[k + 1]; q++) {
        const int m = P.col_mol[q];
        if (B.skip[m]) continue;
        const S t = B.term[m];
        const int l1 = P.locj[m], l2 = P.locj[m + 1];
        for (int lk = l1; lk < l2; lk++) {
            if (comp_eq(P.kcomps[lk], ne) != k) continue;
            const S d = B.dmain[lk];
            eqk = eqk + t;
            B.a[0 * kMaxEq + k] = B.a[0 * kMaxEq + k] + d;
            for (int lm = l1; lm < l2; lm++) {
                const int mm = comp_eq(P.kcomps[lm], ne);
                B.a[mm * kMaxEq + k] = B.a[mm * kMaxEq + k] + d;
            }
        }
        if (P.has_e && P.kcomps[l2 - 1] == e) {
            for (int lk = l1; lk < l2; lk++) {
                const int kk = comp_eq(P.kcomps[lk], ne);
                if (kk != k) continue;
                const S d = B.dcorr[lk];
                if (kk == e) eqk = eqk - t - t;
                B.a[e * kMaxEq + k] = B.a[e * kMaxEq + k] - d - d;
            }
        }
    }
    B.b[k] = eqk;
}

// SOLVIT (nmolec_exact.py:3671-3765): Gauss-Jordan elimination with the
// full pivot search (largest |a| over unpivoted rows and columns, first in
// row-major order on ties; pivots chosen on the values, so with dual numbers
// the derivative is that of the same elimination), rows swapped to put the
// pivot on the diagonal, one matrix entry per thread in the elimination.
// The solution is left in B.b.
template <typename S>
__device__ void solvit_block(BlockShared<S>& B, int n) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid < kMaxEq) B.pcount[tid] = 0;
    __syncthreads();
    for (int step = 0; step < n; step++) {
        double best = 0.0;
        int bi = 0x7fffffff;
        for (int idx = tid; idx < n * n; idx += kPopThreads) {
            const int r = idx / n, c = idx - r * n;
            if (B.pcount[r] == 1 || B.pcount[c] == 1) continue;
            const double v = fabs(val(B.a[r * kMaxEq + c]));
            if (v > best) {  // ascending idx per thread: the first maximum
                best = v;
                bi = idx;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = shfl_xor(best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (lane == 0) {
            B.best[w] = best;
            B.bidx[w] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            double bb = B.best[0];
            int ii = B.bidx[0];
            for (int q = 1; q < kPopThreads / 32; q++)
                if (B.best[q] > bb || (B.best[q] == bb && B.bidx[q] < ii)) {
                    bb = B.best[q];
                    ii = B.bidx[q];
                }
            int irow = 0, icol = 0;
            if (bb > 0.0) {
                irow = ii / n;
                icol = ii - irow * n;
            }
            B.piv_row = irow;
            B.piv_col = icol;
            B.pcount[icol] += 1;
        }
        __syncthreads();
        const int irow = B.piv_row, icol = B.piv_col;
        if (irow != icol) {
            if (tid < n) {
                const S x = B.a[irow * kMaxEq + tid];
                B.a[irow * kMaxEq + tid] = B.a[icol * kMaxEq + tid];
                B.a[icol * kMaxEq + tid] = x;
            }
            if (tid == 0) {
                const S x = B.b[irow];
                B.b[irow] = B.b[icol];
                B.b[icol] = x;
            }
            __syncthreads();
        }
        const S pivot = B.a[icol * kMaxEq + icol];
        __syncthreads();
        if (tid < n) B.a[icol * kMaxEq + tid] = (tid == icol ? lift<S>(1.0) : B.a[icol * kMaxEq + tid]) / pivot;
        if (tid == kPopThreads - 1) B.b[icol] = B.b[icol] / pivot;
        __syncthreads();
        if (tid < n) B.dcol[tid] = B.a[tid * kMaxEq + icol];
        __syncthreads();
        for (int idx = tid; idx < n * n; idx += kPopThreads) {
            const int l = idx / n, c = idx - l * n;
            if (l == icol) continue;
            const S t = B.dcol[l];
            if (val(t) == 0.0) continue;
            const S cur = c == icol ? lift<S>(0.0) : B.a[l * kMaxEq + c];
            B.a[l * kMaxEq + c] = cur - B.a[icol * kMaxEq + c] * t;
        }
        if (tid < n && tid != icol) {
            const S t = B.dcol[tid];
            if (val(t) != 0.0) B.b[tid] = B.b[tid] - B.b[icol] * t;
        }
        __syncthreads();
    }
}

template <typename S>
__global__ void __launch_bounds__(kPopThreads) nmolec_block_kernel(const PopsJobT<S>* __restrict__ jobs, int n_jobs) {
    __shared__ BlockShared<S> B;
    const int job = blockIdx.x;
    if (job >= n_jobs) return;
    const int tid = threadIdx.x;
    const PopsJobT<S> J = jobs[job];
    const PopsTables& P = g_pops;
    const int ne = P.nequa, e = ne - 1, nmol = P.nmol, nloc = P.locj[P.nmol];
    const bool has_e = P.has_e != 0;
    for (int z = tid; z < kNEl; z += kPopThreads) B.xab_all[z] = abundance<S>(J, z);
    __syncthreads();
    if (tid < ne) {
        S x = lift<S>(0.0);
        if (tid >= 1 && P.idequa[tid] < 100) x = smax<S>(B.xab_all[P.idequa[tid] - 1], lift<S>(1e-20));
        B.xab[tid] = x;
    }
    S wtmole = lift<S>(0.0);
    if (tid == 0) wtmole = wtmole_dev<S>(B.xab_all);
    S xne_prev = lift<S>(0.0);
    double p_prev = 0.0;
    __syncthreads();
    for (int j = 0; j < J.n_layers; j++) {
        const LayerState s = layer_state(J.t[j], J.p[j], J.vturb[j]);
        S xne_j;
        if (j == 0) {
            const double x0 = s.xntot / 2.0;
            const double x = x0 / 10.0;
            if (tid < ne) B.xn[tid] = tid == 0 ? lift<S>(x0) : (has_e && tid == e ? lift<S>(x) : x * B.xab[tid]);
            xne_j = lift<S>(x);
        } else {
            const double ratio = s.p / p_prev;
            if (tid < ne) B.xn[tid] = B.xn[tid] * ratio;
            xne_j = xne_prev * ratio;
        }
        if (tid < ne) B.eqold[tid] = lift<S>(0.0);
        for (int m = tid; m < nmol; m += kPopThreads) B.equilj[m] = equilj_dev<S>(m, s, xne_j);
        __syncthreads();
        int it = 0;
        for (it = 1; it <= kMaxIter; it++) {
            for (int m = tid; m < nmol; m += kPopThreads) {
                S t = B.equilj[m];
                if (!(isfinite(val(t)) && val(t) > 0.0)) {
                    B.skip[m] = 1;
                    continue;
                }
                for (int lk = P.locj[m]; lk < P.locj[m + 1]; lk++) {
                    const int kr = P.kcomps[lk];
                    t = kr >= ne ? t / B.xn[e] : t * B.xn[kr];
                }
                B.term[m] = t;
                B.skip[m] = isfinite(val(t)) ? 0 : 1;
            }
            __syncthreads();
            for (int q = tid; q < nloc; q += kPopThreads) {
                const int m = P.slot_mol[q];
                if (B.skip[m]) continue;
                const S t = B.term[m];
                const int kr = P.kcomps[q];
                B.dmain[q] = kr >= ne ? -t / B.xn[e] : t / B.xn[kr];
                B.dcorr[q] = t / B.xn[comp_eq(kr, ne)];
            }
            __syncthreads();
            if (tid < ne) assemble_column_pre<S>(B, tid, s.xntot);
            __syncthreads();
            solvit_block<S>(B, ne);
            if (tid < ne) {
                S d = B.b[tid];
                const S x = B.xn[tid];
                const double dv = val(d), xv = val(x);
                const double ratio = xv == 0.0 ? (dv == 0.0 ? 0.0 : INFINITY) : fabs(dv / xv);
                B.ratio_err[tid] = ratio > 0.001;
                const double eo = val(B.eqold[tid]);
                const bool flip = (eo > 0.0 && dv < 0.0) || (eo < 0.0 && dv > 0.0);
                B.flip[tid] = flip;
                if (flip && isfinite(dv)) d = d * 0.69;
                B.b[tid] = d;
                B.xneq[tid] = (isfinite(xv) && isfinite(val(d)) && fabs(xv) > 2.2250738585072014e-308)
                                  ? x * (1.0 - d / x)
                                  : x - d;
            }
            __syncthreads();
            if (tid == 0) {
                int iferr = 0;
                double scale = 100.0;
                for (int k = 0; k < ne; k++) {
                    if (B.ratio_err[k]) iferr = 1;
                    const S x = B.xn[k];
                    if (val(B.xneq[k]) < val(x) / 100.0) {
                        B.xn[k] = x / scale;
                        if (B.flip[k]) scale = sqrt(scale);
                    } else {
                        B.xn[k] = B.xneq[k];
                    }
                    B.eqold[k] = B.b[k];
                }
                B.iferr = iferr;
            }
            __syncthreads();
            if (B.iferr == 0) break;
        }
        if (it > kMaxIter) it = kMaxIter;
        if (has_e) xne_j = B.xn[e];
        S* xnmol = J.xnmol + (size_t)j * kMaxMol;
        for (int m = tid; m < nmol; m += kPopThreads) {
            S v = B.equilj[m];
            for (int lk = P.locj[m]; lk < P.locj[m + 1]; lk++) {
                const int kr = P.kcomps[lk];
                v = kr >= ne ? v / B.xn[e] : v * B.xn[kr];
            }
            xnmol[m] = v;
        }
        __syncthreads();
        if (tid == 0) {
            J.state[j] = s;
            J.xnes[j] = xne_j;
            J.xnat[j] = B.xn[0];
            store<S>(J.xne, J.d_xne, j, xne_j);
            store<S>(J.rho, J.d_rho, j, B.xn[0] * wtmole * 1.660e-24);
            if (J.xnatom) J.xnatom[j] = val(B.xn[0]);
            if (J.hckt) J.hckt[j] = s.hckt;
            if (J.iterations) J.iterations[j] = it;
            const S h1 = smax<S>(P.row_h1 >= 0 ? xnmol[P.row_h1] : lift<S>(0.0), lift<S>(1e-40));
            store<S>(J.xnf_h, J.d_xnf_h, j, h1);
            store<S>(J.xnf_he1, J.d_xnf_he1, j,
                     smax<S>(P.row_he1 >= 0 ? xnmol[P.row_he1] : lift<S>(0.0), lift<S>(1e-40)));
            S h2 = lift<S>(0.0);
            if (!(s.t > 9000.0)) {
                const double T = s.t;
                const double eqk = exp(4.478 / s.tkev - 4.64584e1 +
                                       (1.63660e-3 +
                                        (-4.93992e-7 +
                                         (1.11822e-10 + (-1.49567e-14 + (1.06206e-18 - 3.08720e-23 * T) * T) * T) *
                                             T) *
                                            T) *
                                           T -
                                       1.5 * s.tlog);
                h2 = h1 * h1 * eqk;
            }
            store<S>(J.xnf_h2, J.d_xnf_h2, j, h2);
        }
        xne_prev = xne_j;
        p_prev = s.p;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// pops_kernel: POPS (pops_exact.py:1855-2025) and Doppler widths (:2027)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double doppler_width(double tk, double mass, double vt) {
    return sqrt(2.0 * tk / mass / 1.660e-24 + vt * vt) / kCcms;
}

template <typename S>
__global__ void __launch_bounds__(128) pops_kernel(const PopsJobT<S>* __restrict__ jobs,
                                                   const int* __restrict__ first, int n_jobs) {
    // block -> (job, layer) through the prefix of layer counts
    int lo = 0, hi = n_jobs - 1;
    const int b = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const PopsJobT<S>& J = jobs[lo];
    const int j = b - first[lo];
    if (j < 0 || j >= J.n_layers) return;
    const PopsTables& P = g_pops;
    const LayerState s = J.state[j];
    const S xne = J.xnes[j];
    const S xnat = J.xnat[j];
    const S* xnmol = J.xnmol + (size_t)j * kMaxMol;
    const size_t row0 = (size_t)j * kNIon * kNSpec;
    const int tid = threadIdx.x;
    for (int sp = tid; sp < kNSpec; sp += blockDim.x) {
        S v[kNIon];
        for (int i = 0; i < kNIon; i++) v[i] = lift<S>(0.0);
        if (sp < kNEl) {
            const int z = sp + 1;
            S F[10], PART[10];
            if (P.elem_mol_branch[sp]) {
                // number density over partition function of each ion from
                // the molecular equilibrium (XNFPMOL, pops_exact.py:130-150)
                for (int ion = 0; ion < kNIon; ion++) {
                    const int row = P.elem_mol_row[sp][ion];
                    if (row < 0) continue;
                    const int ncomp = P.locj[row + 1] - P.locj[row];
                    pfsaha_dev<S>(z, ncomp, s, xne, F, PART);
                    v[ion] = xnmol[row] / PART[ncomp - 1];
                }
            } else {
                const int nion = P.elem_nion[sp];
                const int nion2 = pfsaha_dev<S>(z, nion, s, xne, F, PART);
                const int n = nion < nion2 ? nion : nion2;
                const S ab = abundance<S>(J, sp);
                for (int i = 0; i < n && i < kNIon; i++) v[i] = F[i] / PART[i] * xnat * ab;
            }
        }
        for (int ion = 0; ion < kNIon; ion++) store<S>(J.population, J.d_population, row0 + ion * kNSpec + sp, v[ion]);
    }
    if (!J.doppler) return;
    for (int q = tid; q < kNIon * kNSpec; q += blockDim.x) {
        const int ion = q / kNSpec, sp = q - ion * kNSpec;
        double v = 0.0;
        if (sp < kNEl && P.atmass[sp] > 0.0) v = doppler_width(s.tk, P.atmass[sp], s.vturb);
        if (ion == 4) {
            // iron-group copies (pops_exact.py:2068-2079)
            for (int off = 30; off <= 60; off += 10) {
                const int z = sp - off + 1;
                if (z >= 20 && z <= 28) {
                    const double m = P.atmass[z - 1];
                    v = m > 0.0 ? doppler_width(s.tk, m, s.vturb) : 0.0;
                }
            }
        }
        if (ion == 5 && sp >= 40) {
            const double mm = P.momass[sp - 39];
            if (mm > 0.0) v = doppler_width(s.tk, mm, s.vturb);
        }
        J.doppler[row0 + q] = v;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace ks {
ks_status set_error(ks_status code, const std::string& msg);
}

namespace {

ks_status perr(ks_status code, const std::string& msg) { return ks::set_error(code, msg); }

#define KP_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return perr(KS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// READMOL (readmol_exact.py:20-251): components of each molecule as
// equation numbers; equation 0 is the total particle count, then one per
// element present (ascending Z), the electrons last.
ks_status build_molecules(PopsTables& T, const double* code, const double* equil, int nmol) {
    if (nmol <= 0 || nmol > kMaxMol) return perr(KS_ERR_INVALID, "molecule table: 1..200 entries expected");
    static const double xcode[8] = {1e14, 1e12, 1e10, 1e8, 1e6, 1e4, 1e2, 1e0};
    int ifequa[102] = {0};
    std::vector<int> comps;
    T.locj[0] = 0;
    for (int m = 0; m < nmol; m++) {
        const double c = code[m];
        int ii = -1;
        for (int i = 0; i < 8; i++)
            if (c >= xcode[i]) {
                ii = i;
                break;
            }
        if (ii < 0) return perr(KS_ERR_INVALID, "molecule table: invalid code");
        double x = c;
        for (int i = ii; i < 8; i++) {
            int id = (int)(x / xcode[i]);
            x = x - (double)id * xcode[i];
            if (id == 0) id = 100;
            if (id < 1 || id > 100) return perr(KS_ERR_INVALID, "molecule table: component out of range");
            ifequa[id] = 1;
            comps.push_back(id);
        }
        const int ion = (int)(x * 100.0 + 0.5);
        if (ion >= 1) {
            ifequa[100] = 1;
            ifequa[101] = 1;
            for (int q = 0; q < ion; q++) comps.push_back(101);
        }
        if ((int)comps.size() > kMaxLoc) return perr(KS_ERR_INVALID, "molecule table: too many components");
        T.locj[m + 1] = (int)comps.size();
        T.mol_code[m] = c;
        for (int k = 0; k < 7; k++) T.mol_equil[k * kMaxMol + m] = equil[k * nmol + m];
    }
    int iequa = 1;
    for (int i = 0; i < kMaxEq; i++) T.idequa[i] = 0;
    for (int i = 1; i <= 100; i++) {
        if (ifequa[i] != 1) continue;
        iequa += 1;
        if (iequa > kMaxEq) return perr(KS_ERR_UNSUPPORTED, "molecule table: more than 32 equations");
        ifequa[i] = iequa;
        T.idequa[iequa - 1] = i;
    }
    T.nequa = iequa;
    ifequa[101] = iequa + 1;
    for (size_t q = 0; q < comps.size(); q++) T.kcomps[q] = ifequa[comps[q]] - 1;
    T.nmol = nmol;
    T.has_e = T.idequa[T.nequa - 1] == 100;
    for (int m = 0; m < nmol; m++)
        for (int l = T.locj[m]; l < T.locj[m + 1]; l++) T.slot_mol[l] = m;
    // per equation, the molecules (more than one component) that hold it
    const int ne = T.nequa;
    int n = 0;
    for (int k = 0; k < ne; k++) {
        T.col_off[k] = n;
        for (int m = 0; m < nmol; m++) {
            if (T.locj[m + 1] - T.locj[m] <= 1) continue;
            bool has = false;
            for (int l = T.locj[m]; l < T.locj[m + 1]; l++) {
                const int kr = T.kcomps[l];
                if ((kr >= ne ? ne - 1 : kr) == k) has = true;
            }
            if (has) {
                if (n >= kMaxLoc) return perr(KS_ERR_INVALID, "molecule table: column lists too long");
                T.col_mol[n++] = m;
            }
        }
    }
    T.col_off[ne] = n;
    // the POPS molecular branch per element (pops_exact.py:1871-1900): the
    // CODE of the converter's all-ion call (convert_atm_to_npz.py:2496-2532)
    for (int z = 1; z <= kNEl; z++) {
        double cz;
        if (z == 1) cz = 1.01;
        else if (z == 2) cz = 2.02;
        else if (z <= 5) cz = (double)z + 0.03;
        else if (z <= 16) cz = (double)z + 0.05;
        else if (z <= 19) cz = (double)z + 0.04;
        else if (z <= 28) cz = (double)z + 0.09;
        else cz = (double)z + 0.02;
        const int iz = (int)cz;
        T.elem_nion[z - 1] = (int)((cz - (double)iz) * 100.0 + 1.5);
        int nn = (int)((cz - (double)(int)cz) * 100.0 + 1.5);
        if (nn < 1) nn = 1;
        bool has_int = false;
        for (int m = 0; m < nmol; m++)
            if (std::fabs(T.mol_code[m] - (double)iz) < 1e-3) has_int = true;
        for (int i = 0; i < 10; i++) T.elem_mol_row[z - 1][i] = -1;
        bool matched = false;
        double c = cz;
        for (int i = 1; i <= nn; i++) {
            const int ion = nn - i + 1;
            for (int m = 0; m < nmol; m++)
                if (std::fabs(T.mol_code[m] - c) < 0.001) {
                    if (ion <= 10) T.elem_mol_row[z - 1][ion - 1] = m;
                    matched = true;
                    break;
                }
            c -= 0.01;
        }
        T.elem_mol_branch[z - 1] = (matched || has_int) ? 1 : 0;
    }
    T.row_h1 = T.row_he1 = -1;
    for (int m = 0; m < nmol; m++) {
        if (T.row_h1 < 0 && std::fabs(T.mol_code[m] - 1.00) < 0.001) T.row_h1 = m;
        if (T.row_he1 < 0 && std::fabs(T.mol_code[m] - 2.00) < 0.001) T.row_he1 = m;
    }
    // MOMASS of the first 100 entries (convert_atm_to_npz.py:122-187)
    for (int i = 0; i < 100; i++) {
        T.momass[i] = 0.0;
        if (i >= nmol) continue;
        const double c = T.mol_code[i];
        int start = 0;
        for (int k = 0; k < 8; k++)
            if (c >= xcode[k]) {
                start = k;
                break;
            }
        double rem = c, tot = 0.0;
        for (int k = start; k < 8; k++) {
            const int el = (int)(rem / xcode[k] + 1e-9);
            rem -= el * xcode[k];
            if (el == 0) continue;
            if (el >= 1 && el <= kNEl) tot += T.atmass[el - 1];
        }
        T.momass[i] = tot;
    }
    return KS_OK;
}

ks_status device_pops() {
    int dev = 0;
    KP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) return perr(KS_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_host.ready) return perr(KS_ERR_INVALID, "population tables not initialised (ks_init_pops_tables)");
    if (!g_dev_ready[dev]) {
        KP_CUDA(cudaMemcpyToSymbol(g_pops, &g_host.t, sizeof(PopsTables)));
        g_dev_ready[dev] = true;
    }
    return KS_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    }
};

ks_status check_models(const ks_pops_model* models, int32_t n) {
    if (!models || n <= 0) return perr(KS_ERR_INVALID, "ks_populations: no models");
    for (int i = 0; i < n; i++) {
        const ks_pops_model& m = models[i];
        if (m.n_layers < 1 || m.n_layers > 4096)
            return perr(KS_ERR_INVALID, "ks_populations: n_layers must be 1..4096");
        if (!m.temperature || !m.gas_pressure || !m.vturb || !m.xabund || !m.electron_density || !m.mass_density ||
            !m.hckt || !m.xnf_h || !m.xnf_he1 || !m.xnf_h2 || !m.population || !m.doppler)
            return perr(KS_ERR_INVALID, "ks_populations: null input or output pointer");
    }
    return KS_OK;
}

template <typename S>
size_t job_ws_bytes(Carve& c, size_t L) {
    c.take(sizeof(S) * L * kMaxMol);
    c.take(sizeof(S) * L);
    c.take(sizeof(S) * L);
    c.take(sizeof(LayerState) * L);
    return c.off;
}

size_t pops_ws_bytes(const ks_pops_model* models, int32_t n) {
    Carve c;
    c.take(sizeof(PopsJob) * (size_t)n);
    c.take(sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < n; i++) job_ws_bytes<double>(c, (size_t)models[i].n_layers);
    return c.off + 256;
}

template <typename S>
void fill_job(PopsJobT<S>& J, const ks_pops_model& m, char* base, Carve& c) {
    std::memset(&J, 0, sizeof(J));
    const size_t L = (size_t)m.n_layers;
    J.n_layers = m.n_layers;
    J.dparam = -1;
    J.t = m.temperature;
    J.p = m.gas_pressure;
    J.vturb = m.vturb;
    J.xabund = m.xabund;
    J.xne = m.electron_density;
    J.rho = m.mass_density;
    J.xnatom = m.xnatom;
    J.hckt = m.hckt;
    J.xnf_h = m.xnf_h;
    J.xnf_he1 = m.xnf_he1;
    J.xnf_h2 = m.xnf_h2;
    J.population = m.population;
    J.doppler = m.doppler;
    J.iterations = m.nmolec_iterations;
    J.xnmol = (S*)(base + c.take(sizeof(S) * L * kMaxMol));
    J.xnat = (S*)(base + c.take(sizeof(S) * L));
    J.xnes = (S*)(base + c.take(sizeof(S) * L));
    J.state = (LayerState*)(base + c.take(sizeof(LayerState) * L));
}

}  // namespace

namespace ks {
ks_status pops_build_tables(const ks_pops_tables* t);
}

ks_status ks::pops_build_tables(const ks_pops_tables* t) {
    if (!t || !t->potion || !t->nnn || !t->atmass || !t->pftab || !t->pf_potlo || !t->pf_potlolog || !t->level_e ||
        !t->level_g || !t->level_n || !t->pfg_first || !t->pfg_second || !t->pfg_label || !t->pfg_g0 || !t->pfg_off ||
        !t->pfg_g || !t->pfg_e || !t->mol_code || !t->mol_equil)
        return perr(KS_ERR_INVALID, "ks_init_pops_tables: null table pointer");
    if (t->n_pfg_first > 114 || t->n_pfg_second > 168 || t->n_pfg_label > kPfgRows || t->n_pfg_label < 1)
        return perr(KS_ERR_INVALID, "ks_init_pops_tables: PFGROUND table sizes out of range");
    PopsTables* T = new PopsTables();
    std::memset(T, 0, sizeof(PopsTables));
    std::memcpy(T->potion, t->potion, sizeof(T->potion));
    std::memcpy(T->nnn, t->nnn, sizeof(T->nnn));
    std::memcpy(T->atmass, t->atmass, sizeof(T->atmass));
    std::memcpy(T->pftab, t->pftab, sizeof(T->pftab));
    std::memcpy(T->pf_potlo, t->pf_potlo, sizeof(T->pf_potlo));
    std::memcpy(T->pf_potlolog, t->pf_potlolog, sizeof(T->pf_potlolog));
    int off = 0;
    for (int i = 0; i < kNLevTab; i++) {
        T->lev_off[i] = off;
        if (t->level_n[i] < 1 || off + t->level_n[i] > kLevCap) {
            delete T;
            return perr(KS_ERR_INVALID, "ks_init_pops_tables: level tables out of range");
        }
        off += t->level_n[i];
    }
    T->lev_off[kNLevTab] = off;
    std::memcpy(T->lev_e, t->level_e, sizeof(double) * off);
    std::memcpy(T->lev_g, t->level_g, sizeof(double) * off);
    T->n_first = t->n_pfg_first;
    T->n_second = t->n_pfg_second;
    std::memcpy(T->pfg_first, t->pfg_first, sizeof(int) * t->n_pfg_first);
    std::memcpy(T->pfg_second, t->pfg_second, sizeof(int) * t->n_pfg_second);
    for (int i = 0; i < kPfgLabels; i++) T->pfg_row[i] = -1;
    const int nt = t->pfg_off[t->n_pfg_label];
    if (nt < 0 || nt > kPfgTerms) {
        delete T;
        return perr(KS_ERR_INVALID, "ks_init_pops_tables: too many PFGROUND terms");
    }
    for (int r = 0; r < t->n_pfg_label; r++) {
        const int lab = t->pfg_label[r];
        if (lab < 0 || lab >= kPfgLabels) {
            delete T;
            return perr(KS_ERR_INVALID, "ks_init_pops_tables: PFGROUND label out of range");
        }
        T->pfg_row[lab] = r;
        T->pfg_g0[r] = t->pfg_g0[r];
        T->pfg_off[r] = t->pfg_off[r];
    }
    T->pfg_off[t->n_pfg_label] = nt;
    std::memcpy(T->pfg_g, t->pfg_g, sizeof(double) * nt);
    std::memcpy(T->pfg_e, t->pfg_e, sizeof(double) * nt);
    ks_status st = build_molecules(*T, t->mol_code, t->mol_equil, t->n_mol);
    if (st != KS_OK) {
        delete T;
        return st;
    }
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_host.t = *T;
        g_host.ready = true;
        for (int d = 0; d < kMaxDev; d++) g_dev_ready[d] = false;
    }
    delete T;
    return KS_OK;
}

extern "C" ks_status ks_init_pops_tables(const ks_pops_tables* tables) { return ks::pops_build_tables(tables); }

extern "C" ks_status ks_pops_system(int32_t* n_molecules, int32_t* n_equations, int32_t* equation_element,
                                    int32_t* element_molecular) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_host.ready) return perr(KS_ERR_INVALID, "population tables not initialised (ks_init_pops_tables)");
    const PopsTables& T = g_host.t;
    if (n_molecules) *n_molecules = T.nmol;
    if (n_equations) *n_equations = T.nequa;
    if (equation_element)
        for (int k = 0; k < T.nequa; k++) equation_element[k] = T.idequa[k];
    if (element_molecular)
        for (int z = 0; z < kNEl; z++) element_molecular[z] = T.elem_mol_branch[z];
    return KS_OK;
}

extern "C" ks_status ks_populations_workspace_size(const ks_pops_model* models, int32_t n_models, size_t* bytes) {
    ks_status st = check_models(models, n_models);
    if (st != KS_OK) return st;
    if (!bytes) return perr(KS_ERR_INVALID, "ks_populations_workspace_size: null output");
    *bytes = pops_ws_bytes(models, n_models);
    return KS_OK;
}

extern "C" ks_status ks_populations(const ks_pops_model* models, int32_t n_models, void* workspace,
                                    size_t workspace_bytes, void* stream) {
    ks_status st = check_models(models, n_models);
    if (st != KS_OK) return st;
    if (!workspace) return perr(KS_ERR_INVALID, "ks_populations: null workspace");
    if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
        return perr(KS_ERR_INVALID, "ks_populations: workspace must be 256-byte aligned");
    if (workspace_bytes < pops_ws_bytes(models, n_models))
        return perr(KS_ERR_NOMEM, "ks_populations: workspace smaller than ks_populations_workspace_size");
    st = device_pops();
    if (st != KS_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    char* base = (char*)workspace;
    Carve c;
    const size_t o_jobs = c.take(sizeof(PopsJob) * (size_t)n_models);
    const size_t o_first = c.take(sizeof(int) * ((size_t)n_models + 1));
    std::vector<PopsJob> jobs(n_models);
    std::vector<int> first(n_models + 1);
    int total = 0;
    for (int i = 0; i < n_models; i++) {
        fill_job<double>(jobs[i], models[i], base, c);
        first[i] = total;
        total += models[i].n_layers;
    }
    first[n_models] = total;
    KP_CUDA(cudaMemcpyAsync(base + o_jobs, jobs.data(), sizeof(PopsJob) * n_models, cudaMemcpyHostToDevice, s));
    KP_CUDA(cudaMemcpyAsync(base + o_first, first.data(), sizeof(int) * (n_models + 1), cudaMemcpyHostToDevice, s));
    const PopsJob* dj = (const PopsJob*)(base + o_jobs);
    nmolec_block_kernel<double><<<n_models, kPopThreads, 0, s>>>(dj, n_models);
    KP_CUDA(cudaGetLastError());
    pops_kernel<double><<<total, 128, 0, s>>>(dj, (const int*)(base + o_first), n_models);
    KP_CUDA(cudaGetLastError());
    // the host copies of the job records must outlive the copies: wait for them
    KP_CUDA(cudaStreamSynchronize(s));
    return KS_OK;
}

// ---------------------------------------------------------------------------
// forward-mode derivatives w.r.t. the log10 abundance of one element
// ---------------------------------------------------------------------------

namespace {

ks_status check_tangents(const ks_pops_tangent* t, int32_t n) {
    if (!t || n <= 0) return perr(KS_ERR_INVALID, "ks_populations_tangent: no models");
    for (int i = 0; i < n; i++) {
        const ks_pops_model& m = t[i].model;
        if (m.n_layers < 1 || m.n_layers > 4096)
            return perr(KS_ERR_INVALID, "ks_populations_tangent: n_layers must be 1..4096");
        if (!m.temperature || !m.gas_pressure || !m.vturb || !m.xabund)
            return perr(KS_ERR_INVALID, "ks_populations_tangent: null input pointer");
        if (t[i].element < 0 || t[i].element >= kNEl)
            return perr(KS_ERR_INVALID, "ks_populations_tangent: element must be 0..98 (Z-1)");
        if (!t[i].d_electron_density || !t[i].d_mass_density || !t[i].d_xnf_h || !t[i].d_xnf_he1 ||
            !t[i].d_xnf_h2 || !t[i].d_population)
            return perr(KS_ERR_INVALID, "ks_populations_tangent: null derivative output");
    }
    return KS_OK;
}

size_t tangent_ws_bytes(const ks_pops_tangent* t, int32_t n) {
    Carve c;
    c.take(sizeof(PopsJobT<D1>) * (size_t)n);
    c.take(sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < n; i++) job_ws_bytes<D1>(c, (size_t)t[i].model.n_layers);
    return c.off + 256;
}

}  // namespace

extern "C" ks_status ks_populations_tangent_workspace_size(const ks_pops_tangent* tangents, int32_t n,
                                                           size_t* bytes) {
    ks_status st = check_tangents(tangents, n);
    if (st != KS_OK) return st;
    if (!bytes) return perr(KS_ERR_INVALID, "ks_populations_tangent_workspace_size: null output");
    *bytes = tangent_ws_bytes(tangents, n);
    return KS_OK;
}

extern "C" ks_status ks_populations_tangent(const ks_pops_tangent* tangents, int32_t n, void* workspace,
                                            size_t workspace_bytes, void* stream) {
    ks_status st = check_tangents(tangents, n);
    if (st != KS_OK) return st;
    if (!workspace || (reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
        return perr(KS_ERR_INVALID, "ks_populations_tangent: workspace must be non-null and 256-byte aligned");
    if (workspace_bytes < tangent_ws_bytes(tangents, n))
        return perr(KS_ERR_NOMEM, "ks_populations_tangent: workspace smaller than its workspace size");
    st = device_pops();
    if (st != KS_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    char* base = (char*)workspace;
    Carve c;
    const size_t o_jobs = c.take(sizeof(PopsJobT<D1>) * (size_t)n);
    const size_t o_first = c.take(sizeof(int) * ((size_t)n + 1));
    std::vector<PopsJobT<D1>> jobs(n);
    std::vector<int> first(n + 1);
    int total = 0;
    for (int i = 0; i < n; i++) {
        const ks_pops_tangent& t = tangents[i];
        fill_job<D1>(jobs[i], t.model, base, c);
        PopsJobT<D1>& J = jobs[i];
        J.dparam = t.element;
        J.d_xne = t.d_electron_density;
        J.d_rho = t.d_mass_density;
        J.d_xnf_h = t.d_xnf_h;
        J.d_xnf_he1 = t.d_xnf_he1;
        J.d_xnf_h2 = t.d_xnf_h2;
        J.d_population = t.d_population;
        J.doppler = nullptr;  // the Doppler widths do not depend on the abundances
        first[i] = total;
        total += t.model.n_layers;
    }
    first[n] = total;
    KP_CUDA(cudaMemcpyAsync(base + o_jobs, jobs.data(), sizeof(PopsJobT<D1>) * n, cudaMemcpyHostToDevice, s));
    KP_CUDA(cudaMemcpyAsync(base + o_first, first.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    const PopsJobT<D1>* dj = (const PopsJobT<D1>*)(base + o_jobs);
    nmolec_block_kernel<D1><<<n, kPopThreads, 0, s>>>(dj, n);
    KP_CUDA(cudaGetLastError());
    pops_kernel<D1><<<total, 128, 0, s>>>(dj, (const int*)(base + o_first), n);
    KP_CUDA(cudaGetLastError());
    KP_CUDA(cudaStreamSynchronize(s));
    return KS_OK;
}
