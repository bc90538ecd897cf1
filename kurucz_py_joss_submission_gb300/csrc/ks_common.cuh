// ks_common.cuh -- constants, the Voigt function and small helpers shared by
// the GB300 kernels.  Physics constants are the reference's own
// (synthe_py/physics/line_opacity.py:39-49, engine/radiative.py:14-17).
#pragma once

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace ks {

// Index of a block as its kernel body sees it: the hardware block of a
// single-synthesis launch, or one job's block of a batched launch (the
// batched kernels walk a job table and hand each job's blocks to the same
// bodies).
struct VB {
    int x, y, gx, gy;
};

constexpr double C_LIGHT_NM = 2.99792458e17;
constexpr double C_LIGHT_CM = 2.99792458e10;
constexpr double C_LIGHT_KM = 299792.458;
constexpr double H_PLANCK = 6.62607015e-27;
constexpr double K_BOLTZ = 1.380649e-16;
constexpr int MAX_PROFILE_STEPS = 1000000;  // synthe.for MAXPROF
constexpr int VOIGT_N = 2001;               // H0/H1/H2TAB length, step 1/200
constexpr int EXP_N = 1001;                 // EXTAB/EXTABF length
constexpr int NXTAU = 51;                   // JOSH optical-depth grid
constexpr int MAX_LAYERS = 128;             // per-wavelength column bound
constexpr int MAX_EDGES = 1024;             // continuum edges (the reference's tables have 341)
constexpr int N_REACH_CLASSES = 22;         // reach classes 0..21 (2^20 > MAXPROF)
constexpr int LONG_CLASS = 8;               // default: classes 8+ (reach > 128 bins) in batches of 8 pairs
constexpr int SHORT_CLASS = 7;              // default: classes 0-6 (reach <= 64 bins) one lane per pair
constexpr double EPS38 = 1.0e-38;
constexpr double MAX_OPACITY_REAL4 = 3.4e38;

// Device flags (bit mask written to the stats word on internal limits).
constexpr int FLAG_N10DOP_RANGE = 1;   // n10dop larger than the packed field
constexpr int FLAG_LAYERS = 2;         // more layers than MAX_LAYERS
constexpr int FLAG_MAXJ_NONCONV = 4;   // informational
constexpr int FLAG_HYDROGEN_LINE = 16; // a hydrogen line's row or levels outside the tables
constexpr int FLAG_HELIUM_LINE = 32;   // a helium line's row outside the catalog
constexpr int FLAG_F19_LINE = 64;      // a fort.19 line's row or ion outside the tables

// Kurucz VOIGT H(a, v) approximation (synthe_py/physics/voigt_jit.py:17-69).
// Tables are passed as one pointer to interleaved (h0, h1) pairs plus h2.
template <typename R>
__device__ __forceinline__ R voigt_hv(R v, R a, const R* __restrict__ h0,
                                      const R* __restrict__ h1,
                                      const R* __restrict__ h2) {
    R av = v < R(0) ? -v : v;
    int iv = (int)(av * R(200) + R(0.5));
    iv = iv < 0 ? 0 : (iv > VOIGT_N - 1 ? VOIGT_N - 1 : iv);
    if (a < R(0.2)) {
        if (av > R(10)) return R(0.5642) * a / (v * v);
        return (h2[iv] * a + h1[iv]) * a + h0[iv];
    } else if (a > R(1.4) || (a + av) > R(3.2)) {
        R aa = a * a;
        R vv = v * v;
        R u = (aa + vv) * R(1.4142);
        R val = a * R(0.79788) / u;
        if (a <= R(100)) {
            R aau = aa / u;
            R vvu = vv / u;
            R uu = u * u;
            val = ((((aau - R(10) * vvu) * aau * R(3) + R(15) * vvu * vvu) + R(3) * vv - aa) / uu +
                   R(1)) * val;
        }
        return val;
    } else {
        R vv = v * v;
        R hh0 = h0[iv];
        R hh1 = h1[iv] + hh0 * R(1.12838);
        R hh2 = h2[iv] + hh1 * R(1.12838) - hh0;
        R hh3 = (R(1) - h2[iv]) * R(0.37613) - hh1 * R(0.66667) * vv + hh2 * R(1.12838);
        R hh4 = (R(3) * hh3 - hh1) * R(0.37613) + hh0 * R(0.66667) * vv * vv;
        R pa = (((hh4 * a + hh3) * a + hh2) * a + hh1) * a + hh0;
        R pb = ((R(-0.122727278) * a + R(0.532770573)) * a - R(0.96284325)) * a + R(0.979895032);
        return pa * pb;
    }
}

// Kahan-compensated accumulation of v into (sum, comp).
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
    float y = v - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ int reach_class(int reach) {
    // class 0: reach 0..1; class k: 2^(k-1) < reach <= 2^k
    if (reach <= 1) return 0;
    return 32 - __clz(reach - 1);
}

__host__ __device__ __forceinline__ int64_t class_halo(int k) {
    return (int64_t)1 << k;  // maximum reach of class k
}

}  // namespace ks
