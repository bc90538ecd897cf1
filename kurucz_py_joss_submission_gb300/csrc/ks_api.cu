// ks_api.cu -- the C ABI (include/kurucz_gb300.h): constant tables, workspace
// layout, the precision-independent kernels (grid scalars, line bins, reach-
// class partition) and the pipeline drivers.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kurucz_gb300.h"
#include "ks_common.cuh"
#include "ks_internal.h"
#include "ks_launch.h"

using namespace ks;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string g_last_error;

static ks_status fail(ks_status code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

static ks_status cuda_fail(cudaError_t e, const char* where) {
    return fail(KS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define KS_CUDA(call)                                  \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

extern "C" const char* ks_last_error(void) { return g_last_error.c_str(); }

// Error setter for the other translation units of the library.
ks_status ks::set_error(ks_status code, const std::string& msg) { return fail(code, msg); }

extern "C" ks_status ks_version(int32_t* major, int32_t* minor) {
    if (major) *major = 1;
    if (minor) *minor = 6;
    return KS_OK;
}

// ---------------------------------------------------------------------------
// constant tables
// ---------------------------------------------------------------------------

// Device copies of the constant tables (Voigt H0/H1/H2, FASTEX EXTAB/EXTABF,
// JOSH XTAU/CH).  They are built on the host by ks_init_tables and copied to
// every device on its first use.
__device__ double g_h0d[VOIGT_N], g_h1d[VOIGT_N], g_h2d[VOIGT_N];
__device__ float g_h0f[VOIGT_N], g_h1f[VOIGT_N], g_h2f[VOIGT_N];
__device__ double g_extab[EXP_N], g_extabf[EXP_N];
__device__ float g_extab_f[EXP_N], g_extabf_f[EXP_N];
__device__ double g_xtau[NXTAU], g_ch[NXTAU];
__device__ float g_coefj32[NXTAU * NXTAU];
__device__ double g_coefj64[NXTAU * NXTAU];

struct HostTables {
    bool ready = false;
    std::vector<double> h0, h1, h2, extab, extabf, xtau, ch, coefj;
    CoefJ32 cj;
};
static HostTables g_tables;
static std::mutex g_tables_mu;

struct DevTables {
    const double *h0d, *h1d, *h2d, *extab, *extabf, *xtau, *ch;
    const float *h0f, *h1f, *h2f, *extab_f, *extabf_f, *coefj32;
    const double *coefj64;
};
static const int kMaxDevices = 64;
static bool g_dev_ready[kMaxDevices];
static DevTables g_dev[kMaxDevices];

// MAP1 as used to build the 2001-point H1 table from the 81-point one
// (synthe_py/physics/tables.py:275-391).
static void map1_tables(const double* xold, const double* fold, int nold, const double* xnew,
                        double* fnew, int nnew) {
    std::vector<double> x1(nold + 2), f1(nold + 2);
    for (int i = 0; i < nold; i++) {
        x1[i + 1] = xold[i];
        f1[i + 1] = fold[i];
    }
    int l = 2, ll = 0;
    double a = 0, b = 0, c = 0, abac = 0, bbac = 0, cbac = 0, afor = 0, bfor = 0, cfor = 0;
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
        } else if (l == ll) {
        } else if (l == 2) {
            c = 0.0;
            b = (f1[l] - f1[l - 1]) / (x1[l] - x1[l - 1]);
            a = f1[l] - x1[l] * b;
            ll = l;
        } else {
            int l1 = l - 1;
            bool done = false;
            if (l > ll + 1 || l == 3) {
                int l2 = l - 2;
                double d = (f1[l1] - f1[l2]) / (x1[l1] - x1[l2]);
                cbac = f1[l] / ((x1[l] - x1[l1]) * (x1[l] - x1[l2])) +
                       (f1[l2] / (x1[l] - x1[l2]) - f1[l1] / (x1[l] - x1[l1])) / (x1[l1] - x1[l2]);
                bbac = d - (x1[l1] + x1[l2]) * cbac;
                abac = f1[l2] - x1[l2] * d + x1[l1] * x1[l2] * cbac;
                if (l == nold) {
                    c = cbac; b = bbac; a = abac; ll = l;
                    done = true;
                }
            } else {
                cbac = cfor; bbac = bfor; abac = afor;
                if (l == nold) {
                    c = cbac; b = bbac; a = abac; ll = l;
                    done = true;
                }
            }
            if (!done) {
                double d = (f1[l] - f1[l1]) / (x1[l] - x1[l1]);
                cfor = f1[l + 1] / ((x1[l + 1] - x1[l]) * (x1[l + 1] - x1[l1])) +
                       (f1[l1] / (x1[l + 1] - x1[l1]) - f1[l] / (x1[l + 1] - x1[l])) / (x1[l] - x1[l1]);
                bfor = d - (x1[l] + x1[l1]) * cfor;
                afor = f1[l1] - x1[l1] * d + x1[l] * x1[l1] * cfor;
                double wt = 0.0;
                if (std::fabs(cfor) != 0.0) wt = std::fabs(cfor) / (std::fabs(cfor) + std::fabs(cbac));
                a = afor + wt * (abac - afor);
                b = bfor + wt * (bbac - bfor);
                c = cfor + wt * (cbac - cfor);
                ll = l;
            }
        }
        fnew[k - 1] = a + (b + c * x) * x;
    }
}

// Builds every derived table from the SYNTHE source tables: the Voigt
// tables (tables.py:224-241), FASTEX tables (tables.py:21-27) and the
// single-precision JOSH operator.  Host function; call once per process.
extern "C" ks_status ks_init_tables(const double* tabvi, const double* tabh1, int32_t n_tab,
                                    const double* xtau, const double* ch, const double* coefj) {
    if (!tabvi || !tabh1 || n_tab < 3 || n_tab > 1000 || !xtau || !ch || !coefj)
        return fail(KS_ERR_INVALID, "ks_init_tables: null or invalid table");
    std::lock_guard<std::mutex> lk(g_tables_mu);
    HostTables t;
    t.h0.resize(VOIGT_N);
    t.h1.resize(VOIGT_N);
    t.h2.resize(VOIGT_N);
    std::vector<double> grid(VOIGT_N);
    for (int i = 0; i < VOIGT_N; i++) grid[i] = (double)i / 200.0;
    map1_tables(tabvi, tabh1, n_tab, grid.data(), t.h1.data(), VOIGT_N);
    for (int i = 0; i < VOIGT_N; i++) {
        double v = (double)i / 200.0;
        double vv = v * v;
        t.h0[i] = std::exp(-vv);
        t.h2[i] = t.h0[i] - (vv + vv) * t.h0[i];
    }
    t.extab.resize(EXP_N);
    t.extabf.resize(EXP_N);
    for (int i = 0; i < EXP_N; i++) {
        t.extab[i] = std::exp(-((double)i));
        t.extabf[i] = std::exp(-((double)i) * 0.001);
    }
    t.xtau.assign(xtau, xtau + NXTAU);
    t.ch.assign(ch, ch + NXTAU);
    t.coefj.assign(coefj, coefj + NXTAU * NXTAU);
    for (int i = 0; i < NXTAU * NXTAU; i++) t.cj.c[i] = (float)coefj[i];
    for (int i = 0; i < NXTAU; i++) {
        t.cj.ch[i] = (float)ch[i];
        t.cj.xtau[i] = (float)xtau[i];
    }
    t.ready = true;
    g_tables = std::move(t);
    for (int i = 0; i < kMaxDevices; i++) g_dev_ready[i] = false;
    return KS_OK;
}

// Copies of the host-built tables, for tests.
extern "C" ks_status ks_get_tables(double* h0, double* h1, double* h2, double* extab, double* extabf) {
    std::lock_guard<std::mutex> lk(g_tables_mu);
    if (!g_tables.ready) return fail(KS_ERR_INVALID, "tables not initialised (ks_init_tables)");
    if (h0) std::memcpy(h0, g_tables.h0.data(), sizeof(double) * VOIGT_N);
    if (h1) std::memcpy(h1, g_tables.h1.data(), sizeof(double) * VOIGT_N);
    if (h2) std::memcpy(h2, g_tables.h2.data(), sizeof(double) * VOIGT_N);
    if (extab) std::memcpy(extab, g_tables.extab.data(), sizeof(double) * EXP_N);
    if (extabf) std::memcpy(extabf, g_tables.extabf.data(), sizeof(double) * EXP_N);
    return KS_OK;
}

template <typename T>
static cudaError_t sym_addr(const T& sym, const void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, sym);
    *out = p;
    return e;
}

// Ensures the current device holds the tables; the first call on a device
// uploads them (synchronously), so it must come before any stream capture.
static ks_status device_tables(DevTables* out) {
    int dev = 0;
    KS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KS_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_tables_mu);
    if (!g_tables.ready) return fail(KS_ERR_INVALID, "tables not initialised (ks_init_tables)");
    if (!g_dev_ready[dev]) {
        const HostTables& t = g_tables;
        std::vector<float> f0(VOIGT_N), f1(VOIGT_N), f2(VOIGT_N), ef(EXP_N), eff(EXP_N);
        for (int i = 0; i < VOIGT_N; i++) {
            f0[i] = (float)t.h0[i];
            f1[i] = (float)t.h1[i];
            f2[i] = (float)t.h2[i];
        }
        for (int i = 0; i < EXP_N; i++) {
            ef[i] = (float)t.extab[i];
            eff[i] = (float)t.extabf[i];
        }
        KS_CUDA(cudaMemcpyToSymbol(g_h0d, t.h0.data(), sizeof(double) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_h1d, t.h1.data(), sizeof(double) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_h2d, t.h2.data(), sizeof(double) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_h0f, f0.data(), sizeof(float) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_h1f, f1.data(), sizeof(float) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_h2f, f2.data(), sizeof(float) * VOIGT_N));
        KS_CUDA(cudaMemcpyToSymbol(g_extab, t.extab.data(), sizeof(double) * EXP_N));
        KS_CUDA(cudaMemcpyToSymbol(g_extabf, t.extabf.data(), sizeof(double) * EXP_N));
        KS_CUDA(cudaMemcpyToSymbol(g_extab_f, ef.data(), sizeof(float) * EXP_N));
        KS_CUDA(cudaMemcpyToSymbol(g_extabf_f, eff.data(), sizeof(float) * EXP_N));
        KS_CUDA(cudaMemcpyToSymbol(g_xtau, t.xtau.data(), sizeof(double) * NXTAU));
        KS_CUDA(cudaMemcpyToSymbol(g_ch, t.ch.data(), sizeof(double) * NXTAU));
        KS_CUDA(cudaMemcpyToSymbol(g_coefj32, t.cj.c, sizeof(float) * NXTAU * NXTAU));
        KS_CUDA(cudaMemcpyToSymbol(g_coefj64, t.coefj.data(), sizeof(double) * NXTAU * NXTAU));
        DevTables d;
        const void* p;
        KS_CUDA(sym_addr(g_h0d, &p)); d.h0d = (const double*)p;
        KS_CUDA(sym_addr(g_h1d, &p)); d.h1d = (const double*)p;
        KS_CUDA(sym_addr(g_h2d, &p)); d.h2d = (const double*)p;
        KS_CUDA(sym_addr(g_h0f, &p)); d.h0f = (const float*)p;
        KS_CUDA(sym_addr(g_h1f, &p)); d.h1f = (const float*)p;
        KS_CUDA(sym_addr(g_h2f, &p)); d.h2f = (const float*)p;
        KS_CUDA(sym_addr(g_extab, &p)); d.extab = (const double*)p;
        KS_CUDA(sym_addr(g_extabf, &p)); d.extabf = (const double*)p;
        KS_CUDA(sym_addr(g_extab_f, &p)); d.extab_f = (const float*)p;
        KS_CUDA(sym_addr(g_extabf_f, &p)); d.extabf_f = (const float*)p;
        KS_CUDA(sym_addr(g_xtau, &p)); d.xtau = (const double*)p;
        KS_CUDA(sym_addr(g_ch, &p)); d.ch = (const double*)p;
        KS_CUDA(sym_addr(g_coefj32, &p)); d.coefj32 = (const float*)p;
        KS_CUDA(sym_addr(g_coefj64, &p)); d.coefj64 = (const double*)p;
        g_dev[dev] = d;
        g_dev_ready[dev] = true;
    }
    *out = g_dev[dev];
    return KS_OK;
}

// ---------------------------------------------------------------------------
// host grid
// ---------------------------------------------------------------------------

extern "C" int64_t ks_wavelength_grid(double start, double end, double resolution, double* out,
                                      int64_t cap) {
    if (!(resolution > 0.0) || !(start > 0.0)) {
        g_last_error = "ks_wavelength_grid: resolution and start must be positive";
        return -1;
    }
    double ratio = 1.0 + 1.0 / resolution;
    double rlog = std::log(ratio);
    double ix_floor = std::floor(std::log(start) / rlog);
    if (std::exp(ix_floor * rlog) < start) ix_floor += 1.0;
    double wl = std::exp(ix_floor * rlog);
    int64_t n = 0;
    const double stop = end * (1.0 + 1e-9);
    while (wl <= stop) {
        if (out && n < cap) out[n] = wl;
        n++;
        wl *= ratio;
    }
    return n;
}

// ---------------------------------------------------------------------------
// precision-independent kernels
// ---------------------------------------------------------------------------

// Internal-limit flags raised on this device since the last ks_check_flags.
// Every entry point ends by OR-ing its call's flag word into it on the call's
// stream (flag_sink_kernel), so an overflow in a call that reads no counters
// is kept until the caller asks; ks_check_flags takes and clears it.
static __device__ int g_sticky_flags;
static __device__ int g_taken_flags;

__global__ void flag_sink_kernel(const int* __restrict__ flags) {
    const int f = *flags;
    if (f) atomicOr(&g_sticky_flags, f);
}

__global__ void flag_take_kernel() { g_taken_flags = atomicExch(&g_sticky_flags, 0); }

static ks_status sink_flags(const int* flags, cudaStream_t s) {
    flag_sink_kernel<<<1, 1, 0, s>>>(flags);
    KS_CUDA(cudaGetLastError());
    return KS_OK;
}

static ks_status flags_status(int flags) {
    if (flags & 8) return fail(KS_ERR_DEVICE, "wing bins are not monotone in the line order");
    if (flags & FLAG_HELIUM_LINE) return fail(KS_ERR_DEVICE, "a helium line's row lies outside the catalog");
    if (flags & FLAG_F19_LINE)
        return fail(KS_ERR_DEVICE, "a fort.19 line's row, element or ion lies outside the tables");
    if (flags & FLAG_HYDROGEN_LINE)
        return fail(KS_ERR_DEVICE, "a hydrogen line's row lies outside the catalog or its upper level above 94");
    if (flags & FLAG_N10DOP_RANGE)
        return fail(KS_ERR_DEVICE, "a pair exceeded a packed descriptor field (N10DOP or centre offset)");
    if (flags) return fail(KS_ERR_DEVICE, "a kernel raised device flag " + std::to_string(flags));
    return KS_OK;
}

extern "C" ks_status ks_check_flags(void* stream, int32_t* flags_out) {
    cudaStream_t s = (cudaStream_t)stream;
    int f = 0;
    flag_take_kernel<<<1, 1, 0, s>>>();
    KS_CUDA(cudaGetLastError());
    KS_CUDA(cudaMemcpyFromSymbolAsync(&f, g_taken_flags, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    KS_CUDA(cudaStreamSynchronize(s));
    if (flags_out) *flags_out = f;
    return flags_status(f);
}

// Grid scalars (opacity.py:570-574; line_opacity.py:235-239 RESOLU and
// :1035-1058 WBEGIN / grid offset of the wing bins).
__device__ __forceinline__ void grid_params_kernel_body(VB vb, const double* g, int64_t n, double grid_origin, GridPar* gp) {
    GridPar p;
    p.resolu = 300000.0;
    p.ratiolg = 0.0;
    p.ix_start = 0;
    p.wbegin = 1.0;
    p.grid_offset = 0;
    p.first = n > 0 ? g[0] : 0.0;
    p.last = n > 0 ? g[n - 1] : 0.0;
    if (n > 1) {
        double ratio = g[1] / g[0];
        if (ratio > 1.0) p.resolu = 1.0 / (ratio - 1.0);
        p.ratiolg = log(ratio);
        p.ix_start = (int64_t)(log(g[0]) / p.ratiolg + 0.5);
        double ix_floor = floor(log(grid_origin) / p.ratiolg);
        double wb = exp(ix_floor * p.ratiolg);
        if (wb < grid_origin) {
            ix_floor += 1.0;
            wb = exp(ix_floor * p.ratiolg);
        }
        p.wbegin = wb;
        p.grid_offset = (int64_t)rint(log(g[0] / wb) / p.ratiolg);
    }
    *gp = p;
}
__global__ void grid_params_kernel(const double* g, int64_t n, double grid_origin, GridPar* gp) {
    grid_params_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, g, n, grid_origin, gp);
}


// Centre bins (opacity.py:550-592) and wing bins (line_opacity.py:1030-1059)
// per line, plus the single-precision line copies of the mixed path.  Flags
// non-monotone wing bins (the accumulation searches them); the previous
// line's wing bin comes from the neighbouring lane (lane 0 computes it).
__device__ __forceinline__ int64_t wing_bin(double w, const GridPar& gp) {
    return (int64_t)rint(log(w / gp.wbegin) / gp.ratiolg) - gp.grid_offset;
}

__device__ __forceinline__ void line_bins_kernel_body(VB vb, int64_t n_lines, int64_t n_wl, const double* __restrict__ wl,
                                 const GridPar* __restrict__ gpp, int32_t* center_out,
                                 int32_t* wing_out, const double* cgf, const double* elo,
                                 const double* gr, const double* gs, const double* gw,
                                 const double* gf, LineF* linef, int* flags) {
    const int64_t i = (int64_t)vb.x * blockDim.x + threadIdx.x;
    const bool act = i < n_lines;
    const GridPar gp = *gpp;
    const double w = act ? wl[i] : (n_lines > 0 ? wl[n_lines - 1] : 1.0);
    int64_t c = 0, wb = 0;
    if (n_wl >= 2) {  // uniform across the grid
        c = (int64_t)(log(w) / gp.ratiolg + 0.5) - gp.ix_start;
        if (w < gp.first) c = -1;
        if (w > gp.last) c = n_wl;
        wb = wing_bin(w, gp);
        int64_t wbp = __shfl_up_sync(0xffffffffu, wb, 1);
        const int lane = threadIdx.x & 31;
        if (lane == 0 && act && i > 0) wbp = wing_bin(wl[i - 1], gp);
        if (act && i > 0 && wbp > wb) atomicOr(flags, 8);
    }
    if (!act) return;
    if (center_out) center_out[i] = (int32_t)c;
    if (wing_out) wing_out[i] = (int32_t)wb;
    if (linef) {
        LineF f;
        f.cgf = (float)cgf[i];
        f.elo_hi = (float)elo[i];
        f.elo_lo = (float)(elo[i] - (double)f.elo_hi);
        f.gr = (float)gr[i];
        f.gs = (float)gs[i];
        f.gw = (float)gw[i];
        f.gf = (float)gf[i];
        f.wl = (float)w;
        linef[i] = f;
    }
}
__global__ void line_bins_kernel(int64_t n_lines, int64_t n_wl, const double* __restrict__ wl,
                                 const GridPar* __restrict__ gpp, int32_t* center_out,
                                 int32_t* wing_out, const double* cgf, const double* elo,
                                 const double* gr, const double* gs, const double* gw,
                                 const double* gf, LineF* linef, int* flags) {
    line_bins_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, n_lines, n_wl, wl, gpp, center_out, wing_out, cgf, elo, gr, gs, gw, gf, linef, flags);
}


// ---- deterministic stable partition of the pairs by reach class ----
// Each depth's lines are cut into chunks of kChunk; counts per (depth,
// chunk, class), an exclusive scan per (depth, class) over chunks, then a
// scatter that keeps line order inside every class (warp ballots give each
// lane its rank among equal classes).
static const int kChunk = 4096;
static const int kDefaultTile = 1024;  // accumulation tile (bins) unless ks_options.tile_bins says otherwise
static const int kPartThreads = 256;

__device__ __forceinline__ void class_count_kernel_body(VB vb, const uint8_t* __restrict__ cls, int64_t stride, int nchunks,
                                   int32_t* __restrict__ counts) {
    __shared__ int c[N_REACH_CLASSES];
    int d = vb.y, ch = vb.x;
    if (threadIdx.x < N_REACH_CLASSES) c[threadIdx.x] = 0;
    __syncthreads();
    const uint8_t* base = cls + (int64_t)d * stride + (int64_t)ch * kChunk;
    for (int i = threadIdx.x; i < kChunk; i += blockDim.x) {
        uint8_t k = base[i];
        if (k < N_REACH_CLASSES) atomicAdd(&c[k], 1);
    }
    __syncthreads();
    if (threadIdx.x < N_REACH_CLASSES)
        counts[((int64_t)d * nchunks + ch) * N_REACH_CLASSES + threadIdx.x] = c[threadIdx.x];
}
__global__ void class_count_kernel(const uint8_t* __restrict__ cls, int64_t stride, int nchunks,
                                   int32_t* __restrict__ counts) {
    class_count_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, cls, stride, nchunks, counts);
}


// One block per depth.  chunk_base[d][ch][k] = absolute start of chunk ch's
// class-k lines; class_off[d][k] = absolute start of class k.
__device__ __forceinline__ void class_scan_kernel_body(VB vb, const int32_t* __restrict__ counts, int nchunks, int64_t stride,
                                  int64_t* __restrict__ chunk_base, int64_t* __restrict__ class_off,
                                  unsigned long long* valid_pairs) {
    __shared__ int64_t tot[N_REACH_CLASSES];
    __shared__ int64_t off[N_REACH_CLASSES + 1];
    int d = vb.x;
    int k = threadIdx.x;
    const int32_t* cd = counts + (int64_t)d * nchunks * N_REACH_CLASSES;
    if (k < N_REACH_CLASSES) {
        int64_t s = 0;
        for (int ch = 0; ch < nchunks; ch++) s += cd[(int64_t)ch * N_REACH_CLASSES + k];
        tot[k] = s;
    }
    __syncthreads();
    if (k == 0) {
        int64_t b = (int64_t)d * stride;
        for (int q = 0; q < N_REACH_CLASSES; q++) {
            off[q] = b;
            b += tot[q];
        }
        off[N_REACH_CLASSES] = b;
        for (int q = 0; q <= N_REACH_CLASSES; q++)
            class_off[(int64_t)d * (N_REACH_CLASSES + 1) + q] = off[q];
        if (valid_pairs) atomicAdd(valid_pairs, (unsigned long long)(b - (int64_t)d * stride));
    }
    __syncthreads();
    if (k < N_REACH_CLASSES) {
        int64_t run = off[k];
        int64_t* cb = chunk_base + (int64_t)d * nchunks * N_REACH_CLASSES;
        for (int ch = 0; ch < nchunks; ch++) {
            cb[(int64_t)ch * N_REACH_CLASSES + k] = run;
            run += cd[(int64_t)ch * N_REACH_CLASSES + k];
        }
    }
}
__global__ void class_scan_kernel(const int32_t* __restrict__ counts, int nchunks, int64_t stride,
                                  int64_t* __restrict__ chunk_base, int64_t* __restrict__ class_off,
                                  unsigned long long* valid_pairs) {
    class_scan_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, counts, nchunks, stride, chunk_base, class_off, valid_pairs);
}


__device__ __forceinline__ void class_scatter_kernel_body(VB vb, 
    const uint8_t* __restrict__ cls, int64_t stride, int nchunks,
    const int64_t* __restrict__ chunk_base, int32_t* __restrict__ class_pos) {
    constexpr int NW = kPartThreads / 32;
    constexpr int PER_WARP = kChunk / NW;
    __shared__ int wcount[NW][N_REACH_CLASSES];
    __shared__ int64_t wbase[NW][N_REACH_CLASSES];
    int d = vb.y, ch = vb.x;
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint8_t* base = cls + (int64_t)d * stride + (int64_t)ch * kChunk + warp * PER_WARP;
    if (lane < N_REACH_CLASSES) wcount[warp][lane] = 0;
    __syncwarp();
    for (int r = 0; r < PER_WARP; r += 32) {
        uint8_t k = base[r + lane];
        unsigned peers = __match_any_sync(0xffffffffu, (int)k);
        if (k < N_REACH_CLASSES && (peers & ((1u << lane) - 1)) == 0)
            wcount[warp][k] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x < N_REACH_CLASSES) {
        int k = threadIdx.x;
        int64_t run = chunk_base[((int64_t)d * nchunks + ch) * N_REACH_CLASSES + k];
        for (int w = 0; w < NW; w++) {
            wbase[w][k] = run;
            run += wcount[w][k];
        }
    }
    __syncthreads();
    int64_t line0 = (int64_t)ch * kChunk + warp * PER_WARP;
    for (int r = 0; r < PER_WARP; r += 32) {
        uint8_t k = base[r + lane];
        unsigned peers = __match_any_sync(0xffffffffu, (int)k);
        int rank = __popc(peers & ((1u << lane) - 1));
        if (k < N_REACH_CLASSES) class_pos[wbase[warp][k] + rank] = (int32_t)(line0 + r + lane);
        __syncwarp();
        if (k < N_REACH_CLASSES && rank == 0) wbase[warp][k] += __popc(peers);
        __syncwarp();
    }
}
__global__ void __launch_bounds__(kPartThreads) class_scatter_kernel(
    const uint8_t* __restrict__ cls, int64_t stride, int nchunks,
    const int64_t* __restrict__ chunk_base, int32_t* __restrict__ class_pos) {
    class_scatter_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, cls, stride, nchunks, chunk_base, class_pos);
}


// For every (depth, tile, class): the range of the class's centre-sorted
// list whose wing centres lie within the class's maximum reach (+1 bin) of
// the tile, as offsets from the class start.  One thread per (tile, class),
// two binary searches over wing bins.
__device__ __forceinline__ int64_t lower_bound_wing(const int32_t* __restrict__ pos, int64_t lo, int64_t hi,
                                                    const int32_t* __restrict__ wing, int64_t key) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)wing[pos[mid]] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void tile_ranges_kernel_body(VB vb, const int64_t* __restrict__ class_off, const int32_t* __restrict__ class_pos,
                                   const int32_t* __restrict__ wing, int64_t n_wl, int tile_bins, int ntiles,
                                   int2* __restrict__ rng) {
    const int d = vb.y;
    const int64_t idx = (int64_t)vb.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)ntiles * N_REACH_CLASSES) return;
    const int t = (int)(idx / N_REACH_CLASSES), k = (int)(idx % N_REACH_CLASSES);
    const int64_t* off = class_off + (int64_t)d * (N_REACH_CLASSES + 1);
    const int64_t lo = off[k], hi = off[k + 1];
    const int64_t T0 = (int64_t)t * tile_bins;
    const int64_t T1 = min(T0 + tile_bins, n_wl);
    const int64_t h = class_halo(k) + 1;
    const int64_t s0 = lower_bound_wing(class_pos, lo, hi, wing, T0 - h);
    const int64_t s1 = lower_bound_wing(class_pos, s0, hi, wing, T1 + h);
    rng[((int64_t)d * ntiles + t) * N_REACH_CLASSES + k] = make_int2((int)(s0 - lo), (int)(s1 - lo));
}
__global__ void tile_ranges_kernel(const int64_t* __restrict__ class_off, const int32_t* __restrict__ class_pos,
                                   const int32_t* __restrict__ wing, int64_t n_wl, int tile_bins, int ntiles,
                                   int2* __restrict__ rng) {
    tile_ranges_kernel_body(VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y}, class_off, class_pos, wing, n_wl, tile_bins, ntiles, rng);
}


// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------

struct Carve {
    char* base;
    size_t cap, used;
    bool dry;
    template <typename T>
    T* take(size_t count) {
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        T* p = dry ? nullptr : reinterpret_cast<T*>(base + used);
        used += bytes;
        return p;
    }
};

struct Workspace {
    GridPar* gp;
    DepthPar* depth;
    IonPar* ion;
    LineF* linef;
    int32_t *center, *wing;
    void *cont_abs, *cont_scat, *asynth, *desc;
    uint8_t* cls;
    int32_t* counts;
    int64_t *chunk_base, *class_off;
    int32_t* class_pos;
    unsigned long long* counters;  // [0] valid pairs, [1] evaluations
    int32_t* iters;
    int32_t* tlist;  // wavelengths left to the general transfer kernel
    int2* tile_rng;  // per (depth, tile, class) contributing range
    int ntiles;
    float* coef_f;   // continuum coefficient tables in FP32: absorption, then scattering
    float* freq_f;   // c / lambda per grid point in FP32
    int* flags;
    HydPar* hyd_par;  // hydrogen lines: per (line, depth) state and walk limits
    int2* hyd_walk;
    int hyd_cap;
    HePar* he_par;    // helium lines: per (line, depth) wing parameters and walk limits
    int2* he_walk;
    F19Par* f19_par;  // fort.19 lines: per (line, depth) gates and wing
    int2* f19_walk;
    int64_t stride;
    int nchunks;
};

// Special lines (hydrogen, helium, fort.19) whose per-(line, depth) scratch
// every workspace holds; a synthesis with more allocates the rest on its
// stream (stream-ordered, freed after use); the no-allocation entry point
// takes at most this many of each.
static const int kMaxHydrogenLines = 256;
// Upper bound of special lines of one class in a synthesis.
static const int kMaxSpecialLines = 1 << 16;

static void layout(Carve& c, Workspace& w, int64_t n_lines, int L, int64_t n_wl, int n_ion,
                   int n_elem, bool fp64, bool need_cont, bool need_asynth, int tile_bins = 0) {
    size_t rs = fp64 ? 8 : 4;
    w.stride = ((n_lines + kChunk - 1) / kChunk) * kChunk;
    if (w.stride == 0) w.stride = kChunk;
    w.nchunks = (int)(w.stride / kChunk);
    w.gp = c.take<GridPar>(1);
    w.depth = c.take<DepthPar>(L);
    w.ion = c.take<IonPar>((size_t)L * n_ion * n_elem);
    w.linef = c.take<LineF>(n_lines > 0 ? n_lines : 1);
    w.center = c.take<int32_t>(n_lines > 0 ? n_lines : 1);
    w.wing = c.take<int32_t>(n_lines > 0 ? n_lines : 1);
    w.cont_abs = need_cont ? (void*)c.take<char>(rs * L * n_wl) : nullptr;
    w.cont_scat = need_cont ? (void*)c.take<char>(rs * L * n_wl) : nullptr;
    w.asynth = need_asynth ? (void*)c.take<char>(rs * L * n_wl) : nullptr;
    w.desc = (void*)c.take<char>((fp64 ? sizeof(PairDesc<double>) : sizeof(PairDesc<float>)) *
                                 (size_t)L * w.stride);
    w.cls = c.take<uint8_t>((size_t)L * w.stride);
    w.counts = c.take<int32_t>((size_t)L * w.nchunks * N_REACH_CLASSES);
    w.chunk_base = c.take<int64_t>((size_t)L * w.nchunks * N_REACH_CLASSES);
    w.class_off = c.take<int64_t>((size_t)L * (N_REACH_CLASSES + 1));
    w.class_pos = c.take<int32_t>((size_t)L * w.stride);
    w.counters = c.take<unsigned long long>(4);
    w.iters = c.take<int32_t>(2 * (size_t)(n_wl > 0 ? n_wl : 1));
    w.tlist = c.take<int32_t>(n_wl > 0 ? n_wl : 1);
    w.ntiles = tile_bins > 0 ? (int)((n_wl + tile_bins - 1) / tile_bins) : 0;
    w.tile_rng = c.take<int2>((size_t)L * (w.ntiles > 0 ? w.ntiles : 1) * N_REACH_CLASSES);
    w.coef_f = c.take<float>(2 * (size_t)L * (MAX_EDGES - 1) * 3);
    w.freq_f = c.take<float>(n_wl > 0 ? n_wl : 1);
    w.flags = c.take<int>(1);
    w.hyd_cap = (int)std::max<int64_t>(1, std::min<int64_t>(n_lines, kMaxHydrogenLines));
    w.hyd_par = c.take<HydPar>((size_t)w.hyd_cap * L);
    w.hyd_walk = c.take<int2>((size_t)w.hyd_cap * L * 2);
    w.he_par = c.take<HePar>((size_t)w.hyd_cap * L);
    w.he_walk = c.take<int2>((size_t)w.hyd_cap * L * 2);
    w.f19_par = c.take<F19Par>((size_t)w.hyd_cap * L);
    w.f19_walk = c.take<int2>((size_t)w.hyd_cap * L * 2);
}

extern "C" ks_status ks_workspace_size(int64_t n_lines, int32_t n_layers, int64_t n_wavelengths,
                                       const ks_options* opt, size_t* bytes) {
    if (!bytes || n_lines < 0 || n_layers <= 0 || n_wavelengths < 0)
        return fail(KS_ERR_INVALID, "ks_workspace_size: invalid sizes");
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    Carve c{nullptr, 0, 0, true};
    Workspace w;
    layout(c, w, n_lines, n_layers, n_wavelengths, 6, 139, fp64, true, true,
           opt && opt->tile_bins > 0 ? opt->tile_bins : kDefaultTile);
    *bytes = c.used + 256;
    return KS_OK;
}

// ---------------------------------------------------------------------------
// argument checks
// ---------------------------------------------------------------------------

static ks_status check_atmos(const ks_atmos* a) {
    if (!a) return fail(KS_ERR_INVALID, "atmosphere is NULL");
    if (a->n_layers <= 0) return fail(KS_ERR_INVALID, "atmosphere has no layers");
    if (a->n_layers > MAX_LAYERS)
        return fail(KS_ERR_UNSUPPORTED, "atmosphere has more than 128 layers");
    if (!a->rhox || !a->temperature || !a->electron_density || !a->mass_density || !a->hckt ||
        !a->population || !a->doppler)
        return fail(KS_ERR_INVALID, "atmosphere: required depth array is NULL");
    if (a->n_ion <= 0 || a->n_elem <= 0) return fail(KS_ERR_INVALID, "atmosphere: bad population shape");
    return KS_OK;
}

static ks_status check_cont(const ks_atmos* a) {
    if (!a->wledge || !a->cont_abs_coeff || !a->cont_scat_coeff || a->n_edge < 2)
        return fail(KS_ERR_INVALID,
                    "continuum coefficients are missing (wledge, cont_abs_coeff, cont_scat_coeff)");
    if (a->n_edge > MAX_EDGES) return fail(KS_ERR_UNSUPPORTED, "more than 1024 continuum edges");
    return KS_OK;
}

static ks_status check_grid(const ks_grid* g) {
    if (!g || !g->wavelength) return fail(KS_ERR_INVALID, "grid is NULL");
    if (g->n < 1) return fail(KS_ERR_INVALID, "grid is empty");
    if (g->n > 0x7fffffffLL) return fail(KS_ERR_UNSUPPORTED, "grid larger than 2^31 points");
    return KS_OK;
}

static ks_status check_lines(const ks_lines* l) {
    if (!l) return fail(KS_ERR_INVALID, "lines is NULL");
    if (l->n_lines < 0) return fail(KS_ERR_INVALID, "negative line count");
    if (l->n_lines == 0) return KS_OK;
    if (!l->wavelength || !l->gf || !l->cgf || !l->gamma_rad || !l->gamma_stark || !l->gamma_vdw ||
        !l->elo_cm || !l->element_idx || !l->ion_stage || !l->line_type || !l->process_mask ||
        !l->asynth_mask)
        return fail(KS_ERR_INVALID, "lines: a required column is NULL");
    if (!l->sorted_by_wavelength)
        return fail(KS_ERR_INVALID, "lines must be sorted by wavelength (sorted_by_wavelength = 1)");
    if (l->n_lines > 0x7fffffffLL) return fail(KS_ERR_UNSUPPORTED, "more than 2^31 lines");
    if (l->n_hydrogen < 0 || l->n_hydrogen > l->n_lines)
        return fail(KS_ERR_INVALID, "n_hydrogen must lie in [0, n_lines]");
    if (l->n_hydrogen > kMaxSpecialLines) return fail(KS_ERR_UNSUPPORTED, "more than 65536 hydrogen lines");
    if (l->n_hydrogen > 0 && (!l->hydrogen_rows || !l->hydrogen_n_lower || !l->hydrogen_n_upper))
        return fail(KS_ERR_INVALID, "lines: a hydrogen column is NULL");
    if (l->n_helium < 0 || l->n_helium > l->n_lines)
        return fail(KS_ERR_INVALID, "n_helium must lie in [0, n_lines]");
    if (l->n_helium > kMaxSpecialLines) return fail(KS_ERR_UNSUPPORTED, "more than 65536 helium lines");
    if (l->n_helium > 0 && (!l->helium_rows || !l->helium_ncon || !l->helium_nelionx))
        return fail(KS_ERR_INVALID, "lines: a helium column is NULL");
    if (l->n_f19 < 0 || l->n_f19 > l->n_lines) return fail(KS_ERR_INVALID, "n_f19 must lie in [0, n_lines]");
    if (l->n_f19 > kMaxSpecialLines) return fail(KS_ERR_UNSUPPORTED, "more than 65536 fort.19 lines");
    if (l->n_f19 > 0 && (!l->f19_rows || !l->f19_cgf || !l->f19_gamma_rad || !l->f19_gamma_stark ||
                         !l->f19_gamma_vdw || !l->f19_kind || !l->f19_nlast || !l->f19_nelion ||
                         !l->f19_ncon || !l->f19_nelionx))
        return fail(KS_ERR_INVALID, "lines: a fort.19 column is NULL");
    return KS_OK;
}

// ---------------------------------------------------------------------------
// pipeline pieces
// ---------------------------------------------------------------------------

static PrepArgs prep_args(const ks_atmos* atm, const ks_options* opt, const Workspace& w) {
    PrepArgs p;
    p.n_layers = atm->n_layers;
    p.n_ion = atm->n_ion;
    p.n_elem = atm->n_elem;
    p.rhox = atm->rhox;
    p.temperature = atm->temperature;
    p.electron_density = atm->electron_density;
    p.mass_density = atm->mass_density;
    p.hckt = atm->hckt;
    p.xnf_h = atm->xnf_h;
    p.xnf_he1 = atm->xnf_he1;
    p.xnf_h2 = atm->xnf_h2;
    p.population = atm->population;
    p.doppler = atm->doppler;
    p.microturb_kms = opt ? opt->microturb_kms : 0.0;
    p.rhoxj = opt ? opt->rhoxj : 0.0;
    p.gp = w.gp;
    p.depth = w.depth;
    p.ion = w.ion;
    p.n_coeff = 0;
    p.abs_coeff = p.scat_coeff = nullptr;
    p.abs_coeff_f = p.scat_coeff_f = nullptr;
    return p;
}

static ContArgs cont_args(const ks_atmos* atm, const ks_grid* g) {
    ContArgs c;
    c.n_layers = atm->n_layers;
    c.n_edge = atm->n_edge;
    c.coeff_log10 = atm->coeff_log10;
    c.n = g->n;
    c.grid = g->wavelength;
    c.wledge = atm->wledge;
    c.half_edge = atm->half_edge;
    c.delta_edge = atm->delta_edge;
    c.abs_coeff = atm->cont_abs_coeff;
    c.scat_coeff = atm->cont_scat_coeff;
    c.abs_coeff_f = c.scat_coeff_f = nullptr;
    c.freq_f = nullptr;
    return c;
}

static PairArgs pair_args(const ks_lines* l, const ks_atmos* atm, const ks_grid* g,
                          const ks_options* opt, const Workspace& w, const DevTables& t) {
    PairArgs p;
    std::memset(&p, 0, sizeof(p));
    p.n_lines = l->n_lines;
    p.n_wl = g->n;
    p.stride = w.stride;
    p.n_layers = atm->n_layers;
    p.n_ion = atm->n_ion;
    p.n_elem = atm->n_elem;
    p.cutoff = opt ? opt->cutoff : 1e-3;
    p.cutoff_f = (float)p.cutoff;
    p.gp = w.gp;
    p.wavelength = l->wavelength;
    p.gf = l->gf;
    p.cgf = l->cgf;
    p.gamma_rad = l->gamma_rad;
    p.gamma_stark = l->gamma_stark;
    p.gamma_vdw = l->gamma_vdw;
    p.elo_cm = l->elo_cm;
    p.element_idx = l->element_idx;
    p.ion_stage = l->ion_stage;
    p.line_type = l->line_type;
    p.process_mask = l->process_mask;
    p.asynth_mask = l->asynth_mask;
    p.center_idx = w.center;
    p.wing_idx = w.wing;
    p.linef = w.linef;
    p.depth = w.depth;
    p.ion = w.ion;
    p.extab = t.extab;
    p.extabf = t.extabf;
    p.extab_f = t.extab_f;
    p.extabf_f = t.extabf_f;
    p.h0d = t.h0d;
    p.h1d = t.h1d;
    p.h2d = t.h2d;
    p.h0f = t.h0f;
    p.h1f = t.h1f;
    p.h2f = t.h2f;
    p.flags = w.flags;
    return p;
}

static ks_status run_bins(const ks_lines* l, const ks_grid* g, const Workspace& w, bool mixed,
                          cudaStream_t s) {
    grid_params_kernel<<<1, 1, 0, s>>>(g->wavelength, g->n, g->grid_origin, w.gp);
    KS_CUDA(cudaGetLastError());
    if (l && l->n_lines > 0) {
        line_bins_kernel<<<(unsigned)((l->n_lines + 255) / 256), 256, 0, s>>>(
            l->n_lines, g->n, l->wavelength, w.gp, w.center, w.wing, l->cgf, l->elo_cm,
            l->gamma_rad, l->gamma_stark, l->gamma_vdw, l->gf, mixed ? w.linef : nullptr, w.flags);
        KS_CUDA(cudaGetLastError());
    }
    return KS_OK;
}

static ks_status run_partition(const Workspace& w, int L, int64_t n_wl, int tile_bins, cudaStream_t s) {
    dim3 grid(w.nchunks, L);
    class_count_kernel<<<grid, kPartThreads, 0, s>>>(w.cls, w.stride, w.nchunks, w.counts);
    KS_CUDA(cudaGetLastError());
    class_scan_kernel<<<L, 32, 0, s>>>(w.counts, w.nchunks, w.stride, w.chunk_base, w.class_off,
                                       w.counters);
    KS_CUDA(cudaGetLastError());
    class_scatter_kernel<<<grid, kPartThreads, 0, s>>>(w.cls, w.stride, w.nchunks, w.chunk_base,
                                                       w.class_pos);
    KS_CUDA(cudaGetLastError());
    if (w.ntiles > 0) {
        const int64_t work = (int64_t)w.ntiles * N_REACH_CLASSES;
        dim3 rg((unsigned)((work + 255) / 256), (unsigned)L);
        tile_ranges_kernel<<<rg, 256, 0, s>>>(w.class_off, w.class_pos, w.wing, n_wl, tile_bins, w.ntiles,
                                              w.tile_rng);
        KS_CUDA(cudaGetLastError());
    }
    return KS_OK;
}

// The accumulation tile: a multiple of 32 bins, at most 8192, with 1-16
// warps, whose per-warp copies must fit the 227 KB of shared memory.
static ks_status check_tiling(const ks_options* opt) {
    int t = opt && opt->tile_bins > 0 ? opt->tile_bins : kDefaultTile;
    int w = opt && opt->warps_per_tile > 0 ? opt->warps_per_tile : 8;
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    if ((opt && (opt->tile_bins < 0 || opt->warps_per_tile < 0)) || w > 16 || t % 32 != 0 || t > 8192)
        return fail(KS_ERR_INVALID,
                    "tile_bins must be a multiple of 32 up to 8192 and warps_per_tile 1..16 (0 = defaults 1024, 8)");
    size_t smem = fp64 ? accumulate_smem_bytes_f64(t, w) : accumulate_smem_bytes_f32(t, w);
    if (smem > 227 * 1024)
        return fail(KS_ERR_INVALID, "tile_bins x warps_per_tile needs more than 227 KB of shared memory");
    return KS_OK;
}

static int default_tile(const ks_options* opt, bool fp64) {
    int t = opt && opt->tile_bins > 0 ? opt->tile_bins : kDefaultTile;
    return t;
}
static int default_warps(const ks_options* opt) {
    return opt && opt->warps_per_tile > 0 ? opt->warps_per_tile : 8;
}

static AccArgs acc_args(const ks_lines* l, const ks_atmos* atm, const ks_grid* g,
                        const ks_options* opt, const Workspace& w, const DevTables& t, bool fp64) {
    AccArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n_lines = l->n_lines;
    a.n_wl = g->n;
    a.stride = w.stride;
    a.n_layers = atm->n_layers;
    a.tile_bins = default_tile(opt, fp64);
    a.short_class = !opt || opt->short_class == 0 ? SHORT_CLASS
                    : opt->short_class < 0 ? 0 : min(opt->short_class, N_REACH_CLASSES);
    a.long_class = !opt || opt->long_class <= 0 ? LONG_CLASS : min(opt->long_class, N_REACH_CLASSES);
    a.grid = g->wavelength;
    a.wing_idx = w.wing;
    a.class_pos = w.class_pos;
    a.class_off = w.class_off;
    a.tile_rng = w.tile_rng;
    a.freq_f = w.freq_f;
    a.depth = w.depth;
    a.h0d = t.h0d;
    a.h1d = t.h1d;
    a.h2d = t.h2d;
    a.h0f = t.h0f;
    a.h1f = t.h1f;
    a.h2f = t.h2f;
    a.evals = w.counters + 1;
    return a;
}

static TransferArgs transfer_args(const ks_atmos* atm, const ks_grid* g, const Workspace& w,
                                  const DevTables& t, double* ft, double* fc, bool asynth_mode,
                                  bool fp64) {
    TransferArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->n;
    a.n_layers = atm->n_layers;
    a.asynth_mode = asynth_mode ? 1 : 0;
    a.slinec_mode = fp64 ? 1 : 0;
    a.line_scat = 0;
    a.grid = g->wavelength;
    a.depth = w.depth;
    a.xtau = t.xtau;
    a.ch = t.ch;
    a.coefj32 = t.coefj32;
    a.coefj64 = nullptr;
    a.flux_total = ft;
    a.flux_cont = fc;
    a.iters = w.iters;
    return a;
}

static ks_status collect_stats(const Workspace& w, int64_t n_wl, ks_stats* stats, cudaStream_t s,
                               bool with_iters = true) {
    unsigned long long ctr[2];
    int flags = 0;
    KS_CUDA(cudaMemcpyAsync(ctr, w.counters, sizeof(ctr), cudaMemcpyDeviceToHost, s));
    KS_CUDA(cudaMemcpyAsync(&flags, w.flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (!with_iters) n_wl = 0;
    std::vector<int32_t> it(2 * (size_t)n_wl);
    if (n_wl > 0)
        KS_CUDA(cudaMemcpyAsync(it.data(), w.iters, sizeof(int32_t) * 2 * n_wl,
                                cudaMemcpyDeviceToHost, s));
    KS_CUDA(cudaStreamSynchronize(s));
    if (stats) {
        stats->valid_pairs = (int64_t)ctr[0];
        stats->evaluations = (int64_t)ctr[1];
        int64_t maxj = 0, iters = 0;
        for (int64_t j = 0; j < n_wl; j++) {
            int32_t v = it[2 * j + 1];
            if (v < 0) maxj++;
            iters += (v < 0 ? -v : v) + (it[2 * j] < 0 ? -it[2 * j] : it[2 * j]);
        }
        stats->maxj_wavelengths = maxj;
        stats->iterations = iters;
        stats->device_flags = flags;
    }
    return flags_status(flags);
}

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------

extern "C" ks_status ks_line_bins(const ks_grid* grid, const double* wavelength, int64_t n_lines,
                                  int32_t* center_out, int32_t* wing_out, void* stream) {
    ks_status st = check_grid(grid);
    if (st) return st;
    if (n_lines < 0 || (n_lines > 0 && !wavelength)) return fail(KS_ERR_INVALID, "ks_line_bins: bad lines");
    cudaStream_t s = (cudaStream_t)stream;
    GridPar* gp = nullptr;
    int* flags = nullptr;
    KS_CUDA(cudaMallocAsync((void**)&gp, sizeof(GridPar) + 256, s));
    flags = reinterpret_cast<int*>(reinterpret_cast<char*>(gp) + sizeof(GridPar) + 64);
    KS_CUDA(cudaMemsetAsync(flags, 0, sizeof(int), s));
    grid_params_kernel<<<1, 1, 0, s>>>(grid->wavelength, grid->n, grid->grid_origin, gp);
    KS_CUDA(cudaGetLastError());
    if (n_lines > 0) {
        line_bins_kernel<<<(unsigned)((n_lines + 255) / 256), 256, 0, s>>>(
            n_lines, grid->n, wavelength, gp, center_out, wing_out, nullptr, nullptr, nullptr,
            nullptr, nullptr, nullptr, nullptr, flags);
        KS_CUDA(cudaGetLastError());
    }
    ks_status fs = sink_flags(flags, s);
    KS_CUDA(cudaFreeAsync(gp, s));
    return fs;
}

extern "C" ks_status ks_continuum(const ks_atmos* atm, const ks_grid* grid, int32_t precision,
                                  void* cont_abs, void* cont_scat, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_cont(atm);
    if (st) return st;
    if (!cont_abs || !cont_scat) return fail(KS_ERR_INVALID, "ks_continuum: NULL output");
    cudaStream_t s = (cudaStream_t)stream;
    ContArgs c = cont_args(atm, grid);
    if (precision == KS_PREC_FP64) KS_CUDA(launch_continuum_f64(c, (double*)cont_abs, (double*)cont_scat, s));
    else KS_CUDA(launch_continuum_f32(c, (float*)cont_abs, (float*)cont_scat, s));
    return KS_OK;
}

extern "C" ks_status ks_transp(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                               const ks_options* opt, const double* cont_kapmin, double* transp_out,
                               uint8_t* valid_out, int32_t* center_out, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (st) return st;
    if (!cont_kapmin || (lines->n_lines > 0 && (!transp_out || !valid_out)))
        return fail(KS_ERR_INVALID, "ks_transp: NULL input/output");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, true, false, false);
    char* buf = nullptr;
    KS_CUDA(cudaMallocAsync((void**)&buf, dry.used + 256, s));
    Carve c{buf, dry.used + 256, 0, false};
    layout(c, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, true, false, false);
    KS_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int), s));
    PrepArgs pa = prep_args(atm, opt, w);
    if ((st = run_bins(lines, grid, w, false, s))) return st;
    KS_CUDA(launch_prep_f64(pa, s));
    PairArgs p = pair_args(lines, atm, grid, opt, w, t);
    p.transp_out = transp_out;
    p.valid_out = valid_out;
    KS_CUDA(launch_pair_setup_f64(p, true, cont_kapmin, nullptr, (PairDesc<double>*)w.desc, w.cls, s));
    if (center_out && lines->n_lines > 0)
        KS_CUDA(cudaMemcpyAsync(center_out, w.center, sizeof(int32_t) * lines->n_lines,
                                cudaMemcpyDeviceToDevice, s));
    if ((st = sink_flags(w.flags, s))) return st;
    KS_CUDA(cudaFreeAsync(buf, s));
    return KS_OK;
}

extern "C" ks_status ks_asynth(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                               const ks_options* opt, const double* transp, const uint8_t* valid,
                               const double* cont_kapmin, void* workspace, size_t workspace_bytes,
                               double* asynth_out, ks_stats* stats, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (st) return st;
    if (!cont_kapmin || !asynth_out || (lines->n_lines > 0 && (!transp || !valid)))
        return fail(KS_ERR_INVALID, "ks_asynth: NULL input/output");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, true, false, false,
           default_tile(opt, true));
    if (!workspace || workspace_bytes < dry.used)
        return fail(KS_ERR_NOMEM, "ks_asynth: workspace too small (see ks_workspace_size)");
    Carve c{(char*)workspace, workspace_bytes, 0, false};
    layout(c, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, true, false, false,
           default_tile(opt, true));
    KS_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int), s));
    KS_CUDA(cudaMemsetAsync(w.counters, 0, 4 * sizeof(unsigned long long), s));
    KS_CUDA(cudaMemsetAsync(w.cls, 0xff, (size_t)atm->n_layers * w.stride, s));
    if ((st = run_bins(lines, grid, w, false, s))) return st;
    KS_CUDA(launch_prep_f64(prep_args(atm, opt, w), s));
    PairArgs p = pair_args(lines, atm, grid, opt, w, t);
    p.transp_in = transp;
    p.valid_in = valid;
    KS_CUDA(launch_pair_setup_f64(p, false, cont_kapmin, nullptr, (PairDesc<double>*)w.desc, w.cls, s));
    if ((st = run_partition(w, atm->n_layers, grid->n, default_tile(opt, true), s))) return st;
    AccArgs a = acc_args(lines, atm, grid, opt, w, t, true);
    KS_CUDA(launch_accumulate_f64(a, default_warps(opt), (const PairDesc<double>*)w.desc, asynth_out, s));
    if ((st = sink_flags(w.flags, s))) return st;
    if (stats) return collect_stats(w, 0, stats, s);
    return KS_OK;
}

extern "C" ks_status ks_formal_solution(const ks_atmos* atm, const ks_grid* grid, int32_t precision,
                                        const void* cont_abs, const void* cont_scat,
                                        const void* line_opacity, const void* line_scattering,
                                        const void* line_source, double* flux_total,
                                        double* flux_cont, ks_stats* stats, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (st) return st;
    if (!cont_abs || !cont_scat || !line_opacity || !flux_total || !flux_cont)
        return fail(KS_ERR_INVALID, "ks_formal_solution: NULL input/output");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    bool fp64 = precision == KS_PREC_FP64;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, 0, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false);
    char* buf = nullptr;
    KS_CUDA(cudaMallocAsync((void**)&buf, dry.used + 256, s));
    Carve c{buf, dry.used + 256, 0, false};
    layout(c, w, 0, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false);
    KS_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int), s));
    KS_CUDA(cudaMemsetAsync(w.counters, 0, 4 * sizeof(unsigned long long), s));
    if ((st = run_bins(nullptr, grid, w, false, s))) return st;
    KS_CUDA(fp64 ? launch_prep_f64(prep_args(atm, nullptr, w), s) : launch_prep_f32(prep_args(atm, nullptr, w), s));
    TransferArgs ta = transfer_args(atm, grid, w, t, flux_total, flux_cont, false, fp64);
    ta.slinec_mode = 0;
    if (fp64)
        KS_CUDA(launch_transfer_f64(ta, &g_tables.cj, (const double*)cont_abs, (const double*)cont_scat,
                                    (const double*)line_opacity, (const double*)line_scattering,
                                    (const double*)line_source, s));
    else
        KS_CUDA(launch_transfer_f32(ta, &g_tables.cj, (const float*)cont_abs, (const float*)cont_scat,
                                    (const float*)line_opacity, (const float*)line_scattering,
                                    (const float*)line_source, s));
    if ((st = sink_flags(w.flags, s))) return st;
    if (stats) {
        st = collect_stats(w, grid->n, stats, s);
        cudaFreeAsync(buf, s);
        return st;
    }
    KS_CUDA(cudaFreeAsync(buf, s));
    return KS_OK;
}

// Optional per-stage CUDA events of one synthesis (ks_options.profile).
struct StageTimer {
    bool on = false;
    cudaEvent_t ev[8];
    cudaEvent_t ev_special;  // end of the special-line kernels (after the accumulation mark)
    bool special = false;
    int n = 0;
    cudaStream_t s = nullptr;
    void start(cudaStream_t st, bool enable) {
        on = enable;
        s = st;
        special = false;
        if (!on) return;
        for (int i = 0; i < 8; i++) cudaEventCreate(&ev[i]);
        cudaEventCreate(&ev_special);
        cudaEventRecord(ev[0], s);
        n = 1;
    }
    void mark() {
        if (on && n < 8) cudaEventRecord(ev[n++], s);
    }
    // the hydrogen/helium/fort.19 kernels, queued right after the accumulation mark
    void mark_special() {
        if (on && n == 6) {
            cudaEventRecord(ev_special, s);
            special = true;
        }
    }
    void finish(ks_stats* stats) {
        if (!on) return;
        cudaEventSynchronize(ev[n - 1]);
        if (stats) {
            for (int i = 0; i < 8; i++) stats->stage_ms[i] = 0.f;
            for (int i = 1; i < n && i <= 6; i++) cudaEventElapsedTime(&stats->stage_ms[i - 1], ev[i - 1], ev[i]);
            if (special) {
                // stage 6: special lines; the transfer counts from their end
                cudaEventElapsedTime(&stats->stage_ms[6], ev[5], ev_special);
                if (n > 6) cudaEventElapsedTime(&stats->stage_ms[5], ev_special, ev[6]);
            }
            cudaEventElapsedTime(&stats->stage_ms[7], ev[0], ev[n - 1]);
        }
        for (int i = 0; i < 8; i++) cudaEventDestroy(ev[i]);
        cudaEventDestroy(ev_special);
        on = false;
    }
};

// The JOSH stage of the fused path (radiative.py:282-494 over ASYNTH split
// by FSCAT, opacity.py:2408-2420): FP64 per-column kernel, or the FP32
// streaming pass (per-column kernel on request).
template <typename R>
static ks_status run_transfer(const ks_atmos* atm, const ks_grid* grid, const ks_options* opt,
                              const Workspace& w, const DevTables& t, const R* cabs, const R* cscat,
                              const R* asynth, double* flux_total, double* flux_cont, cudaStream_t s) {
    constexpr bool fp64 = sizeof(R) == 8;
    TransferArgs ta = transfer_args(atm, grid, w, t, flux_total, flux_cont, true, fp64);
    ta.line_scat = (opt && opt->rhoxj > 0.0) ? 1 : 0;
    if (fp64 && opt && opt->exact_sweeps) ta.coefj64 = t.coefj64;
    if constexpr (fp64)
        KS_CUDA(launch_transfer_f64(ta, &g_tables.cj, cabs, cscat, asynth, nullptr, nullptr, s));
    else if (opt && opt->transfer_path == 1)
        KS_CUDA(launch_transfer_f32(ta, &g_tables.cj, cabs, cscat, asynth, nullptr, nullptr, s));
    else
        KS_CUDA(launch_transfer_stream_f32(ta, &g_tables.cj, cabs, cscat, asynth, w.tlist, w.counters + 2, s));
    return KS_OK;
}

static int fused_launches(bool has_lines, bool fp64, const ks_options* opt, bool with_transfer) {
    // grid parameters, prep, continuum, accumulation, the flag sink; line
    // bins, pair setup, three partition passes and the tile ranges; the
    // transfer (FP32: streaming pass + list pass)
    const bool stream_pass = !fp64 && !(opt && opt->transfer_path == 1);
    return 5 + (has_lines ? 6 : 0) + (with_transfer ? (stream_pass ? 2 : 1) : 0);
}

// Hydrogen lines (HPROF4 profiles) onto the line opacity cube, after the
// accumulation of the catalog's other lines (synthe_py/engine/opacity.py:2465-2503:
// with RHOXJ = 0 the transfer's line opacity is ASYNTH + AHLINE).
template <typename R>
static ks_status run_hydrogen(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                              const ks_options* opt, const Workspace& w, const DevTables& t, const R* cabs,
                              const R* cscat, R* cube, cudaStream_t s) {
    if (!atm->turbulent_velocity)
        return fail(KS_ERR_INVALID, "hydrogen lines need ks_atmos.turbulent_velocity");
    if (atm->n_ion < 2 || atm->n_elem < 1)
        return fail(KS_ERR_INVALID, "hydrogen lines need the H I and H II populations (n_ion >= 2)");
    if (lines->n_hydrogen > w.hyd_cap) return fail(KS_ERR_INVALID, "hydrogen lines exceed the workspace");
    const HydTables* tab = nullptr;
    ks_status st = hydrogen_device_tables(&tab);
    if (st) return st;
    HydArgs h;
    h.n_h = lines->n_hydrogen;
    h.n_layers = atm->n_layers;
    h.n_ion = atm->n_ion;
    h.n_elem = atm->n_elem;
    h.n_wl = grid->n;
    h.n_lines = lines->n_lines;
    h.flags = w.flags;
    h.rows = lines->hydrogen_rows;
    h.n_lower = lines->hydrogen_n_lower;
    h.n_upper = lines->hydrogen_n_upper;
    h.wavelength = lines->wavelength;
    h.gf = lines->gf;
    h.elo = lines->elo_cm;
    h.center = w.center;
    h.grid = grid->wavelength;
    h.temperature = atm->temperature;
    h.xne = atm->electron_density;
    h.rho = atm->mass_density;
    h.hckt = atm->hckt;
    h.vturb = atm->turbulent_velocity;
    h.xnf_he1 = atm->xnf_he1;
    h.xnf_h2 = atm->xnf_h2;
    h.population = atm->population;
    h.doppler = atm->doppler;
    h.cutoff = opt ? opt->cutoff : 1e-3;
    h.microturb_kms = opt ? opt->microturb_kms : 0.0;
    h.cabs = cabs;
    h.cscat = cscat;
    h.extab = t.extab;
    h.extabf = t.extabf;
    h.tab = tab;
    h.par = w.hyd_par;
    h.walk = w.hyd_walk;
    cudaError_t e;
    if constexpr (sizeof(R) == 8) e = launch_hydrogen_f64(h, cube, s);
    else e = launch_hydrogen_f32(h, cube, s);
    if (e != cudaSuccess) return fail(KS_ERR_CUDA, std::string("hydrogen lines: ") + cudaGetErrorString(e));
    return KS_OK;
}

// fort.19 NORMAL (NBLO/NBUP set) and autoionizing lines: _add_fort19_asynth's
// profiles, TMP x STIM onto ASYNTH before the hydrogen lines
// (synthe_py/engine/opacity.py:1335-1541, called at :2366).
template <typename R>
static ks_status run_f19(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid, const ks_options* opt,
                         const Workspace& w, const DevTables& t, const R* cabs, const R* cscat, R* cube,
                         cudaStream_t s) {
    if (!atm->turbulent_velocity)
        return fail(KS_ERR_INVALID, "fort.19 lines need ks_atmos.turbulent_velocity");
    if (lines->n_f19 > w.hyd_cap) return fail(KS_ERR_INVALID, "fort.19 lines exceed the workspace");
    F19Args f;
    f.n_f19 = lines->n_f19;
    f.n_layers = atm->n_layers;
    f.n_ion = atm->n_ion;
    f.n_elem = atm->n_elem;
    f.n_wl = grid->n;
    f.n_lines = lines->n_lines;
    f.flags = w.flags;
    f.rows = lines->f19_rows;
    f.kind = lines->f19_kind;
    f.nlast = lines->f19_nlast;
    f.nelion = lines->f19_nelion;
    f.ncon = lines->f19_ncon;
    f.nelionx = lines->f19_nelionx;
    const HydTables* tab = nullptr;
    ks_status st = hydrogen_device_tables(&tab);
    if (st) return st;
    f.tab = tab;
    f.cgf = lines->f19_cgf;
    f.gamma_rad = lines->f19_gamma_rad;
    f.gamma_stark = lines->f19_gamma_stark;
    f.gamma_vdw = lines->f19_gamma_vdw;
    f.wavelength = lines->wavelength;
    f.elo = lines->elo_cm;
    f.element_idx = lines->element_idx;
    f.ion_stage = lines->ion_stage;
    f.center = w.center;
    f.grid = grid->wavelength;
    f.temperature = atm->temperature;
    f.vturb = atm->turbulent_velocity;
    f.population = atm->population;
    f.depth = w.depth;
    f.cutoff = opt ? opt->cutoff : 1e-3;
    f.microturb_kms = opt ? opt->microturb_kms : 0.0;
    f.cabs = cabs;
    f.cscat = cscat;
    f.extab = t.extab;
    f.extabf = t.extabf;
    f.h0 = t.h0d;
    f.h1 = t.h1d;
    f.h2 = t.h2d;
    f.par = w.f19_par;
    f.walk = w.f19_walk;
    cudaError_t e;
    if constexpr (sizeof(R) == 8) e = launch_f19_f64(f, cube, s);
    else e = launch_f19_f32(f, cube, s);
    if (e != cudaSuccess) return fail(KS_ERR_CUDA, std::string("fort.19 lines: ") + cudaGetErrorString(e));
    return KS_OK;
}

// Helium lines: the reference's helium wing pass, AHE x STIM onto the line
// opacity cube after the hydrogen lines (synthe_py/engine/opacity.py:3650-3660).
template <typename R>
static ks_status run_helium(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                            const ks_options* opt, const Workspace& w, const DevTables& t, const R* cabs,
                            const R* cscat, R* cube, cudaStream_t s) {
    if (atm->n_ion < 2 || atm->n_elem < 2)
        return fail(KS_ERR_INVALID, "helium lines need the He populations (n_ion >= 2, n_elem >= 2)");
    if (lines->n_helium > w.hyd_cap) return fail(KS_ERR_INVALID, "helium lines exceed the workspace");
    HeArgs h;
    h.n_he = lines->n_helium;
    h.n_layers = atm->n_layers;
    h.n_ion = atm->n_ion;
    h.n_elem = atm->n_elem;
    h.n_wl = grid->n;
    h.n_lines = lines->n_lines;
    h.flags = w.flags;
    h.rows = lines->helium_rows;
    h.ncon = lines->helium_ncon;
    h.nelionx = lines->helium_nelionx;
    const HydTables* tab = nullptr;
    ks_status st = hydrogen_device_tables(&tab);
    if (st) return st;
    h.tab = tab;
    h.wavelength = lines->wavelength;
    h.gf = lines->gf;
    h.elo = lines->elo_cm;
    h.gamma_rad = lines->gamma_rad;
    h.gamma_stark = lines->gamma_stark;
    h.gamma_vdw = lines->gamma_vdw;
    h.ion_stage = lines->ion_stage;
    h.line_type = lines->line_type;
    h.center = w.center;
    h.grid = grid->wavelength;
    h.temperature = atm->temperature;
    h.population = atm->population;
    h.doppler = atm->doppler;
    h.depth = w.depth;
    h.cutoff = opt ? opt->cutoff : 1e-3;
    h.cabs = cabs;
    h.cscat = cscat;
    h.extab = t.extab;
    h.extabf = t.extabf;
    h.h0 = t.h0d;
    h.h1 = t.h1d;
    h.h2 = t.h2d;
    h.par = w.he_par;
    h.walk = w.he_walk;
    cudaError_t e;
    if constexpr (sizeof(R) == 8) e = launch_helium_f64(h, cube, s);
    else e = launch_helium_f32(h, cube, s);
    if (e != cudaSuccess) return fail(KS_ERR_CUDA, std::string("helium lines: ") + cudaGetErrorString(e));
    return KS_OK;
}

template <typename R>
static ks_status synthesize_impl(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                                 const ks_options* opt, Workspace& w, const DevTables& t,
                                 double* flux_total, double* flux_cont, R* asynth,
                                 cudaStream_t s, StageTimer& tm, bool do_transfer = true,
                                 bool allow_alloc = true) {
    constexpr bool fp64 = sizeof(R) == 8;
    ks_status st;
    const int L = atm->n_layers;
    KS_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int), s));
    KS_CUDA(cudaMemsetAsync(w.counters, 0, 4 * sizeof(unsigned long long), s));
    // class bytes of the padding slots [n_lines, stride) of every depth (the
    // pair setup writes the others)
    if (w.stride > lines->n_lines)
        KS_CUDA(cudaMemset2DAsync(w.cls + lines->n_lines, (size_t)w.stride, 0xff,
                                  (size_t)(w.stride - lines->n_lines), (size_t)L, s));
    PrepArgs pa = prep_args(atm, opt, w);
    ContArgs ca = cont_args(atm, grid);
    if constexpr (!fp64) {
        // the prep kernel converts the continuum tables once; the continuum
        // kernel then reads them in FP32 and leaves c/lambda for the
        // accumulation epilogue
        const int64_t nc = (int64_t)L * (atm->n_edge - 1) * 3;
        pa.n_coeff = nc;
        pa.abs_coeff = atm->cont_abs_coeff;
        pa.scat_coeff = atm->cont_scat_coeff;
        pa.abs_coeff_f = w.coef_f;
        pa.scat_coeff_f = w.coef_f + (size_t)L * (MAX_EDGES - 1) * 3;
        ca.abs_coeff_f = pa.abs_coeff_f;
        ca.scat_coeff_f = pa.scat_coeff_f;
        ca.freq_f = w.freq_f;
    }
    R* cabs = (R*)w.cont_abs;
    R* cscat = (R*)w.cont_scat;
    if ((st = run_bins(lines, grid, w, !fp64, s))) return st;
    if constexpr (fp64) KS_CUDA(launch_prep_f64(pa, s));
    else KS_CUDA(launch_prep_f32(pa, s));
    tm.mark();
    if constexpr (fp64) KS_CUDA(launch_continuum_f64(ca, cabs, cscat, s));
    else KS_CUDA(launch_continuum_f32(ca, cabs, cscat, s));
    tm.mark();
    if (lines->n_lines > 0) {
        PairArgs p = pair_args(lines, atm, grid, opt, w, t);
        if constexpr (fp64)
            KS_CUDA(launch_pair_setup_f64(p, true, cabs, cscat, (PairDesc<double>*)w.desc, w.cls, s));
        else
            KS_CUDA(launch_pair_setup_f32(p, true, cabs, cscat, (PairDesc<float>*)w.desc, w.cls, s));
        tm.mark();
        if ((st = run_partition(w, L, grid->n, default_tile(opt, fp64), s))) return st;
        tm.mark();
    } else {
        // no lines: every class list is empty
        KS_CUDA(cudaMemsetAsync(w.class_off, 0, sizeof(int64_t) * L * (N_REACH_CLASSES + 1), s));
        KS_CUDA(cudaMemsetAsync(w.tile_rng, 0, sizeof(int2) * L * w.ntiles * N_REACH_CLASSES, s));
        tm.mark();
        tm.mark();
    }
    AccArgs a = acc_args(lines, atm, grid, opt, w, t, fp64);
    int warps = default_warps(opt);
    if constexpr (fp64)
        KS_CUDA(launch_accumulate_f64(a, warps, (const PairDesc<double>*)w.desc, asynth, s));
    else
        KS_CUDA(launch_accumulate_f32(a, warps, (const PairDesc<float>*)w.desc, asynth, s));
    tm.mark();
    const int n_special = std::max(lines->n_f19, std::max(lines->n_hydrogen, lines->n_helium));
    if (n_special > 0) {
        // more special lines than the workspace's scratch holds: the rest on
        // the stream (freed once the special-line kernels are queued)
        Workspace ws = w;
        char* extra = nullptr;
        if (n_special > w.hyd_cap) {
            if (!allow_alloc)
                return fail(KS_ERR_UNSUPPORTED, "more than 256 special lines of one class need stream-ordered "
                                                "scratch, which this entry point does not allocate");
            const size_t per = sizeof(HydPar) + sizeof(HePar) + sizeof(F19Par) + 6 * sizeof(int2);
            const size_t bytes = (size_t)n_special * L * per + 1024;
            KS_CUDA(cudaMallocAsync((void**)&extra, bytes, s));
            Carve c{extra, bytes, 0, false};
            ws.hyd_cap = n_special;
            ws.hyd_par = c.take<HydPar>((size_t)n_special * L);
            ws.hyd_walk = c.take<int2>((size_t)n_special * L * 2);
            ws.he_par = c.take<HePar>((size_t)n_special * L);
            ws.he_walk = c.take<int2>((size_t)n_special * L * 2);
            ws.f19_par = c.take<F19Par>((size_t)n_special * L);
            ws.f19_walk = c.take<int2>((size_t)n_special * L * 2);
        }
        st = KS_OK;
        if (lines->n_f19 > 0) st = run_f19<R>(lines, atm, grid, opt, ws, t, cabs, cscat, asynth, s);
        if (!st && lines->n_hydrogen > 0) st = run_hydrogen<R>(lines, atm, grid, opt, ws, t, cabs, cscat, asynth, s);
        if (!st && lines->n_helium > 0) st = run_helium<R>(lines, atm, grid, opt, ws, t, cabs, cscat, asynth, s);
        if (extra) {
            cudaError_t fe = cudaFreeAsync(extra, s);
            if (!st && fe != cudaSuccess) st = fail(KS_ERR_CUDA, std::string("cudaFreeAsync: ") + cudaGetErrorString(fe));
        }
        if (st) return st;
        tm.mark_special();
    }
    if (do_transfer) {
        if ((st = run_transfer<R>(atm, grid, opt, w, t, cabs, cscat, asynth, flux_total, flux_cont, s)))
            return st;
        tm.mark();
    }
    return sink_flags(w.flags, s);
}

extern "C" ks_status ks_synthesize(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                                   const ks_options* opt, void* workspace, size_t workspace_bytes,
                                   double* flux_total, double* flux_cont, void* asynth_out,
                                   ks_stats* stats, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (!st) st = check_cont(atm);
    if (st) return st;
    if (!flux_total || !flux_cont) return fail(KS_ERR_INVALID, "ks_synthesize: NULL flux output");
    if ((st = check_tiling(opt))) return st;
    if (opt && (opt->transfer_path < 0 || opt->transfer_path > 1))
        return fail(KS_ERR_INVALID, "transfer_path must be 0 (streaming) or 1 (per-column)");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    bool need_asynth = asynth_out == nullptr;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, true, need_asynth,
           default_tile(opt, fp64));
    if (!workspace || workspace_bytes < dry.used)
        return fail(KS_ERR_NOMEM, "ks_synthesize: workspace too small (see ks_workspace_size)");
    Carve c{(char*)workspace, workspace_bytes, 0, false};
    layout(c, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, true, need_asynth,
           default_tile(opt, fp64));
    void* asy = asynth_out ? asynth_out : w.asynth;
    StageTimer tm;
    tm.start(s, stats && opt && opt->profile);
    if (fp64) st = synthesize_impl<double>(lines, atm, grid, opt, w, t, flux_total, flux_cont, (double*)asy, s, tm);
    else st = synthesize_impl<float>(lines, atm, grid, opt, w, t, flux_total, flux_cont, (float*)asy, s, tm);
    tm.finish(stats);
    if (st) return st;
    if (stats) {
        st = collect_stats(w, grid->n, stats, s);
        stats->kernel_launches = fused_launches(lines->n_lines > 0, fp64, opt, true);
        return st;
    }
    return KS_OK;
}

// ---------------------------------------------------------------------------
// the fused path in two halves, for depth-sharded runs
// ---------------------------------------------------------------------------

// Everything of ks_synthesize before the transfer, on the layers given
// (any contiguous block of an atmosphere: each stage is per layer), with the
// ASYNTH and continuum cubes [n_layers, n] written to the caller's buffers.
extern "C" ks_status ks_opacity(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                                const ks_options* opt, void* workspace, size_t workspace_bytes,
                                void* asynth_out, void* cont_abs_out, void* cont_scat_out,
                                ks_stats* stats, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (!st) st = check_cont(atm);
    if (st) return st;
    if (!asynth_out || !cont_abs_out || !cont_scat_out)
        return fail(KS_ERR_INVALID, "ks_opacity: NULL output cube");
    if ((st = check_tiling(opt))) return st;
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false,
           default_tile(opt, fp64));
    if (!workspace || workspace_bytes < dry.used)
        return fail(KS_ERR_NOMEM, "ks_opacity: workspace too small (see ks_workspace_size)");
    Carve c{(char*)workspace, workspace_bytes, 0, false};
    layout(c, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false,
           default_tile(opt, fp64));
    w.cont_abs = cont_abs_out;
    w.cont_scat = cont_scat_out;
    StageTimer tm;
    tm.start(s, stats && opt && opt->profile);
    if (fp64) st = synthesize_impl<double>(lines, atm, grid, opt, w, t, nullptr, nullptr, (double*)asynth_out, s, tm, false);
    else st = synthesize_impl<float>(lines, atm, grid, opt, w, t, nullptr, nullptr, (float*)asynth_out, s, tm, false);
    tm.finish(stats);
    if (st) return st;
    if (stats) {
        st = collect_stats(w, grid->n, stats, s, false);
        stats->kernel_launches = fused_launches(lines->n_lines > 0, fp64, opt, false);
        return st;
    }
    return KS_OK;
}

// The transfer of ks_synthesize on opacity cubes [n_layers, n] that
// ks_opacity produced (possibly layer block by layer block, regathered for
// a wavelength slice of the grid): the same arithmetic, so a spectrum
// assembled from slices equals the unsharded one.  Allocates its small
// workspace on the stream.
extern "C" ks_status ks_transfer_opacity(const ks_atmos* atm, const ks_grid* grid, const ks_options* opt,
                                         const void* cont_abs, const void* cont_scat, const void* asynth,
                                         double* flux_total, double* flux_cont, ks_stats* stats,
                                         void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (st) return st;
    if (!cont_abs || !cont_scat || !asynth || !flux_total || !flux_cont)
        return fail(KS_ERR_INVALID, "ks_transfer_opacity: NULL input/output");
    if (opt && (opt->transfer_path < 0 || opt->transfer_path > 1))
        return fail(KS_ERR_INVALID, "transfer_path must be 0 (streaming) or 1 (per-column)");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, 0, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false);
    char* buf = nullptr;
    KS_CUDA(cudaMallocAsync((void**)&buf, dry.used + 256, s));
    Carve c{buf, dry.used + 256, 0, false};
    layout(c, w, 0, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, false, false);
    st = KS_OK;
    if (cudaMemsetAsync(w.flags, 0, sizeof(int), s) != cudaSuccess ||
        cudaMemsetAsync(w.counters, 0, 4 * sizeof(unsigned long long), s) != cudaSuccess)
        st = fail(KS_ERR_CUDA, "ks_transfer_opacity: memset failed");
    if (!st) st = run_bins(nullptr, grid, w, false, s);
    if (!st) {
        PrepArgs pa = prep_args(atm, opt, w);
        cudaError_t e = fp64 ? launch_prep_f64(pa, s) : launch_prep_f32(pa, s);
        if (e != cudaSuccess) st = fail(KS_ERR_CUDA, cudaGetErrorString(e));
    }
    if (!st) {
        if (fp64)
            st = run_transfer<double>(atm, grid, opt, w, t, (const double*)cont_abs, (const double*)cont_scat,
                                      (const double*)asynth, flux_total, flux_cont, s);
        else
            st = run_transfer<float>(atm, grid, opt, w, t, (const float*)cont_abs, (const float*)cont_scat,
                                     (const float*)asynth, flux_total, flux_cont, s);
    }
    if (!st) st = sink_flags(w.flags, s);
    if (!st && stats) {
        st = collect_stats(w, grid->n, stats, s);
        const bool stream_pass = !fp64 && !(opt && opt->transfer_path == 1);
        stats->kernel_launches = 3 + (stream_pass ? 2 : 1);
    }
    cudaFreeAsync(buf, s);
    return st;
}

// ---------------------------------------------------------------------------
// gradients (the differentiable form)
// ---------------------------------------------------------------------------

// The FP64 fused synthesis with the JOSH system solved to 1e-13, then the
// adjoints of the transfer and of the accumulation for a loss whose
// derivative with respect to F_total is g_flux_total: gradients with respect
// to log10 gf and the three log10 damping constants of every line.
static ks_status adjoint_impl(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                              const ks_options* opt, void* workspace, size_t workspace_bytes,
                              const double* g_flux_total, double* flux_total, double* flux_cont,
                              double* d_log_gf, double* d_log_gamma_rad, double* d_log_gamma_stark,
                              double* d_log_gamma_vdw, const ks_atm_grad* ag, ks_stats* stats, void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (!st) st = check_cont(atm);
    if (st) return st;
    if (!opt || opt->precision != KS_PREC_FP64)
        return fail(KS_ERR_INVALID, "ks_synthesize_adjoint: options with precision KS_PREC_FP64 are required");
    if (opt->rhoxj > 0.0 || opt->microturb_kms > 0.0)
        return fail(KS_ERR_UNSUPPORTED, "ks_synthesize_adjoint: line scattering and microturbulence are not covered");
    if (lines->n_hydrogen > 0 || lines->n_helium > 0 || lines->n_f19 > 0)
        return fail(KS_ERR_UNSUPPORTED, "ks_synthesize_adjoint: hydrogen, helium and fort.19 lines are not covered");
    if (!g_flux_total || !flux_total || !flux_cont || !d_log_gf || !d_log_gamma_rad || !d_log_gamma_stark ||
        !d_log_gamma_vdw)
        return fail(KS_ERR_INVALID, "ks_synthesize_adjoint: NULL input/output");
    if ((st = check_tiling(opt))) return st;
    if (ag && (!ag->d_ln_population || !ag->d_ln_mass_density || !ag->d_electron_density || !ag->d_txnxn ||
               ag->n_groups < 0 || (ag->n_groups > 0 && (!ag->line_order || !ag->group_first || !ag->group_species))))
        return fail(KS_ERR_INVALID, "ks_synthesize_adjoint_atmos: incomplete ks_atm_grad record");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    ks_options o = *opt;
    o.exact_sweeps = 1;
    o.profile = 0;
    const int L = atm->n_layers;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, L, grid->n, atm->n_ion, atm->n_elem, true, true, true, default_tile(&o, true));
    if (!workspace || workspace_bytes < dry.used)
        return fail(KS_ERR_NOMEM, "ks_synthesize_adjoint: workspace too small (see ks_workspace_size, FP64)");
    Carve c{(char*)workspace, workspace_bytes, 0, false};
    layout(c, w, lines->n_lines, L, grid->n, atm->n_ion, atm->n_elem, true, true, true, default_tile(&o, true));
    StageTimer tm;
    st = synthesize_impl<double>(lines, atm, grid, &o, w, t, flux_total, flux_cont, (double*)w.asynth, s, tm);
    if (st) return st;
    // adjoint scratch
    const size_t n_asy = (size_t)L * grid->n, n_slot = (size_t)L * w.stride;
    char* buf = nullptr;
    const size_t n_part = ag ? (size_t)L * (size_t)ag->n_groups * 3 : 0;
    const size_t bytes = sizeof(double) * (n_asy + 2 * n_slot + n_part) + 256;
    KS_CUDA(cudaMallocAsync((void**)&buf, bytes, s));
    double* g_asy = (double*)buf;
    double* g_gf = g_asy + n_asy;
    double* g_a = g_gf + n_slot;
    double* part = g_a + n_slot;
    unsigned long long* skipped = w.counters + 3;
    AdjArgs aa;
    aa.n = grid->n;
    aa.n_layers = L;
    aa.grid = grid->wavelength;
    aa.depth = w.depth;
    aa.xtau = t.xtau;
    aa.ch = t.ch;
    aa.coefj64 = t.coefj64;
    aa.cont_abs = (const double*)w.cont_abs;
    aa.cont_scat = (const double*)w.cont_scat;
    aa.asynth = (const double*)w.asynth;
    aa.g_flux = g_flux_total;
    aa.g_asy = g_asy;
    aa.skipped = skipped;
    LineAdjArgs la;
    la.n_lines = lines->n_lines;
    la.n_wl = grid->n;
    la.stride = w.stride;
    la.n_layers = L;
    la.desc = (const PairDesc<double>*)w.desc;
    la.cls = w.cls;
    la.g_asy = g_asy;
    la.h0 = t.h0d;
    la.h1 = t.h1d;
    la.h2 = t.h2d;
    la.g_gf = g_gf;
    la.g_a = g_a;
    LineGradArgs lg;
    lg.n_lines = lines->n_lines;
    lg.stride = w.stride;
    lg.n_layers = L;
    lg.n_ion = atm->n_ion;
    lg.n_elem = atm->n_elem;
    lg.cls = w.cls;
    lg.g_gf = g_gf;
    lg.g_a = g_a;
    lg.depth = w.depth;
    lg.ion = w.ion;
    lg.desc = (const PairDesc<double>*)w.desc;
    lg.element_idx = lines->element_idx;
    lg.ion_stage = lines->ion_stage;
    lg.gamma_rad = lines->gamma_rad;
    lg.gamma_stark = lines->gamma_stark;
    lg.gamma_vdw = lines->gamma_vdw;
    lg.d_loggf = d_log_gf;
    lg.d_loggr = d_log_gamma_rad;
    lg.d_loggs = d_log_gamma_stark;
    lg.d_loggw = d_log_gamma_vdw;
    cudaError_t e = launch_transfer_adjoint(aa, s);
    if (e == cudaSuccess) e = launch_line_adjoint(la, s);
    if (e == cudaSuccess) e = launch_line_grad(lg, s);
    if (e == cudaSuccess && ag) {
        AtmGradArgs g;
        g.stride = w.stride;
        g.n_layers = L;
        g.n_ion = atm->n_ion;
        g.n_elem = atm->n_elem;
        g.n_groups = ag->n_groups;
        g.cls = w.cls;
        g.g_gf = g_gf;
        g.g_a = g_a;
        g.ion = w.ion;
        g.desc = (const PairDesc<double>*)w.desc;
        g.element_idx = lines->element_idx;
        g.ion_stage = lines->ion_stage;
        g.gamma_stark = lines->gamma_stark;
        g.gamma_vdw = lines->gamma_vdw;
        g.order = ag->line_order;
        g.group_first = ag->group_first;
        g.group_species = ag->group_species;
        g.part = part;
        g.d_ln_pop = ag->d_ln_population;
        g.d_ln_rho = ag->d_ln_mass_density;
        g.d_xne = ag->d_electron_density;
        g.d_txnxn = ag->d_txnxn;
        e = cudaMemsetAsync(ag->d_ln_population, 0, sizeof(double) * (size_t)L * atm->n_ion * atm->n_elem, s);
        if (e == cudaSuccess) e = launch_atm_grad(g, s);
    }
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return fail(KS_ERR_CUDA, cudaGetErrorString(e));
    if (stats) {
        st = collect_stats(w, grid->n, stats, s);
        unsigned long long sk = 0;
        KS_CUDA(cudaMemcpyAsync(&sk, skipped, sizeof(sk), cudaMemcpyDeviceToHost, s));
        KS_CUDA(cudaStreamSynchronize(s));
        stats->maxj_wavelengths = (int64_t)sk;  // columns given zero gradient (MAXJ = 1 or masked layers)
        stats->kernel_launches = fused_launches(lines->n_lines > 0, true, &o, true) + 3 +
                                 (ag ? (ag->n_groups > 0 ? 2 : 1) : 0);
        return st;
    }
    return KS_OK;
}

extern "C" ks_status ks_synthesize_adjoint(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                                           const ks_options* opt, void* workspace, size_t workspace_bytes,
                                           const double* g_flux_total, double* flux_total, double* flux_cont,
                                           double* d_log_gf, double* d_log_gamma_rad, double* d_log_gamma_stark,
                                           double* d_log_gamma_vdw, ks_stats* stats, void* stream) {
    return adjoint_impl(lines, atm, grid, opt, workspace, workspace_bytes, g_flux_total, flux_total, flux_cont,
                        d_log_gf, d_log_gamma_rad, d_log_gamma_stark, d_log_gamma_vdw, nullptr, stats, stream);
}

extern "C" ks_status ks_synthesize_adjoint_atmos(const ks_lines* lines, const ks_atmos* atm, const ks_grid* grid,
                                                 const ks_options* opt, void* workspace, size_t workspace_bytes,
                                                 const double* g_flux_total, double* flux_total, double* flux_cont,
                                                 double* d_log_gf, double* d_log_gamma_rad,
                                                 double* d_log_gamma_stark, double* d_log_gamma_vdw,
                                                 const ks_atm_grad* atm_grad, ks_stats* stats, void* stream) {
    if (!atm_grad) return fail(KS_ERR_INVALID, "ks_synthesize_adjoint_atmos: NULL ks_atm_grad");
    return adjoint_impl(lines, atm, grid, opt, workspace, workspace_bytes, g_flux_total, flux_total, flux_cont,
                        d_log_gf, d_log_gamma_rad, d_log_gamma_stark, d_log_gamma_vdw, atm_grad, stats, stream);
}

// ---------------------------------------------------------------------------
// synthesis without any device allocation
// ---------------------------------------------------------------------------

// Scratch of ks_synthesize_noalloc: a fixed 64 MiB array in the library's own
// device image.  Every GPU that loads the library holds it until the process
// exits.  All calls on a device share it, so calls that overlap on the GPU
// (concurrent streams, or threads) race on it and must be serialised by the
// caller.  Host code must not use the symbol itself as a device address: the
// address comes from cudaGetSymbolAddress, per device.
static const size_t kNoAllocScratchBytes = (size_t)64 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static void* g_noalloc_ptr[kMaxDevices];
static std::mutex g_noalloc_mu;

extern "C" ks_status ks_synthesize_noalloc(const ks_lines* lines, const ks_atmos* atm,
                                           const ks_grid* grid, const ks_options* opt,
                                           double* flux_total, double* flux_cont, void* asynth_out,
                                           void* stream) {
    ks_status st = check_atmos(atm);
    if (!st) st = check_grid(grid);
    if (!st) st = check_lines(lines);
    if (!st) st = check_cont(atm);
    if (st) return st;
    if (!flux_total || !flux_cont) return fail(KS_ERR_INVALID, "ks_synthesize_noalloc: NULL flux output");
    if (lines->n_hydrogen > kMaxHydrogenLines || lines->n_helium > kMaxHydrogenLines ||
        lines->n_f19 > kMaxHydrogenLines)
        return fail(KS_ERR_UNSUPPORTED, "ks_synthesize_noalloc: more than 256 special lines of one class "
                                        "(their scratch would be allocated); use ks_synthesize");
    if ((st = check_tiling(opt))) return st;
    if (opt && (opt->transfer_path < 0 || opt->transfer_path > 1))
        return fail(KS_ERR_INVALID, "transfer_path must be 0 (streaming) or 1 (per-column)");
    bool fp64 = opt && opt->precision == KS_PREC_FP64;
    bool need_asynth = asynth_out == nullptr;
    Carve dry{nullptr, 0, 0, true};
    Workspace w;
    layout(dry, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, true, need_asynth,
           default_tile(opt, fp64));
    if (dry.used > kNoAllocScratchBytes)
        return fail(KS_ERR_NOMEM,
                    "ks_synthesize_noalloc: these sizes need " + std::to_string(dry.used) +
                        " bytes of scratch, more than the 64 MiB (67108864 bytes) the no-allocation "
                        "entry point holds; use ks_synthesize with a caller workspace");
    DevTables t;
    if ((st = device_tables(&t))) return st;
    int dev = 0;
    KS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KS_ERR_UNSUPPORTED, "device index out of range");
    void* scratch = nullptr;
    {
        // set-up, once per device (this device is current): the device
        // address of the scratch array
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    Carve c{(char*)scratch, kNoAllocScratchBytes, 0, false};
    layout(c, w, lines->n_lines, atm->n_layers, grid->n, atm->n_ion, atm->n_elem, fp64, true, need_asynth,
           default_tile(opt, fp64));
    void* asy = asynth_out ? asynth_out : w.asynth;
    StageTimer tm;  // off: no profiling in this entry point
    // synthesize_impl clears the counters, flags and reach classes in the
    // scratch before use; everything else is written before it is read.
    if (fp64)
        st = synthesize_impl<double>(lines, atm, grid, opt, w, t, flux_total, flux_cont, (double*)asy, s, tm, true,
                                     false);
    else
        st = synthesize_impl<float>(lines, atm, grid, opt, w, t, flux_total, flux_cont, (float*)asy, s, tm, true,
                                    false);
    return st;
}

// ---------------------------------------------------------------------------
// batched synthesis: every stage once over all jobs
// ---------------------------------------------------------------------------

#define KS_BATCH_LOOP(...)                                                       \
    const int64_t total = g.first[g.n_jobs];                                    \
    int j = -1;                                                                 \
    int64_t j_first = 0, j_end = -1;                                            \
    for (int64_t v = blockIdx.x; v < total; v += gridDim.x) {                   \
        int x, y, gx, gy;                                                       \
        if (v >= j_end) { /* a new job: search the prefix */                    \
            j = batch_locate(g, v, x, y, gx, gy);                               \
            j_first = g.first[j];                                               \
            j_end = g.first[j + 1];                                             \
        } else {                                                                \
            const int64_t local = v - j_first;                                  \
            gx = g.dims[2 * j];                                                 \
            gy = g.dims[2 * j + 1];                                             \
            x = (int)(local % gx);                                              \
            y = (int)(local / gx);                                              \
        }                                                                       \
        const VB vb{x, y, gx, gy};                                              \
        __VA_ARGS__;                                                            \
        __syncthreads();                                                        \
    }

// Per job and depth (virtual block (0, d)): clear the job's flag word and
// counters, set its class bytes of the padding slots to 0xff and, for a job
// without lines, empty its class lists and tile ranges (the memsets that
// synthesize_impl issues for one synthesis).
__global__ void __launch_bounds__(256) reset_batch_kernel(const ResetJob* __restrict__ jobs, BatchGrid g) {
    KS_BATCH_LOOP({
        const ResetJob& J = jobs[j];
        const int d = vb.y;
        if (d == 0 && threadIdx.x == 0) {
            *J.flags = 0;
            for (int k = 0; k < 4; k++) J.counters[k] = 0ull;
        }
        uint8_t* row = J.cls + (int64_t)d * J.stride;
        for (int64_t i = J.n_lines + threadIdx.x; i < J.stride; i += blockDim.x) row[i] = 0xff;
        if (J.n_lines == 0) {
            for (int k = threadIdx.x; k <= N_REACH_CLASSES; k += blockDim.x)
                J.class_off[(int64_t)d * (N_REACH_CLASSES + 1) + k] = 0;
            for (int64_t k = threadIdx.x; k < (int64_t)J.ntiles * N_REACH_CLASSES; k += blockDim.x)
                J.tile_rng[(int64_t)d * J.ntiles * N_REACH_CLASSES + k] = make_int2(0, 0);
        }
    })
}

__global__ void __launch_bounds__(32) grid_params_batch_kernel(const BinsJob* __restrict__ jobs, BatchGrid g) {
    KS_BATCH_LOOP(if (threadIdx.x == 0) grid_params_kernel_body(vb, jobs[j].grid, jobs[j].n_wl,
                                                                 jobs[j].grid_origin, jobs[j].gp))
}

__global__ void __launch_bounds__(256) line_bins_batch_kernel(const BinsJob* __restrict__ jobs, BatchGrid g) {
    KS_BATCH_LOOP({
        const BinsJob& J = jobs[j];
        line_bins_kernel_body(vb, J.n_lines, J.n_wl, J.wavelength, J.gp, J.center, J.wing, J.cgf, J.elo, J.gr,
                              J.gs, J.gw, J.gf, J.linef, J.flags);
    })
}

__global__ void __launch_bounds__(kPartThreads) class_count_batch_kernel(const PartJob* __restrict__ jobs,
                                                                        BatchGrid g) {
    KS_BATCH_LOOP(class_count_kernel_body(vb, jobs[j].cls, jobs[j].stride, jobs[j].nchunks, jobs[j].counts))
}

__global__ void __launch_bounds__(32) class_scan_batch_kernel(const PartJob* __restrict__ jobs, BatchGrid g) {
    KS_BATCH_LOOP(class_scan_kernel_body(vb, jobs[j].counts, jobs[j].nchunks, jobs[j].stride, jobs[j].chunk_base,
                                         jobs[j].class_off, jobs[j].counters))
}

__global__ void __launch_bounds__(kPartThreads) class_scatter_batch_kernel(const PartJob* __restrict__ jobs,
                                                                          BatchGrid g) {
    KS_BATCH_LOOP(class_scatter_kernel_body(vb, jobs[j].cls, jobs[j].stride, jobs[j].nchunks, jobs[j].chunk_base,
                                            jobs[j].class_pos))
}

__global__ void __launch_bounds__(256) tile_ranges_batch_kernel(const PartJob* __restrict__ jobs, BatchGrid g) {
    KS_BATCH_LOOP(tile_ranges_kernel_body(vb, jobs[j].class_off, jobs[j].class_pos, jobs[j].wing, jobs[j].n_wl,
                                          jobs[j].tile_bins, jobs[j].ntiles, jobs[j].tile_rng))
}

__global__ void __launch_bounds__(32) flag_sink_batch_kernel(int* const* __restrict__ flags, BatchGrid g) {
    KS_BATCH_LOOP(if (threadIdx.x == 0) {
        const int f = *flags[j];
        if (f) atomicOr(&g_sticky_flags, f);
    })
}

#undef KS_BATCH_LOOP

namespace {

enum BatchStage {
    BS_RESET, BS_GRID, BS_BINS, BS_PREP, BS_CONT, BS_PAIR, BS_COUNT, BS_SCAN, BS_SCATTER, BS_RANGES, BS_ACC,
    BS_TRANS, BS_LIST, BS_SINK, BS_N
};
const int kBatchThreads[BS_N] = {256, 32, 256, 256, 256, 128, kPartThreads, 32, kPartThreads, 256, 0, 0, 0, 32};

// Device tables of one stage: job records, block prefix and per-job grids.
struct StageTable {
    void* jobs = nullptr;
    int64_t* first = nullptr;
    int* dims = nullptr;
    int64_t total = 0;
    int grid = 1;
};

}  // namespace

// A job's special lines (hydrogen, helium, fort.19): its view of the shared
// list with its own special rows (relative to the job's slice, in the job's
// block of the workspace), and the records the special-line kernels read when
// the batch runs.
struct BatchSpecial {
    bool any = false;
    ks_lines lines{};
    ks_atmos atm{};
    ks_grid grid{};
};

struct ks_batch {
    int n_jobs = 0;
    int dev = 0;
    bool fp64 = false, stream_pass = true, profile = false;
    int tile = 0, warps = 0;
    StageTable st[BS_N];
    std::vector<Workspace> ws;
    std::vector<int64_t> n_wl;
    std::vector<BatchSpecial> spec;
    bool any_special = false;
    ks_options opt{};
    bool has_opt = false;
};

namespace {

struct BatchLayout {
    size_t table_bytes = 0;
    std::vector<size_t> job_off, job_bytes, rows_off;  // rows_off: the job's special rows
    size_t total = 0;
};

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

ks_status batch_check(const ks_lines* lines, const ks_job* jobs, int32_t n_jobs, const ks_options* opt) {
    ks_status st = check_lines(lines);
    if (st) return st;
    if (n_jobs <= 0 || !jobs) return fail(KS_ERR_INVALID, "ks_batch: no jobs");
    if ((st = check_tiling(opt))) return st;
    if (opt && (opt->transfer_path < 0 || opt->transfer_path > 1))
        return fail(KS_ERR_INVALID, "transfer_path must be 0 (streaming) or 1 (per-column)");
    for (int i = 0; i < n_jobs; i++) {
        const ks_job& J = jobs[i];
        if (!J.atm || !J.grid || !J.flux_total || !J.flux_cont)
            return fail(KS_ERR_INVALID, "ks_batch: job " + std::to_string(i) + " has a NULL record or output");
        if ((st = check_atmos(J.atm)) || (st = check_grid(J.grid)) || (st = check_cont(J.atm))) return st;
        if (J.line_first < 0 || J.line_count < 0 || J.line_first + J.line_count > lines->n_lines)
            return fail(KS_ERR_INVALID, "ks_batch: job " + std::to_string(i) + " line slice outside the list");
    }
    return KS_OK;
}

// Rows [line_first, line_first + line_count) of the shared list as a ks_lines view.
ks_lines job_lines(const ks_lines* l, const ks_job& J) {
    ks_lines v = *l;
    const int64_t o = J.line_first;
    v.n_lines = J.line_count;
    v.wavelength = l->wavelength + o;
    v.gf = l->gf + o;
    v.cgf = l->cgf + o;
    v.gamma_rad = l->gamma_rad + o;
    v.gamma_stark = l->gamma_stark + o;
    v.gamma_vdw = l->gamma_vdw + o;
    v.elo_cm = l->elo_cm + o;
    v.element_idx = l->element_idx + o;
    v.ion_stage = l->ion_stage + o;
    v.line_type = l->line_type + o;
    v.process_mask = l->process_mask + o;
    v.asynth_mask = l->asynth_mask + o;
    return v;
}

// Bytes of one job's records over all stage tables.
size_t batch_job_record_bytes(bool fp64) {
    size_t r = sizeof(ResetJob) + sizeof(BinsJob) + sizeof(PrepArgs) + sizeof(PartJob) + sizeof(int*);
    r += fp64 ? sizeof(ContJob<double>) + sizeof(PairJob<double>) + sizeof(AccJob<double>) + sizeof(TransferJob<double>)
              : sizeof(ContJob<float>) + sizeof(PairJob<float>) + sizeof(AccJob<float>) + sizeof(TransferJob<float>);
    return r;
}

BatchLayout batch_layout(const ks_lines* lines, const ks_job* jobs, int32_t n_jobs, const ks_options* opt) {
    BatchLayout b;
    const bool fp64 = opt && opt->precision == KS_PREC_FP64;
    // job records (9 tables), then per stage the block prefix and the grids,
    // each table 64-byte aligned
    b.table_bytes = batch_job_record_bytes(fp64) * (size_t)n_jobs + 64 * (9 + 2 * BS_N) +
                    BS_N * (sizeof(int64_t) * (n_jobs + 1) + sizeof(int) * 2 * (size_t)n_jobs);
    size_t off = al256(b.table_bytes);
    for (int i = 0; i < n_jobs; i++) {
        Carve dry{nullptr, 0, 0, true};
        Workspace w;
        layout(dry, w, jobs[i].line_count, jobs[i].atm->n_layers, jobs[i].grid->n, jobs[i].atm->n_ion,
               jobs[i].atm->n_elem, fp64, true, true, default_tile(opt, fp64));
        // room for the job's special rows: at most its slice's lines of each class
        const int64_t cnt = jobs[i].line_count;
        const int64_t n_rows = std::min<int64_t>(cnt, lines->n_hydrogen) + std::min<int64_t>(cnt, lines->n_helium) +
                               std::min<int64_t>(cnt, lines->n_f19);
        const size_t rows_bytes = al256((size_t)n_rows * sizeof(int32_t));
        b.job_off.push_back(off);
        b.rows_off.push_back(off + al256(dry.used));
        b.job_bytes.push_back(al256(dry.used) + rows_bytes);
        off += al256(dry.used) + rows_bytes;
    }
    b.total = off;
    return b;
}

// The jobs' special lines.  The shared list's special rows ascend (catalog
// order), so a job's lines of each class are one contiguous run of them: its
// per-line columns are the shared ones offset to the run, its rows are copied
// relative to the job's slice into the job's block.  Synchronous (plan time).
ks_status batch_special_build(ks_batch* b, const ks_lines* lines, const ks_job* jobs, int32_t n, char* base,
                              const BatchLayout& lay) {
    b->spec.assign(n, BatchSpecial{});
    b->any_special = false;
    if (lines->n_hydrogen <= 0 && lines->n_helium <= 0 && lines->n_f19 <= 0) return KS_OK;
    auto fetch = [](const int32_t* d, int32_t cnt, std::vector<int32_t>& h) -> cudaError_t {
        h.resize(cnt > 0 ? cnt : 0);
        return cnt > 0 ? cudaMemcpy(h.data(), d, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost) : cudaSuccess;
    };
    std::vector<int32_t> hr, her, fr;
    KS_CUDA(fetch(lines->hydrogen_rows, lines->n_hydrogen, hr));
    KS_CUDA(fetch(lines->helium_rows, lines->n_helium, her));
    KS_CUDA(fetch(lines->f19_rows, lines->n_f19, fr));
    if (!std::is_sorted(hr.begin(), hr.end()) || !std::is_sorted(her.begin(), her.end()) ||
        !std::is_sorted(fr.begin(), fr.end()))
        return fail(KS_ERR_INVALID, "ks_batch: the special lines' rows must ascend (catalog order)");
    if (lines->n_hydrogen > 0 || lines->n_helium > 0 || lines->n_f19 > 0) {
        // the hydrogen tables' first copy to this device happens here, not in a captured run
        const HydTables* tab = nullptr;
        ks_status st = hydrogen_device_tables(&tab);
        if (st) return st;
    }
    for (int i = 0; i < n; i++) {
        const ks_job& J = jobs[i];
        const int64_t r0 = J.line_first, r1 = J.line_first + J.line_count;
        auto run = [&](const std::vector<int32_t>& v, int64_t* lo) -> int32_t {
            const auto a = std::lower_bound(v.begin(), v.end(), r0);
            const auto z = std::lower_bound(v.begin(), v.end(), r1);
            *lo = a - v.begin();
            return (int32_t)(z - a);
        };
        int64_t lh = 0, le = 0, lf = 0;
        const int32_t nh = run(hr, &lh), ne = run(her, &le), nf = run(fr, &lf);
        if (nh + ne + nf == 0) continue;
        if (nh > kMaxHydrogenLines || ne > kMaxHydrogenLines || nf > kMaxHydrogenLines)
            return fail(KS_ERR_UNSUPPORTED, "ks_batch: job " + std::to_string(i) +
                                                " has more than 256 special lines of one class");
        if (nh > 0 && (!J.atm->turbulent_velocity || J.atm->n_ion < 2))
            return fail(KS_ERR_INVALID, "ks_batch: job " + std::to_string(i) +
                                            ": hydrogen lines need ks_atmos.turbulent_velocity and n_ion >= 2");
        std::vector<int32_t> local;
        local.reserve((size_t)nh + ne + nf);
        for (int32_t k = 0; k < nh; k++) local.push_back((int32_t)(hr[lh + k] - r0));
        for (int32_t k = 0; k < ne; k++) local.push_back((int32_t)(her[le + k] - r0));
        for (int32_t k = 0; k < nf; k++) local.push_back((int32_t)(fr[lf + k] - r0));
        int32_t* d = (int32_t*)(base + lay.rows_off[i]);
        KS_CUDA(cudaMemcpy(d, local.data(), sizeof(int32_t) * local.size(), cudaMemcpyHostToDevice));
        BatchSpecial& sp = b->spec[i];
        sp.any = true;
        sp.atm = *J.atm;
        sp.grid = *J.grid;
        ks_lines& v = sp.lines;
        v = job_lines(lines, J);
        v.n_hydrogen = nh;
        v.hydrogen_rows = nh ? d : nullptr;
        v.hydrogen_n_lower = nh ? lines->hydrogen_n_lower + lh : nullptr;
        v.hydrogen_n_upper = nh ? lines->hydrogen_n_upper + lh : nullptr;
        v.n_helium = ne;
        v.helium_rows = ne ? d + nh : nullptr;
        v.helium_ncon = ne ? lines->helium_ncon + le : nullptr;
        v.helium_nelionx = ne ? lines->helium_nelionx + le : nullptr;
        v.n_f19 = nf;
        v.f19_rows = nf ? d + nh + ne : nullptr;
        v.f19_cgf = nf ? lines->f19_cgf + lf : nullptr;
        v.f19_gamma_rad = nf ? lines->f19_gamma_rad + lf : nullptr;
        v.f19_gamma_stark = nf ? lines->f19_gamma_stark + lf : nullptr;
        v.f19_gamma_vdw = nf ? lines->f19_gamma_vdw + lf : nullptr;
        v.f19_kind = nf ? lines->f19_kind + lf : nullptr;
        v.f19_nlast = nf ? lines->f19_nlast + lf : nullptr;
        v.f19_nelion = nf ? lines->f19_nelion + lf : nullptr;
        v.f19_ncon = nf ? lines->f19_ncon + lf : nullptr;
        v.f19_nelionx = nf ? lines->f19_nelionx + lf : nullptr;
        b->any_special = true;
    }
    return KS_OK;
}

// Queues every job's special-line kernels (fort.19 into ASYNTH, then the
// hydrogen and helium lines), in the order a single synthesis runs them,
// between the batch's accumulation and transfer launches.
template <typename R>
ks_status batch_special_run(ks_batch* b, cudaStream_t s) {
    DevTables t;
    ks_status st = device_tables(&t);
    if (st) return st;
    const ks_options* opt = b->has_opt ? &b->opt : nullptr;
    for (int i = 0; i < b->n_jobs; i++) {
        const BatchSpecial& sp = b->spec[i];
        if (!sp.any) continue;
        const Workspace& w = b->ws[i];
        const R* cabs = (const R*)w.cont_abs;
        const R* cscat = (const R*)w.cont_scat;
        R* cube = (R*)w.asynth;
        if (sp.lines.n_f19 > 0 && (st = run_f19<R>(&sp.lines, &sp.atm, &sp.grid, opt, w, t, cabs, cscat, cube, s)))
            return st;
        if (sp.lines.n_hydrogen > 0 &&
            (st = run_hydrogen<R>(&sp.lines, &sp.atm, &sp.grid, opt, w, t, cabs, cscat, cube, s)))
            return st;
        if (sp.lines.n_helium > 0 &&
            (st = run_helium<R>(&sp.lines, &sp.atm, &sp.grid, opt, w, t, cabs, cscat, cube, s)))
            return st;
    }
    return KS_OK;
}

template <typename R>
ks_status batch_build(ks_batch* b, const ks_lines* lines, const ks_job* jobs, int32_t n, const ks_options* opt,
                      char* base, const BatchLayout& lay, const DevTables& t) {
    constexpr bool fp64 = sizeof(R) == 8;
    std::vector<ResetJob> reset(n);
    std::vector<BinsJob> bins(n);
    std::vector<PrepArgs> prep(n);
    std::vector<ContJob<R>> cont(n);
    std::vector<PairJob<R>> pair(n);
    std::vector<PartJob> part(n);
    std::vector<AccJob<R>> acc(n);
    std::vector<TransferJob<R>> tr(n);
    std::vector<int*> sink(n);
    std::vector<std::vector<int>> dims(BS_N, std::vector<int>(2 * (size_t)n, 1));
    b->ws.resize(n);
    b->n_wl.resize(n);
    for (int i = 0; i < n; i++) {
        const ks_job& J = jobs[i];
        const ks_atmos* atm = J.atm;
        const ks_grid* grid = J.grid;
        const ks_lines lv = job_lines(lines, J);
        const int L = atm->n_layers;
        Carve c{base + lay.job_off[i], lay.job_bytes[i], 0, false};
        Workspace& w = b->ws[i];
        layout(c, w, lv.n_lines, L, grid->n, atm->n_ion, atm->n_elem, fp64, true, true, b->tile);
        b->n_wl[i] = grid->n;
        reset[i] = ResetJob{w.flags, w.counters, w.cls, lv.n_lines, w.stride, L, w.ntiles, w.class_off, w.tile_rng};
        dims[BS_RESET][2 * i + 1] = L;
        BinsJob& bj = bins[i];
        bj.grid = grid->wavelength;
        bj.n_wl = grid->n;
        bj.grid_origin = grid->grid_origin;
        bj.gp = w.gp;
        bj.n_lines = lv.n_lines;
        bj.wavelength = lv.wavelength;
        bj.cgf = lv.cgf;
        bj.elo = lv.elo_cm;
        bj.gr = lv.gamma_rad;
        bj.gs = lv.gamma_stark;
        bj.gw = lv.gamma_vdw;
        bj.gf = lv.gf;
        bj.center = w.center;
        bj.wing = w.wing;
        bj.linef = fp64 ? nullptr : w.linef;
        bj.flags = w.flags;
        dims[BS_BINS][2 * i] = (int)((lv.n_lines + 255) / 256);
        dims[BS_BINS][2 * i + 1] = lv.n_lines > 0 ? 1 : 0;
        PrepArgs pa = prep_args(atm, opt, w);
        ContArgs ca = cont_args(atm, grid);
        if constexpr (!fp64) {
            pa.n_coeff = (int64_t)L * (atm->n_edge - 1) * 3;
            pa.abs_coeff = atm->cont_abs_coeff;
            pa.scat_coeff = atm->cont_scat_coeff;
            pa.abs_coeff_f = w.coef_f;
            pa.scat_coeff_f = w.coef_f + (size_t)L * (MAX_EDGES - 1) * 3;
            ca.abs_coeff_f = pa.abs_coeff_f;
            ca.scat_coeff_f = pa.scat_coeff_f;
            ca.freq_f = w.freq_f;
        }
        prep[i] = pa;
        dims[BS_PREP][2 * i] = (int)(((int64_t)L * atm->n_ion * atm->n_elem + 255) / 256);
        cont[i] = ContJob<R>{ca, (R*)w.cont_abs, (R*)w.cont_scat};
        dims[BS_CONT][2 * i] = (int)((grid->n + 255) / 256);
        pair[i] = PairJob<R>{pair_args(&lv, atm, grid, opt, w, t), (const R*)w.cont_abs, (const R*)w.cont_scat,
                             (PairDesc<R>*)w.desc, w.cls};
        const int Lp = lv.n_lines > 0 ? L : 0;
        dims[BS_PAIR][2 * i] = (int)((lv.n_lines + 127) / 128);
        dims[BS_PAIR][2 * i + 1] = Lp;
        PartJob& pj = part[i];
        pj.cls = w.cls;
        pj.stride = w.stride;
        pj.n_wl = grid->n;
        pj.nchunks = w.nchunks;
        pj.ntiles = w.ntiles;
        pj.tile_bins = b->tile;
        pj.counts = w.counts;
        pj.chunk_base = w.chunk_base;
        pj.class_off = w.class_off;
        pj.class_pos = w.class_pos;
        pj.wing = w.wing;
        pj.tile_rng = w.tile_rng;
        pj.counters = w.counters;
        dims[BS_COUNT][2 * i] = w.nchunks;
        dims[BS_COUNT][2 * i + 1] = Lp;
        dims[BS_SCAN][2 * i] = Lp;
        dims[BS_SCATTER][2 * i] = w.nchunks;
        dims[BS_SCATTER][2 * i + 1] = Lp;
        dims[BS_RANGES][2 * i] = (int)(((int64_t)w.ntiles * N_REACH_CLASSES + 255) / 256);
        dims[BS_RANGES][2 * i + 1] = w.ntiles > 0 ? Lp : 0;
        acc[i] = AccJob<R>{acc_args(&lv, atm, grid, opt, w, t, fp64), (const PairDesc<R>*)w.desc, (R*)w.asynth};
        dims[BS_ACC][2 * i] = (int)((grid->n + b->tile - 1) / b->tile);
        dims[BS_ACC][2 * i + 1] = L;
        TransferArgs ta = transfer_args(atm, grid, w, t, J.flux_total, J.flux_cont, true, fp64);
        ta.line_scat = (opt && opt->rhoxj > 0.0) ? 1 : 0;
        if (fp64 && opt && opt->exact_sweeps) ta.coefj64 = t.coefj64;
        tr[i] = TransferJob<R>{ta, (const R*)w.cont_abs, (const R*)w.cont_scat, (const R*)w.asynth, w.tlist,
                               w.counters + 2};
        dims[BS_TRANS][2 * i] = (int)((grid->n + 127) / 128);
        // the hand-over list may hold any of the job's columns (hot or
        // saturated columns all go there): one virtual block per 128 of them;
        // blocks past the list's length return at once
        dims[BS_LIST][2 * i] = b->stream_pass ? (int)((grid->n + 127) / 128) : 0;
        sink[i] = w.flags;
    }
    std::vector<char> host(lay.table_bytes, 0);
    size_t off = 0;
    bool overflow = false;
    auto put = [&](const void* src, size_t bytes) -> void* {
        off = (off + 63) & ~size_t(63);
        if (off + bytes > host.size()) {
            overflow = true;
            return nullptr;
        }
        std::memcpy(host.data() + off, src, bytes);
        void* dptr = base + off;
        off += bytes;
        return dptr;
    };
    void* d_reset = put(reset.data(), sizeof(ResetJob) * n);
    void* d_bins = put(bins.data(), sizeof(BinsJob) * n);
    void* d_prep = put(prep.data(), sizeof(PrepArgs) * n);
    void* d_cont = put(cont.data(), sizeof(ContJob<R>) * n);
    void* d_pair = put(pair.data(), sizeof(PairJob<R>) * n);
    void* d_part = put(part.data(), sizeof(PartJob) * n);
    void* d_acc = put(acc.data(), sizeof(AccJob<R>) * n);
    void* d_tr = put(tr.data(), sizeof(TransferJob<R>) * n);
    void* d_sink = put(sink.data(), sizeof(int*) * n);
    void* stage_jobs[BS_N] = {d_reset, d_bins, d_bins, d_prep, d_cont, d_pair, d_part,
                              d_part, d_part, d_part, d_acc, d_tr, d_tr, d_sink};
    for (int s = 0; s < BS_N; s++) {
        std::vector<int64_t> first(n + 1, 0);
        for (int i = 0; i < n; i++) first[i + 1] = first[i] + (int64_t)dims[s][2 * i] * dims[s][2 * i + 1];
        for (int i = 0; i < n; i++)
            if (dims[s][2 * i] <= 0) dims[s][2 * i] = 1;  // a job without blocks: keep the divisor valid
        StageTable& T = b->st[s];
        T.jobs = stage_jobs[s];
        T.first = (int64_t*)put(first.data(), sizeof(int64_t) * (n + 1));
        T.dims = (int*)put(dims[s].data(), sizeof(int) * 2 * n);
        T.total = first[n];
    }
    if (overflow) return fail(KS_ERR_NOMEM, "ks_batch: internal table overflow");
    KS_CUDA(cudaMemcpy(base, host.data(), off, cudaMemcpyHostToDevice));
    ks_status sst = batch_special_build(b, lines, jobs, n, base, lay);
    if (sst) return sst;
    // persistent grids
    int64_t totals[6] = {b->st[BS_PREP].total, b->st[BS_CONT].total, b->st[BS_PAIR].total, b->st[BS_ACC].total,
                         b->st[BS_TRANS].total, b->st[BS_LIST].total};
    int grids[6];
    KS_CUDA(fp64 ? batch_grids_f64(b->warps, b->tile, b->stream_pass, totals, grids)
                 : batch_grids_f32(b->warps, b->tile, b->stream_pass, totals, grids));
    b->st[BS_PREP].grid = grids[0];
    b->st[BS_CONT].grid = grids[1];
    b->st[BS_PAIR].grid = grids[2];
    b->st[BS_ACC].grid = grids[3];
    b->st[BS_TRANS].grid = grids[4];
    b->st[BS_LIST].grid = grids[5];
    const void* fns[BS_N] = {(const void*)reset_batch_kernel, (const void*)grid_params_batch_kernel,
                             (const void*)line_bins_batch_kernel, nullptr, nullptr, nullptr,
                             (const void*)class_count_batch_kernel, (const void*)class_scan_batch_kernel,
                             (const void*)class_scatter_batch_kernel, (const void*)tile_ranges_batch_kernel,
                             nullptr, nullptr, nullptr, (const void*)flag_sink_batch_kernel};
    int sms = 0;
    KS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->dev));
    for (int s = 0; s < BS_N; s++) {
        if (!fns[s]) continue;
        int per = 0;
        KS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fns[s], kBatchThreads[s], 0));
        const int64_t g = (int64_t)sms * (per > 0 ? per : 1);
        const int64_t tot = b->st[s].total;
        b->st[s].grid = (int)(tot < g ? (tot > 0 ? tot : 1) : g);
    }
    return KS_OK;
}

BatchGrid bgrid(const StageTable& T, int n) { return BatchGrid{T.first, T.dims, n}; }

}  // namespace

extern "C" ks_status ks_batch_workspace_size(const ks_lines* lines, const ks_job* jobs, int32_t n_jobs,
                                             const ks_options* opt, size_t* bytes) {
    ks_status st = batch_check(lines, jobs, n_jobs, opt);
    if (st) return st;
    if (!bytes) return fail(KS_ERR_INVALID, "ks_batch_workspace_size: NULL output");
    *bytes = batch_layout(lines, jobs, n_jobs, opt).total;
    return KS_OK;
}

extern "C" ks_status ks_batch_create(const ks_lines* lines, const ks_job* jobs, int32_t n_jobs,
                                     const ks_options* opt, void* workspace, size_t workspace_bytes,
                                     ks_batch** out) {
    if (!out) return fail(KS_ERR_INVALID, "ks_batch_create: NULL output");
    *out = nullptr;
    ks_status st = batch_check(lines, jobs, n_jobs, opt);
    if (st) return st;
    DevTables t;
    if ((st = device_tables(&t))) return st;
    BatchLayout lay = batch_layout(lines, jobs, n_jobs, opt);
    if (!workspace || workspace_bytes < lay.total)
        return fail(KS_ERR_NOMEM, "ks_batch_create: workspace too small (see ks_batch_workspace_size)");
    if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
        return fail(KS_ERR_INVALID, "ks_batch_create: workspace must be 256-byte aligned");
    ks_batch* b = new ks_batch();
    b->n_jobs = n_jobs;
    b->fp64 = opt && opt->precision == KS_PREC_FP64;
    b->stream_pass = !b->fp64 && !(opt && opt->transfer_path == 1);
    b->profile = opt && opt->profile;
    b->tile = default_tile(opt, b->fp64);
    b->warps = default_warps(opt);
    if (opt) {
        b->opt = *opt;
        b->has_opt = true;
    }
    cudaError_t e = cudaGetDevice(&b->dev);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "cudaGetDevice");
    }
    st = b->fp64 ? batch_build<double>(b, lines, jobs, n_jobs, opt, (char*)workspace, lay, t)
                 : batch_build<float>(b, lines, jobs, n_jobs, opt, (char*)workspace, lay, t);
    if (st) {
        delete b;
        return st;
    }
    *out = b;
    return KS_OK;
}

extern "C" ks_status ks_batch_run(ks_batch* b, ks_stats* stats, void* stream) {
    if (!b) return fail(KS_ERR_INVALID, "ks_batch_run: NULL plan");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = b->n_jobs;
    auto G = [&](int stage) { return bgrid(b->st[stage], n); };
    StageTimer tm;
    tm.start(s, stats != nullptr && b->profile);
    reset_batch_kernel<<<b->st[BS_RESET].grid, 256, 0, s>>>((const ResetJob*)b->st[BS_RESET].jobs, G(BS_RESET));
    KS_CUDA(cudaGetLastError());
    grid_params_batch_kernel<<<b->st[BS_GRID].grid, 32, 0, s>>>((const BinsJob*)b->st[BS_GRID].jobs, G(BS_GRID));
    KS_CUDA(cudaGetLastError());
    line_bins_batch_kernel<<<b->st[BS_BINS].grid, 256, 0, s>>>((const BinsJob*)b->st[BS_BINS].jobs, G(BS_BINS));
    KS_CUDA(cudaGetLastError());
    KS_CUDA(b->fp64 ? launch_prep_batch_f64((const PrepArgs*)b->st[BS_PREP].jobs, G(BS_PREP), b->st[BS_PREP].grid, s)
                    : launch_prep_batch_f32((const PrepArgs*)b->st[BS_PREP].jobs, G(BS_PREP), b->st[BS_PREP].grid, s));
    tm.mark();
    KS_CUDA(b->fp64 ? launch_continuum_batch_f64(b->st[BS_CONT].jobs, G(BS_CONT), b->st[BS_CONT].grid, s)
                    : launch_continuum_batch_f32(b->st[BS_CONT].jobs, G(BS_CONT), b->st[BS_CONT].grid, s));
    tm.mark();
    KS_CUDA(b->fp64 ? launch_pair_setup_batch_f64(b->st[BS_PAIR].jobs, G(BS_PAIR), b->st[BS_PAIR].grid, s)
                    : launch_pair_setup_batch_f32(b->st[BS_PAIR].jobs, G(BS_PAIR), b->st[BS_PAIR].grid, s));
    tm.mark();
    class_count_batch_kernel<<<b->st[BS_COUNT].grid, kPartThreads, 0, s>>>((const PartJob*)b->st[BS_COUNT].jobs,
                                                                           G(BS_COUNT));
    KS_CUDA(cudaGetLastError());
    class_scan_batch_kernel<<<b->st[BS_SCAN].grid, 32, 0, s>>>((const PartJob*)b->st[BS_SCAN].jobs, G(BS_SCAN));
    KS_CUDA(cudaGetLastError());
    class_scatter_batch_kernel<<<b->st[BS_SCATTER].grid, kPartThreads, 0, s>>>(
        (const PartJob*)b->st[BS_SCATTER].jobs, G(BS_SCATTER));
    KS_CUDA(cudaGetLastError());
    tile_ranges_batch_kernel<<<b->st[BS_RANGES].grid, 256, 0, s>>>((const PartJob*)b->st[BS_RANGES].jobs,
                                                                  G(BS_RANGES));
    KS_CUDA(cudaGetLastError());
    tm.mark();
    KS_CUDA(b->fp64 ? launch_accumulate_batch_f64(b->st[BS_ACC].jobs, G(BS_ACC), b->st[BS_ACC].grid, b->warps,
                                                  b->tile, s)
                    : launch_accumulate_batch_f32(b->st[BS_ACC].jobs, G(BS_ACC), b->st[BS_ACC].grid, b->warps,
                                                  b->tile, s));
    tm.mark();
    if (b->any_special) {
        const ks_status sst = b->fp64 ? batch_special_run<double>(b, s) : batch_special_run<float>(b, s);
        if (sst) return sst;
        tm.mark_special();
    }
    KS_CUDA(b->fp64 ? launch_transfer_batch_f64(b->st[BS_TRANS].jobs, G(BS_TRANS), G(BS_LIST), &g_tables.cj,
                                                b->st[BS_TRANS].grid, b->st[BS_LIST].grid, false, s)
                    : launch_transfer_batch_f32(b->st[BS_TRANS].jobs, G(BS_TRANS), G(BS_LIST), &g_tables.cj,
                                                b->st[BS_TRANS].grid, b->st[BS_LIST].grid, b->stream_pass, s));
    tm.mark();
    flag_sink_batch_kernel<<<b->st[BS_SINK].grid, 32, 0, s>>>((int* const*)b->st[BS_SINK].jobs, G(BS_SINK));
    KS_CUDA(cudaGetLastError());
    tm.finish(stats);
    if (stats) {
        int64_t vp = 0, ev = 0, maxj = 0, iters = 0;
        int flags = 0;
        ks_status first_err = KS_OK;
        for (int i = 0; i < n; i++) {
            ks_stats one;
            std::memset(&one, 0, sizeof(one));
            ks_status st = collect_stats(b->ws[i], b->n_wl[i], &one, s);
            vp += one.valid_pairs;
            ev += one.evaluations;
            maxj += one.maxj_wavelengths;
            iters += one.iterations;
            flags |= one.device_flags;
            if (st && !first_err) first_err = st;
        }
        stats->valid_pairs = vp;
        stats->evaluations = ev;
        stats->maxj_wavelengths = maxj;
        stats->iterations = iters;
        stats->device_flags = flags;
        stats->kernel_launches = b->stream_pass ? 15 : 14;
        return first_err;
    }
    return KS_OK;
}

extern "C" void ks_batch_free(ks_batch* b) { delete b; }

extern "C" ks_status ks_synthesize_batch(const ks_lines* lines, const ks_job* jobs, int32_t n_jobs,
                                         const ks_options* opt, void* workspace, size_t workspace_bytes,
                                         ks_stats* stats, void* stream) {
    ks_batch* b = nullptr;
    ks_status st = ks_batch_create(lines, jobs, n_jobs, opt, workspace, workspace_bytes, &b);
    if (st) return st;
    st = ks_batch_run(b, stats, stream);
    ks_batch_free(b);
    return st;
}
