// ks_internal.h -- argument records shared by the host API and the kernels.
#pragma once

#include <cstddef>
#include <cstdint>

namespace ks {

// Scalars derived from the wavelength grid (opacity.py:570-574,
// line_opacity.py:1035-1058, :235-239), computed on the device.
struct GridPar {
    double ratiolg, wbegin, resolu, first, last;
    int64_t ix_start, grid_offset;
};

// Per-depth state (populations.py:160-204, line_opacity.py:1009-1016,
// radiative.py:33, opacity.py:2408-2414).
struct DepthPar {
    double rho, xne, txnxn, hckt, hkt, hkt_asynth, temperature, rhox, fscat;
    float hckt_hi, hckt_lo, xne_f, txnxn_f, hkt_f, rhox_f, fscat_f, pad;
};

// Per (depth, ion, element) entry.
struct IonPar {
    double pop, dop, dop_transp, xnfdop, dvoigt;
    float xnfdop_f, dop_f, dvoigt_f, pop_over_rho_f, dopw_f;
    int n10dop;
    int ok;  // bit 0: TRANSP may use it (pop, DOPPLE, rho > 0); bit 1: wings (pop, DOPPLE > 0)
};

// Per-line single-precision copies for the mixed path.
struct LineF {
    float cgf, elo_hi, elo_lo, gr, gs, gw, gf, wl;
};

// Wing descriptor of one valid (line, depth) pair.
//   ctr_n10:     bits 0-3 centre-add code (0 none, else centre bin = wing_c +
//                code - 8), bits 8-31 N10DOP
//   maxstep_far: bits 0-30 MAXSTEP, bit 31 set when the far wing is used
template <typename R>
struct __align__(sizeof(R) == 4 ? 32 : 64) PairDesc {
    R kappa0, adamp, dvoigt, xfar, kapcen;
    int wing_c, maxstep_far, ctr_n10;
};

struct PrepArgs {
    int n_layers, n_ion, n_elem;
    const double *rhox, *temperature, *electron_density, *mass_density, *hckt;
    const double *xnf_h, *xnf_he1, *xnf_h2, *population, *doppler;
    double microturb_kms, rhoxj;
    const GridPar *gp;
    DepthPar *depth;
    IonPar *ion;
    // single-precision copies of the continuum coefficient tables (optional)
    int64_t n_coeff;
    const double *abs_coeff, *scat_coeff;
    float *abs_coeff_f, *scat_coeff_f;
};

struct ContArgs {
    int n_layers, n_edge, coeff_log10;
    int64_t n;
    const double *grid, *wledge, *half_edge, *delta_edge, *abs_coeff, *scat_coeff;
    const float *abs_coeff_f, *scat_coeff_f;  // FP32 path: the same tables in single precision
    float *freq_f;                            // optional out: c / lambda per grid point, FP32
};

struct LineBinArgs {
    int64_t n_lines, n_wl;
    const double *grid, *wavelength;
    double grid_origin;
    int32_t *center_out, *wing_out;
    // optional mixed-path per-line copies
    const double *cgf, *elo, *gr, *gs, *gw, *gf;
    LineF *linef;
    int *flags;
};

struct PairArgs {
    int64_t n_lines, n_wl, stride;
    int n_layers, n_ion, n_elem;
    double cutoff;
    float cutoff_f;  // the same in single precision (mixed path)
    const GridPar *gp;
    const double *wavelength, *gf, *cgf, *gamma_rad, *gamma_stark, *gamma_vdw, *elo_cm;
    const int32_t *element_idx, *ion_stage, *line_type;
    const uint8_t *process_mask, *asynth_mask;
    const int32_t *center_idx, *wing_idx;
    const LineF *linef;
    const DepthPar *depth;
    const IonPar *ion;
    const double *extab, *extabf;
    const float *extab_f, *extabf_f;
    const double *h0d, *h1d, *h2d;
    const float *h0f, *h1f, *h2f;
    // seam mode inputs (FP64, [n_lines, L])
    const double *transp_in;
    const uint8_t *valid_in;
    // optional TRANSP outputs ([n_lines, L])
    double *transp_out;
    uint8_t *valid_out;
    int *flags;
};

struct AccArgs {
    int64_t n_lines, n_wl, stride;
    int n_layers, tile_bins;
    int short_class;            // reach classes below it are accumulated one lane per pair
    int long_class;             // reach classes from it are dealt in batches of 8 pairs
    const double *grid;
    const int32_t *wing_idx;
    const int32_t *class_pos;   // per depth, per class: line positions, ascending
    const int64_t *class_off;   // [L][N_REACH_CLASSES + 1] absolute offsets into class_pos
    const int2 *tile_rng;       // [L][tiles][N_REACH_CLASSES] contributing range within each class
    const float *freq_f;        // c / lambda per grid point (FP32 path)
    const DepthPar *depth;
    const double *h0d, *h1d, *h2d;
    const float *h0f, *h1f, *h2f;
    unsigned long long *evals;
};

struct TransferArgs {
    int64_t n;
    int n_layers;
    int asynth_mode;   // line opacity given as ASYNTH (split by FSCAT here)
    int slinec_mode;   // source = SLINEC of the driver's frequency (FP64 path)
    int line_scat;     // some layer has FSCAT > 0 (RHOXJ > 0): line scattering present
    const double *grid;
    const DepthPar *depth;
    const double *xtau, *ch;
    const float *coefj32;
    const double *coefj64;  // non-null: FP64 path solves Gauss-Seidel in FP64 to 1e-13 (differentiable form)
    double *flux_total, *flux_cont;
    int32_t *iters;
};

// Adjoint of the transfer (differentiable form, FP64).
struct AdjArgs {
    int64_t n;
    int n_layers;
    const double *grid;
    const DepthPar *depth;
    const double *xtau, *ch, *coefj64;
    const double *cont_abs, *cont_scat, *asynth;  // [L, n]
    const double *g_flux;                         // [n] dLoss/dF_total
    double *g_asy;                                // [L, n] out: dLoss/dASYNTH * STIM
    unsigned long long *skipped;                  // columns given zero
};

// Adjoint of the accumulation, per (line, depth) pair.
struct LineAdjArgs {
    int64_t n_lines, n_wl, stride;
    int n_layers;
    const PairDesc<double>* desc;
    const uint8_t* cls;
    const double* g_asy;  // [L, n] dLoss/dASYNTH * STIM
    const double *h0, *h1, *h2;
    double* g_gf;  // [L, stride] out: sum G c
    double* g_a;   // [L, stride] out: sum G dc/da (wings, and the centre through KAPCEN)
};

// Per-line gradients from the per-pair sums.
struct LineGradArgs {
    int64_t n_lines, stride;
    int n_layers, n_ion, n_elem;
    const uint8_t* cls;
    const double *g_gf, *g_a;
    const DepthPar* depth;
    const IonPar* ion;
    const PairDesc<double>* desc;
    const int32_t *element_idx, *ion_stage;
    const double *gamma_rad, *gamma_stark, *gamma_vdw;
    double *d_loggf, *d_loggr, *d_loggs, *d_loggw;  // [n_lines] out
};

// Atmosphere terms of the adjoint: per depth, the per-pair sums of the line
// adjoint gathered by species (lines grouped by the caller, each group in
// row order, so every sum has a fixed order).
struct AtmGradArgs {
    int64_t stride;
    int n_layers, n_ion, n_elem, n_groups;
    const uint8_t* cls;
    const double *g_gf, *g_a;
    const IonPar* ion;
    const PairDesc<double>* desc;
    const int32_t *element_idx, *ion_stage;
    const double *gamma_stark, *gamma_vdw;
    const int32_t *order, *group_first, *group_species;
    double* part;             // scratch [L, n_groups, 3]: sum G c, sum G dc/da * gs/dop, * gw/dop
    double* d_ln_pop;         // [L, n_ion, n_elem] out (entries of the groups' species)
    double *d_ln_rho, *d_xne, *d_txnxn;  // [L] out
};

// Hydrogen line profile tables (HPROF4, synthe_py/physics/profiles/hydrogen.py),
// resident on the device.
struct HydTables {
    double propbm[7 * 5 * 15], c[5 * 7], d[5 * 7], pp[5], beta[15];
    double stalph[34], stwtal[34], stcomp[5 * 4], stcpwt[5 * 4];
    int istal[4], lnghal[4], lncomp[4];
    double cutoff_h2_plus[111], cutoff_h2[91], asum_lyman[100], asum[96], y1wtm[2 * 2], xknmtb[4 * 3];
    double ehyd[8], conth[15];
    double contx[26 * 17];  // continuum edges of the fort.19 merge limits, [NCON][NELIONX]
};

// One (hydrogen line, depth): gates, walk limits and the hydrogen depth state.
// The wavelength-independent part of one HPROF4 (n, m) profile at one layer:
// line frequency and wavelength, the widths and the Stark constants.
struct HprofConst {
    double freqnm, wavenm, dbeta, dop, hfwidth, hhw, hwres, hwvdw, hwrad, c1, c2, g1, gamma0;
    int mmn, nwid;
};

struct HydPar {
    double wl0, kappa0, wcon, wtail, wlm1, wlm2, wlp1, wlp2, redcut, bluecut;
    double pp, fo, y1b, y1s, t3nhe, t3nh2, c1d, c2d, gcon1, gcon2, xnfph0, xnfph1, dopph, xne, hkt;
    int ci, nl, nu, d, active;
    HprofConst k_line, k_red, k_blue;  // (NBLO, NBUP), (NBLO, max(NBUP-2, NBLO+1)), (NBLO, NBUP+2)
};

struct HydArgs {
    int n_h, n_layers, n_ion, n_elem;
    int64_t n_wl, n_lines;
    int* flags;                               // FLAG_HYDROGEN_LINE
    const int32_t *rows, *n_lower, *n_upper;  // per hydrogen line: catalog row, NBLO, NBUP
    const double *wavelength, *gf, *elo;      // catalog columns
    const int32_t* center;                    // centre bins of every catalog row
    const double* grid;
    const double *temperature, *xne, *rho, *hckt, *vturb, *xnf_he1, *xnf_h2, *population, *doppler;
    double cutoff, microturb_kms;
    const void *cabs, *cscat;                 // continuum cubes (the precision's type)
    const double *extab, *extabf;             // FASTEX tables
    const HydTables* tab;
    HydPar* par;                              // [n_h, L]
    int2* walk;                               // [n_h, L, 2] walk offsets [x, y), red then blue
};

// One (helium line, depth) of the helium wing pass: the gated kappa (3He:
// / 1.155), the Doppler width in nm (3He: x 1.155) and the damping.
struct HePar {
    double wl0, keff, dop, adamp;
    double wcon, wtail;  // fort.19 continuum-merge limits (nm; <= 0: none)
    int ci, d, active, pad;
};

struct HeArgs {
    int n_he, n_layers, n_ion, n_elem;
    int64_t n_wl, n_lines;
    int* flags;                               // FLAG_HELIUM_LINE
    const int32_t* rows;                      // per helium line: catalog row, in catalog order
    const int32_t *ncon, *nelionx;            // per helium line: fort.19 NCON and CONTX column (0: none)
    const HydTables* tab;                     // CONTX
    const double *wavelength, *gf, *elo, *gamma_rad, *gamma_stark, *gamma_vdw;  // catalog columns
    const int32_t *ion_stage, *line_type, *center;
    const double* grid;
    const double *temperature, *population, *doppler;
    const DepthPar* depth;                    // XNE, TXNXN, HCKT, RHO per layer
    double cutoff;
    const void *cabs, *cscat;                 // continuum cubes (the precision's type)
    const double *extab, *extabf;             // FASTEX tables
    const double *h0, *h1, *h2;               // Voigt tables (FP64)
    HePar* par;                               // [n_he, L]
    int2* walk;                               // [n_he, L, 2] walk offsets [x, y), red then blue
};

// One (fort.19 NORMAL line, depth): gates, KAPCEN and the wing of
// _accumulate_metal_profile_kernel (near profile to N10DOP or the first value
// below KAPMIN, else far wings X / n^2 to MAXSTEP).
// Autoionizing lines (kind 1) use kappa0, kapcen (= kappa0 at the centre
// bin cc), and tabstep/dvoigt/x_far as the line frequency, the width and
// ASHORE, adamp as BSHORE, with their walks in F19Args::walk.  Merged-
// continuum records (kind 2) use kappa0 (KAPPA), tabstep (the wavelength),
// cc / n10 / nstep / early as the first bin, the merge bin, the tail bin and
// the ramp's denominator, with their walk (absolute bins) in F19Args::walk.
struct F19Par {
    double kappa0, adamp, tabstep, dvoigt, x_far, kapcen;
    double wcon, wtail;  // NORMAL lines: continuum-merge limits (nm; <= 0: none)
    int ci, cc, n10, nstep, early, active, kc_ok, d, kind;
    int bw_con, bw_tail;  // grid points at or below WCON (last index, -1: none) and below WTAIL (count)
};

struct F19Args {
    int n_f19, n_layers, n_ion, n_elem;
    int64_t n_wl, n_lines;
    int* flags;                               // FLAG_F19_LINE
    const int32_t* rows;                      // per line: catalog row, in catalog order
    const int32_t* kind;                      // per line: 0 NORMAL, 1 autoionizing, 2 merged continuum
    const int32_t *nlast, *nelion;            // per line (merged continuum): NLAST, the ion index
    const int32_t *ncon, *nelionx;            // per line (NORMAL): NCON and the CONTX column (0: none)
    const HydTables* tab;                     // CONTX
    const double *cgf, *gamma_rad, *gamma_stark, *gamma_vdw;  // per line: fort.19 record values
                                              // (single-precision values held in double; the
                                              // autoionizing lines' gf in cgf)
    const double *wavelength, *elo;           // catalog columns
    const int32_t *element_idx, *ion_stage, *center;
    const double* grid;
    const double *temperature, *vturb, *population;
    const DepthPar* depth;
    double cutoff, microturb_kms;
    const void *cabs, *cscat;
    const double *extab, *extabf, *h0, *h1, *h2;
    F19Par* par;                              // [n_f19, L]
    int2* walk;                               // [n_f19, L, 2] autoionizing walks [x, y), red, blue
};

// ---- batched launches -------------------------------------------------------
//
// A batch runs every stage once over all its jobs: the launch walks a job
// table, job j owning virtual blocks [first[j], first[j + 1]) laid out on its
// own grid dims[j] (x, y) -- the grid a single synthesis of that job would
// launch.  Blocks take virtual blocks v = blockIdx.x + k gridDim.x (a static,
// atomic-free schedule, so a persistent grid of a few blocks per SM covers any
// batch) and run the same kernel body as a single synthesis.
struct BatchGrid {
    const int64_t* first;  // [n_jobs + 1] prefix of the jobs' block counts
    const int* dims;       // [2 n_jobs] grid x, y per job
    int n_jobs;
};

template <typename R>
struct ContJob {
    ContArgs a;
    R *cont_abs, *cont_scat;
};

template <typename R>
struct PairJob {
    PairArgs a;
    const R *kap_a, *kap_b;
    PairDesc<R>* desc;
    uint8_t* cls;
};

template <typename R>
struct AccJob {
    AccArgs a;
    const PairDesc<R>* desc;
    R* out;
};

template <typename R>
struct TransferJob {
    TransferArgs a;
    const R *cab, *csc, *lop;
    int32_t* list;               // FP32 streaming pass: columns left to the per-column code
    unsigned long long* count;   // its length
};

// The per-job arguments of the precision-independent stages.
struct BinsJob {
    const double* grid;
    int64_t n_wl;
    double grid_origin;
    GridPar* gp;
    int64_t n_lines;
    const double *wavelength, *cgf, *elo, *gr, *gs, *gw, *gf;
    int32_t *center, *wing;
    LineF* linef;  // FP32 path
    int* flags;
};

struct PartJob {
    const uint8_t* cls;
    int64_t stride, n_wl;
    int nchunks, ntiles, tile_bins;
    int32_t* counts;
    int64_t *chunk_base, *class_off;
    int32_t* class_pos;
    const int32_t* wing;
    int2* tile_rng;
    unsigned long long* counters;
};

struct ResetJob {
    int* flags;
    unsigned long long* counters;  // [4]
    uint8_t* cls;                  // padding slots [n_lines, stride) of every depth set to 0xff
    int64_t n_lines, stride;
    int n_layers, ntiles;
    int64_t* class_off;            // jobs without lines: class lists and tile ranges empty
    int2* tile_rng;
};

#ifdef __CUDACC__
__device__ __forceinline__ int batch_locate(const BatchGrid& g, int64_t v, int& x, int& y, int& gx, int& gy) {
    int lo = 0, hi = g.n_jobs - 1;  // the last job whose first block is <= v
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g.first[mid] <= v) lo = mid; else hi = mid - 1;
    }
    const int64_t local = v - g.first[lo];
    gx = g.dims[2 * lo];
    gy = g.dims[2 * lo + 1];
    x = (int)(local % gx);
    y = (int)(local / gx);
    return lo;
}
#endif

}  // namespace ks
