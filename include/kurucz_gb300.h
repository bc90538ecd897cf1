/*
 * kurucz_gb300.h -- C ABI of the GB300 line-opacity and transfer library.
 *
 * The reference (synthe_py) is Python; its seams for this path are Python
 * functions, listed beside each entry point that replaces one.  All entry
 * points take plain pointers and sizes, return a ks_status and run on the
 * CUDA stream they are given.  The fused entry points (ks_synthesize,
 * ks_asynth) work in caller-provided workspace; the smaller seam helpers
 * (ks_line_bins, ks_transp, ks_formal_solution) take stream-ordered
 * temporaries (cudaMallocAsync) for a few bytes per line or wavelength.
 * Device pointers are marked "device"; the library never frees caller
 * memory.  ks_init_tables must be called once per process first; the first
 * compute call on each device copies the tables to it synchronously, so that
 * call must come before any CUDA-graph capture on that device.
 *
 * Errors: every call returns KS_OK or an error code; ks_last_error() returns
 * the message of the last failure on the calling thread.  Numerical
 * problems inside the data (NaN/Inf opacities) are masked as the reference
 * masks them, not raised.  Internal limits that a kernel meets (a packed
 * descriptor field overflowing, wing bins out of order) raise a device flag:
 * a call given a ks_stats pointer returns KS_ERR_DEVICE for its own flags;
 * every call also ORs its flags into a per-device sticky word, which
 * ks_check_flags reads and clears, so calls without stats (and CUDA-graph
 * replays of them) lose no error.
 *
 * Threading: calls are thread-safe; each call only touches the buffers and
 * stream it is given.
 */
#ifndef KURUCZ_GB300_H
#define KURUCZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t ks_status;
enum {
    KS_OK = 0,
    KS_ERR_INVALID = 1,     /* bad argument (null pointer, size out of range) */
    KS_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    KS_ERR_NOMEM = 3,       /* workspace too small / allocation failed */
    KS_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
    KS_ERR_IO = 5,          /* file could not be read */
    KS_ERR_UNSUPPORTED = 6, /* input outside what the kernels handle */
    KS_ERR_DEVICE = 7       /* a kernel flagged an internal limit */
};

/* Arithmetic of the fused path.
 * KS_PREC_MIXED: FP32 Voigt and profile evaluation with Kahan-compensated
 *   tile sums, FP32 continuum and Planck, compensated FP32 tau integration,
 *   FP32 Gauss-Seidel sweeps (the reference's own sweep precision).
 * KS_PREC_FP64: every step in FP64 (the all-FP64 GPU path).              */
typedef enum { KS_PREC_MIXED = 0, KS_PREC_FP64 = 1 } ks_precision;

/* One model atmosphere, device pointers (synthe_py/io/atmosphere.py:17
 * AtmosphereModel fields; sizes as in the converted .npz). */
typedef struct {
    int32_t n_layers;               /* L */
    const double *rhox;             /* [L] column mass ("depth") */
    const double *temperature;      /* [L] */
    const double *electron_density; /* [L] */
    const double *mass_density;     /* [L] */
    const double *hckt;             /* [L] hc/kT per cm^-1 */
    const double *xnf_h;            /* [L] (TXNXN inputs, populations.py:204) */
    const double *xnf_he1;          /* [L] */
    const double *xnf_h2;           /* [L] */
    const double *population;       /* [L, n_ion, n_elem] population_per_ion */
    const double *doppler;          /* [L, n_ion, n_elem] doppler_per_ion */
    int32_t n_ion;                  /* 6 */
    int32_t n_elem;                 /* 139 */
    const double *wledge;           /* [n_edge] continuum edges (nm) */
    const double *half_edge;        /* [n_edge-1] */
    const double *delta_edge;       /* [n_edge-1] */
    int32_t n_edge;
    const double *cont_abs_coeff;   /* [L, n_edge-1, 3] log10 coefficients */
    const double *cont_scat_coeff;  /* [L, n_edge-1, 3] */
    int32_t coeff_log10;            /* 1: coefficients are log10 (always in practice) */
    const double *turbulent_velocity; /* [L] cm/s (the H Doppler width of hydrogen lines; may be
                                         NULL when the lines hold no hydrogen line) */
} ks_atmos;

/* The log-lambda grid, device pointer. */
typedef struct {
    int64_t n;                      /* number of grid points */
    const double *wavelength;       /* [n] nm, built by ks_wavelength_grid */
    double grid_origin;             /* first point of the unsubsampled grid */
} ks_grid;

/* Line catalog (LineCatalog, synthe_py/io/lines/atomic.py:237), device
 * pointers, n_lines entries each, in catalog order. */
typedef struct {
    int64_t n_lines;
    const double *wavelength;       /* nm (vacuum, from the level energies) */
    const double *gf;               /* 10**log_gf */
    const double *cgf;              /* 0.026538/1.77245 * gf / freq */
    const double *gamma_rad;        /* normalised by 4 pi nu (atomic.py:501-504) */
    const double *gamma_stark;
    const double *gamma_vdw;
    const double *elo_cm;           /* lower-level energy, cm^-1 */
    const int32_t *element_idx;     /* Z-1, or -1 when unknown */
    const int32_t *ion_stage;       /* 1 = neutral */
    const int32_t *line_type;       /* 0 plain; see atomic.py:566-582 */
    const uint8_t *process_mask;    /* 1 = TRANSP processes it (line_opacity.py:740-765) */
    const uint8_t *asynth_mask;     /* 1 = centre added to ASYNTH (line_opacity.py:1094) */
    int32_t sorted_by_wavelength;   /* 1 if wavelength is non-decreasing */
    /* hydrogen lines (line types -1/-2 of neutral H), added with the HPROF4
     * profile (synthe_py/engine/opacity.py:1706): their rows, in catalog
     * order, and their principal quantum numbers (device; n_hydrogen = 0 for
     * none; at most 65536: beyond 256 lines of a
     * class ks_synthesize allocates their scratch on its stream, the
     * no-allocation entry point rejects them) */
    int32_t n_hydrogen;
    const int32_t *hydrogen_rows;
    const int32_t *hydrogen_n_lower;
    const int32_t *hydrogen_n_upper;
    /* helium lines (line types -3/-4/-6: He I, 3He I, He II; their fort.19
     * continuum-merge limits in helium_ncon / helium_nelionx): the helium wing pass (synthe_py/engine/opacity.py:
     * 2515-3590, Voigt wings of _apply_fort19_profile :996-1061), added to the
     * line opacity as AHE x STIM (:3650-3660); their rows in catalog order
     * (device; n_helium = 0 for none; at most 65536: beyond 256 lines of a
     * class ks_synthesize allocates their scratch on its stream, the
     * no-allocation entry point rejects them) */
    int32_t n_helium;
    const int32_t *helium_rows;
    /* fort.19 lines: NORMAL ones (NBLO/NBUP set, line type 0; their continuum-
     * merge limits in f19_ncon / f19_nelionx): the profiles of _add_fort19_asynth (synthe_py/engine/
     * opacity.py:1335-1488) added to ASYNTH; their rows in catalog order and
     * the fort.19 record's CGF and damping constants, rounded to single
     * precision as the record stores them (io/lines/fort19.py:368-402);
     * device; n_f19 = 0 for none; at most 65536, see above */
    int32_t n_f19;
    const int32_t *f19_rows;
    const double *f19_cgf, *f19_gamma_rad, *f19_gamma_stark, *f19_gamma_vdw;
    /* per fort.19 line: 0 NORMAL, 1 autoionizing, 2 merged continuum (the AUT tag: the profile
     * of _accumulate_autoionizing_profile, opacity.py:901-963, with KAPPA0 =
     * BSHORE GF XNFPEL BOLT; f19_cgf then holds gf and f19_gamma_* the
     * record's unnormalised GAMMAR, ASHORE, BSHORE, fort19.py:352-373) */
    const int32_t *f19_kind;
    /* per fort.19 line, merged-continuum records (kind 2: LABELP CONTINUU,
     * NLAST > 3; _accumulate_merged_continuum, opacity.py:863-898, f19_cgf
     * holding gf (2 XJ + 1)): NLAST and the record's ion index NELION
     * (fort19.py:323-328); unread for the other kinds */
    const int32_t *f19_nlast, *f19_nelion;
    /* fort.19 continuum-merge limits (opacity.py:657-702): per helium line
     * and per fort.19 line, NCON (ISO2 when ISO1 is 0) and the CONTX column
     * NELIONX of the record's species (fort19.py:330-338); 0 for none */
    const int32_t *helium_ncon, *helium_nelionx;
    const int32_t *f19_ncon, *f19_nelionx;
} ks_lines;

typedef struct {
    double cutoff;          /* KAPMIN = continuum * cutoff (default 1e-3) */
    double microturb_kms;   /* synthesis microturbulence (default 0) */
    double rhoxj;           /* scattering scale height (0 = LTE, fscat = 0) */
    int32_t precision;      /* ks_precision */
    int32_t tile_bins;      /* accumulation tile width in bins, a multiple of 32; 0 = 1024 */
    int32_t warps_per_tile; /* warps per accumulation CTA, 1..16; 0 = 8 */
    int32_t profile;        /* 1: time each stage with CUDA events into ks_stats.stage_ms
                               (only when a ks_stats pointer is given) */
    int32_t short_class;    /* reach classes 0..short_class-1 (wing reach <= 2^(short_class-1)
                               bins) are accumulated one lane per pair; 0 = default (7),
                               negative = none */
    int32_t transfer_path;  /* single precision, fused: 0 = streaming pass (columns it cannot
                               take go to the per-column kernel), 1 = per-column kernel only */
    int32_t long_class;     /* reach classes >= long_class are dealt to the accumulation warps in
                               batches of 8 pairs instead of 32; 0 = default (8) */
    int32_t exact_sweeps;   /* FP64 precision only: 1 = solve the JOSH Gauss-Seidel system in FP64
                               to 1e-13 instead of the reference's FP32 sweep at 1e-5 (the
                               forward of the differentiable form, smooth in the inputs) */
} ks_options;

/* Counters of one synthesis (filled when a pointer is given). */
typedef struct {
    int64_t valid_pairs;        /* (line, depth) pairs that passed both KAPMIN gates */
    int64_t evaluations;        /* line.depth.lambda contributions accumulated */
    int64_t maxj_wavelengths;   /* total-flux solves that took the MAXJ=1 path */
    int64_t iterations;         /* Gauss-Seidel sweeps summed over all solves */
    int32_t device_flags;       /* nonzero when a kernel hit an internal limit */
    int32_t kernel_launches;    /* kernels this call launched */
    float stage_ms[8];          /* with ks_options.profile: bins+prep, continuum, pair setup,
                                   partition, accumulation, transfer, special lines (hydrogen,
                                   helium, fort.19; 0 without), total */
} ks_stats;

/* ---- library ---------------------------------------------------------- */

/* Version of this ABI. */
ks_status ks_version(int32_t *major, int32_t *minor);

/* Message of the last failed call on this thread ("" if none). */
const char *ks_last_error(void);

/* Synchronises `stream` (the current device's stream), then takes and clears
 * the device's sticky flag word: the OR of the internal-limit flags raised by
 * every call on this device since the last ks_check_flags.  Returns
 * KS_ERR_DEVICE (message names the limit) when it was nonzero; *flags_out
 * (may be NULL) receives the word.  Call it after a batch of asynchronous
 * calls or graph replays.  No reference counterpart: the reference raises
 * Python exceptions synchronously. */
ks_status ks_check_flags(void *stream, int32_t *flags_out);

/* Builds the constant tables from the SYNTHE source tables (host memory):
 * the 81-point H1 Voigt table tabvi/tabh1 (synthe_py/physics/tables.py:249,
 * expanded to 2001 points as VoigtTables.build does, :224), and the JOSH
 * grid xtau[51], surface weights ch[51] and operator coefj[51*51]
 * (synthe_py/physics/josh_tables.py:6,120,177).  Once per process. */
ks_status ks_init_tables(const double *tabvi, const double *tabh1, int32_t n_tab,
                         const double *xtau, const double *ch, const double *coefj);

/* The hydrogen line profile tables (host memory, the package's
 * data/hydrogen_tables.npz): the Stark-profile corrections PROPBM [7*5*15],
 * C and D [5*7], PP [5], BETA [15], the fine-structure components STALPH and
 * STWTAL [34], STCOMP and STCPWT [5*4], ISTAL, LNGHAL and LNCOMP [4], the
 * Lyman cutoff tables [111] and [91], ASUMLYMAN [100], ASUM [96], Y1WTM
 * [2*2] and XKNMTB [4*3] (synthe_py/physics/profiles/hydrogen.py:23-1405),
 * the level energies EHYD [8] (synthe_py/engine/opacity.py:49) and the
 * continuum edges CONTH [15] (synthe_py/physics/tables.py:152), all
 * row-major.  Once per process, before a synthesis with hydrogen lines. */
typedef struct {
    const double *propbm, *c, *d, *pp, *beta, *stalph, *stwtal, *stcomp, *stcpwt;
    const int32_t *istal, *lnghal, *lncomp;
    const double *cutoff_h2_plus, *cutoff_h2, *asum_lyman, *asum, *y1wtm, *xknmtb, *ehyd, *conth;
    const double *contx; /* [26*17] continuum edges of the fort.19 merge limits (tables.py:173) */
} ks_hydrogen_tables;
ks_status ks_init_hydrogen_tables(const ks_hydrogen_tables *tables);

/* Host copies of the derived tables (2001-point H0/H1/H2, 1001-point
 * EXTAB/EXTABF of tables.py:14-42), for verification.  Any pointer may be
 * NULL. */
ks_status ks_get_tables(double *h0, double *h1, double *h2, double *extab, double *extabf);

/* ---- wavelength grid and bins ----------------------------------------- */

/* Replaces synthe_py/engine/opacity.py:526 _build_wavelength_grid.
 * Host function.  Returns the number of points; writes at most `cap`
 * points to `out` (out may be NULL to query the size). */
int64_t ks_wavelength_grid(double start, double end, double resolution,
                           double *out, int64_t cap);

/* Replaces synthe_py/engine/opacity.py:550 _nearest_grid_indices (centre
 * bins, -1 / n outside the grid) and line_opacity.py:1030-1059 (wing bins
 * relative to grid_origin).  wavelength, center_out, wing_out: device. */
ks_status ks_line_bins(const ks_grid *grid, const double *wavelength, int64_t n_lines,
                       int32_t *center_out, int32_t *wing_out, void *stream);

/* ---- continuum --------------------------------------------------------- */

/* Replaces synthe_py/physics/continuum.py:73 build_depth_continuum.
 * Writes ACONT and SIGMAC, [L, n] row-major, as double (KS_PREC_FP64) or
 * float (KS_PREC_MIXED).  Outputs: device. */
ks_status ks_continuum(const ks_atmos *atm, const ks_grid *grid, int32_t precision,
                       void *cont_abs, void *cont_scat, void *stream);

/* ---- TRANSP ------------------------------------------------------------ */

/* Replaces synthe_py/physics/line_opacity.py:620 compute_transp (with the
 * Boltzmann factors of physics/populations.py:131).  FP64.
 *   cont_kapmin: [L, n] ACONT+SIGMAC (device, double)
 *   transp_out:  [n_lines, L] line-centre opacity (device, double)
 *   valid_out:   [n_lines, L] 1 where both KAPMIN gates pass (device)
 *   center_out:  [n_lines] centre bins (device, may be NULL)           */
ks_status ks_transp(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                    const ks_options *opt, const double *cont_kapmin,
                    double *transp_out, uint8_t *valid_out, int32_t *center_out,
                    void *stream);

/* ---- ASYNTH ------------------------------------------------------------ */

/* Scratch bytes ks_asynth / ks_synthesize need for these sizes. */
ks_status ks_workspace_size(int64_t n_lines, int32_t n_layers, int64_t n_wavelengths,
                            const ks_options *opt, size_t *bytes);

/* Replaces synthe_py/physics/line_opacity.py:946 compute_asynth_from_transp
 * (plain lines; stimulated emission applied).  FP64 in, FP64 out.
 *   transp, valid: as produced by ks_transp (device)
 *   asynth_out:    [L, n] (device, double)
 *   workspace:     ks_workspace_size bytes of device memory            */
ks_status ks_asynth(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                    const ks_options *opt, const double *transp, const uint8_t *valid,
                    const double *cont_kapmin, void *workspace, size_t workspace_bytes,
                    double *asynth_out, ks_stats *stats, void *stream);

/* ---- formal solution ---------------------------------------------------- */

/* Replaces synthe_py/engine/radiative.py:282 solve_lte_spectrum (JOSH
 * surface flux, physics/josh_solver.py:367).  Field arrays [L, n] in the
 * precision's type (double for KS_PREC_FP64, float for KS_PREC_MIXED);
 * line_source may be NULL (Planck).  Fluxes are F_nu (device, double). */
ks_status ks_formal_solution(const ks_atmos *atm, const ks_grid *grid, int32_t precision,
                             const void *cont_abs, const void *cont_scat,
                             const void *line_opacity, const void *line_scattering,
                             const void *line_source, double *flux_total,
                             double *flux_cont, ks_stats *stats, void *stream);

/* ---- fused synthesis ------------------------------------------------------ */

/* The hot section of synthe_py/engine/opacity.py:2084 run_synthesis, fused:
 * continuum -> TRANSP -> ASYNTH -> line source -> JOSH, for one atmosphere.
 * Fluxes are F_nu at the surface (device, double, [n]); the caller converts
 * to F_lambda as opacity.py:3855-3861 does.  asynth_out (optional, device,
 * [L, n], float for MIXED / double for FP64) receives the line opacity. */
ks_status ks_synthesize(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                        const ks_options *opt, void *workspace, size_t workspace_bytes,
                        double *flux_total, double *flux_cont, void *asynth_out,
                        ks_stats *stats, void *stream);

/* ks_synthesize in two halves, for runs sharded over GPUs by layer: each
 * stage before the transfer works layer by layer (the same split as the
 * reference's depth loops in line_opacity.py:56-184 and :946-1340), and the
 * transfer wavelength by wavelength (radiative.py:282-494).
 *
 * ks_opacity: continuum -> TRANSP -> ASYNTH on the layers of `atm` (any
 * contiguous block of an atmosphere's layers), writing the ASYNTH and
 * continuum (absorption, scattering) cubes, device, [n_layers, n], float for
 * MIXED / double for FP64.  Workspace as ks_synthesize.  No reference
 * counterpart: the reference runs the whole path in one process. */
ks_status ks_opacity(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                     const ks_options *opt, void *workspace, size_t workspace_bytes,
                     void *asynth_out, void *cont_abs_out, void *cont_scat_out,
                     ks_stats *stats, void *stream);

/* ks_transfer_opacity: the transfer of ks_synthesize (line source, FSCAT
 * split, two JOSH solves) on cubes [n_layers, n] holding every layer of
 * `atm` for the wavelengths of `grid` (a slice of the full grid is allowed):
 * a spectrum stitched from slices is identical to the unsharded one.
 * Allocates its small scratch on the stream.  Replaces the tail of
 * opacity.py:2084 run_synthesis from :3788 (solve_lte_spectrum). */
ks_status ks_transfer_opacity(const ks_atmos *atm, const ks_grid *grid, const ks_options *opt,
                              const void *cont_abs, const void *cont_scat, const void *asynth,
                              double *flux_total, double *flux_cont, ks_stats *stats,
                              void *stream);

/* The differentiable form: the FP64 fused synthesis (precision must be
 * KS_PREC_FP64; the JOSH system is solved in FP64 to 1e-13 so the fluxes are
 * smooth in the inputs), then hand-written adjoints of the transfer and of
 * the line accumulation.  g_flux_total (device, double, [n]) is
 * dLoss/dF_total of the caller's loss (F_nu; the continuum flux does not
 * depend on the lines); the outputs are dLoss/dlog10(gf) and
 * dLoss/dlog10(gamma_rad, gamma_stark, gamma_vdw) per line (device, double,
 * [n_lines], sorted order).  The TRANSP gates and the wing reach are held
 * fixed (they are step functions of the parameters).  Wavelengths that take
 * the MAXJ = 1 branch contribute no gradient; their count is returned in
 * stats->maxj_wavelengths.  Not covered: line scattering (rhoxj > 0),
 * microturbulence.  No counterpart in the reference (it has no gradients). */
ks_status ks_synthesize_adjoint(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                                const ks_options *opt, void *workspace, size_t workspace_bytes,
                                const double *g_flux_total, double *flux_total, double *flux_cont,
                                double *d_log_gf, double *d_log_gamma_rad, double *d_log_gamma_stark,
                                double *d_log_gamma_vdw, ks_stats *stats, void *stream);

/* The adjoint of ks_synthesize_adjoint, plus the atmosphere terms that carry
 * the gradient on to the populations (and through ks_populations_tangent to
 * the abundances).  Lines are grouped by species by the caller: line_order
 * holds the rows of `lines` grouped by (element_idx, ion_stage), each group
 * in ascending row order, group g = line_order[group_first[g] ..
 * group_first[g+1]) with species (ion_stage - 1) * n_elem + element_idx in
 * group_species[g] (device arrays), so every sum has a fixed order.  Out
 * (device, double): dLoss/d ln population_per_ion [L, n_ion, n_elem] (zero
 * for species without lines), dLoss/d ln mass_density [L] (through
 * XNFDOP = POP / (RHO DOPPLE)), dLoss/dXNE and dLoss/dTXNXN [L] (through the
 * Stark and van der Waals damping).  The continuum opacity tables, the TRANSP
 * gates and the wing reach are held fixed.  No counterpart in the
 * reference. */
typedef struct {
    const int32_t *line_order;
    const int32_t *group_first;
    const int32_t *group_species;
    int32_t n_groups;
    double *d_ln_population;
    double *d_ln_mass_density;
    double *d_electron_density;
    double *d_txnxn;
} ks_atm_grad;

ks_status ks_synthesize_adjoint_atmos(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                                      const ks_options *opt, void *workspace, size_t workspace_bytes,
                                      const double *g_flux_total, double *flux_total, double *flux_cont,
                                      double *d_log_gf, double *d_log_gamma_rad, double *d_log_gamma_stark,
                                      double *d_log_gamma_vdw, const ks_atm_grad *atm_grad, ks_stats *stats,
                                      void *stream);

/* The fused synthesis of ks_synthesize for callers that cannot allocate
 * device memory: a plug-in running inside a host application that owns all
 * device memory, or a runtime reached through an FFI with no CUDA allocator,
 * cannot hand over a workspace.  This entry point allocates nothing (no
 * cudaMalloc, no cudaFree, no allocating library routine): its scratch is a
 * fixed 64 MiB array inside the library.  A call is rejected with
 * KS_ERR_NOMEM when the scratch it needs exceeds 64 MiB; that need is never
 * more than ks_workspace_size for the same sizes (which assumes the full
 * 6 x 139 population table, room for the ASYNTH cube even when asynth_out is
 * given, and 256 bytes of slack), so a problem whose ks_workspace_size is at
 * most 64 MiB always runs (on a 72-layer atmosphere and a 6,000-point grid
 * about 20,000 lines fit in KS_PREC_MIXED, 8,000 in KS_PREC_FP64).  The
 * caller still passes
 * inputs and outputs.  All calls on a device share the array: calls that
 * overlap on the GPU race and must be serialised.  The first call on each
 * device looks up the array's device address (and, like every entry point,
 * copies the constant tables), so make it before any stream capture on that
 * device.  No stats are returned.  This entry point has no counterpart in the
 * reference. */
ks_status ks_synthesize_noalloc(const ks_lines *lines, const ks_atmos *atm, const ks_grid *grid,
                                const ks_options *opt, double *flux_total, double *flux_cont,
                                void *asynth_out, void *stream);

/* ---- batched synthesis -------------------------------------------------------- */

/* One job of a batch: an atmosphere, its own wavelength grid (window), the
 * rows of the batch's shared line list that lie in the window, and where its
 * fluxes go.  atm and grid are host pointers to records whose arrays are on
 * the device; they are read when the plan is made. */
typedef struct {
    const ks_atmos *atm;
    const ks_grid *grid;
    int64_t line_first;     /* first row of the shared (wavelength-sorted) list */
    int64_t line_count;     /* rows in the job's window */
    double *flux_total;     /* device, [grid->n], F_nu at the surface */
    double *flux_cont;      /* device, [grid->n] */
} ks_job;

/* A plan for running many syntheses over one shared line list as one batch:
 * every stage of ks_synthesize (bins, per-depth state, continuum, TRANSP and
 * wing setup, reach-class partition, accumulation, transfer) is one
 * persistent launch over all jobs -- blocks walk a device table of
 * (job, block) work items with a precomputed per-job prefix, no atomics --
 * 15 launches per batch whatever the number of jobs.  Each job gets the
 * results a ks_synthesize call with the same options gives (bit for bit).
 * Special lines (hydrogen, helium, fort.19) of the shared list are taken:
 * their rows must ascend (catalog order), a job's are those in its slice
 * (at most 256 of each class per job, else KS_ERR_UNSUPPORTED), and each
 * job with some runs the special-line kernels of ks_synthesize between the
 * accumulation and the transfer launch (a few launches per such job).
 * The options (precision, tiling, cutoff, microturbulence, RHOXJ) are shared
 * by all jobs.  No reference counterpart: the reference synthesises one
 * atmosphere per run (synthe_py/engine/opacity.py:2084); this replaces a
 * loop of run_synthesis calls.
 *
 * ks_batch_workspace_size: device bytes the plan needs (its job tables plus
 * one ks_synthesize workspace per job).
 * ks_batch_create: lays the jobs out in `workspace` (device, 256-byte
 * aligned, owned by the caller and kept alive with the plan) and copies the
 * job tables to it synchronously -- call it before any stream capture.
 * ks_batch_run: enqueues the batch on `stream` (launches only, so it can be
 * recorded in a CUDA graph and replayed); with stats it synchronises and
 * returns the counters summed over the jobs (profile option: stage times).
 * ks_batch_free: releases the host plan (not the workspace).
 * ks_synthesize_batch: create, run and free in one call. */
typedef struct ks_batch ks_batch;
ks_status ks_batch_workspace_size(const ks_lines *lines, const ks_job *jobs, int32_t n_jobs,
                                  const ks_options *opt, size_t *bytes);
ks_status ks_batch_create(const ks_lines *lines, const ks_job *jobs, int32_t n_jobs,
                          const ks_options *opt, void *workspace, size_t workspace_bytes,
                          ks_batch **out);
ks_status ks_batch_run(ks_batch *plan, ks_stats *stats, void *stream);
void ks_batch_free(ks_batch *plan);
ks_status ks_synthesize_batch(const ks_lines *lines, const ks_job *jobs, int32_t n_jobs,
                              const ks_options *opt, void *workspace, size_t workspace_bytes,
                              ks_stats *stats, void *stream);

/* ---- populations (FP64) ------------------------------------------------------ */

/* Data tables of the population stage, host memory (the package's
 * data/pops_tables.npz).  Once per process, before ks_populations.
 *   potion [999], nnn [6 * 374] (row-major), atmass [99]:
 *       synthe_py/data/fortran_data.npz as pops_exact.py:748 loads it;
 *   pftab [7 * 56 * 10 * 9], pf_potlo / pf_potlolog [7]: the PFIRON table
 *       (synthe_py/data/pfiron_data.npz, pops_exact.py:831);
 *   level_e / level_g, level_n [14]: the explicit level sums of PFSAHA,
 *       concatenated in the order H I, He I, He II, C I, C II, O I, Mg I,
 *       Mg II, Al I, Si I, Si II, Na I, B I, K I (pops_exact.py:520-741);
 *   pfg_first [n_pfg_first], pfg_second [n_pfg_second]: PFGROUND labels per
 *       NELION; per label row r < n_pfg_label: pfg_label[r], the constant
 *       pfg_g0[r] and the terms pfg_off[r] .. pfg_off[r+1]-1 of
 *       (pfg_g, pfg_e) = weight * exp(-hc/kT * energy)
 *       (synthe_py/tools/_pfground_table.py);
 *   mol_code [n_mol], mol_equil [7 * n_mol] (row-major (7, n_mol)): the
 *       molecular equilibrium table lines/molecules.dat as READMOL reads it
 *       (synthe_py/tools/readmol_exact.py:20). */
typedef struct {
    const double *potion;
    const int32_t *nnn;
    const double *atmass;
    const double *pftab;
    const double *pf_potlo;
    const double *pf_potlolog;
    const double *level_e;
    const double *level_g;
    const int32_t *level_n;
    const int32_t *pfg_first;
    int32_t n_pfg_first;
    const int32_t *pfg_second;
    int32_t n_pfg_second;
    const int32_t *pfg_label;
    const double *pfg_g0;
    const int32_t *pfg_off;
    int32_t n_pfg_label;
    const double *pfg_g;
    const double *pfg_e;
    const double *mol_code;
    const double *mol_equil;
    int32_t n_mol;
} ks_pops_tables;

ks_status ks_init_pops_tables(const ks_pops_tables *tables);

/* The molecular system built from the table (READMOL): number of molecules,
 * of equations, the element of each equation (0 = total particles, 100 =
 * electrons) and, per element Z-1, 1 when POPS takes its populations from
 * the molecular equilibrium.  Host; any pointer may be NULL (arrays of 32
 * and 99 entries). */
ks_status ks_pops_system(int32_t *n_molecules, int32_t *n_equations, int32_t *equation_element,
                         int32_t *element_molecular);

/* One model atmosphere for ks_populations: the columns of an ATLAS .atm model,
 * layers in order of increasing column mass (device pointers). */
typedef struct {
    int32_t n_layers;               /* L, 1..4096 */
    const double *temperature;      /* [L] K */
    const double *gas_pressure;     /* [L] dyn cm^-2 */
    const double *vturb;            /* [L] cm s^-1 */
    const double *xabund;           /* [99] abundances as number fractions (the converter's
                                       XABUND, convert_atm_to_npz.py:1775-1800) */
    /* outputs (device) -- the fields of the converted atmosphere the synthesis reads */
    double *electron_density;       /* [L] XNE after the molecular equilibrium */
    double *mass_density;           /* [L] XNATOM * WTMOLE * 1.660e-24 */
    double *hckt;                   /* [L] hc/kT */
    double *xnf_h;                  /* [L] neutral H number density */
    double *xnf_he1;                /* [L] neutral He number density */
    double *xnf_h2;                 /* [L] H2 number density */
    double *population;             /* [L, 6, 139] population_per_ion (number / partition
                                       function, per element Z-1 and ion) */
    double *doppler;                /* [L, 6, 139] doppler_per_ion (Doppler width / c) */
    double *xnatom;                 /* [L] XNATOM (may be NULL) */
    int32_t *nmolec_iterations;     /* [L] Newton iterations per layer (may be NULL) */
} ks_pops_model;

/* Replaces the population stage of synthe_py/tools/convert_atm_to_npz.py
 * (:1860-2650): the molecular equilibrium NMOLEC (tools/nmolec_exact.py:1742,
 * Newton iteration per layer, surface first), the ion populations POPS /
 * PFSAHA (tools/pops_exact.py:1639, :941) of elements 1-99 and the Doppler
 * widths (tools/pops_exact.py:2027), all in FP64, for n_models atmospheres
 * in one launch per stage (one warp per model for the molecular
 * equilibrium).  Workspace: ks_populations_workspace_size bytes of device
 * memory, 256-byte aligned.  The call copies the model records to the
 * workspace and returns when the results are ready (it synchronises the
 * stream). */
ks_status ks_populations_workspace_size(const ks_pops_model *models, int32_t n_models, size_t *bytes);
ks_status ks_populations(const ks_pops_model *models, int32_t n_models, void *workspace,
                         size_t workspace_bytes, void *stream);

/* Forward-mode derivatives of the population stage with respect to the log10
 * abundance (dex) of one element: `model` as for ks_populations (its value
 * outputs may be NULL, except none are needed), `element` = Z-1, and device
 * arrays receiving d(field)/d(log10 XABUND[element]) for the fields the
 * synthesis reads (the Doppler widths and hc/kT do not depend on the
 * abundances).  Every step of ks_populations is differentiated as computed
 * (dual numbers through the Newton iterations, the same pivots and iteration
 * counts), one warp per (model, element) pair, so any number of pairs cost
 * about one model's time.  No counterpart in the reference (it has no
 * gradients). */
typedef struct {
    ks_pops_model model;
    int32_t element;
    double *d_electron_density;     /* [L] */
    double *d_mass_density;         /* [L] */
    double *d_xnf_h;                /* [L] */
    double *d_xnf_he1;              /* [L] */
    double *d_xnf_h2;               /* [L] */
    double *d_population;           /* [L, 6, 139] */
} ks_pops_tangent;

ks_status ks_populations_tangent_workspace_size(const ks_pops_tangent *tangents, int32_t n,
                                                size_t *bytes);
ks_status ks_populations_tangent(const ks_pops_tangent *tangents, int32_t n, void *workspace,
                                 size_t workspace_bytes, void *stream);

/* ---- gfall reader ---------------------------------------------------------- */

/* Native reader of gfall line lists (synthe_py/io/lines/atomic.py:299
 * load_catalog: fixed-width records, or the whitespace form for lines
 * shorter than 98 columns; :762 filter_by_range DELLIM window; the TRANSP
 * routing of physics/line_opacity.py:740-765 and the ASYNTH centre classes
 * of :1094).  Host memory.  ks_gfall_read parses the file and keeps lines
 * inside [wl_min - margin, wl_max + margin] (wl_max <= 0 keeps all);
 * ks_gfall_sort orders them by wavelength (stable); ks_gfall_count gives the
 * size; ks_gfall_fetch copies columns (any pointer may be NULL;
 * catalog_index = position in the window-filtered catalog order, i.e. the
 * reference's line index); ks_gfall_free releases the handle.  potion: the
 * 999 ionisation potentials for the Stark/van der Waals defaults (may be
 * NULL). */
typedef struct ks_gfall ks_gfall;
ks_status ks_gfall_read(const char *path, double wl_min, double wl_max,
                        const double *potion, int32_t n_potion, ks_gfall **out);
ks_status ks_gfall_sort(ks_gfall *g);
int64_t ks_gfall_count(const ks_gfall *g);
ks_status ks_gfall_fetch(const ks_gfall *g, double *wavelength, double *log_gf, double *gf,
                         double *cgf, double *elo_cm, double *gamma_rad, double *gamma_stark,
                         double *gamma_vdw, int32_t *element_idx, int32_t *ion_stage,
                         int32_t *line_type, uint8_t *process_mask, uint8_t *asynth_mask,
                         double *code, int64_t *catalog_index);
/* NBLO / NBUP of every record (columns 103-106 of the fixed-width form,
 * synthe_py/io/lines/atomic.py:520-532): the principal quantum numbers of
 * hydrogen lines, 0 when blank.  Same order as ks_gfall_fetch. */
ks_status ks_gfall_fetch_levels(const ks_gfall *g, int32_t *n_lower, int32_t *n_upper);
/* ISO1 / ISO2 of every record (columns 107-109 and 117-119,
 * synthe_py/io/lines/atomic.py:344-346, :535-546), 0 when blank; fort.19
 * takes ISO2 as the continuum index NCON when ISO1 is 0
 * (io/lines/fort19.py:338).  Same order as ks_gfall_fetch. */
ks_status ks_gfall_fetch_iso(const ks_gfall *g, int32_t *iso1, int32_t *iso2);
/* The GR / GS / GW fields of every record as read (log10 damping constants,
 * 0 when blank; synthe_py/io/lines/atomic.py:341-343): fort.19 keeps them
 * unnormalised for autoionizing lines (io/lines/fort19.py:352-373).  Same
 * order as ks_gfall_fetch. */
ks_status ks_gfall_fetch_gamma_logs(const ks_gfall *g, double *gamma_rad_log, double *gamma_stark_log,
                                    double *gamma_vdw_log);
/* XJ / XJP of every record (columns 37-41, 65-69) and whether its LABELP
 * begins with CONTINUU (io/lines/atomic.py:338-340): fort.19 turns such a
 * record into a merged-continuum record with NLAST = XJP (or NBUP) and gf x
 * (2 XJ + 1) (io/lines/fort19.py:304-307).  Same order as ks_gfall_fetch. */
ks_status ks_gfall_fetch_j(const ks_gfall *g, double *xj, double *xjp, uint8_t *continuum_label);
void ks_gfall_free(ks_gfall *g);

#ifdef __cplusplus
}
#endif

#endif /* KURUCZ_GB300_H */
