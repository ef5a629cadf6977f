/*
 * trvg.h -- C ABI of the GB300-native mesh-based clustering estimators.
 *
 * Drop-in boundary for Triumvirate's FFT-based three-point (and two-point)
 * estimators.  Every entry point replaces one reference C++ function of
 * MikeSWang/Triumvirate (paths relative to src/triumvirate/):
 *
 *   trvg_compute_bispec_in_gpp_box  <- trv::compute_bispec_in_gpp_box
 *                                      (include/threept.hpp:274)
 *   trvg_compute_bispec             <- trv::compute_bispec
 *                                      (include/threept.hpp:237)
 *   trvg_compute_3pcf_in_gpp_box    <- trv::compute_3pcf_in_gpp_box
 *                                      (include/threept.hpp:290)
 *   trvg_compute_3pcf               <- trv::compute_3pcf
 *                                      (include/threept.hpp:257)
 *   trvg_compute_3pcf_window        <- trv::compute_3pcf_window
 *                                      (include/threept.hpp:310)
 *   trvg_hankel_*                   <- trv::maths::HankelTransform
 *                                      (include/fftlog.hpp:68-257)
 *   trvg_dcat_*                     <- trv::ParticleCatalogue loading and
 *                                      preparation (particles.cpp:94-510,
 *                                      570-888) and the Python
 *                                      ParticleCatalogue's centre / pad /
 *                                      periodise / compute_los
 *                                      (catalogue.py:437-676)
 *   trvg_compute_powspec_in_gpp_box <- trv::compute_powspec_in_gpp_box
 *                                      (include/twopt.hpp:283)
 *   trvg_compute_powspec            <- trv::compute_powspec
 *                                      (include/twopt.hpp:246)
 *   trvg_calc_grid_based_powlaw_norm<- trv::MeshField::
 *                                      calc_grid_based_powlaw_norm
 *                                      (include/field.hpp:426), the kernel of
 *                                      calc_{bispec,powspec}_normalisation_
 *                                      from_mesh (threept.hpp:150,
 *                                      twopt.hpp:101)
 *   trvg_assign_weighted_field_to_mesh <- trv::MeshField::
 *                                      assign_weighted_field_to_mesh
 *                                      (include/field.hpp:165)
 *
 * Conventions
 *  - Plain pointers and sizes only.  Particle arrays may live in host or
 *    device memory (trvg_catalogue.memory); results are written to
 *    caller-owned HOST arrays of length `dim` (complex values interleaved
 *    re, im).  The reference returns the same vectors by value in
 *    BispecMeasurements / ThreePCFMeasurements / PowspecMeasurements
 *    (include/dataobjs.hpp:202-283).
 *  - Errors: every function returns a TRVG_* status; the message of the
 *    last failure on the calling thread is given by trvg_last_error().
 *    TRVG_ERR_INVALID_PARAMETER maps to trv::sys::InvalidParameterError,
 *    TRVG_ERR_INVALID_DATA to trv::sys::InvalidDataError and
 *    TRVG_ERR_UNIMPLEMENTED to trv::sys::UnimplementedError
 *    (include/monitor.hpp:683-780).
 *  - Threading: a context owns one CUDA stream, its FFT plans and device
 *    workspace; calls on one context must not overlap.  Different contexts
 *    may be used from different threads.
 *  - Parameters arrive already validated and derived as the reference's
 *    ParameterSet::validate leaves them (parameters.cpp:466-1270): e.g.
 *    interlacing is off for three-point statistics and 'full' form with
 *    ell1 == ell2 is passed as TRVG_SHAPE_TRIU.
 */
#ifndef TRVG_H_INCLUDED
#define TRVG_H_INCLUDED

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define TRVG_OK                     0
#define TRVG_ERR_INVALID_PARAMETER  1
#define TRVG_ERR_INVALID_DATA       2
#define TRVG_ERR_UNIMPLEMENTED      3
#define TRVG_ERR_CUDA               4
#define TRVG_ERR_CUFFT              5
#define TRVG_ERR_ALLOC              6

/* Data-vector shapes (ParameterSet::shape, parameters.cpp:829-848). */
#define TRVG_SHAPE_DIAG     0
#define TRVG_SHAPE_OFFDIAG  1
#define TRVG_SHAPE_ROW      2
#define TRVG_SHAPE_FULL     3
#define TRVG_SHAPE_TRIU     4

/* Arithmetic of meshes and transforms.  FP64: all-double path.
 * FP32_MIXED: float meshes and FFTs; particle offsets, Y_lm recurrences,
 * mode counts, mesh-wide reductions, normalisation and shot-noise
 * subtraction stay in double. */
#define TRVG_PREC_FP64        0
#define TRVG_PREC_FP32_MIXED  1

/* Where the arrays of a trvg_catalogue live. */
#define TRVG_MEM_HOST    0
#define TRVG_MEM_DEVICE  1

typedef struct trvg_context trvg_context;

/* The subset of trv::ParameterSet (include/parameters.hpp:58-290) that
 * the mesh estimators read. */
typedef struct trvg_params {
  double boxsize[3];
  int ngrid[3];
  int assignment_order;   /* 1 NGP, 2 CIC, 3 TSC, 4 PCS */
  int interlace;          /* 0 or 1 */
  int ell1, ell2, ELL;    /* multipole degrees */
  int shape;              /* TRVG_SHAPE_* */
  int idx_bin;            /* row / off-diagonal index */
  int precision;          /* TRVG_PREC_* */
  int verbose;            /* 0 silent; >= 20 stage log on stderr */
  int i_wa, j_wa;         /* wide-angle orders (3PCF window only) */
} trvg_params;

/* trv::Binning (include/dataobjs.hpp:58): edges and centres, host memory. */
typedef struct trvg_binning {
  int num_bins;
  const double* bin_edges;    /* num_bins + 1 */
  const double* bin_centres;  /* num_bins */
} trvg_binning;

/* A particle catalogue in structure-of-arrays form.  Replaces
 * trv::ParticleCatalogue (include/particles.hpp:78) plus the
 * LineOfSight arrays (include/dataobjs.hpp:186) of the survey estimators.
 * Positions are box coordinates (the caller has centred / periodised).
 * `w` is the overall weight ws * wc (NULL = unit weights).  `los_*` are
 * unit line-of-sight vectors (survey estimators only; may be NULL for the
 * periodic-box ones). */
typedef struct trvg_catalogue {
  int64_t n;
  const double* x;
  const double* y;
  const double* z;
  const double* w;
  const double* los_x;
  const double* los_y;
  const double* los_z;
  int memory;             /* TRVG_MEM_HOST or TRVG_MEM_DEVICE */
} trvg_catalogue;

/* trv::BispecMeasurements / trv::ThreePCFMeasurements
 * (include/dataobjs.hpp:249-283).  For the 3PCF, coord/eff hold r values
 * and counts hold npairs.  Caller-owned host arrays of length `dim`
 * (2 * dim doubles for the complex ones). */
typedef struct trvg_threept_out {
  int dim;
  double* coord1_bin;
  double* coord1_eff;
  int32_t* count_1;
  double* coord2_bin;
  double* coord2_eff;
  int32_t* count_2;
  double* raw;    /* complex, interleaved */
  double* shot;   /* complex, interleaved */
} trvg_threept_out;

/* trv::PowspecMeasurements (include/dataobjs.hpp:202). */
typedef struct trvg_powspec_out {
  int dim;
  double* kbin;
  double* keff;
  int32_t* nmodes;
  double* pk_raw;   /* complex, interleaved */
  double* pk_shot;  /* complex, interleaved */
} trvg_powspec_out;

/* Per-call counters of the last estimator call on a context. */
typedef struct trvg_stats {
  double ms_total;        /* wall time of the call on its stream (events) */
  double ms_h2d;          /* host->device copies of particle arrays */
  int64_t h2d_bytes;      /* bytes copied host->device */
  int64_t kernel_launches;/* launches of this library's kernels */
  int64_t fft_launches;   /* cuFFT executions */
  int pruned_grid[3];     /* evaluation grid of the shell fields (== ngrid
                             when the full mesh is used) */
  int64_t graph_replays;  /* mocks of the last batch replayed from its
                             captured CUDA graph */
} trvg_stats;

/* ---- Context -------------------------------------------------------- */

/* Create a context on CUDA device `device`. */
int trvg_context_create(int device, trvg_context** ctx);
int trvg_context_destroy(trvg_context* ctx);
/* Message of the last failure on this thread ("" if none). */
const char* trvg_last_error(void);
/* Library version string. */
const char* trvg_version(void);
/* Counters of the last estimator call on `ctx`. */
int trvg_get_stats(const trvg_context* ctx, trvg_stats* out);
/* Release cached device workspace and FFT plans of `ctx`. */
int trvg_release_workspace(trvg_context* ctx);

/* Run the context's work on `stream` (a cudaStream_t of the calling
 * framework, e.g. its current stream); NULL restores the context's own
 * stream.  No counterpart in the reference (which has no streams). */
int trvg_context_set_stream(trvg_context* ctx, void* stream);
/* Context options (no counterpart in the reference):
 *   "full_mesh_shells" 0/1: evaluate the shell-filtered fields on the full
 *                           mesh instead of the smallest exact grid;
 *   "profiling"        0/1: time every kernel / FFT launch with CUDA events
 *                           (read back with trvg_kernel_time_*);
 *   "shotnoise_fp64"   0/1: FP32-mixed: transform the shot-noise field in
 *                           FP64 (default FP32);
 *   "shell_fields_fp64" 0/1: FP32-mixed: evaluate the shell-filtered and
 *                           compensated fields in FP64 (default FP32);
 *   "sort_catalogue"   0/1: order catalogues of >= 65536 particles by mesh
 *                           tile before the deposit (default 1);
 *   "ff_transforms"    FP32-mixed periodic-box bispectra with real shell
 *                           fields: 1 (default) compute the spectrum modes
 *                           of the shell fields and the evaluation-grid
 *                           transforms in float-float arithmetic, 2 only
 *                           the forward transform of the mesh (rounded once
 *                           to FP32 before FP32 inverse transforms), 0
 *                           neither;
 *   "gram_per_pair"    0/1: FP32 shell-field pair sums one data-vector
 *                           entry per thread instead of the register-tiled
 *                           Gram form (default 0);
 *   "graph_batch"      0/1: FP32-mixed batches: capture one mock as a CUDA
 *                           graph and replay it for the others (default 1;
 *                           off while profiling);
 *   "autotune"         0/1: time candidate launch shapes (catalogue-sort
 *                           tile side, pair-reduction bin batch) on first
 *                           use and keep the fastest (default 1; 0 also
 *                           forgets earlier choices);
 *   "overlap"          0/1: run the shot-noise field of an FP32
 *                           periodic-box bispectrum on a second stream next
 *                           to the float-float shell fields (default 1; off
 *                           while profiling and in batch replays);
 *   "side_priority"    0/1: create the second stream at the default (0)
 *                           or the device's greatest priority (1);
 *   "xi_octant"        0/1: FP32 periodic-box bispectra with m = 0 legs of
 *                           even total degree: keep the shot-noise field
 *                           averaged over sign flips on one octant (three
 *                           DCT-I passes) instead of the full mesh
 *                           (default 1);
 *   "fused_ylm"        0/1: FP32 meshes: build the Y_lm-weighted fields of
 *                           every order of a survey estimate in one fused
 *                           pass per catalogue (default 1);
 *   "assign_path"      FP32 real meshes of sorted catalogues: 0 the
 *                           autotuner's choice (default), 1 the
 *                           shared-memory tiled deposit (32^3 tiles),
 *                           2 per-particle global atomics (finer tiles);
 *                           the tiled deposit serves uncompensated meshes;
 *   "mesh_comp"        FP32-mixed: deposit with float-float windows and
 *                           compensated atomics, each FP32 mesh keeping
 *                           its rounding errors in a second FP32 mesh:
 *                           0 never, 1 always, 2 (default) for fields of
 *                           several catalogues (data minus alpha randoms,
 *                           whose sum cancels);
 *   "mesh_renorm"      0/1: FP32-mixed: round every compensated mesh to
 *                           its correctly rounded FP32 sum before the FP32
 *                           transforms (default 0: only fields of several
 *                           catalogues are). */
int trvg_set_option(trvg_context* ctx, const char* key, int64_t value);
/* Launch shapes the autotuner chose so far: key and value. */
int trvg_tuned_count(const trvg_context* ctx, int* count);
int trvg_tuned_get(const trvg_context* ctx, int index, char* key,
                   int key_len, int64_t* value);
/* Per-kernel device time of the last call (profiling on). */
int trvg_kernel_time_count(const trvg_context* ctx, int* count);
int trvg_kernel_time_get(const trvg_context* ctx, int index, char* name,
                         int name_len, double* ms, int64_t* launches);

/* ---- FFTLog Hankel transforms (fftlog.cpp) --------------------------- */

typedef struct trvg_hankel trvg_hankel;

/* trv::maths::HankelTransform(mu, q) followed by
 * initialise(sample_pts, kr_c, lowring, extrap, extrap_exp)
 * (include/fftlog.hpp:90, 164): n log-spaced points x, pivot kr_c (adjusted
 * by the low-ringing condition when lowring != 0), native extrapolation 0
 * none, 1 zero, 2 constant, 3 linear, 4 log-linear to the power of 2 >=
 * extrap_exp n. */
int trvg_hankel_create(double mu, double q, const double* x, int n,
                       double kr_c, int lowring, int extrap,
                       double extrap_exp, trvg_hankel** out);
/* Sample size, transform size, pivot, log spacing, and the n points before
 * and after the transform (any output may be NULL). */
int trvg_hankel_info(const trvg_hankel* h, int* n, int* n_trans,
                     double* pivot, double* logres, double* pre_sampts,
                     double* post_sampts);
/* HankelTransform::biased_transform (include/fftlog.hpp:187) of `batch`
 * rows of n complex samples at once: a and b are host arrays of
 * 2 n batch doubles (re, im interleaved, row after row); rows are taken as
 * real when extrapolating. */
int trvg_hankel_transform(trvg_context* ctx, const trvg_hankel* h, int batch,
                          const double* a, double* b);
int trvg_hankel_destroy(trvg_hankel* h);

/* ---- Device-resident particle catalogues (particles.cpp) ------------- */

/* A catalogue whose columns x, y, z, nz, ws, wc and w = ws wc (and, once
 * computed, the lines of sight) live in device memory of the context's
 * GPU.  trvg_dcat_view hands it to every estimator as a TRVG_MEM_DEVICE
 * trvg_catalogue without a copy. */
typedef struct trvg_dcat trvg_dcat;

/* ParticleCatalogue::load_catalogue_file (particles.cpp:94-510) for text
 * files: `path` may join sub-files with "::"; `columns` names the file's
 * columns, comma-separated, from x, y, z, nz, ws, wc (others are skipped);
 * lines that are empty or start with '#' are skipped.  Absent columns take
 * nz = ntotal / volume (0 if volume <= 0) and ws = wc = 1.  HDF5 paths
 * (.h5, .hdf5) give TRVG_ERR_INVALID_DATA, as a build without HDF5 does.
 * Parsing runs on all host threads; the columns are copied to the device
 * once. */
int trvg_dcat_read_text(trvg_context* ctx, const char* path,
                        const char* columns, double volume, trvg_dcat** out);
/* A catalogue from n host particles; nz, ws, wc may be NULL (0, 1, 1). */
int trvg_dcat_from_host(trvg_context* ctx, int64_t n, const double* x,
                        const double* y, const double* z, const double* nz,
                        const double* ws, const double* wc, trvg_dcat** out);
/* One catalogue holding `count` catalogues back to back (device-to-device
 * copies; lines of sight kept when every part has them), e.g. the
 * particles of a batch of mocks. */
int trvg_dcat_concat(trvg_context* ctx, const trvg_dcat* const* cats,
                     int count, trvg_dcat** out);
/* Size, weight totals (calc_total_weights, particles.cpp:570-602) and
 * coordinate extents (calc_pos_extents, particles.cpp:604-656); any output
 * may be NULL.  The totals come from a fixed-order device reduction. */
int trvg_dcat_info(trvg_context* ctx, const trvg_dcat* c, int64_t* n,
                   double* wtotal, double* wstotal, double* pos_min,
                   double* pos_max);
/* x -= dpos[0], y -= dpos[1], z -= dpos[2]
 * (offset_coords, particles.cpp:658-676). */
int trvg_dcat_offset(trvg_context* ctx, trvg_dcat* c, const double* dpos);
/* centre_in_box (particles.cpp:701-778; catalogue.py:490-545): the
 * mid-point of ref's extents (c's if ref is NULL) moves to boxsize / 2 and
 * both catalogues move by the same offset. */
int trvg_dcat_centre(trvg_context* ctx, trvg_dcat* c, trvg_dcat* ref,
                     const double* boxsize);
/* pad_in_box / pad_grids (particles.cpp:780-888): the minimum of ref's
 * extents (c's if ref is NULL) moves to boxsize_pad * boxsize, or to
 * ngrid_pad * boxsize / ngrid evaluated left to right as pad_grids does;
 * give exactly one of boxsize_pad and ngrid_pad (three values each). */
int trvg_dcat_pad(trvg_context* ctx, trvg_dcat* c, trvg_dcat* ref,
                  const double* boxsize, const double* boxsize_pad,
                  const double* ngrid, const double* ngrid_pad);
/* offset_coords_for_periodicity (particles.cpp:678-699): coordinates
 * x >= L become fmod(x, L) and x < 0 become fmod(x, L) + L. */
int trvg_dcat_wrap_box(trvg_context* ctx, trvg_dcat* c,
                       const double* boxsize);
/* ParticleCatalogue.periodise (catalogue.py:648-676): each coordinate
 * becomes (x + L/2 - (max + min)/2) mod L with the remainder taking the
 * sign of L, bit for bit as numpy computes it. */
int trvg_dcat_periodise(trvg_context* ctx, trvg_dcat* c,
                        const double* boxsize);
/* ParticleCatalogue.compute_los (catalogue.py:437-458): unit end-point
 * lines of sight x / |x| (1 where |x| = 0), kept on the device and
 * included in trvg_dcat_view. */
int trvg_dcat_compute_los(trvg_context* ctx, trvg_dcat* c);
/* Set 'nz', 'ws' or 'wc' to a constant (w follows); compute_mean_density
 * (catalogue.py:460-488) is nz = ntotal / volume. */
int trvg_dcat_set_column(trvg_context* ctx, trvg_dcat* c, const char* column,
                         double value);
/* Replace column x, y, z, nz, ws, wc, los_x, los_y or los_z with n host
 * doubles (w follows ws and wc). */
int trvg_dcat_upload(trvg_context* ctx, trvg_dcat* c, const char* column,
                     const double* values);
/* sum ws nz^(order-1) wc^order over the particles, the denominator of the
 * particle normalisation (order 2: twopt.cpp:56-99; order 3:
 * threept.cpp:96-136), and the number of particles with nz != 0; either
 * output may be NULL. */
int trvg_dcat_norm_sum(trvg_context* ctx, const trvg_dcat* c, int order,
                       double* sum, int64_t* nonzero_nz);
/* A TRVG_MEM_DEVICE trvg_catalogue over c's columns (valid until c is
 * destroyed or its lines of sight are first computed). */
int trvg_dcat_view(const trvg_dcat* c, trvg_catalogue* out);
/* Copy column x, y, z, nz, ws, wc, w, los_x, los_y or los_z to n host
 * doubles. */
int trvg_dcat_download(trvg_context* ctx, const trvg_dcat* c,
                       const char* column, double* out);
int trvg_dcat_destroy(trvg_dcat* c);

/* Length of the data vector of a three-point measurement
 * (threept.cpp:1495-1521). */
int trvg_data_vector_dim(int shape, int num_bins, int idx_bin, int* dim);

/* ---- Estimators ------------------------------------------------------ */

/* Bispectrum, periodic box, global plane-parallel line of sight. */
int trvg_compute_bispec_in_gpp_box(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_binning* kbinning,
  double norm_factor, trvg_threept_out* out);

/* Bispectra of n_mocks periodic-box catalogues in one call (the reference
 * calls trv::compute_bispec_in_gpp_box once per catalogue).  `particles`
 * holds the catalogues back to back: mock i is the slice
 * [offsets[i], offsets[i + 1]) of every column (offsets[0] = 0,
 * offsets[n_mocks] = particles->n); norm_factors[i] and outs[i] belong to
 * mock i.  Plans, workspace, spline tables and the catalogue-independent
 * mode counts are shared by the whole batch. */
/* Adjoint of the raw periodic-box bispectrum of degrees (0, 0, 0); the
 * reference has no derivatives.  For the cotangent
 * cotangent[2 i] = dL / d Re(raw_i) of every data-vector entry (raw B_000
 * is real, so cotangent[2 i + 1] is not used) it writes, each optional and
 * in the memory kind of `data`:
 *   grad_mesh  dL/dm of the weighted count mesh m that the assignment
 *              deposits (ngrid[0] * ngrid[1] * ngrid[2] doubles, z fastest);
 *   grad_w     dL/dw_i (n doubles);
 *   grad_pos   dL/dx_i, dL/dy_i, dL/dz_i (3 n doubles: every x, then every
 *              y, then every z), for positions in [0, L);
 * and, if `out` is given, the raw values themselves (shot left at 0: shot
 * noise is not differentiated).  Needs even mesh numbers or a pruned
 * evaluation grid. */
int trvg_bispec_gpp_adjoint(
  trvg_context* ctx, const trvg_params* params, const trvg_catalogue* data,
  const trvg_binning* kbinning, double norm_factor, const double* cotangent,
  double* grad_mesh, double* grad_w, double* grad_pos, trvg_threept_out* out);

/* Vector-Jacobian product of the periodic-box B_000 (degrees 0, 0, 0),
 * raw AND shot noise; the reference has no derivatives.  The input is
 * either the particles `data` (mesh = NULL) or a count mesh `mesh` (data
 * = NULL): ngrid[0] * ngrid[1] * ngrid[2] FP32 values in DEVICE memory,
 * z fastest, the weight per cell the assignment deposits; its fluctuation
 * is taken about its own mean, and it has no shot noise.  cot_raw[2 i] =
 * dL / d Re(raw_i) and, for particles, cot_shot[2 i] = dL / d Re(shot_i)
 * (NULL: shot noise not differentiated).  Outputs as for
 * trvg_bispec_gpp_adjoint; grad_mesh in device memory for a mesh input;
 * grad_w and grad_pos must be NULL for a mesh input. */
int trvg_bispec_gpp_vjp(
  trvg_context* ctx, const trvg_params* params, const trvg_catalogue* data,
  const float* mesh, const trvg_binning* kbinning, double norm_factor,
  const double* cot_raw, const double* cot_shot, double* grad_mesh,
  double* grad_w, double* grad_pos, trvg_threept_out* out);

int trvg_compute_bispec_in_gpp_box_batch(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* particles, int n_mocks, const int64_t* offsets,
  const trvg_binning* kbinning, const double* norm_factors,
  trvg_threept_out* outs);

/* Bispectrum, survey-type catalogues, local plane-parallel line of sight.
 * `alpha` = wstotal_data / wstotal_rand (threept.cpp:271). */
int trvg_compute_bispec(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_catalogue* rand, double alpha,
  const trvg_binning* kbinning, double norm_factor, trvg_threept_out* out);

/* Three-point correlation function, periodic box. */
int trvg_compute_3pcf_in_gpp_box(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_binning* rbinning,
  double norm_factor, trvg_threept_out* out);

/* Three-point correlation function, survey-type catalogues. */
int trvg_compute_3pcf(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_catalogue* rand, double alpha,
  const trvg_binning* rbinning, double norm_factor, trvg_threept_out* out);

/* Three-point correlation function window from a random catalogue: the
 * survey estimator on alpha * (random field) alone, the shot-noise
 * amplitude alpha^3 sum y w^3, and with `wide_angle` the power-law kernel
 * r^-(i_wa + j_wa) applied to G in configuration space. */
int trvg_compute_3pcf_window(
  trvg_context* ctx, const trvg_params* params, const trvg_catalogue* rand,
  double alpha, const trvg_binning* rbinning, double norm_factor,
  int wide_angle, trvg_threept_out* out);

/* Power spectrum multipole (ELL = params->ELL), periodic box. */
int trvg_compute_powspec_in_gpp_box(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_binning* kbinning,
  double norm_factor, trvg_powspec_out* out);

/* Power spectrum multipole, survey-type catalogues. */
int trvg_compute_powspec(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* data, const trvg_catalogue* rand, double alpha,
  const trvg_binning* kbinning, double norm_factor, trvg_powspec_out* out);

/* 1 / (dV sum_x n(x)^order) of the weighted mesh n (no interlacing),
 * the mesh normalisation of calc_*_normalisation_from_mesh. */
int trvg_calc_grid_based_powlaw_norm(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* particles, int order, double* norm_factor);

/* Allocation-free variant of trvg_calc_grid_based_powlaw_norm; it has no
 * counterpart in the reference.  It allocates no device memory and creates
 * no context: the mesh and reduction slots live in one static device array
 * of 2^21 cells (128^3, 16 MiB), so meshes with more cells are rejected
 * (TRVG_ERR_INVALID_PARAMETER).  It serves callers whose device memory is
 * held by another allocator, or that must not call cudaMalloc / cudaFree
 * (both synchronise the device) once running.
 *  - `particles` must be device-resident (TRVG_MEM_DEVICE);
 *  - runs on the calling thread's current device, on `stream` (a
 *    cudaStream_t; NULL for the legacy default stream), always in FP64,
 *    and waits for `stream` before writing *norm_factor (host);
 *  - the call zeroes the scratch it uses itself; nothing must be zero on
 *    entry;
 *  - the scratch is one per device: overlapping calls on one device race
 *    and must be serialised by the caller;
 *  - the call synchronises `stream` to read its result back, so it must
 *    not be made while `stream` (or, in global capture mode, any stream)
 *    is being captured;
 *  - the first call on a device also looks up the scratch address on
 *    that device (a one-off host-side step). */
int trvg_calc_grid_based_powlaw_norm_noalloc(
  const trvg_params* params, const trvg_catalogue* particles, int order,
  void* stream, double* norm_factor);

/* The weighted mesh n(x) = sum_i w_i W(x - x_i) / dV (real weights) or its
 * interlacing shadow (`shadow` = 1), written to `mesh_out` (host, ngrid[0]
 * * ngrid[1] * ngrid[2] doubles, row-major, z fastest). */
int trvg_assign_weighted_field_to_mesh(
  trvg_context* ctx, const trvg_params* params,
  const trvg_catalogue* particles, int shadow, double* mesh_out);

/* ---- Host maths (no GPU needed) ------------------------------------- */

/* Wigner 3-j symbol (maths.cpp:167-169). */
double trvg_wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3);
/* j_ell(x) by the library's own evaluation (double). */
double trvg_sph_bessel(int ell, double x);
/* j_ell(x) through the natural-cubic-spline table the GPU kernels use
 * (maths.cpp:309-375: dx = 0.05 up to max(1000, ell^2), direct above). */
int trvg_sph_bessel_spline(int ell, const double* x, int64_t n, double* out);
/* Reduced spherical harmonic y_lm(v) of n vectors (maths.cpp:171-220),
 * evaluated by the same code the kernels use, on the host. */
int trvg_reduced_ylm(int ell, int m, const double* v3, int64_t n,
                     double* out_complex);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* TRVG_H_INCLUDED */
