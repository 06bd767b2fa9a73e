/*
 * holodeck_gb300 C ABI: GB300 (sm_103a) kernels for holodeck's semi-analytic-model
 * gravitational-wave-background path.
 *
 * Conventions shared by every entry point
 * - All array arguments are DEVICE pointers to C-contiguous float64 (or int32 where
 *   stated) arrays laid out exactly like the numpy arrays of the holodeck function the
 *   entry point replaces: (M, Q, Z) grids are m-major, (M, Q, Z, F) grids carry the
 *   frequency index fastest.
 * - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Every
 *   call only enqueues work; results are ready once the stream is synchronised.
 * - `d_status` (may be NULL) is a device int32 word.  Kernels OR HGB_STATUS_* bits into
 *   it when a bounded device loop runs out or an input check fails on the device; the
 *   caller zeroes it before the call and reads it after synchronising.
 * - Functions that need scratch memory take `workspace`/`workspace_bytes`; the matching
 *   *_workspace_bytes() query returns the size.  No entry point allocates device memory.
 * - Return value: HGB_OK or an HGB_ERR_* code (argument errors are detected on the
 *   host before anything is enqueued).  hgb_error_string() describes a code.
 */
#ifndef HOLODECK_GB300_H
#define HOLODECK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes */
#define HGB_OK 0
#define HGB_ERR_INVALID_ARGUMENT 1
#define HGB_ERR_CUDA 2
#define HGB_ERR_WORKSPACE 3
#define HGB_ERR_CAPACITY 4   /* input larger than a static scratch array holds */
#define HGB_ERR_DEVICE_LIMIT 5   /* a bounded device wait gave up: the call's outputs are not valid */

/* ---- device status bits (OR-ed into *d_status) */
#define HGB_STATUS_ITERATION_LIMIT 1   /* a bounded sampling / root-finding loop ran out */
#define HGB_STATUS_INVALID_REDSHIFT 2  /* redz < 0 and != -1 (single_sources.py:95-98) */
#define HGB_STATUS_TABLE_RANGE 4       /* an interpolation argument left its table */
#define HGB_STATUS_GRADIENT_NOT_CONVERGED 8  /* scatter gradient solve hit grad_maxiter (scipy only warns) */
#define HGB_STATUS_BOUNDS 16           /* an index left its array; the access was skipped (only a library
                                          built with HGB_BOUNDS_CHECK checks, see holodeck_gb300/build.py) */

/* ---- realization modes for hgb_loudest_hc_from_sorted / hgb_sam_poisson_gwb */
#define HGB_RNG_PHILOX 0   /* counter-based Philox4x32-10 draws keyed by (seed, bin, realization, frequency) */
#define HGB_RNG_REPLAY 1   /* consume caller-supplied draws (bit-exact replay of numpy's stream) */

/* Cosmology consumed by the kernels: flat matter + Lambda, no radiation.
 * Tables are device pointers; they match holodeck's cosmo._grid_z (decreasing),
 * cosmo._grid_age (increasing, s) and cosmo._grid_dcom (cm)  (sam_cyutils.pyx:476, :494). */
typedef struct {
    double H0;              /* [1/s] */
    double Om0;
    double Ode0;
    double age_pref;        /* 2 / (3 H0 sqrt(Ode0))         age(z) = age_pref * asinh(age_c1 (1+z)^-1.5) */
    double age_c1;          /* sqrt(Ode0 / Om0) */
    double tz_c2;           /* 1.5 H0 sqrt(Ode0)             z(t) = (age_c1 / sinh(tz_c2 t))^(2/3) - 1 */
    double age_limit;       /* age(0) rounded through Gyr, the stall threshold of utils.py:46, :1797-1806 */
    double hubble_distance; /* c / H0 [cm] */
    const double *grid_z;   /* [grid_size] */
    const double *grid_age; /* [grid_size] */
    const double *grid_dcom;/* [grid_size] */
    int grid_size;
    /* comoving distance D_C as a function of u = sqrt(1/(1+z)) on u = k / dc_n, k = 0..dc_n:
     * values [cm] and derivatives dD/du [cm]; cubic Hermite interpolation between nodes */
    const double *dc_val;   /* [dc_n + 1] */
    const double *dc_der;   /* [dc_n + 1] */
    int dc_n;
    /* the same distance for the FP32 entry points (may be NULL for the FP64 ones), written as
     * D_C = hubble_distance (1 - u) g(u) so that it keeps its relative precision as z -> 0:
     * g (dimensionless) and dg/du on the same nodes u = k / dc_n, cubic Hermite between them */
    const float *dcg_val;   /* [dc_n + 1] */
    const float *dcg_der;   /* [dc_n + 1] */
} hgb_cosmo;

/* Galaxy / black-hole population model (holodeck/sams/components.py, host_relations.py). */
#define HGB_GSMF_SCHECHTER 0         /* GSMF_Schechter (components.py:110-172) */
#define HGB_GSMF_DOUBLE_SCHECHTER 1  /* GSMF_Double_Schechter (components.py:276-330) */
#define HGB_RATE_GPF_GMT 0           /* GPF_Power_Law / GMT_Power_Law (components.py:520-675) */
#define HGB_RATE_GMR 1               /* GMR_Illustris (components.py:380-483), optional GMT */
typedef struct {
    int gsmf_kind;
    /* GSMF_Schechter: phi0, phiz, mchar0 [g], mcharz, alpha0, alphaz
     * GSMF_Double_Schechter: log10_phi1[3], log10_phi2[3], log10_mstar[3], alpha1, alpha2 */
    double gsmf[11];
    int rate_kind;
    int use_gmt;            /* 1 if a GMT is present (always 1 for HGB_RATE_GPF_GMT) */
    double gpf[6];          /* frac_norm, mref [g], malpha, zbeta, qgamma, max_frac */
    double gmt[5];          /* time_norm [s], mref [g], malpha, zbeta, qgamma */
    double gmr[11];         /* norm0 [1/s], normz, malpha0, malphaz, mdelta0, mdeltaz, qgamma0, qgammaz, qgammam, mref_delta [g], mref [g] */
    double mmb[4];          /* mamp [g], mplaw, mref [g], bulge_frac */
    int gsmf_uses_mtot, gpf_uses_mtot, gmt_uses_mtot;   /* sam.py:55-59 */
} hgb_sam_model;

/* ---- library */
int hgb_version(void);
const char *hgb_error_string(int code);
/* last CUDA error text of the calling thread after HGB_ERR_CUDA */
const char *hgb_last_cuda_error(void);

/* Static binary density before M-Mbulge scatter, plus the galaxy-merger time and the
 * redshift after the merger (-1 past the age of the Universe).
 * Replaces Semi_Analytic_Model.static_binary_density, sam.py:280-365 (+ mass_stellar
 * sam.py:250-278, components.py:132-172, :556-586, :620-675, utils.py:1772-1808).
 * density/gmt_time/redz_prime are (M, Q, Z); gmt_time/redz_prime are left untouched
 * when the model has no GMT. */
int hgb_static_density(const hgb_sam_model *model, const hgb_cosmo *cosmo,
                       const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                       const double *redz, int n_redz,
                       double *density, double *gmt_time, double *redz_prime,
                       int *d_status, void *stream);

/* density[i] = 0 where redz_prime[i] < 0 (sam.py:392-394). */
int hgb_zero_stalled(double *density, const double *redz_prime, long n, void *stream);

/* ---- M-Mbulge scatter (sam.py:1291-1394, add_scatter_to_masses)
 * Per redshift slice: Clough-Tocher interpolation of the density from the (log10 m1, log10 m2)
 * points of the (mtot, mrat) grid onto a (refine*M)^2 regular log grid (gradients by the
 * minimum-norm-network Gauss-Seidel solve, tolerance 1e-6, 400 sweeps), nearest-point repair of
 * NaN / negative nodes, Gaussian redistribution W^T G W along both mass axes, bilinear
 * interpolation back to the points.  The geometry depends only on the grid and is built once on
 * the host by hgb_scatter_plan_build (HOST pointers), copied to the device by the caller and
 * passed as hgb_scatter_plan (DEVICE pointers). */
typedef struct {
    int n_pts;      /* M*Q points */
    int n_tri;      /* triangles */
    int n_nbr;      /* directed point-neighbour entries */
    int n_grid;     /* refine*M nodes per axis */
    int n_levels;   /* Gauss-Seidel wavefront levels */
} hgb_scatter_sizes;

typedef struct {    /* host arrays, sized by hgb_scatter_plan_bounds */
    double *pts;        /* [n_pts][2] (log10 m1, log10 m2), m-major */
    int32_t *tri;       /* [n_tri][3] counter-clockwise point indices */
    double *tri_kappa;  /* [n_tri][3] cross-derivative coefficient of the edge opposite each vertex */
    double *vtx_qinv;   /* [n_pts][4] inverse normal matrix of the gradient update */
    int32_t *nbr_ptr;   /* [n_pts+1] */
    int32_t *nbr_idx;   /* [n_nbr] */
    double *nbr_w;      /* [n_nbr][4] edge vector and edge vector / length^3 */
    int32_t *level_ptr; /* [n_levels+1] */
    int32_t *level_vtx; /* [n_pts] points ordered by level */
    int32_t *grid_tri;  /* [n_grid^2] containing triangle, -1 outside the hull */
    double *grid_bary;  /* [n_grid^2][3] barycentric coordinates */
    int32_t *grid_near; /* [n_grid^2] nearest point */
    double *grid_axis;  /* [n_grid] log10 mass of the regular grid */
    double *weights;    /* [n_grid][n_grid] W[source][target] */
    int32_t *back_idx;  /* [n_pts][2] lower grid cell */
    double *back_t;     /* [n_pts][2] fractional offsets */
    double *back_w;     /* [n_pts][2][n_grid] (1-ty) bw and ty bw, bw = (1-tx) (W W)[:, a] + tx (W W)[:, a+1] */
    /* the neighbourhoods again, indexed by level-order position p (point level_vtx[p]) */
    int32_t *lv_nbr_ptr; /* [n_pts+1] */
    int32_t *lv_nbr;    /* [n_nbr] neighbour positions, in the order of nbr_idx */
    double *lv_nbr_w;   /* [n_nbr][4]: -2 w0, -2 w1, w2, w3 of nbr_w, in level order */
    double *lv_qinv;    /* [n_pts][4] */
} hgb_scatter_host_plan;

typedef struct {    /* the same arrays on the device */
    int n_mtot, n_mrat, n_grid, n_tri, n_levels;
    const double *pts;
    const int32_t *tri;
    const double *tri_kappa;
    const double *vtx_qinv;
    const int32_t *nbr_ptr;
    const int32_t *nbr_idx;
    const double *nbr_w;
    const int32_t *level_ptr;
    const int32_t *level_vtx;
    const int32_t *grid_tri;
    const double *grid_bary;
    const int32_t *grid_near;
    const double *weights;
    const int32_t *back_idx;
    const double *back_t;
    const double *back_w;
    const int32_t *lv_nbr_ptr;
    const int32_t *lv_nbr;
    const double *lv_nbr_w;
    const double *lv_qinv;
    double grad_tol;    /* 1e-6 in the reference */
    int grad_maxiter;   /* 400 in the reference */
} hgb_scatter_plan;

/* Upper bounds of the plan array sizes (n_grid is exact). */
int hgb_scatter_plan_bounds(int n_mtot, int n_mrat, int refine, hgb_scatter_sizes *out);
/* Build the geometry on the host; mtot / mrat are HOST arrays; writes the actual sizes. */
int hgb_scatter_plan_build(const double *mtot, int n_mtot, const double *mrat, int n_mrat, int refine,
                           double scatter_dex, hgb_scatter_host_plan *plan, hgb_scatter_sizes *sizes);
size_t hgb_scatter_workspace_bytes(int n_mtot, int n_mrat, int n_redz, int n_grid);
/* dens (M, Q, Z) is replaced by its scattered version. */
int hgb_add_scatter_to_masses(const hgb_scatter_plan *plan, double *dens, int n_redz,
                              void *workspace, size_t workspace_bytes, int *d_status, void *stream);

/* log10 hardening-rate normalisation per (mtot, mrat) cell such that the two-power-law
 * lifetime equals target_time: Brent root on [-20, 20], xtol 1e-3, rtol 1e-5, 100 iterations
 * (0 when the interval brackets no root, like scipy's cython brentq).  `norm` (may be NULL)
 * receives 10**norm_log10, the Fixed_Time_2PL_SAM._norm of hardening.py:1412-1416.
 * Replaces sam_cyutils.find_2pwl_hardening_norm, sam_cyutils.pyx:289-398. */
int hgb_find_2pwl_hardening_norm(double target_time, const double *mtot, const double *mrat, int n,
                                 double sepa_init, double rchar, double gamma_inner, double gamma_outer,
                                 int nsteps, double *norm_log10, double *norm, int *d_status, void *stream);

/* x[i] = sqrt(x[i]) (the hc^2 -> hc step of single_sources.py:166-167). */
int hgb_sqrt_inplace(double *x, long n, void *stream);

/* Differential binary number d^4N/[dlog10M dq dz dlnf] and the redshift at each target
 * frequency for Fixed_Time_2PL_SAM hardening.  Replaces _dynamic_binary_number_at_fobs_2pwl,
 * sam_cyutils.pyx:510-781.  redz_final / diff_num are (M, Q, Z, F) and fully written
 * (-1 / 0 where no target is reached).  fobs_sorted = 1 asserts fobs_orb is ascending. */
int hgb_dbn_2pwl(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                 const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                 const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                 const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                 double *redz_final, double *diff_num, void *stream);

/* hgb_dbn_2pwl in two phases, so that the first can overlap the M-Mbulge scatter: phase 1 walks the
 * separation steps (needs gmt_time, not the density; nden may be NULL) and leaves, per element, the
 * bracketing step index in redz_final and the target's time in diff_num; phase 2 turns them into
 * redz_final / diff_num with the final density nden.  phase 3 is both (= hgb_dbn_2pwl). */
int hgb_dbn_2pwl_phase(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                       const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                       const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                       const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                       double *redz_final, double *diff_num, int phase, void *stream);

/* FP32 production mode of hgb_dbn_2pwl_phase: same arguments and outputs.  Phase 1 (the
 * separation-step walk, i.e. the hardening residence-time integral) is the FP64 walk; phase 2 keeps
 * the age -> redshift inversion and its comoving distance in FP64 and evaluates the residence time
 * and the cosmological factor in FP32 (relative error of diff_num about 1e-6). */
int hgb_dbn_2pwl_phase_f32(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                           const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                           const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                           const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                           double *redz_final, double *diff_num, int phase, void *stream);

/* Same for Hard_GW (GW-only) hardening.  Replaces _dynamic_binary_number_at_fobs_gw,
 * sam_cyutils.pyx:788-899.  redz_prime is (M, Q, Z). */
int hgb_dbn_gw(const double *fobs_orb, int n_freq, const double *nden, const double *mtot, int n_mtot,
               const double *mrat, int n_mrat, int n_redz, const double *redz_prime,
               const hgb_cosmo *cosmo, double *redz_final, double *diff_num, void *stream);

/* number (M-1, Q-1, Z-1, F) = 8-vertex mean of dnum x dlog10M dq dz x dlnf.
 * Replaces _integrate_differential_number_3dx1d, sam_cyutils.pyx:170-216; takes the arguments of
 * that Cython kernel: log10(mtot) edges, mrat and redz edges, and dln_freq = diff(ln(fobs_orb_edges))
 * as its Python wrapper (sam_cyutils.pyx:115-167) prepares them. */
int hgb_integrate_3dx1d(const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat,
                        const double *redz, int n_redz, const double *dln_freq, int n_freq,
                        const double *dnum, double *number, void *stream);

/* h2fdf (M-1, Q-1, Z-1, F) = h_s^2 f/df at bin centres from the 3-axis midpoint of redz_final.
 * Replaces gravwaves.char_strain_sq_from_bin_edges_redz, gravwaves.py:694-724.
 * gw_src_const is holodeck.utils._GW_SRC_CONST (utils.py:40). */
int hgb_char_strain_sq(const double *mtot, int n_mtot, const double *mrat, int n_mrat, int n_redz,
                       const double *fobs_orb_edges, int n_freq, const double *redz_final, double gw_src_const,
                       const hgb_cosmo *cosmo, double *h2fdf, int *d_status, void *stream);

/* Both of the above in one pass over the (M, Q, Z, F) grids (the sequence of gwb(), sam.py:930-935).
 * Also flags redz_final values < 0 and != -1 (single_sources.py:95-98) in *d_status. */
int hgb_number_and_strain(const double *mtot, const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat,
                          const double *redz, int n_redz, const double *fobs_orb_edges, const double *dln_freq,
                          int n_freq, const double *dnum, const double *redz_final, double gw_src_const,
                          const hgb_cosmo *cosmo, double *number, double *h2fdf, int *d_status, void *stream);

/* FP32 production mode of hgb_number_and_strain: same arguments, arrays and status bits; the
 * vertex sums run in FP32 with Kahan compensation, the strain product in FP32 with power-of-two
 * scale factors (so nothing becomes subnormal), and only the redshift midpoints of bins whose
 * corners mix the -1 sentinel with redshifts are formed in FP64 (the reference's midpoint cancels
 * there).  Relative error of number and h2fdf about 1e-6.  Needs cosmo->dcg_val / dcg_der. */
int hgb_number_and_strain_f32(const double *mtot, const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat,
                              const double *redz, int n_redz, const double *fobs_orb_edges, const double *dln_freq,
                              int n_freq, const double *dnum, const double *redz_final, double gw_src_const,
                              const hgb_cosmo *cosmo, double *number, double *h2fdf, int *d_status, void *stream);

/* order[k] = flat bin index of the k-th largest h2fdf[..., 0] (single_sources.py:89).
 * Equal keys are put in ascending bin index.  This is a deterministic choice of this library,
 * not the reference's behaviour: the reference orders with numpy's default (unstable) argsort,
 * whose order among equal keys depends on the sort's partitioning.  Bins whose keys tie can
 * therefore be visited in another order than the reference visits them; callers that must
 * reproduce the reference's visiting order exactly pass its order to the realization entry
 * points instead.  -0.0 ties with +0.0 and NaN keys come last, as in numpy's argsort of the
 * negated keys.  The sort is this library's own stable radix sort (8 passes of 8 bits, 25 kernel
 * launches); workspace: hgb_sort_workspace_bytes(n_bins), about 20 bytes per bin. */
size_t hgb_sort_workspace_bytes(long n_bins);
int hgb_argsort_f0_desc(const double *h2fdf, long n_bins, int n_freq, int32_t *order,
                        void *workspace, size_t workspace_bytes, void *stream);

/* No reference counterpart.  Allocation-free variant of hgb_argsort_f0_desc for callers that
 * cannot supply a workspace: same arguments without workspace/workspace_bytes, same `order`.
 * Equal keys are ordered as hgb_argsort_f0_desc orders them (ascending bin index).
 * Its scratch is a file-scope device array of HGB_SORT_STATIC_BYTES (24 MiB) per device, so
 * n_bins <= HGB_SORT_STATIC_MAX_BINS (2^20); larger inputs return HGB_ERR_CAPACITY with nothing
 * enqueued.  The first call on each device (with that device current) looks the array up with
 * cudaGetSymbolAddress, which loads the module: make that first call before any stream capture.
 * Every call on a device shares the one array, so calls that overlap in time (different streams
 * or host threads) race; the caller serialises them. */
#define HGB_SORT_STATIC_MAX_BINS 1048576L
#define HGB_SORT_STATIC_BYTES (24UL << 20)
int hgb_argsort_f0_desc_static(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *stream);

/* Poisson realizations with the loudest-L split.  Replaces cyutils.loudest_hc_from_sorted,
 * cyutils.pyx:1220-1344: for every realization r and frequency f the bins are visited in
 * `order`; each bin draws n ~ Poisson(number) (Normal(number, sqrt(number)) above 1e10),
 * the first `nloud` sources fill hc2ss[f, r, :] and the rest add n*h2fdf to hc2bg[f, r].
 * number / h2fdf are (B, F) (the (M-1, Q-1, Z-1, F) grids flattened); hc2ss is (F, R, L),
 * hc2bg (F, R), both fully written.
 * mode HGB_RNG_PHILOX: draws from Philox4x32-10 keyed by seed.
 * mode HGB_RNG_REPLAY: replay[(r*F + f)*B + k] is the draw of the k-th sorted bin. */
#define HGB_MAX_NREALS (65535L * 1024L)   /* realizations per call: 65535 grid rows of 1024 */
size_t hgb_loudest_workspace_bytes(long n_bins, int n_freq, int nreals, int nloud, int mode);
int hgb_loudest_hc_from_sorted(const double *number, const double *h2fdf, long n_bins, int n_freq,
                               int nreals, int nloud, const int32_t *order, int mode, uint64_t seed,
                               const double *replay, double *hc2ss, double *hc2bg,
                               void *workspace, size_t workspace_bytes, int *d_status, void *stream);

/* hgb_loudest_hc_from_sorted on a run of frequencies that starts at global frequency index
 * freq_offset: number / h2fdf / hc2ss / hc2bg hold only the n_freq frequencies of the run, and the
 * Philox counters use the global index, so splitting the frequencies over several calls gives the
 * same draws as one call (order is still the loudest-first order of the first global frequency). */
int hgb_loudest_hc_from_sorted_ex(const double *number, const double *h2fdf, long n_bins, int n_freq, int nreals,
                                  int nloud, const int32_t *order, int mode, uint64_t seed, const double *replay,
                                  double *hc2ss, double *hc2bg, void *workspace, size_t workspace_bytes,
                                  int *d_status, void *stream, int freq_offset);

/* hgb_loudest_hc_from_sorted (HGB_RNG_PHILOX, freq_offset 0) for many independent samples: the
 * realization stage of a library, where librarian/lib_tools.py:714-842 (run_model) calls
 * single_sources.ss_gws_redz -> cyutils.loudest_hc_from_sorted once per sample.  Each sample's
 * gather, scan and loudest slots run as in the single call; the bulk background of every sample
 * runs in ONE launch whose blocks take (sample, chunk, frequency, realization group) items from a
 * device work list.  Every sample's hc2ss / hc2bg equal those of its own hgb_loudest_hc_from_sorted
 * call with the same seed and the same hgb_set_bulk_waves setting, bit for bit.
 * samples: HOST array; each entry's arrays are device pointers as in hgb_loudest_hc_from_sorted,
 * all samples share n_freq and nloud, and each has its own workspace
 * (hgb_loudest_workspace_bytes(n_bins, n_freq, nreals, nloud, HGB_RNG_PHILOX)) and status word.
 * blocks_per_sm: 0 = one block per item (blocks retire as items finish, so kernels of other
 * streams interleave); 1..6 = a persistent grid of that many blocks per SM, each taking items
 * from an atomic counter.  workspace: hgb_loudest_batch_workspace_bytes(samples, ...) bytes for
 * the work list, written before the launch. */
typedef struct {
    const double *number;      /* (n_bins, n_freq) */
    const double *h2fdf;       /* (n_bins, n_freq) */
    const int32_t *order;      /* (n_bins) loudest-first order */
    long n_bins;
    int nreals;
    uint64_t seed;
    double *hc2ss;             /* (n_freq, nreals, nloud) */
    double *hc2bg;             /* (n_freq, nreals) */
    void *workspace;
    size_t workspace_bytes;
    int *d_status;             /* may be NULL */
} hgb_loudest_sample;
size_t hgb_loudest_batch_workspace_bytes(const hgb_loudest_sample *samples, int n_samples, int n_freq);
int hgb_loudest_hc_batch(const hgb_loudest_sample *samples, int n_samples, int n_freq, int nloud, int blocks_per_sm,
                         void *workspace, size_t workspace_bytes, void *stream);

/* Parameter grids of ss_gws_redz(params=True) (single_sources.py:117-143) on the (B, F) bins:
 * redz_mid = the redshift midpoints of redz_final along mtot, mrat, redz (-1 where <= 0),
 * dcom = comoving distance of redz_mid (+inf where it is -1), sepa = Kepler separation
 * (G mt / (2 pi fobs_orb_cent (1 + redz_mid))^2)^(1/3) with mt the bin-centre total mass, and
 * angs = sepa / (dcom / (1 + redz_mid)).  mt_cent (M-1) and fobs_orb_cent (F) are device arrays of
 * the axis midpoints; nwtg is the gravitational constant of holodeck.constants (astropy's).
 * scale_log2 (device int[4], may be NULL) receives, per output grid, the exponent e of
 * max |finite value| (frexp convention, over bins with a nonzero h2fdf when h2fdf is given). */
int hgb_param_grids(const double *mt_cent, int n_mtot, int n_mrat, int n_redz, const double *fobs_orb_cent,
                    int n_freq, const double *redz_final, double nwtg, const hgb_cosmo *cosmo,
                    const double *h2fdf, double *redz_mid, double *dcom, double *sepa, double *angs,
                    int *scale_log2, void *stream);

/* Loudest-L split with source parameters.  Replaces cyutils.loudest_hc_and_par_from_sorted_redz,
 * cyutils.pyx:1541-1770: as hgb_loudest_hc_from_sorted, but bins with h2fdf == 0 are skipped
 * (neither slots nor background), each filled slot also records
 * sspar[0..3, f, r, l] = (mt_cent[m], mr_cent[q], rz_cent[z], redz_mid[b, f]) of its bin
 * b = (m, q, z), and bgpar[k, f, r] = sum(n h2fdf p_k) / sum(n h2fdf) over the background
 * sources for the seven parameters p = (mt, mr, rz, redz_mid, dcom, sepa, angs) (0/0 = NaN as in
 * the reference).  The grids are the outputs of hgb_param_grids; scale_log2 (device int[7]: the
 * frexp exponents of max |p_k| for mt, mr, rz and the four grids) sets the FP32 scaling of the
 * Philox-mode background sums.  sspar is (4, F, R, L), bgpar (7, F, R).  Replay mode reproduces
 * the reference bit for bit. */
size_t hgb_loudest_par_workspace_bytes(long n_bins, int n_freq, int nreals, int nloud, int mode);
int hgb_loudest_hc_and_par_from_sorted(const double *number, const double *h2fdf, int n_m, int n_q, int n_z,
                                       int n_freq, int nreals, int nloud, const int32_t *order, int mode,
                                       uint64_t seed, const double *replay, const double *mt_cent,
                                       const double *mr_cent, const double *rz_cent, const double *redz_mid,
                                       const double *dcom, const double *sepa, const double *angs,
                                       const int *scale_log2, double *hc2ss, double *hc2bg, double *sspar,
                                       double *bgpar, void *workspace, size_t workspace_bytes, int *d_status,
                                       void *stream);

/* Model details of a library run.  Replaces librarian/lib_tools.py:845-943 (_calc_model_details):
 * with w = h2fdf * number on the (M-1, Q-1, Z-1, F) bins, gwb_m (M-1, Z-1, F), gwb_q (Q-1, Z-1, F)
 * and gwb_z (Z-1, F) are the sums of w over the other mass axes divided by denom[f] = sum(w);
 * gwb_rz (Z-1, F) and gwb_mrz (M-1, Z-1, F) bin w by the final redshift at bin centres over the
 * redz edges (scipy.stats.binned_statistic's rule); num_* are the same sums of number, undivided.
 * n_mtot, n_mrat, n_redz are edge counts; redz_final is (M, Q, Z, F); redz_edges (Z) device. */
int hgb_model_details(const double *number, const double *h2fdf, const double *redz_final, const double *redz_edges,
                      int n_mtot, int n_mrat, int n_redz, int n_freq, double *gwb_m, double *gwb_q, double *gwb_z,
                      double *gwb_rz, double *num_m, double *num_q, double *num_z, double *num_rz, double *gwb_mrz,
                      double *num_mrz, double *denom, void *stream);

/* No reference counterpart.  Measurement hook for the realization kernel: with enable != 0,
 * hgb_loudest_hc_from_sorted (HGB_RNG_PHILOX) records CUDA events on its stream immediately
 * before and after its bulk-background kernel, on the calling host thread.
 * hgb_bulk_last_ms() returns the time between the last recorded pair in ms (call it after
 * synchronising the stream), or -1 when nothing was recorded since hgb_bulk_timing(). */
int hgb_bulk_timing(int enable);
float hgb_bulk_last_ms(void);

/* No reference counterpart.  Schedule knob of the realization kernels, set by the batched-library
 * autotuner: the chunk count of k_bulk aims for `waves` waves of resident blocks (counted at six
 * per SM, the kernel's launch-bounds minimum; seven fit) over the device's SMs (default 12).
 * Applies to every later launch in the process; workspace sizes are always computed for
 * HGB_BULK_WAVES_MAX, so changing it never invalidates a workspace. */
#define HGB_BULK_WAVES_MAX 16
int hgb_set_bulk_waves(int waves);   /* 1 <= waves <= HGB_BULK_WAVES_MAX, else HGB_ERR_INVALID_ARGUMENT */
int hgb_get_bulk_waves(void);

/* Second-pass GWB without the loudest split.  Replaces cyutils.sam_poisson_gwb,
 * cyutils.pyx:854-897; gwb is (F, R).  replay[(b*F + f)*R + r] in REPLAY mode (no workspace needed). */
size_t hgb_sam_poisson_gwb_workspace_bytes(long n_bins, int n_freq, int nreals);
int hgb_sam_poisson_gwb(const double *number, const double *hc2, long n_bins, int n_freq, int nreals,
                        int mode, uint64_t seed, const double *replay, double *gwb,
                        void *workspace, size_t workspace_bytes, int *d_status, void *stream);

/* ---- Emulator MLP ensemble (no reference counterpart: the reference's emulators are Gaussian
 * processes, holodeck/gps/gp_utils.py; this network is trained on libraries the GPU SAM writes).
 * E members, each dims[0] -> dims[1] -> ... -> dims[n_layers] with SiLU after every layer but the
 * last.  Every width is a multiple of 16 in [16, 256] (inputs are zero-padded to 16).  Per member
 * the fp32 parameters are laid out layer by layer as W_l [dims[l+1]][dims[l]] (row-major) then
 * b_l [dims[l+1]] (P values, hgb_mlp_param_count); `weights` holds bf16 copies of the W_l only
 * (Pw values, hgb_mlp_weight_count), kept in step by hgb_mlp_adamw / hgb_mlp_pack_weights.
 * bf16 buffers are passed as uint16_t bit patterns.  Hidden activations live in buffers with a row
 * stride of 256: act and pre hold layers 0..n_layers-2 as [layer][member][batch][256] (bf16 and
 * fp32), out is [member][batch][dims[n_layers]] fp32.  All products accumulate in fp32 on the
 * tensor cores (tcgen05, accumulators in tensor memory). */
#define HGB_MLP_MAX_LAYERS 8
#define HGB_MLP_SPLIT_ROWS 128   /* batch rows per partial of a weight gradient */
typedef struct {
    int n_layers;
    int n_members;
    int dims[HGB_MLP_MAX_LAYERS + 1];
    const float *params;       /* fp32 [E][P] */
    const uint16_t *weights;   /* bf16 [E][Pw] */
} hgb_mlp;

long hgb_mlp_param_count(const hgb_mlp *net);    /* P, or -1 for an invalid description */
long hgb_mlp_weight_count(const hgb_mlp *net);   /* Pw, or -1 */
/* x: bf16 [batch][dims[0]] per member (x_member_stride elements apart; 0 = one input for all);
 * pre may be NULL (inference). */
int hgb_mlp_forward(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, uint16_t *act,
                    float *pre, float *out, int *d_status, void *stream);
/* The same outputs as hgb_mlp_forward (out [member][batch][dims[n_layers]]) for batch <=
 * HGB_MLP_FUSED_MAX_BATCH in ONE launch: a cluster of 8 CTAs per member holds every layer's
 * weights (bulk-copied into shared memory at the start) and the activations on chip, with the
 * products on the CUDA cores (fp32 sums, bf16 activations as in hgb_mlp_forward; the summation
 * order differs).  For query latency; no act / pre buffers.  `weights` must be 16-byte aligned.
 * x, out and d_status are accessed with plain loads and stores, so they may also be pinned host
 * memory; d_status's bit is set by a plain read-modify-write (do not share the word with kernels
 * that run concurrently). */
#define HGB_MLP_FUSED_MAX_BATCH 16
int hgb_mlp_forward_fused(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, float *out,
                          int *d_status, void *stream);
/* No reference counterpart.  One emulator query end to end on the calling host thread, for query
 * latency: params (HOST, [n_queries][n_params], n_queries <= HGB_MLP_FUSED_MAX_BATCH) are mapped to
 * 2 (p - lo) / (hi - lo) - 1, rounded to bf16 into x_host ([n_queries][dims[0]], zero-padded), the
 * fused forward runs on `stream` reading x_host and writing out_host ([member][n_queries][dims[L]])
 * and status_host, the stream is synchronised, and result (HOST, [n_queries][n_out], double) receives
 * mean over members of out * sd + mu for the first n_out outputs.  x_host, out_host and status_host
 * must be pinned (device-accessible) host memory; lo, hi (n_params), mu, sd (n_out) are host arrays.
 * Returns HGB_ERR_DEVICE_LIMIT when the kernel's bounded wait gave up (result not written). */
int hgb_emulator_query(const hgb_mlp *net, const double *params, int n_queries, int n_params, const double *lo,
                       const double *hi, const double *mu, const double *sd, int n_out, uint16_t *x_host,
                       float *out_host, int *status_host, double *result, void *stream);
size_t hgb_mlp_backward_workspace_bytes(const hgb_mlp *net, int batch);
/* Mean-squared-error loss against target [batch][dims[n_layers]] (target_member_stride apart) of the
 * outputs of the last hgb_mlp_forward (with pre): loss[e] (may be NULL) and grad [E][P] fp32. */
int hgb_mlp_backward(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, const uint16_t *act,
                     const float *pre, const float *out, const float *target, long target_member_stride,
                     float *grad, float *loss, void *workspace, size_t workspace_bytes, int *d_status,
                     void *stream);
/* Decoupled AdamW step `step` (>= 1) on params [E][P] with moments m1, m2 [E][P]; weights, not
 * biases, decay; writes the bf16 weight copies. */
int hgb_mlp_adamw(const hgb_mlp *net, float *params, const float *grad, float *m1, float *m2, uint16_t *weights,
                  int step, float lr, float beta1, float beta2, float eps, float weight_decay, void *stream);
int hgb_mlp_pack_weights(const hgb_mlp *net, const float *params, uint16_t *weights, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HOLODECK_GB300_H */
