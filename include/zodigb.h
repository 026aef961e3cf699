/*
 * zodigb.h — C ABI of the GB300 (sm_103a) zodiacal-light line-of-sight integrator.
 *
 * This library replaces the numeric core that ZodiPy runs below
 * `Model._evaluate` (zodipy/model.py:205-279): the per-component line-of-sight
 * range (zodipy/line_of_sight.py:64-105), the Gauss-Legendre quadrature
 * (zodipy/line_of_sight.py:55-61) of the Kelsall integrand
 * (zodipy/brightness.py:21-56) with the four Kelsall-98 densities
 * (zodipy/number_density.py:47-181) or of the Rowan-Robinson & May integrand
 * (zodipy/brightness.py:59-83) with its eight densities
 * (zodipy/number_density.py:184-404), the blackbody lookup
 * (zodipy/blackbody.py:16-30 + np.interp) and scattering
 * (zodipy/scattering.py:11-59).  Everything above that seam (units, frames,
 * ephemerides, spectral unpacking) stays in the host language.
 *
 * Conventions
 *  - Plain C types only.  Every array argument named *_dev is a CUDA device
 *    pointer owned by the caller; the library allocates nothing except where
 *    an entry point says so.
 *  - `stream` is a cudaStream_t passed as void*; all work is enqueued on it
 *    and no entry point synchronises.
 *  - Every entry point returns 0 on success or a negative ZL_ERR_* code; the
 *    message of the last failure on the calling thread is read with
 *    zl_last_error().  Nothing aborts the process.
 */
#ifndef ZODIGB_H
#define ZODIGB_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ZL_API __attribute__((visibility("default")))
#else
#define ZL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define ZL_ABI_VERSION 3

#define ZL_MAX_COMPS 8   /* components per model (DIRBE has 6) */
#define ZL_MAX_RANGES 8  /* distinct (inner, outer) cutoff pairs per model */
#define ZL_MAX_SPEC 4    /* spectral sets (wavelengths / bandpasses) fused in one launch */
#define ZL_MAX_NODES 128 /* Gauss-Legendre degree */
#define ZL_MAX_TEMPS 128 /* blackbody table length (the reference uses 100) */

/* Component type codes (zodipy/number_density.py:406-419). */
enum {
  ZL_CLOUD = 0, ZL_BAND = 1, ZL_RING = 2, ZL_FEATURE = 3,      /* Kelsall et al. (1998) */
  ZL_FAN = 4, ZL_COMET = 5, ZL_INTERSTELLAR = 6,               /* Rowan-Robinson & May (2013) */
  ZL_NARROW_BAND = 7, ZL_BROAD_BAND = 8, ZL_RING_RRM = 9, ZL_FEATURE_RRM = 10
};

/* Model families: the integrand (zodipy/zodiacal_light_model.py:70-102). */
enum {
  ZL_KELSALL = 0, /* (1-A) eps B(T) + A S Phi / R^2, one T_0/delta (brightness.py:21-56) */
  ZL_RRM = 1      /* B(T) x calibration, T_0/delta per component (brightness.py:59-83) */
};

/* Arithmetic of the integrand. */
enum {
  ZL_PREC_F64 = 0, /* plain method: float64 throughout, the GPU oracle */
  ZL_PREC_F32 = 1  /* float32 bulk; float-float geometry near the ring/feature, compensated sums */
};

enum {
  ZL_OK = 0,
  ZL_ERR_ARG = -1,    /* invalid argument (null pointer, size, layout) */
  ZL_ERR_CUDA = -2,   /* a CUDA runtime call failed */
  ZL_ERR_MODEL = -3,  /* model description out of range */
  ZL_ERR_SPACE = -4   /* caller-provided workspace too small */
};

/* One zodiacal component; geometry derived like zodipy/component.py:39-44. */
typedef struct ZlComponent {
  int32_t type;       /* ZL_CLOUD .. ZL_FEATURE_RRM */
  int32_t range;      /* index into ZlModel.cutoff */
  double offset[3];   /* x_0, y_0, z_0 [AU] */
  double sin_i, cos_i, sin_Omega, cos_Omega;
  double n_0;         /* unused by fan, comet, interstellar, narrow and broad band */
  /* own parameters, in the order of the reference's dataclass fields (component.py:47-204):
   * cloud:        alpha, beta, gamma, mu
   * band:         delta_zeta [rad], v, p, delta_r
   * ring:         R, sigma_r, sigma_z
   * feature:      R, sigma_r, sigma_z, theta [rad], sigma_theta [rad]
   * fan:          gamma, Z_0, Q, P, R_outer
   * comet:        gamma, Z_0, P, amp, R_inner, R_outer
   * interstellar: amp
   * narrow band:  gamma, A, G, R_inner, R_outer, beta_nb [deg]
   * broad band:   gamma, A, R_inner, R_outer, beta_bb [deg], sigma_bb [deg]
   * ring (RRM):   R, sigma_r, sigma_z, A
   * feature (RRM): R, sigma_r, sigma_z, theta [rad], sigma_theta [rad], A */
  double p[6];
} ZlComponent;

/* Spectral quantities of one wavelength / bandpass
 * (zodipy/unpack_model.py:23-107, zodipy/blackbody.py:33-49). */
typedef struct ZlSpectrum {
  double emissivity[ZL_MAX_COMPS];
  double albedo[ZL_MAX_COMPS];
  double C1, C2, C3;           /* phase-function coefficients */
  double solar_irradiance;     /* [MJy/sr] at 1 AU */
  double calibration;          /* ZL_RRM only: [Jy/cm] (unpack_model.py:121-131); Kelsall ignores it */
  double bb[ZL_MAX_TEMPS];     /* blackbody table [MJy/sr] at ZlModel.temps */
} ZlSpectrum;

/* A complete model evaluated at ZL_MAX_SPEC or fewer spectral sets.  For
 * ZL_KELSALL emissivity/albedo/C1..C3/solar_irradiance apply and T_0/delta are
 * shared; for ZL_RRM only calibration applies and T_0/delta are per component
 * (components that share a range must then share T_0 and delta too). */
typedef struct ZlModel {
  int32_t abi_version;         /* = ZL_ABI_VERSION */
  int32_t n_comps, n_ranges, n_spec, n_nodes, n_temps;
  int32_t family;              /* ZL_KELSALL or ZL_RRM */
  int32_t reserved;
  double T_0, delta;           /* T(R) = T_0 R^-delta (zodipy/blackbody.py:16-30), ZL_KELSALL */
  double comp_T_0[ZL_MAX_COMPS], comp_delta[ZL_MAX_COMPS]; /* per component, ZL_RRM */
  double cutoff[ZL_MAX_RANGES][2]; /* inner, outer cutoff radius [AU] (line_of_sight.py:19-26) */
  double temps[ZL_MAX_TEMPS];  /* table temperatures [K], uniformly spaced, increasing */
  double gl_x[ZL_MAX_NODES];   /* Gauss-Legendre nodes on [-1, 1] */
  double gl_w[ZL_MAX_NODES];   /* Gauss-Legendre weights */
  ZlComponent comp[ZL_MAX_COMPS];
  ZlSpectrum spec[ZL_MAX_SPEC];
} ZlModel;

/* One observer (one instant).  Pixels [pix_begin, next observer's pix_begin)
 * belong to it; the last observer runs to n_pix.  `outside` is filled by
 * zl_observer_flags(). */
typedef struct ZlObserver {
  double obs[3];      /* heliocentric ecliptic observer position [AU] */
  double earth[3];    /* heliocentric ecliptic Earth position [AU] */
  int64_t pix_begin;
  uint32_t outside;   /* bit 2r: start of range r collapses to eps; bit 2r+1: stop does */
  uint32_t reserved;
} ZlObserver;

/* Which kernel serves a call (ZlLaunch.kernel).  float32: AUTO, ONE_PIXEL, TWO_PIXEL,
 * PLAIN_GEOMETRY; float64 forward: AUTO (= ONE_PIXEL) or WARP_PER_PIXEL; adjoint: AUTO or
 * ONE_PIXEL.  Any other pairing is refused with ZL_ERR_ARG. */
enum {
  ZL_KERNEL_AUTO = 0,           /* the fastest measured kernel for the model's layout */
  ZL_KERNEL_ONE_PIXEL = 1,      /* one pixel per thread, components in order (forward and adjoint) */
  ZL_KERNEL_TWO_PIXEL = 2,      /* float32 forward: two pixels per thread on packed float32 (built-in layouts) */
  ZL_KERNEL_PLAIN_GEOMETRY = 3, /* float32 forward, DIRBE layout: all-float32 geometry (a precision study) */
  ZL_KERNEL_WARP_PER_PIXEL = 4  /* float64 forward: one warp per pixel, nodes across the lanes, shuffle
                                   sums (no work queue); the sum over nodes is associated differently
                                   from the reference's sequential sum (last bits) */
};

/* Launch options of one call (NULL = the defaults).  The library keeps no launch
 * state between calls: each call's options apply to that call only, so callers
 * with different options (an autotuner, another model) never affect each other.
 *
 * Work queue: with tile > 0 the forward's blocks pull tiles of `tile` items (pixels;
 * pixel pairs for the two-pixel kernel) from the counter queue_dev[0] until the
 * work runs out, instead of a fixed block-to-tile assignment.  queue_dev is two
 * uint32 words of device memory owned by the caller, zero before the first call;
 * each call leaves them zero again (the last block to finish resets them), so a
 * call can be replayed from a CUDA graph.  Calls that share a queue must not
 * overlap on the GPU.  No block waits for another.
 *
 * out_index_dev: pixel i's outputs go to column out_index_dev[i] (a permutation of
 * 0 .. n_pix-1) instead of column i; lets a caller evaluate its pixels in another
 * order (for example sorted by latitude, so that a warp's lines of sight are alike)
 * and still receive them in its own layout. */
typedef struct ZlLaunch {
  int32_t threads_per_block; /* 32 .. 128, a multiple of 32; 0 = 128 */
  int32_t blocks_per_sm;     /* cap of the grid in blocks per SM, 0 .. 65536; 0 = the default of the
                                entry point (float32 forward: one block per tile; float64 forward: 8;
                                adjoint: 96) */
  int32_t kernel;            /* ZL_KERNEL_* */
  int32_t band_tails;        /* two-pixel kernel: 1 = skip the bands' zero tails (coherent inputs:
                                a HEALPix ring, directions sorted by latitude), 0 = evaluate every
                                node (the default; no effect on the results, only on speed) */
  int32_t tile;              /* > 0: work-queue tile in items, a multiple of threads_per_block; 0 = no queue */
  int32_t reserved;
  uint32_t* queue_dev;       /* tile > 0: the queue's two words (see above) */
  const int64_t* out_index_dev; /* NULL or n_pix output columns */
} ZlLaunch;

/* Version of the library (== ZL_ABI_VERSION of the build). */
ZL_API int zl_abi_version(void);

/* Copy the message of the calling thread's last failure into buf (NUL-terminated). */
ZL_API int zl_last_error(char* buf, size_t len);

/* Check a model description; returns ZL_OK or ZL_ERR_MODEL with a message. */
ZL_API int zl_model_check(const ZlModel* model);

/* Fill ZlObserver.outside for n_obs host-side records, reproducing the rule
 * of zodipy/line_of_sight.py:72-73: a cutoff radius collapses to eps when the
 * observer lies strictly outside that sphere.  With any_mode != 0 the flags of
 * all records are OR-ed together, which is the reference's behaviour when one
 * call carries a position per pixel (time-ordered data). */
ZL_API int zl_observer_flags(const ZlModel* model, ZlObserver* obs_host, int64_t n_obs, int32_t any_mode);

/* Forward pass: the emission of every component at every pixel.
 * Replaces model.py:253-277 (and the sum of model.py:203).
 *  unit_vectors_dev: float64 [3][n_pix], heliocentric-ecliptic unit vectors (SoA)
 *  observers_dev:    n_obs ZlObserver records sorted by pix_begin, first = 0
 *  out_comps_dev:    float64 [n_spec][n_comps][n_pix] or NULL
 *  out_total_dev:    float64 [n_spec][n_pix] or NULL; the component sum in
 *                    component order, so it equals out_comps summed over axis 0
 *  precision:        ZL_PREC_F64 or ZL_PREC_F32 */
ZL_API int zl_forward(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
               const ZlObserver* observers_dev, int32_t n_obs, int32_t precision,
               double* out_comps_dev, double* out_total_dev, void* stream);

/* zl_forward with launch options (NULL = zl_forward).  Forward entry point for
 * autotuners and batched callers: launch shape, kernel choice, work queue and
 * output permutation per call (ZlLaunch). */
ZL_API int zl_forward_ex(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                         const ZlObserver* observers_dev, int32_t n_obs, int32_t precision, double* out_comps_dev,
                         double* out_total_dev, const ZlLaunch* launch, void* stream);

/* Forward pass for time-ordered data: one observer and one Earth position per
 * pixel (zodipy/model.py:119-203 with obstime.size == n_pix and obspos of shape
 * (3, n_pix)).  Replaces the same loop as zl_forward; the cutoff rule of
 * line_of_sight.py:72-73 is applied to the whole call (a range collapses to
 * eps for every pixel when any sample's observer lies outside it), as the
 * reference does.
 *  obs_xyz_dev, earth_xyz_dev: float64 [3][n_pix] heliocentric ecliptic [AU];
 *      earth_xyz_dev may be NULL when no component is a feature
 *  flags_dev: one uint32_t of device scratch; it receives the OR of the
 *      samples' cutoff flags (it is zeroed and filled on `stream` first) */
ZL_API int zl_forward_tod(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                          const double* obs_xyz_dev, const double* earth_xyz_dev, uint32_t* flags_dev,
                          int32_t precision, double* out_comps_dev, double* out_total_dev, void* stream);

/* ---- Adjoint -------------------------------------------------------------
 * Gradient of a loss L with respect to every model parameter, given the
 * upstream gradient dL/d(output) of the float32 forward pass (no counterpart
 * in the reference, which has no derivatives; parameters and their order follow
 * the reference's parameter dictionary, zodipy/zodiacal_light_model.py:38-55).
 * Gradient vector layout (float64):
 *   per component c, in model order: d/d x_0, y_0, z_0, i [deg], Omega [deg],
 *     n_0, then cloud: alpha, beta, gamma, mu | band: delta_zeta [deg], v, p,
 *     delta_r | ring: R, sigma_r, sigma_z | feature: R, sigma_r, sigma_z,
 *     theta [deg], sigma_theta [deg]
 *   d/d T_0, d/d delta
 *   per spectral set s: d/d emissivity[c] (c = 0..n_comps-1), d/d albedo[c],
 *     d/d C1, C2, C3, d/d solar_irradiance (the interpolated scalars)
 * for ZL_KELSALL models with the built-in component layouts (cloud, 3 bands[, ring,
 * feature]), and for ZL_RRM models (zodipy/zodiacal_light_model.py:90-102):
 *   per component c, in model order: d/d x_0, y_0, z_0, i [deg], Omega [deg], then
 *     the type's own parameters in ZlComponent order (fan: gamma, Z_0, Q, P, R_outer |
 *     comet: gamma, Z_0, P, amp, R_inner, R_outer | narrow band: gamma, A, G, R_inner,
 *     R_outer, beta_nb [deg] | broad band: gamma, A, R_inner, R_outer, beta_bb [deg],
 *     sigma_bb [deg] | interstellar: amp | ring: n_0, R, sigma_r, sigma_z, A |
 *     feature: n_0, R, sigma_r, sigma_z, theta [deg], sigma_theta [deg], A)
 *   d/d T_0 of every component, then d/d delta of every component
 *   d/d calibration of every spectral set
 * (a mask edge -- R_inner, R_outer, beta_nb where it cuts -- contributes nothing: the
 * quadrature's nodes do not move with it).  The sum over pixels is deterministic:
 * fixed 128-pixel tiles reduced in a fixed order, independent of the launch. */

/* Number of entries of the gradient vector for this model. */
ZL_API int zl_grad_count(const ZlModel* model, int32_t* count);

/* Device workspace zl_backward needs for n_pix pixels (the caller allocates it). */
ZL_API int zl_backward_workspace_bytes(const ZlModel* model, int64_t n_pix, size_t* bytes);

/* Backward pass.  Exactly one of
 *   g_comps_dev: float64 [n_spec][n_comps][n_pix]  dL/d out_comps
 *   g_total_dev: float64 [n_spec][n_pix]            dL/d out_total
 * is non-NULL.  grad_out_dev receives zl_grad_count() float64 values
 * (overwritten, not accumulated).  workspace_dev holds at least
 * zl_backward_workspace_bytes() bytes; ZL_ERR_SPACE if it is smaller. */
ZL_API int zl_backward(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                       const ZlObserver* observers_dev, int32_t n_obs, const double* g_comps_dev,
                       const double* g_total_dev, double* grad_out_dev, void* workspace_dev,
                       size_t workspace_bytes, void* stream);

/* zl_backward with launch options (NULL = zl_backward): blocks_per_sm and kernel
 * (ZL_KERNEL_AUTO or ZL_KERNEL_ONE_PIXEL) apply; the adjoint's 128-pixel tiles are
 * fixed, and the gradient does not depend on the options (same bits). */
ZL_API int zl_backward_ex(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                          const ZlObserver* observers_dev, int32_t n_obs, const double* g_comps_dev,
                          const double* g_total_dev, double* grad_out_dev, void* workspace_dev, size_t workspace_bytes,
                          const ZlLaunch* launch, void* stream);

/* Backward pass without a caller-allocated workspace, for callers that cannot
 * allocate device memory (a host that owns all device memory through its own
 * pool, an allocation-free real-time loop, a binding without an allocator).
 * No counterpart in the reference.  Same inputs and outputs as zl_backward;
 * the scratch is a 32 MiB array inside the library, held by every GPU that
 * loads it until exit.  Returns ZL_ERR_SPACE when zl_backward_workspace_bytes()
 * exceeds 32 MiB (single-band DIRBE: up to 3.4 million pixels).  Calls that
 * overlap on the GPU share the array and race: serialise them.  The first call
 * on a device looks up the array's address; make it before any stream capture.
 * That address is kept for the life of the process: after cudaDeviceReset() (or
 * anything else that destroys the device's primary context) it no longer holds,
 * so a process that resets a device must not call zl_backward_static again. */
ZL_API int zl_backward_static(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                              const ZlObserver* observers_dev, int32_t n_obs, const double* g_comps_dev,
                              const double* g_total_dev, double* grad_out_dev, void* stream);

/* zl_backward for time-ordered data (positions and flags as zl_forward_tod). */
ZL_API int zl_backward_tod(const ZlModel* model, const double* unit_vectors_dev, int64_t n_pix,
                           const double* obs_xyz_dev, const double* earth_xyz_dev, uint32_t* flags_dev,
                           const double* g_comps_dev, const double* g_total_dev, double* grad_out_dev,
                           void* workspace_dev, size_t workspace_bytes, void* stream);

/* ---- Time-ordered inputs on the device (zodipy/model.py:177-180, bodies.py:16-50) ---- */

/* Positions at n sample times from a cubic spline through n_knots ascending
 * knots: replaces the evaluation of scipy's CubicSpline in
 * get_interp_bodypos (bodies.py:22-35).  coef_dev is the piecewise polynomial
 * the host builds over the knots, float64 [4][n_knots-1][3] with the cubic
 * coefficient first (scipy's PPoly.c layout for a (3, n_knots) array
 * interpolated along its last axis).  The value at t is the power sum of
 * interval j (knots[j] <= t < knots[j+1]; ends extrapolate), accumulated from
 * the constant term up as scipy does.  out_dev: float64 [3][n]. */
ZL_API int zl_spline_eval(const double* knots_dev, int32_t n_knots, const double* coef_dev, const double* t_dev,
                          int64_t n, double* out_dev, void* stream);

#define ZL_SEMB_L2_SCRATCH 1024 /* doubles of scratch zl_semb_l2 needs with whole_array_norm */

/* SEMB-L2 observer (bodies.py:38-50): Earth's direction from the Sun scaled
 * to |E| + l2_distance.  With whole_array_norm == 0, |E| is each sample's own
 * distance (the reference's result for a single time); with whole_array_norm
 * != 0, |E| is the norm of the whole [3][n] array, which is what the
 * reference's numpy.linalg.norm(earthpos) computes for a sequence of times.
 * The second form needs scratch_dev of ZL_SEMB_L2_SCRATCH doubles. */
ZL_API int zl_semb_l2(const double* earth_xyz_dev, int64_t n, double l2_distance, int32_t whole_array_norm,
                      double* scratch_dev, int64_t scratch_len, double* out_dev, void* stream);

/* Unit vectors of (lon, lat) [rad] rotated into the ecliptic frame:
 * u = R (cos lat cos lon, cos lat sin lon, sin lat), R a row-major 3x3 host
 * matrix (NULL = identity).  Replaces the frame transform of model.py:244-251
 * for frames that differ from the ecliptic by a fixed rotation (ICRS,
 * Galactic).  unit_vectors_dev: float64 [3][n]. */
ZL_API int zl_directions(const double* lon_dev, const double* lat_dev, int64_t n, const double* rotation_host,
                         double* unit_vectors_dev, void* stream);

/* Number densities of every component on a Cartesian mesh, float64
 * (replaces the evaluation loop of zodipy/number_density.py:482-536).
 * x_dev[nx], y_dev[ny], z_dev[nz]: heliocentric ecliptic coordinates [AU];
 * earth_xyz_host[3]: Earth's position (the feature's longitude origin);
 * out_dev: float64 [n_comps][ny][nx][nz], the layout of
 * numpy.meshgrid(x, y, z) with its default 'xy' indexing. */
ZL_API int zl_density_grid(const ZlModel* model, const double* x_dev, int32_t nx, const double* y_dev, int32_t ny,
                           const double* z_dev, int32_t nz, const double* earth_xyz_host, double* out_dev,
                           void* stream);

/* Device address of page-locked host memory (cudaHostGetDevicePointer).  On
 * GPUs that reach host memory over a coherent link (Grace-Blackwell NVLink-C2C)
 * the kernels can read their inputs from and write their outputs to such
 * memory directly: pass the returned pointers to zl_forward instead of device
 * buffers.  Returns ZL_ERR_CUDA when the memory is not mapped. */
ZL_API int zl_mapped_pointer(const void* host_ptr, void** dev_ptr);

/* Diagnostics: launch a pipe-throughput probe on `stream` (which = 0: MUFU
 * ex2, which = 1: FP32 FMA, which = 2: packed FP32 FMA counted per FMA), `iters` iterations of 8 independent chains per
 * thread; *ops_per_launch receives the number of probe instructions.  The
 * caller times the launch.  sink_dev must hold >= 8 * SM-count floats. */
ZL_API int zl_diag_pipe_probe(int32_t which, int32_t iters, float* sink_dev, int32_t sink_len,
                              double* ops_per_launch, void* stream);

/* Diagnostics: out[i] = the kernels' branch-free float32 atan2(y[i], x[i]) (the
 * per-node angle of the feature and of scattering), n device floats each, on
 * `stream`.  For checking it against a reference atan2. */
ZL_API int zl_diag_atan2(const float* y_dev, const float* x_dev, float* out_dev, int64_t n, void* stream);

/* Diagnostics: the kernels' conversion of doubles without float64 instructions.  For
 * each of n device doubles d[i], out[3i], out[3i+1] receive the float-float pair (hi, lo)
 * the kernels split d[i] into and out[3i+2] the float value they round d[i] to (an
 * upstream gradient's conversion); out holds 3n device floats.  For checking them
 * against the conversion instruction. */
ZL_API int zl_diag_d2f(const double* d_dev, float* out_dev, int64_t n, void* stream);

/* Diagnostics: the kernels' float-to-double conversion of their results without float64
 * instructions: out[i] = (double)f[i] for n device floats.  For checking it against the
 * conversion instruction. */
ZL_API int zl_diag_f2d(const float* f_dev, double* out_dev, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ZODIGB_H */
