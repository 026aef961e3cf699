// C ABI of the line-of-sight integrator (declared in include/zodigb.h).
//
// Host code only: argument validation, derivation of the per-launch kernel
// parameter blocks from a ZlModel, and kernel launch on the caller's stream.
// No entry point allocates device memory or synchronises.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "zl_common.cuh"

namespace zl {
cudaError_t launch_fwd_f64(const KParamsF64& P, bool warp, const double* u, int64_t n, const ObsArgs& obs,
                           double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);
cudaError_t launch_fwd_f32(const KParamsF32& P, int layout, int kernel, bool tails, const double* u, int64_t n,
                           const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);
int grad_count_layout(int layout, int n_spec);
int bwd_groups(int layout);
cudaError_t launch_bwd_f32(const KParamsF32& P, const KGradAux& A, int layout, bool unpaired, const double* u,
                           int64_t n, const ObsArgs& obs, const double* g_comps, const double* g_total,
                           double* partials, int64_t n_tiles, cudaStream_t st, int bps, int num_sms);
cudaError_t launch_reduce_tiles(const double* partials, int64_t n_rows, int ng, double* out, cudaStream_t st);
int rrm_grad_count(const ZlModel& m);
cudaError_t launch_bwd_rrm(const ZlModel& m, const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs,
                           const double* g_comps, const double* g_total, double* partials, int64_t n_tiles,
                           double* grad_out, cudaStream_t st, int bps, int num_sms);
constexpr int kRrmPartialSlots = 20;  // doubles per component and tile (zl_bwd_rrm.cu)
cudaError_t launch_tod_flags(const ZlModel& m, const double* obs, int64_t n, uint32_t* flags, cudaStream_t st,
                             int num_sms);
cudaError_t launch_density_grid(const ZlModel& M, const double* x, int nx, const double* y, int ny, const double* z,
                                int nz, double ex, double ey, double* out, cudaStream_t st, int num_sms);
}  // namespace zl

using namespace zl;

namespace {
thread_local char g_err[512] = "";
}  // namespace

namespace zl {
// Record the calling thread's last error (read back with zl_last_error) and return code.
int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}
}  // namespace zl

namespace {

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(ZL_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// blocks per SM large enough that every launcher's grid reaches its cap of one block per
// 128 pixels (or tiles) for any map below ~1.3e9 pixels; bounds the grid at 152 x 65536 blocks
constexpr int kBpsOnePixelPerThread = 1 << 16;
constexpr int kMaxQueueTile = 1 << 20;

// SM count of the current device, queried once per device and cached so that
// launches recorded into a CUDA graph make no device queries.
int sm_count(int* out) {
  static int cache[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev >= 0 && dev < 64 && cache[dev] > 0) {
    *out = cache[dev];
    return ZL_OK;
  }
  e = cudaDeviceGetAttribute(out, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  if (dev >= 0 && dev < 64) cache[dev] = *out;
  return ZL_OK;
}

bool is_finite(double x) { return std::isfinite(x); }

void split(double d, float* hi, float* lo) {
  *hi = (float)d;
  *lo = (float)(d - (double)*hi);
}

}  // namespace

extern "C" ZL_API int zl_abi_version(void) { return ZL_ABI_VERSION; }

extern "C" ZL_API int zl_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return ZL_ERR_ARG;
  strncpy(buf, g_err, len - 1);
  buf[len - 1] = '\0';
  return ZL_OK;
}

extern "C" ZL_API int zl_model_check(const ZlModel* m) {
  if (!m) return fail(ZL_ERR_ARG, "model is NULL");
  if (m->abi_version != ZL_ABI_VERSION)
    return fail(ZL_ERR_MODEL, "model abi_version %d != library %d", m->abi_version, ZL_ABI_VERSION);
  if (m->n_comps < 1 || m->n_comps > ZL_MAX_COMPS) return fail(ZL_ERR_MODEL, "n_comps=%d out of [1,%d]", m->n_comps, ZL_MAX_COMPS);
  if (m->n_ranges < 1 || m->n_ranges > ZL_MAX_RANGES) return fail(ZL_ERR_MODEL, "n_ranges=%d out of [1,%d]", m->n_ranges, ZL_MAX_RANGES);
  if (m->n_spec < 1 || m->n_spec > ZL_MAX_SPEC) return fail(ZL_ERR_MODEL, "n_spec=%d out of [1,%d]", m->n_spec, ZL_MAX_SPEC);
  if (m->n_nodes < 1 || m->n_nodes > ZL_MAX_NODES) return fail(ZL_ERR_MODEL, "n_nodes=%d out of [1,%d]", m->n_nodes, ZL_MAX_NODES);
  if (m->n_temps < 2 || m->n_temps > ZL_MAX_TEMPS) return fail(ZL_ERR_MODEL, "n_temps=%d out of [2,%d]", m->n_temps, ZL_MAX_TEMPS);
  for (int t = 1; t < m->n_temps; ++t)
    if (!(m->temps[t] > m->temps[t - 1])) return fail(ZL_ERR_MODEL, "temps must increase (index %d)", t);
  const double dt = (m->temps[m->n_temps - 1] - m->temps[0]) / (m->n_temps - 1);
  for (int t = 0; t < m->n_temps; ++t)
    if (std::fabs(m->temps[t] - (m->temps[0] + t * dt)) > 1e-9 * std::fabs(m->temps[m->n_temps - 1]))
      return fail(ZL_ERR_MODEL, "temps must be uniformly spaced (index %d)", t);
  if (m->family != ZL_KELSALL && m->family != ZL_RRM) return fail(ZL_ERR_MODEL, "bad model family %d", m->family);
  for (int c = 0; c < m->n_comps; ++c) {
    const ZlComponent& C = m->comp[c];
    if (C.type < ZL_CLOUD || C.type > ZL_FEATURE_RRM) return fail(ZL_ERR_MODEL, "component %d: bad type %d", c, C.type);
    if (C.range < 0 || C.range >= m->n_ranges) return fail(ZL_ERR_MODEL, "component %d: range %d out of [0,%d)", c, C.range, m->n_ranges);
    if (m->family == ZL_RRM)
      for (int j = 0; j < c; ++j)
        if (m->comp[j].range == C.range && (m->comp_T_0[j] != m->comp_T_0[c] || m->comp_delta[j] != m->comp_delta[c]))
          return fail(ZL_ERR_MODEL, "components %d and %d share range %d but not T_0/delta", j, c, C.range);
  }
  for (int r = 0; r < m->n_ranges; ++r)
    if (!(m->cutoff[r][0] >= 0.0) || !is_finite(m->cutoff[r][1]) || !(m->cutoff[r][1] > 0.0))
      return fail(ZL_ERR_MODEL, "range %d: bad cutoffs (%g, %g)", r, m->cutoff[r][0], m->cutoff[r][1]);
  return ZL_OK;
}

extern "C" ZL_API int zl_observer_flags(const ZlModel* m, ZlObserver* obs, int64_t n_obs, int32_t any_mode) {
  int rc = zl_model_check(m);
  if (rc) return rc;
  if (!obs || n_obs < 1) return fail(ZL_ERR_ARG, "observers: NULL or n_obs < 1");
  uint32_t all = 0;
  for (int64_t o = 0; o < n_obs; ++o) {
    const double* p = obs[o].obs;
    // line_of_sight.py:71-73
    const double r_obs = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    uint32_t f = 0;
    for (int r = 0; r < m->n_ranges; ++r) {
      if (r_obs > m->cutoff[r][0]) f |= 1u << (2 * r);
      if (r_obs > m->cutoff[r][1]) f |= 1u << (2 * r + 1);
    }
    obs[o].outside = f;
    all |= f;
  }
  if (any_mode)
    for (int64_t o = 0; o < n_obs; ++o) obs[o].outside = all;
  return ZL_OK;
}

namespace {

// A call's launch options, checked, with the defaults filled in (NULL = all defaults).
int launch_options(const ZlLaunch* in, ZlLaunch* out) {
  ZlLaunch d;
  memset(&d, 0, sizeof(d));
  if (in) d = *in;
  if (d.threads_per_block == 0) d.threads_per_block = 128;
  if (d.threads_per_block < 32 || d.threads_per_block > 128 || d.threads_per_block % 32)
    return fail(ZL_ERR_ARG, "threads_per_block %d not in {32..128 step 32}", d.threads_per_block);
  if (d.blocks_per_sm < 0 || d.blocks_per_sm > kBpsOnePixelPerThread)
    return fail(ZL_ERR_ARG, "blocks_per_sm %d out of [0,%d]", d.blocks_per_sm, kBpsOnePixelPerThread);
  if (d.kernel < ZL_KERNEL_AUTO || d.kernel > ZL_KERNEL_WARP_PER_PIXEL) return fail(ZL_ERR_ARG, "bad kernel %d", d.kernel);
  if (d.band_tails != 0 && d.band_tails != 1) return fail(ZL_ERR_ARG, "band_tails %d not 0 or 1", d.band_tails);
  if (d.tile < 0 || d.tile > kMaxQueueTile) return fail(ZL_ERR_ARG, "tile %d out of [0,%d]", d.tile, kMaxQueueTile);
  if (d.tile > 0 && (d.tile % d.threads_per_block))
    return fail(ZL_ERR_ARG, "tile %d is not a multiple of threads_per_block %d", d.tile, d.threads_per_block);
  if (d.tile > 0 && !d.queue_dev) return fail(ZL_ERR_ARG, "tile > 0 needs queue_dev");
  if (d.tile == 0) d.queue_dev = nullptr;
  *out = d;
  return ZL_OK;
}

void first_in_range(const ZlModel& m, int32_t* out) {
  for (int c = 0; c < m.n_comps; ++c) out[c] = (c == 0 || m.comp[c].range != m.comp[c - 1].range) ? 1 : 0;
}

// 1 = DIRBE-like (cloud | 3 bands on one range | ring | feature), 2 = Planck-like, 3 = the
// registry's RRM arrangement (Lay<kLayoutRRM>), 0 = generic
int detect_layout(const ZlModel& m) {
  if (m.family == ZL_RRM) {
    static const int rrm_t[8] = {ZL_FAN, ZL_COMET, ZL_NARROW_BAND, ZL_NARROW_BAND, ZL_BROAD_BAND, ZL_INTERSTELLAR,
                                 ZL_RING_RRM, ZL_FEATURE_RRM};
    static const int rrm_r[8] = {0, 1, 2, 2, 2, 3, 4, 5};
    if (m.n_comps != 8) return 0;
    for (int c = 0; c < 8; ++c)
      if (m.comp[c].type != rrm_t[c] || m.comp[c].range != rrm_r[c]) return 0;
    return 3;
  }
  if (m.family != ZL_KELSALL) return 0;
  int32_t first[ZL_MAX_COMPS];
  first_in_range(m, first);
  static const int dirbe_t[6] = {ZL_CLOUD, ZL_BAND, ZL_BAND, ZL_BAND, ZL_RING, ZL_FEATURE};
  static const int dirbe_f[6] = {1, 0, 0, 0, 1, 1};
  static const int dirbe_r[6] = {0, 0, 0, 0, 1, 2};
  if (m.n_comps == 6) {
    bool ok = true;
    for (int c = 0; c < 6; ++c)
      ok = ok && m.comp[c].type == dirbe_t[c] && first[c] == dirbe_f[c] && m.comp[c].range == dirbe_r[c];
    if (ok) return 1;
  }
  if (m.n_comps == 4) {
    bool ok = true;
    for (int c = 0; c < 4; ++c)
      ok = ok && m.comp[c].type == dirbe_t[c] && first[c] == dirbe_f[c] && m.comp[c].range == dirbe_r[c];
    if (ok) return 2;
  }
  return 0;
}

void build_f64(const ZlModel& m, KParamsF64* P) {
  memset(P, 0, sizeof(*P));
  P->m = m;
  for (int s = 0; s < m.n_spec; ++s) {
    for (int t = 0; t + 1 < m.n_temps; ++t)
      P->slope[s][t] = (m.spec[s].bb[t + 1] - m.spec[s].bb[t]) / (m.temps[t + 1] - m.temps[t]);
    const double C1 = m.spec[s].C1, C2 = m.spec[s].C2, C3 = m.spec[s].C3;
    // scattering.py:53-59
    const double t1 = 2 * M_PI, t2 = 2 * C1, t3 = M_PI * C2, t4 = (std::exp(C3 * M_PI) + 1) / (C3 * C3 + 1);
    P->phase_norm[s] = 1 / (t1 * (t2 + t3 + t4));
  }
  first_in_range(m, P->first_in_range);
  for (int c = 0; c < m.n_comps; ++c) {
    const int r = m.comp[c].range;
    P->range_T0[r] = m.family == ZL_RRM ? m.comp_T_0[c] : m.T_0;
    P->range_delta[r] = m.family == ZL_RRM ? m.comp_delta[c] : m.delta;
    if (m.family == ZL_KELSALL)
      for (int s = 0; s < m.n_spec; ++s)
        if (m.spec[s].albedo[c] != 0.0) P->range_scat[r] = 1;
  }
}

void build_f32(const ZlModel& m, KParamsF32* P) {
  memset(P, 0, sizeof(*P));
  const double L2E = 1.4426950408889634;
  P->n_comps = m.n_comps;
  P->n_ranges = m.n_ranges;
  P->n_spec = m.n_spec;
  P->n_nodes = m.n_nodes;
  P->n_temps = m.n_temps;
  P->T0 = (float)m.T_0;
  P->neg_delta = (float)(-m.delta);
  P->neg_half_delta = (float)(-0.5 * m.delta);
  P->t_min = (float)m.temps[0];
  P->t_max = (float)m.temps[m.n_temps - 1];
  P->inv_dt = (float)((m.n_temps - 1) / (m.temps[m.n_temps - 1] - m.temps[0]));
  for (int r = 0; r < m.n_ranges; ++r) {
    P->cut_in[r] = m.cutoff[r][0];
    P->cut_out[r] = m.cutoff[r][1];
    split(m.cutoff[r][0] * m.cutoff[r][0], &P->cut_in_hi[r], &P->cut_in_lo[r]);
    split(m.cutoff[r][1] * m.cutoff[r][1], &P->cut_out_hi[r], &P->cut_out_lo[r]);
  }
  for (int k = 0; k < m.n_nodes; ++k) {
    split(m.gl_x[k], &P->gl_x_hi[k], &P->gl_x_lo[k]);
    P->gl_w[k] = (float)m.gl_w[k];
  }
  int32_t first[ZL_MAX_COMPS];
  first_in_range(m, first);
  for (int c = 0; c < m.n_comps; ++c) {
    const ZlComponent& C = m.comp[c];
    KCompF32& K = P->comp[c];
    K.type = C.type;
    K.range = C.range;
    K.first_in_range = first[c];
    K.zero_offset = (C.offset[0] == 0.0 && C.offset[1] == 0.0 && C.offset[2] == 0.0) ? 1 : 0;
    K.share_t4 = -1;
    K.T0 = (float)(m.family == ZL_RRM ? m.comp_T_0[c] : m.T_0);
    K.neg_delta = (float)(-(m.family == ZL_RRM ? m.comp_delta[c] : m.delta));
    if (C.type == ZL_BAND)
      for (int j = 0; j < c; ++j) {
        const ZlComponent& Cj = m.comp[j];
        if (Cj.type == ZL_BAND && Cj.range == C.range && Cj.p[3] == C.p[3] && Cj.offset[0] == C.offset[0] &&
            Cj.offset[1] == C.offset[1] && Cj.offset[2] == C.offset[2]) {
          K.share_t4 = j;
          break;
        }
      }
    // same symmetry plane and centre as the previous component (the ring and the Earth-trailing
    // feature): the kernels keep that component's plane projections
    K.same_plane_prev = 0;
    if (c > 0) {
      const ZlComponent& Cp = m.comp[c - 1];
      K.same_plane_prev = (Cp.sin_Omega == C.sin_Omega && Cp.cos_Omega == C.cos_Omega && Cp.sin_i == C.sin_i &&
                           Cp.cos_i == C.cos_i && Cp.offset[0] == C.offset[0] && Cp.offset[1] == C.offset[1] &&
                           Cp.offset[2] == C.offset[2])
                              ? 1
                              : 0;
    }
    split(C.sin_Omega * C.sin_i, &K.nx, &K.nx_lo);
    split(-C.cos_Omega * C.sin_i, &K.ny, &K.ny_lo);
    split(C.cos_i, &K.nz, &K.nz_lo);
    split(C.offset[0], &K.ox, &K.ox_lo);
    split(C.offset[1], &K.oy, &K.oy_lo);
    split(C.offset[2], &K.oz, &K.oz_lo);
    const double* p = C.p;
    switch (C.type) {
      case ZL_CLOUD:
        K.c[0] = (float)C.n_0;
        K.c[1] = (float)p[0];
        K.c[2] = (float)(p[1] * L2E);
        K.c[3] = (float)p[2];
        K.c[4] = (float)p[3];
        K.c[5] = (float)(1.0 / (2.0 * p[3]));
        K.c[6] = (float)(p[3] / 2.0);
        K.c[7] = (float)(-0.5 * p[0]);
        break;
      case ZL_BAND:
        K.c[0] = (float)(3.0 * C.n_0);
        K.c[1] = (float)(1.0 / p[0]);
        K.c[2] = (float)(1.0 / p[1]);
        K.c[3] = (float)p[2];
        K.c[4] = (float)(1.0 / (p[3] * p[3]));
        K.c[5] = (p[2] == 4.0) ? 1.0f : 0.0f;
        break;
      case ZL_RING:
      case ZL_FEATURE:
      case ZL_RING_RRM:
      case ZL_FEATURE_RRM:
        K.c[0] = (float)(C.type == ZL_RING_RRM ? p[3] * C.n_0 : C.type == ZL_FEATURE_RRM ? p[5] * C.n_0 : C.n_0);
        K.c[1] = (float)p[0];
        K.c[2] = (float)(L2E / (p[1] * p[1]));
        K.c[3] = (float)(L2E / p[2]);
        split(p[0] * p[0], &K.c[4], &K.c[5]);
        if (featurelike(C.type)) {
          K.c[6] = (float)p[3];
          K.c[7] = (float)(L2E / (p[4] * p[4]));
        }
        break;
      case ZL_INTERSTELLAR:
        K.c[0] = (float)p[0];
        break;
      case ZL_FAN:  // gamma, Z_0, Q, P, R_outer
        K.c[0] = 1.0f;
        K.c[1] = (float)(-p[0]);
        K.c[2] = (float)(0.5 * p[2]);
        K.c[3] = (float)(-p[3] * L2E);
        K.c[4] = (float)(1.0 / p[1]);
        split(p[4] * p[4], &K.c[10], &K.c[11]);
        break;
      case ZL_COMET:  // gamma, Z_0, P, amp, R_inner, R_outer
        K.c[0] = (float)p[3];
        K.c[1] = (float)(-p[0]);
        K.c[3] = (float)(-p[2] * L2E);
        K.c[4] = (float)(1.0 / p[1]);
        split(p[4] * p[4], &K.c[8], &K.c[9]);
        split(p[5] * p[5], &K.c[10], &K.c[11]);
        break;
      case ZL_NARROW_BAND: {  // gamma, A, G, R_inner, R_outer, beta_nb [deg]
        K.c[0] = (float)p[1];
        K.c[1] = (float)(-p[0]);
        K.c[2] = (float)(p[2] * L2E);
        K.c[3] = (float)p[5];
        K.c[5] = (float)(p[0] * std::log2(p[4]));
        // |beta| < beta_nb  <=>  (Z/R)^2 < sin^2(beta_nb) for beta_nb in (0, 90]
        const double sb = p[5] <= 0.0 ? 0.0 : (p[5] >= 90.0 ? 1.0 : std::sin(p[5] * (M_PI / 180.0)));
        split(sb * sb, &K.c[6], &K.c[7]);
        split(p[3] * p[3], &K.c[8], &K.c[9]);
        split(p[4] * p[4], &K.c[10], &K.c[11]);
        break;
      }
      case ZL_BROAD_BAND:  // gamma, A, R_inner, R_outer, beta_bb [deg], sigma_bb [deg]
        K.c[0] = (float)p[1];
        K.c[1] = (float)(-p[0]);
        K.c[2] = (float)p[4];
        K.c[3] = (float)(1.0 / p[5]);
        K.c[5] = (float)(p[0] * std::log2(p[3]));
        split(p[2] * p[2], &K.c[8], &K.c[9]);
        split(p[3] * p[3], &K.c[10], &K.c[11]);
        break;
    }
  }
  for (int s = 0; s < m.n_spec; ++s) {
    const ZlSpectrum& S = m.spec[s];
    KSpecF32& K = P->spec[s];
    for (int c = 0; c < m.n_comps; ++c) {
      const double c0 = (double)P->comp[c].c[0];  // density prefactor (n_0, 3 n_0, A, amp ...)
      if (m.family == ZL_RRM) {  // brightness.py:83: B(T) n calibration
        K.em1[c] = (float)S.calibration;
        K.alb[c] = 0.f;
        K.outer[c] = (float)(c0 * S.calibration);
        K.outer_alb[c] = 0.f;
        continue;
      }
      K.em1[c] = (float)((1.0 - S.albedo[c]) * S.emissivity[c]);
      K.alb[c] = (float)S.albedo[c];
      K.outer[c] = (float)(c0 * ((1.0 - S.albedo[c]) * S.emissivity[c]));
      K.outer_alb[c] = (float)(c0 * S.albedo[c]);
      if (S.albedo[c] != 0.0) P->has_scat = 1;
    }
    const double t1 = 2 * M_PI, t2 = 2 * S.C1, t3 = M_PI * S.C2, t4 = (std::exp(S.C3 * M_PI) + 1) / (S.C3 * S.C3 + 1);
    K.C1 = (float)S.C1;
    K.C2 = (float)S.C2;
    K.C3l2e = (float)(S.C3 * L2E);
    K.S = (float)S.solar_irradiance;
    K.N = (float)(1 / (t1 * (t2 + t3 + t4)));
    for (int t = 0; t < m.n_temps; ++t) {
      const double slope = (t + 1 < m.n_temps) ? (S.bb[t + 1] - S.bb[t]) / (m.temps[t + 1] - m.temps[t]) : 0.0;
      P->table[s][t] = make_float4((float)m.temps[t], (float)S.bb[t], (float)slope, 0.f);
    }
  }
}

}  // namespace

namespace {

// zl_forward / zl_forward_ex / zl_forward_tod after the observer source is set up.
int forward_impl(const ZlModel* model, const double* u, int64_t n_pix, const ObsArgs& OA, int32_t precision,
                 double* out_comps, double* out_total, const ZlLaunch* launch, void* stream) {
  int rc = 0;
  if (!u) return fail(ZL_ERR_ARG, "unit_vectors is NULL");
  if (!out_comps && !out_total) return fail(ZL_ERR_ARG, "both outputs are NULL");
  if (precision != ZL_PREC_F64 && precision != ZL_PREC_F32) return fail(ZL_ERR_ARG, "bad precision %d", precision);
  ZlLaunch opt;
  if ((rc = launch_options(launch, &opt))) return rc;
  // the queue's counter is 32-bit: every tile plus each block's final fetch must fit
  if (opt.queue_dev && n_pix / opt.tile >= (int64_t)1 << 30)
    return fail(ZL_ERR_ARG, "%lld pixels in tiles of %d overflow the work queue", (long long)n_pix, opt.tile);
  int nsm = 0;
  if ((rc = sm_count(&nsm))) return rc;
  LaunchArgs L{opt.threads_per_block, opt.blocks_per_sm, nsm, Sched{opt.queue_dev, opt.tile, opt.out_index_dev}};
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (precision == ZL_PREC_F64) {
    static thread_local KParamsF64 P;
    build_f64(*model, &P);
    const bool warp = opt.kernel == ZL_KERNEL_WARP_PER_PIXEL;
    if (opt.kernel != ZL_KERNEL_AUTO && opt.kernel != ZL_KERNEL_ONE_PIXEL && !warp)
      return fail(ZL_ERR_ARG, "the float64 forward has no kernel %d", opt.kernel);
    if (warp && opt.queue_dev) return fail(ZL_ERR_ARG, "the warp-per-pixel kernel takes no work queue");
    if (!L.bps) L.bps = 8;
    e = launch_fwd_f64(P, warp, u, n_pix, OA, out_comps, out_total, st, L);
  } else {
    static thread_local KParamsF32 P;
    build_f32(*model, &P);
    // default: one block per tile (one pixel or pixel pair per thread) without a queue.  Pixels
    // cost different amounts (a warp whose pixels are all past a band's zero tail skips it), so
    // many short blocks balance the SMs better than a few long-running ones (DIRBE 25 um at nside
    // 512: 1.48 ms with 8 blocks per SM, 1.33 ms); a queued launch defaults to 8 blocks per SM.
    if (opt.kernel == ZL_KERNEL_WARP_PER_PIXEL) return fail(ZL_ERR_ARG, "the float32 forward has no warp-per-pixel kernel");
    if (!L.bps) L.bps = opt.queue_dev ? 8 : kBpsOnePixelPerThread;
    e = launch_fwd_f32(P, detect_layout(*model), opt.kernel, opt.band_tails != 0, u, n_pix, OA, out_comps, out_total,
                       st, L);
  }
  if (e != cudaSuccess) return cuda_fail(e, "zl_forward launch");
  return ZL_OK;
}

bool needs_earth(const ZlModel& m) {
  for (int c = 0; c < m.n_comps; ++c)
    if (featurelike(m.comp[c].type)) return true;
  return false;
}

// Checks and flag reduction shared by the time-ordered entry points.
int tod_setup(const ZlModel* model, int64_t n_pix, const double* obs_xyz, const double* earth_xyz, uint32_t* flags,
              void* stream, ObsArgs* OA) {
  if (!obs_xyz || !flags) return fail(ZL_ERR_ARG, "obs_xyz or flags is NULL");
  if (!earth_xyz && needs_earth(*model)) return fail(ZL_ERR_ARG, "earth_xyz is NULL but the model has a feature");
  int nsm = 0, rc = 0;
  if ((rc = sm_count(&nsm))) return rc;
  cudaError_t e = launch_tod_flags(*model, obs_xyz, n_pix, flags, (cudaStream_t)stream, nsm);
  if (e != cudaSuccess) return cuda_fail(e, "cutoff flags launch");
  *OA = ObsArgs{nullptr, 0, obs_xyz, earth_xyz, flags};
  return ZL_OK;
}

}  // namespace

extern "C" ZL_API int zl_forward(const ZlModel* model, const double* u, int64_t n_pix, const ZlObserver* obs, int32_t n_obs,
                          int32_t precision, double* out_comps, double* out_total, void* stream) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (n_pix < 0) return fail(ZL_ERR_ARG, "n_pix < 0");
  if (n_pix == 0) return ZL_OK;
  if (!u) return fail(ZL_ERR_ARG, "unit_vectors is NULL");
  if (!obs || n_obs < 1) return fail(ZL_ERR_ARG, "observers: NULL or n_obs < 1");
  const ObsArgs OA{obs, n_obs, nullptr, nullptr, nullptr};
  return forward_impl(model, u, n_pix, OA, precision, out_comps, out_total, nullptr, stream);
}

extern "C" ZL_API int zl_forward_ex(const ZlModel* model, const double* u, int64_t n_pix, const ZlObserver* obs,
                                    int32_t n_obs, int32_t precision, double* out_comps, double* out_total,
                                    const ZlLaunch* launch, void* stream) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (n_pix < 0) return fail(ZL_ERR_ARG, "n_pix < 0");
  if (n_pix == 0) return ZL_OK;
  if (!u) return fail(ZL_ERR_ARG, "unit_vectors is NULL");
  if (!obs || n_obs < 1) return fail(ZL_ERR_ARG, "observers: NULL or n_obs < 1");
  const ObsArgs OA{obs, n_obs, nullptr, nullptr, nullptr};
  return forward_impl(model, u, n_pix, OA, precision, out_comps, out_total, launch, stream);
}

extern "C" ZL_API int zl_forward_tod(const ZlModel* model, const double* u, int64_t n_pix, const double* obs_xyz,
                                     const double* earth_xyz, uint32_t* flags, int32_t precision, double* out_comps,
                                     double* out_total, void* stream) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (n_pix < 0) return fail(ZL_ERR_ARG, "n_pix < 0");
  if (n_pix == 0) return ZL_OK;
  if (!u) return fail(ZL_ERR_ARG, "unit_vectors is NULL");
  if (!out_comps && !out_total) return fail(ZL_ERR_ARG, "both outputs are NULL");
  if (precision != ZL_PREC_F64 && precision != ZL_PREC_F32) return fail(ZL_ERR_ARG, "bad precision %d", precision);
  ObsArgs OA;
  if ((rc = tod_setup(model, n_pix, obs_xyz, earth_xyz, flags, stream, &OA))) return rc;
  return forward_impl(model, u, n_pix, OA, precision, out_comps, out_total, nullptr, stream);
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
namespace {

constexpr int kBwdTile = 128;

int64_t bwd_tiles(int64_t n_pix) { return (n_pix + kBwdTile - 1) / kBwdTile; }

// Adjoint kernel family of a model: the Kelsall layouts 1 (DIRBE) and 2 (Planck), or -1 for an
// RRM model (one launch per component, zl_bwd_rrm.cu).
int bwd_layout(const ZlModel& m, int* layout) {
  if (m.family == ZL_RRM) {
    *layout = -1;
    return ZL_OK;
  }
  const int l = detect_layout(m);
  if (l == 0)
    return fail(ZL_ERR_MODEL,
                "the adjoint supports the built-in component layouts (cloud, 3 bands[, ring, feature]); "
                "this model has %d components in another arrangement", m.n_comps);
  *layout = l;
  return ZL_OK;
}

void build_aux(const ZlModel& m, KGradAux* A) {
  memset(A, 0, sizeof(*A));
  const double deg = M_PI / 180.0;
  for (int c = 0; c < m.n_comps; ++c) {
    const ZlComponent& C = m.comp[c];
    A->dni[c][0] = (float)(C.sin_Omega * C.cos_i * deg);
    A->dni[c][1] = (float)(-C.cos_Omega * C.cos_i * deg);
    A->dni[c][2] = (float)(-C.sin_i * deg);
    A->dnO[c][0] = (float)(C.cos_Omega * C.sin_i * deg);
    A->dnO[c][1] = (float)(C.sin_Omega * C.sin_i * deg);
    A->n0[c] = (float)(C.type == ZL_BAND ? 3.0 * C.n_0 : C.n_0);  // the density's prefactor (bands: 3 n_0)
    const double* p = C.p;
    // derivative constants, with every division done here in float64
    switch (C.type) {
      case ZL_CLOUD:  // alpha, beta, gamma, mu, 1/mu
        for (int k = 0; k < 4; ++k) A->q[c][k] = (float)p[k];
        A->q[c][4] = (float)(1.0 / p[3]);
        break;
      case ZL_BAND:  // delta_zeta [deg], v, p, delta_r, 1/delta_zeta [deg], -20/delta_r
        A->q[c][0] = (float)(p[0] / deg);
        A->q[c][1] = (float)p[1];
        A->q[c][2] = (float)p[2];
        A->q[c][3] = (float)p[3];
        A->q[c][4] = (float)(deg / p[0]);
        A->q[c][5] = (float)(-20.0 / p[3]);
        break;
      default:  // R, 1/sigma_r^2, 1/sigma_z, 2/sigma_r^3, 1/sigma_z^2, 1/sigma_theta^2, 2 deg/sigma_theta^3
        A->q[c][0] = (float)p[0];
        A->q[c][1] = (float)(1.0 / (p[1] * p[1]));
        A->q[c][2] = (float)(1.0 / p[2]);
        A->q[c][3] = (float)(2.0 / (p[1] * p[1] * p[1]));
        A->q[c][4] = (float)(1.0 / (p[2] * p[2]));
        if (C.type == ZL_FEATURE) {
          A->q[c][5] = (float)(1.0 / (p[4] * p[4]));
          A->q[c][6] = (float)(2.0 * deg / (p[4] * p[4] * p[4]));
        }
    }
    for (int s = 0; s < m.n_spec; ++s) {
      A->eps[s][c] = (float)m.spec[s].emissivity[c];
      A->one_m_alb[s][c] = (float)(1.0 - m.spec[s].albedo[c]);
    }
  }
  for (int s = 0; s < m.n_spec; ++s) {
    // phase normalisation N = 1 / (2 pi I) (scattering.py:53-59) and dN/dC_j = -2 pi N^2 dI/dC_j
    const double C1 = m.spec[s].C1, C2 = m.spec[s].C2, C3 = m.spec[s].C3;
    const double e = std::exp(M_PI * C3), d = C3 * C3 + 1;
    const double I = 2 * C1 + M_PI * C2 + (e + 1) / d;
    const double N = 1 / (2 * M_PI * I);
    const double k = -2 * M_PI * N * N;
    A->dN[s][0] = (float)(k * 2);
    A->dN[s][1] = (float)(k * M_PI);
    A->dN[s][2] = (float)(k * (M_PI * e * d - 2 * C3 * (e + 1)) / (d * d));
  }
}

}  // namespace

extern "C" ZL_API int zl_grad_count(const ZlModel* model, int32_t* count) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (!count) return fail(ZL_ERR_ARG, "count is NULL");
  int layout = 0;
  if ((rc = bwd_layout(*model, &layout))) return rc;
  *count = layout < 0 ? rrm_grad_count(*model) : grad_count_layout(layout, model->n_spec);
  return ZL_OK;
}

extern "C" ZL_API int zl_backward_workspace_bytes(const ZlModel* model, int64_t n_pix, size_t* bytes) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (!bytes || n_pix < 0) return fail(ZL_ERR_ARG, "bytes is NULL or n_pix < 0");
  int layout = 0;
  if ((rc = bwd_layout(*model, &layout))) return rc;
  if (layout < 0) {
    *bytes = (size_t)model->n_comps * (size_t)bwd_tiles(n_pix) * kRrmPartialSlots * sizeof(double);
    return ZL_OK;
  }
  const int ng = grad_count_layout(layout, model->n_spec);
  *bytes = (size_t)bwd_groups(layout) * (size_t)bwd_tiles(n_pix) * ng * sizeof(double);
  return ZL_OK;
}

namespace {

int backward_impl(const ZlModel* model, int layout, const double* u, int64_t n_pix, const ObsArgs& OA,
                  const double* g_comps, const double* g_total, double* grad_out, void* workspace,
                  size_t workspace_bytes, const ZlLaunch* launch, void* stream) {
  int rc = 0;
  ZlLaunch opt;
  if ((rc = launch_options(launch, &opt))) return rc;
  if (opt.kernel != ZL_KERNEL_AUTO && opt.kernel != ZL_KERNEL_ONE_PIXEL)
    return fail(ZL_ERR_ARG, "the adjoint has no kernel %d", opt.kernel);
  size_t need = 0;
  if ((rc = zl_backward_workspace_bytes(model, n_pix, &need))) return rc;
  if (workspace_bytes < need || (need > 0 && !workspace))
    return fail(ZL_ERR_SPACE, "workspace of %zu bytes is smaller than the %zu required", workspace_bytes, need);
  int nsm = 0;
  if ((rc = sm_count(&nsm))) return rc;
  // default: 96 blocks per SM, 1.7 tiles per block at nside 512 (per-tile cost varies as in the
  // forward; 2.62 ms with 4 blocks per SM, 2.39 ms)
  const int bps = opt.blocks_per_sm > 0 ? opt.blocks_per_sm : 96;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n_tiles = bwd_tiles(n_pix);
  double* partials = (double*)workspace;
  static thread_local KParamsF32 P;
  build_f32(*model, &P);
  if (layout < 0) {  // RRM: one launch per component, then the fixed-order reduction
    if (n_tiles == 0) {
      const cudaError_t z = cudaMemsetAsync(grad_out, 0, sizeof(double) * rrm_grad_count(*model), st);
      return z == cudaSuccess ? ZL_OK : cuda_fail(z, "zl_backward zero gradient");
    }
    const cudaError_t er = launch_bwd_rrm(*model, P, u, n_pix, OA, g_comps, g_total, partials, n_tiles, grad_out, st,
                                          bps, nsm);
    return er == cudaSuccess ? ZL_OK : cuda_fail(er, "zl_backward launch (RRM)");
  }
  const int ng = grad_count_layout(layout, model->n_spec);
  static thread_local KGradAux A;
  build_aux(*model, &A);
  cudaError_t e = cudaSuccess;
  if (n_tiles > 0)
    e = launch_bwd_f32(P, A, layout, opt.kernel == ZL_KERNEL_ONE_PIXEL, u, n_pix, OA, g_comps, g_total, partials,
                       n_tiles, st, bps, nsm);
  if (e != cudaSuccess) return cuda_fail(e, "zl_backward launch");
  e = launch_reduce_tiles(partials, n_tiles * bwd_groups(layout), ng, grad_out, st);
  if (e != cudaSuccess) return cuda_fail(e, "zl_backward reduce");
  return ZL_OK;
}

int backward_args(const ZlModel* model, const double* u, int64_t n_pix, const double* g_comps, const double* g_total,
                  double* grad_out, int* layout) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if ((rc = bwd_layout(*model, layout))) return rc;
  if (n_pix < 0) return fail(ZL_ERR_ARG, "n_pix < 0");
  if (!grad_out) return fail(ZL_ERR_ARG, "grad_out is NULL");
  if (n_pix > 0 && !u) return fail(ZL_ERR_ARG, "unit_vectors is NULL");
  if ((g_comps == nullptr) == (g_total == nullptr)) return fail(ZL_ERR_ARG, "pass exactly one of g_comps, g_total");
  return ZL_OK;
}

}  // namespace

extern "C" ZL_API int zl_backward(const ZlModel* model, const double* u, int64_t n_pix, const ZlObserver* obs,
                                  int32_t n_obs, const double* g_comps, const double* g_total, double* grad_out,
                                  void* workspace, size_t workspace_bytes, void* stream) {
  int layout = 0;
  int rc = backward_args(model, u, n_pix, g_comps, g_total, grad_out, &layout);
  if (rc) return rc;
  if (!obs || n_obs < 1) return fail(ZL_ERR_ARG, "observers: NULL or n_obs < 1");
  const ObsArgs OA{obs, n_obs, nullptr, nullptr, nullptr};
  return backward_impl(model, layout, u, n_pix, OA, g_comps, g_total, grad_out, workspace, workspace_bytes, nullptr,
                       stream);
}

extern "C" ZL_API int zl_backward_ex(const ZlModel* model, const double* u, int64_t n_pix, const ZlObserver* obs,
                                     int32_t n_obs, const double* g_comps, const double* g_total, double* grad_out,
                                     void* workspace, size_t workspace_bytes, const ZlLaunch* launch, void* stream) {
  int layout = 0;
  int rc = backward_args(model, u, n_pix, g_comps, g_total, grad_out, &layout);
  if (rc) return rc;
  if (!obs || n_obs < 1) return fail(ZL_ERR_ARG, "observers: NULL or n_obs < 1");
  const ObsArgs OA{obs, n_obs, nullptr, nullptr, nullptr};
  return backward_impl(model, layout, u, n_pix, OA, g_comps, g_total, grad_out, workspace, workspace_bytes, launch,
                       stream);
}

extern "C" ZL_API int zl_backward_tod(const ZlModel* model, const double* u, int64_t n_pix, const double* obs_xyz,
                                      const double* earth_xyz, uint32_t* flags, const double* g_comps,
                                      const double* g_total, double* grad_out, void* workspace,
                                      size_t workspace_bytes, void* stream) {
  int layout = 0;
  int rc = backward_args(model, u, n_pix, g_comps, g_total, grad_out, &layout);
  if (rc) return rc;
  ObsArgs OA{nullptr, 0, nullptr, nullptr, nullptr};
  if (n_pix > 0 && (rc = tod_setup(model, n_pix, obs_xyz, earth_xyz, flags, stream, &OA))) return rc;
  return backward_impl(model, layout, u, n_pix, OA, g_comps, g_total, grad_out, workspace, workspace_bytes, nullptr,
                       stream);
}

// ---------------------------------------------------------------------------
// Densities on a mesh
// ---------------------------------------------------------------------------
extern "C" ZL_API int zl_density_grid(const ZlModel* model, const double* x, int32_t nx, const double* y, int32_t ny,
                                      const double* z, int32_t nz, const double* earth_xyz, double* out,
                                      void* stream) {
  int rc = zl_model_check(model);
  if (rc) return rc;
  if (nx < 0 || ny < 0 || nz < 0) return fail(ZL_ERR_ARG, "negative grid size");
  if ((int64_t)nx * ny * nz == 0) return ZL_OK;
  if (!x || !y || !z || !out || !earth_xyz) return fail(ZL_ERR_ARG, "NULL pointer argument");
  int nsm = 0;
  if ((rc = sm_count(&nsm))) return rc;
  cudaError_t e = launch_density_grid(*model, x, nx, y, ny, z, nz, earth_xyz[0], earth_xyz[1], out,
                                      (cudaStream_t)stream, nsm);
  if (e != cudaSuccess) return cuda_fail(e, "zl_density_grid launch");
  return ZL_OK;
}

// ---------------------------------------------------------------------------
// Host memory the device can address directly
// ---------------------------------------------------------------------------
extern "C" ZL_API int zl_mapped_pointer(const void* host_ptr, void** dev_ptr) {
  if (!host_ptr || !dev_ptr) return fail(ZL_ERR_ARG, "NULL pointer argument");
  void* d = nullptr;
  const cudaError_t e = cudaHostGetDevicePointer(&d, const_cast<void*>(host_ptr), 0);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // not mapped: clear the error state and report
    *dev_ptr = nullptr;
    return fail(ZL_ERR_CUDA, "host pointer is not mapped for device access: %s", cudaGetErrorName(e));
  }
  *dev_ptr = d;
  return ZL_OK;
}
