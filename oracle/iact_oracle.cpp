// ORACLE — test infrastructure only (see iact_oracle.hpp). C entry points
// over the templated restatement: FP64 (the oracle) and FP32 (the index
// restatement, multi-threaded as the timed CPU baseline).
//
// All descriptor pointers are HOST pointers here; the descriptor layout is
// the product's C ABI (include/iactrace_gb300.h) so the same packed tables
// feed the CUDA path and this oracle.
#include <omp.h>

#include <cstdio>
#include <vector>

#include "iact_oracle.hpp"

using namespace oracle;

namespace {

bool scene_ok(const iact_scene_t* sc, const iact_sensor_t* sn, int S) {
  if (!sc || !sn || S < 0) return false;
  if (sc->n_facets < 0 || sc->n_samples < 0) return false;
  if (sn->n_pixels <= 0) return false;
  return true;
}

template <typename T>
void deposit_ray(const iact_sensor_t& sn, T x, T y, T v, T* row) {
  if (sn.type == IACT_SENSOR_SQUARE || sn.type == IACT_SENSOR_HEX) {
    int32_t p = bin_hard<T>(sn, x, y, nullptr);
    if (p >= 0) row[p] += v;
  } else if (sn.type == IACT_SENSOR_SOFT_SQUARE) {
    splat_square<T>(sn, x, y, v, [&](int32_t p, T w) { row[p] += w; });
  } else {
    splat_hex<T>(sn, x, y, v, [&](int32_t p, T w) { row[p] += w; });
  }
}

// core/render.py:174-220 render (mode IMAGE) and :271-324
// render_response_matrix (mode RESPONSE); the facet sum order is the
// reference's lax.scan order when n_threads == 1.
template <typename T>
int render_impl(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                const float* values, int S, int mode, T* out, int n_threads, uint32_t seed) {
  const int SS = src_type == IACT_SRC_EXTENDED ? 4 : 3;
  if (!scene_ok(sc, sn, S)) return IACT_E_INVALID;
  const size_t P = (size_t)sn->n_pixels;
  const size_t F = (size_t)sc->n_facets, M = (size_t)sc->n_samples;
  const size_t rows = (mode == IACT_MODE_RESPONSE) ? (size_t)S : 1;
  std::fill(out, out + rows * P, T(0));
  if (F == 0 || M == 0 || S == 0) return IACT_OK;
  World<T> w = transform_to_world<T>(*sc);
  Prepared<T> pr = prepare<T>(*sc, *sn);
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  if (mode == IACT_MODE_RESPONSE) {
    // each thread owns whole source rows: no reduction needed
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
    for (int s = 0; s < S; ++s) {
      T* row = out + (size_t)s * P;
      for (size_t f = 0; f < F; ++f) {
        for (size_t m = 0; m < M; ++m) {
          RayOut<T> r = trace_ray<T>(*sc, pr, w, f * M + m, src_type, sources + SS * s, T(values[s]), seed, s);
          deposit_ray<T>(*sn, r.x, r.y, r.val, row);
        }
      }
    }
    return IACT_OK;
  }
  // image: per-thread accumulators over facets, summed at the end
  std::vector<std::vector<T>> acc((size_t)n_threads, std::vector<T>(P, T(0)));
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
  for (long f = 0; f < (long)F; ++f) {
    T* img = acc[(size_t)omp_get_thread_num()].data();
    for (int s = 0; s < S; ++s)
      for (size_t m = 0; m < M; ++m) {
        RayOut<T> r = trace_ray<T>(*sc, pr, w, (size_t)f * M + m, src_type, sources + SS * s, T(values[s]),
                                   seed, s);
        deposit_ray<T>(*sn, r.x, r.y, r.val, img);
      }
  }
  for (int t = 0; t < n_threads; ++t)
    for (size_t p = 0; p < P; ++p) out[p] += acc[(size_t)t][p];
  return IACT_OK;
}

// core/render.py:223-268 render_debug, ray = (f*S + s)*M + m
template <typename T>
int debug_impl(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
               const float* values, int S, T* pts, T* vals, int32_t* pix, int32_t* hit_mirror,
               T* margin, uint32_t seed) {
  const int SS = src_type == IACT_SRC_EXTENDED ? 4 : 3;
  if (!scene_ok(sc, sn, S)) return IACT_E_INVALID;
  const size_t F = (size_t)sc->n_facets, M = (size_t)sc->n_samples;
  if (F == 0 || M == 0 || S == 0) return IACT_OK;
  World<T> w = transform_to_world<T>(*sc);
  Prepared<T> pr = prepare<T>(*sc, *sn);
#pragma omp parallel for schedule(static)
  for (long f = 0; f < (long)F; ++f)
    for (int s = 0; s < S; ++s)
      for (size_t m = 0; m < M; ++m) {
        size_t i = ((size_t)f * S + s) * M + m;
        RayOut<T> r = trace_ray<T>(*sc, pr, w, (size_t)f * M + m, src_type, sources + SS * s, T(values[s]),
                                   seed, s);
        pts[2 * i] = r.x;
        pts[2 * i + 1] = r.y;
        vals[i] = r.val;
        T mg = 0;
        int32_t p = -1;
        if (sn->type == IACT_SENSOR_SQUARE || sn->type == IACT_SENSOR_HEX ||
            sn->type == IACT_SENSOR_SOFT_SQUARE || sn->type == IACT_SENSOR_SOFT_HEX) {
          iact_sensor_t hard = *sn;
          if (hard.type == IACT_SENSOR_SOFT_SQUARE) hard.type = IACT_SENSOR_SQUARE;
          if (hard.type == IACT_SENSOR_SOFT_HEX) hard.type = IACT_SENSOR_HEX;
          p = bin_hard<T>(hard, r.x, r.y, &mg);
        }
        if (pix) pix[i] = p;
        if (hit_mirror) hit_mirror[i] = r.hit_mirror;
        if (margin) margin[i] = mg;
      }
  return IACT_OK;
}

}  // namespace

extern "C" {

int oracle_render_f64(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                      const float* sources, const float* values, int S, int mode, double* out,
                      int n_threads, uint32_t seed) {
  return render_impl<double>(sc, sn, src_type, sources, values, S, mode, out, n_threads, seed);
}

int oracle_render_f32(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                      const float* sources, const float* values, int S, int mode, float* out,
                      int n_threads, uint32_t seed) {
  return render_impl<float>(sc, sn, src_type, sources, values, S, mode, out, n_threads, seed);
}

int oracle_render_debug_f64(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                            const float* sources, const float* values, int S, double* pts,
                            double* vals, int32_t* pix, int32_t* hit_mirror, double* margin,
                            uint32_t seed) {
  return debug_impl<double>(sc, sn, src_type, sources, values, S, pts, vals, pix, hit_mirror, margin, seed);
}

int oracle_render_debug_f32(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                            const float* sources, const float* values, int S, float* pts,
                            float* vals, int32_t* pix, int32_t* hit_mirror, float* margin,
                            uint32_t seed) {
  return debug_impl<float>(sc, sn, src_type, sources, values, S, pts, vals, pix, hit_mirror, margin, seed);
}

// telescope/mirrors.py:64-79 transform_to_world, for direct checks
int oracle_transform_f64(const iact_scene_t* sc, double* tp, double* tn, double* tw) {
  World<double> w = transform_to_world<double>(*sc);
  for (size_t i = 0; i < w.tw.size(); ++i) {
    tp[3 * i] = w.tp[i].x;
    tp[3 * i + 1] = w.tp[i].y;
    tp[3 * i + 2] = w.tp[i].z;
    tn[3 * i] = w.tn[i].x;
    tn[3 * i + 1] = w.tn[i].y;
    tn[3 * i + 2] = w.tn[i].z;
    tw[i] = w.tw[i];
  }
  return IACT_OK;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

// core/integrators.py:97-187 MCIntegrator.sample_group with the device
// sampler's counter-based variates (include/iactrace_gb300.h,
// iact_sample_facets), replayed in FP64 on host arrays: utils/sampling.py:8-67
// (disk, area-weighted fan triangles), core/surfaces.py:25-65 (point, normal
// through the analytic sag gradient), core/reflection.py:22-49 (delta),
// weights cos_z / area * n_samples.
int oracle_sample_facets(const iact_sampler_t* s, double* pts, double* nrm, double* dlt, double* wts) {
  const int F = s->n_facets, M = s->n_samples;
  const double c = s->curvature, k = s->conic;
  auto sag = [&](double r2) {
    double z = r2 * c / (1.0 + std::sqrt(1.0 - (1.0 + k) * c * c * r2));
    for (int i = 0; i < s->n_asph; ++i) z += (double)s->asph[i] * std::pow(r2, 2 * (i + 1));
    return z;
  };
  auto sag_dr2 = [&](double r2) {
    const double alpha = (1.0 + k) * c * c, q = std::sqrt(1.0 - alpha * r2), den = 1.0 + q;
    double dz = c / den + (r2 * c) * alpha / (2.0 * q * den * den);
    for (int i = 0; i < s->n_asph; ++i) dz += (double)s->asph[i] * (2.0 * (i + 1)) * std::pow(r2, 2 * (i + 1) - 1);
    return dz;
  };
  const double sc = 1.0 / 16777216.0;
  for (int f = 0; f < F; ++f)
    for (int m = 0; m < M; ++m) {
      const size_t i = (size_t)f * M + m;
      uint32_t w[4] = {(uint32_t)m, (uint32_t)f, 0x5A3D1u, 0u};
      philox4x32_10(w, s->seed, 0x53414D50u);
      const double u0 = (w[0] >> 8) * sc, u1 = (w[1] >> 8) * sc, u2 = (w[2] >> 8) * sc;
      double x, y, area;
      if (s->aperture == IACT_APERTURE_DISK) {
        const double R = s->radii[f], r = std::sqrt(u0) * R, th = 2.0 * M_PI * u1;
        x = r * std::cos(th);
        y = r * std::sin(th);
        area = M_PI * R * R;
      } else {
        const float* v = s->vertices + (size_t)f * s->n_vert * 2;
        const int nt = s->n_vert - 2;
        std::vector<double> ar(nt);
        double tot = 0.0;
        for (int t = 0; t < nt; ++t) {
          ar[t] = std::fabs((v[2 * t + 2] - (double)v[0]) * (v[2 * t + 5] - (double)v[1]) -
                            (v[2 * t + 4] - (double)v[0]) * (v[2 * t + 3] - (double)v[1])) / 2.0;
          tot += ar[t];
        }
        int idx = 0;
        double cdf = 0.0;
        for (int t = 0; t < nt; ++t) {
          cdf += ar[t] / tot;
          if (cdf <= u0) ++idx;
        }
        idx = std::min(idx, nt - 1);
        const double u = std::sqrt(u1), a = 1.0 - u, b = u * (1.0 - u2), cc = u * u2;
        x = a * v[0] + b * v[2 * idx + 2] + cc * v[2 * idx + 4];
        y = a * v[1] + b * v[2 * idx + 3] + cc * v[2 * idx + 5];
        double sh = 0.0;
        for (int j = 0; j < s->n_vert; ++j) {
          const int jn = (j + 1) % s->n_vert;
          sh += (double)v[2 * j] * v[2 * jn + 1] - (double)v[2 * jn] * v[2 * j + 1];
        }
        area = 0.5 * std::fabs(sh);
      }
      const double ox = s->offsets[2 * f], oy = s->offsets[2 * f + 1];
      const double xs = x + ox, ys = y + oy;
      const double z = sag(xs * xs + ys * ys) - sag(ox * ox + oy * oy);
      const double g = sag_dr2(xs * xs + ys * ys);
      double n[3] = {-(g * 2.0 * xs), -(g * 2.0 * ys), 1.0};
      const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (double& e : n) e /= nn;
      uint32_t w2[4] = {(uint32_t)m, (uint32_t)f, 0x5A3D1u, 1u};
      philox4x32_10(w2, s->seed, 0x53414D50u);
      const double v1 = ((w2[0] >> 8) + 1u) * sc, v2 = (w2[1] >> 8) * sc;
      const double rad = std::sqrt(-2.0 * std::log(v1));
      const double th1 = rad * std::cos(2.0 * M_PI * v2), th2 = rad * std::sin(2.0 * M_PI * v2);
      const double ref[3] = {std::fabs(n[2]) > 0.9 ? 1.0 : 0.0, 0.0, std::fabs(n[2]) > 0.9 ? 0.0 : 1.0};
      double t1[3] = {n[1] * ref[2] - n[2] * ref[1], n[2] * ref[0] - n[0] * ref[2], n[0] * ref[1] - n[1] * ref[0]};
      const double tn = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
      for (double& e : t1) e /= tn;
      const double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
      pts[3 * i] = x;
      pts[3 * i + 1] = y;
      pts[3 * i + 2] = z;
      for (int a = 0; a < 3; ++a) {
        nrm[3 * i + a] = n[a];
        dlt[3 * i + a] = th1 * t1[a] + th2 * t2[a];
      }
      wts[i] = n[2] / area * M;
    }
  return IACT_OK;
}

}  // extern "C"
