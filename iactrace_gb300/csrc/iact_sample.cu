// Monte-Carlo facet sampling on the device (core/integrators.py:97-187
// MCIntegrator.sample_group), one thread per (facet, sample).
//
// Variates: Philox4x32-10 with key (seed, 0x53414D50) and counters
// (m, f, 0x5A3D1, 0) -> aperture position, (m, f, 0x5A3D1, 1) -> the two
// N(0, 1) roughness coefficients (Box-Muller). Uniforms are the top 24 bits
// of a word scaled by 2^-24. The arithmetic is FP64 (sampling runs once per
// scene, F*M threads) and the arrays are stored as float32, as the reference
// stores them.
#include <cuda_runtime.h>

#include <cmath>

#include "iact_device.cuh"
#include "iact_internal.h"

namespace iact {

struct SamplerK {
  int F, M, aperture, n_vert, n_asph;
  double c, k, asph[IACT_MAX_ASPH];
  const float* offsets;
  const float* radii;
  const float* vertices;
  uint32_t seed;
};

// core/surfaces.py:25-39 _sag_raw and d/d(r2), FP64 (IEEE square root and division)
__device__ __forceinline__ double smp_sag(const SamplerK& s, double r2) {
  double z = r2 * s.c / (1.0 + sqrt(1.0 - (1.0 + s.k) * s.c * s.c * r2));
  double p = r2 * r2, r4 = r2 * r2;
  for (int i = 0; i < s.n_asph; ++i) {
    z += s.asph[i] * p;
    p *= r4;
  }
  return z;
}
__device__ __forceinline__ double smp_sag_dr2(const SamplerK& s, double r2) {
  const double alpha = (1.0 + s.k) * s.c * s.c;
  const double q = sqrt(1.0 - alpha * r2), den = 1.0 + q;
  double dz = s.c / den + (r2 * s.c) * alpha / (2.0 * q * den * den);
  double pm1 = r2, r4 = r2 * r2;
  for (int i = 0; i < s.n_asph; ++i) {
    dz += s.asph[i] * (double)(2 * (i + 1)) * pm1;
    pm1 *= r4;
  }
  return dz;
}

__global__ void __launch_bounds__(256) k_sample(const SamplerK s, float* __restrict__ pts, float* __restrict__ nrm,
                                                float* __restrict__ dlt, float* __restrict__ wts) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)s.F * s.M) return;
  const int f = (int)(i / s.M), m = (int)(i - (long long)f * s.M);
  uint32_t c[4] = {(uint32_t)m, (uint32_t)f, 0x5A3D1u, 0u};
  philox4x32_10(c, s.seed, 0x53414D50u);
  const double sc = 1.0 / 16777216.0;
  const double u0 = (double)(c[0] >> 8) * sc, u1 = (double)(c[1] >> 8) * sc, u2 = (double)(c[2] >> 8) * sc;
  double x, y, area;
  if (s.aperture == IACT_APERTURE_DISK) {
    // utils/sampling.py:8-27 scaled by the radius (core/integrators.py:116)
    const double R = s.radii[f];
    const double r = sqrt(u0) * R;
    double sn, cs;
    sincospi(2.0 * u1, &sn, &cs);
    x = r * cs;
    y = r * sn;
    area = 3.141592653589793 * R * R;
  } else {
    // utils/sampling.py:30-67: fan triangles from vertex 0, chosen by area
    const float* v = s.vertices + (size_t)f * s.n_vert * 2;
    const int nt = s.n_vert - 2;
    double tot = 0.0, ar[IACT_MAX_POLY];
    for (int t = 0; t < nt; ++t) {
      const double ax = v[0], ay = v[1], bx = v[2 * t + 2], by = v[2 * t + 3], cx = v[2 * t + 4], cy = v[2 * t + 5];
      ar[t] = fabs((bx - ax) * (cy - ay) - (cx - ax) * (by - ay)) * 0.5;
      tot += ar[t];
    }
    int idx = 0;
    double cdf = 0.0;
    for (int t = 0; t < nt; ++t) {  // number of cumulative probabilities <= u0
      cdf += ar[t] / tot;
      idx += (cdf <= u0) ? 1 : 0;
    }
    idx = min(idx, nt - 1);
    const double u = sqrt(u1), a = 1.0 - u, b = u * (1.0 - u2), cc = u * u2;
    x = a * v[0] + b * v[2 * idx + 2] + cc * v[2 * idx + 4];
    y = a * v[1] + b * v[2 * idx + 3] + cc * v[2 * idx + 5];
    double sh = 0.0;  // shoelace area (core/integrators.py:171-173)
    for (int j = 0; j < s.n_vert; ++j) {
      const int jn = (j + 1 == s.n_vert) ? 0 : j + 1;
      sh += (double)v[2 * j] * v[2 * jn + 1] - (double)v[2 * jn] * v[2 * j + 1];
    }
    area = 0.5 * fabs(sh);
  }
  // core/surfaces.py:41-65 point and normal at the offset
  const double ox = s.offsets[2 * f], oy = s.offsets[2 * f + 1];
  const double xs = x + ox, ys = y + oy;
  const double z = smp_sag(s, xs * xs + ys * ys) - smp_sag(s, ox * ox + oy * oy);
  const double g = smp_sag_dr2(s, xs * xs + ys * ys);
  double nx = -(g * 2.0 * xs), ny = -(g * 2.0 * ys), nz = 1.0;
  const double nn = sqrt(nx * nx + ny * ny + 1.0);
  nx /= nn;
  ny /= nn;
  nz /= nn;
  // core/reflection.py:22-49 perturbation delta (unit sigma)
  uint32_t c2[4] = {(uint32_t)m, (uint32_t)f, 0x5A3D1u, 1u};
  philox4x32_10(c2, s.seed, 0x53414D50u);
  const double v1 = (double)((c2[0] >> 8) + 1u) * sc, v2 = (double)(c2[1] >> 8) * sc;
  const double rad = sqrt(-2.0 * log(v1));
  double sn2, cs2;
  sincospi(2.0 * v2, &sn2, &cs2);
  const double th1 = rad * cs2, th2 = rad * sn2;
  const bool zref = fabs(nz) <= 0.9;  // ref = z unless the normal is near z, then x
  const double rx = zref ? 0.0 : 1.0, rz = zref ? 1.0 : 0.0;
  double t1x = ny * rz, t1y = nz * rx - nx * rz, t1z = -ny * rx;  // n x ref
  const double tn = sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
  t1x /= tn;
  t1y /= tn;
  t1z /= tn;
  const double t2x = ny * t1z - nz * t1y, t2y = nz * t1x - nx * t1z, t2z = nx * t1y - ny * t1x;
  pts[3 * i] = (float)x;
  pts[3 * i + 1] = (float)y;
  pts[3 * i + 2] = (float)z;
  nrm[3 * i] = (float)nx;
  nrm[3 * i + 1] = (float)ny;
  nrm[3 * i + 2] = (float)nz;
  dlt[3 * i] = (float)(th1 * t1x + th2 * t2x);
  dlt[3 * i + 1] = (float)(th1 * t1y + th2 * t2y);
  dlt[3 * i + 2] = (float)(th1 * t1z + th2 * t2z);
  wts[i] = (float)(nz / area * (double)s.M);  // core/integrators.py:124-127
}

}  // namespace iact

using namespace iact;

extern "C" int iact_sample_facets(const iact_sampler_t* s, float* points, float* normals, float* delta,
                                  float* weights, void* stream) {
  if (!s) return set_error(IACT_E_INVALID, "iact_sample_facets: sampler is NULL");
  if (s->n_facets < 0 || s->n_samples < 0) return set_error(IACT_E_INVALID, "negative facet or sample count");
  if ((long long)s->n_facets * s->n_samples > (1LL << 30))
    return set_error(IACT_E_UNSUPPORTED, "more than 2^30 samples");
  if (s->n_asph < 0 || s->n_asph > IACT_MAX_ASPH) return set_error(IACT_E_INVALID, "n_asph outside [0, IACT_MAX_ASPH]");
  if (s->aperture == IACT_APERTURE_DISK) {
    if (s->n_facets > 0 && !s->radii) return set_error(IACT_E_INVALID, "disk sampler: radii is NULL");
  } else if (s->aperture == IACT_APERTURE_POLYGON) {
    if (s->n_vert < 3 || s->n_vert > IACT_MAX_POLY)
      return set_error(IACT_E_INVALID, "polygon sampler: n_vert outside [3, IACT_MAX_POLY]");
    if (s->n_facets > 0 && !s->vertices) return set_error(IACT_E_INVALID, "polygon sampler: vertices is NULL");
  } else {
    return set_error(IACT_E_INVALID, "unknown aperture type");
  }
  const long long n = (long long)s->n_facets * s->n_samples;
  if (n == 0) return IACT_OK;
  if (!s->offsets || !points || !normals || !delta || !weights)
    return set_error(IACT_E_INVALID, "iact_sample_facets: NULL array");
  SamplerK k;
  k.F = s->n_facets; k.M = s->n_samples; k.aperture = s->aperture; k.n_vert = s->n_vert; k.n_asph = s->n_asph;
  k.c = s->curvature; k.k = s->conic;
  for (int i = 0; i < IACT_MAX_ASPH; ++i) k.asph[i] = i < s->n_asph ? (double)s->asph[i] : 0.0;
  k.offsets = s->offsets; k.radii = s->radii; k.vertices = s->vertices; k.seed = s->seed;
  k_sample<<<(int)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(k, points, normals, delta, weights);
  return check_cuda(cudaGetLastError(), "k_sample launch");
}
