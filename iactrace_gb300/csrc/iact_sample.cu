// Monte-Carlo facet sampling on the device (core/integrators.py:97-187
// MCIntegrator.sample_group), one thread per (facet, sample), and its
// reverse with respect to the shared surface.
//
// Variates: Philox4x32-10 with key (seed, 0x53414D50) and counters
// (m, f, 0x5A3D1, 0) -> aperture position, (m, f, 0x5A3D1, 1) -> the two
// N(0, 1) roughness coefficients (Box-Muller). Uniforms are the top 24 bits
// of a word scaled by 2^-24. The arithmetic is FP64 (sampling runs once per
// scene or optimiser step, F*M threads) and the arrays are stored as
// float32, as the reference stores them.
#include <cuda_runtime.h>

#include <cmath>

#include "iact_device.cuh"
#include "iact_internal.h"

namespace iact {

struct SamplerK {
  int F, M, aperture, n_vert, n_asph;
  double c, k, asph[IACT_MAX_ASPH];
  const float* surface;  // optional device [2 + n_asph] replacing c, k, asph
  const float* offsets;
  const float* radii;
  const float* vertices;
  uint32_t seed;
};

// The surface of one launch: by value, or read from device memory.
struct Surf {
  double c, k, a[IACT_MAX_ASPH];
  int na;
};
__device__ __forceinline__ Surf load_surface(const SamplerK& s) {
  Surf u;
  u.na = s.n_asph;
  if (s.surface) {
    u.c = s.surface[0];
    u.k = s.surface[1];
#pragma unroll
    for (int i = 0; i < IACT_MAX_ASPH; ++i) u.a[i] = i < s.n_asph ? (double)s.surface[2 + i] : 0.0;
  } else {
    u.c = s.c;
    u.k = s.k;
#pragma unroll
    for (int i = 0; i < IACT_MAX_ASPH; ++i) u.a[i] = s.asph[i];
  }
  return u;
}

// core/surfaces.py:25-39 _sag_raw and d/d(r2), FP64 (IEEE square root and division)
__device__ __forceinline__ double smp_sag(const Surf& s, double r2) {
  double z = r2 * s.c / (1.0 + sqrt(1.0 - (1.0 + s.k) * s.c * s.c * r2));
  double p = r2 * r2, r4 = r2 * r2;
  for (int i = 0; i < s.na; ++i) {
    z += s.a[i] * p;
    p *= r4;
  }
  return z;
}
__device__ __forceinline__ double smp_sag_dr2(const Surf& s, double r2) {
  const double alpha = (1.0 + s.k) * s.c * s.c;
  const double q = sqrt(1.0 - alpha * r2), den = 1.0 + q;
  double dz = s.c / den + (r2 * s.c) * alpha / (2.0 * q * den * den);
  double pm1 = r2, r4 = r2 * r2;
  for (int i = 0; i < s.na; ++i) {
    dz += s.a[i] * (double)(2 * (i + 1)) * pm1;
    pm1 *= r4;
  }
  return dz;
}

// One sample's construction: aperture position, surface point and normal,
// tangent basis and roughness coefficients, weight.
struct SampleGeo {
  double x, y, z, xs, ys, r2, r02, g;      // g = dS/dr2 at the point
  double nx, ny, nz, nn;                  // unit normal, |(-2g xs, -2g ys, 1)|
  double rx, rz;                          // tangent reference (z unless the normal is near z, then x)
  double t1x, t1y, t1z, tn, t2x, t2y, t2z;  // tangent basis, |n x ref|
  double th1, th2, area;
};

__device__ __forceinline__ void sample_geo(const SamplerK& s, const Surf& u, int f, int m, SampleGeo& o) {
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
    const double uu = sqrt(u1), a = 1.0 - uu, b = uu * (1.0 - u2), cc = uu * u2;
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
  o.x = x;
  o.y = y;
  o.area = area;
  o.xs = x + ox;
  o.ys = y + oy;
  o.r2 = o.xs * o.xs + o.ys * o.ys;
  o.r02 = ox * ox + oy * oy;
  o.z = smp_sag(u, o.r2) - smp_sag(u, o.r02);
  o.g = smp_sag_dr2(u, o.r2);
  const double nx = -(o.g * 2.0 * o.xs), ny = -(o.g * 2.0 * o.ys);
  o.nn = sqrt(nx * nx + ny * ny + 1.0);
  o.nx = nx / o.nn;
  o.ny = ny / o.nn;
  o.nz = 1.0 / o.nn;
  // core/reflection.py:22-49 perturbation delta (unit sigma)
  uint32_t c2[4] = {(uint32_t)m, (uint32_t)f, 0x5A3D1u, 1u};
  philox4x32_10(c2, s.seed, 0x53414D50u);
  const double v1 = (double)((c2[0] >> 8) + 1u) * sc, v2 = (double)(c2[1] >> 8) * sc;
  const double rad = sqrt(-2.0 * log(v1));
  double sn2, cs2;
  sincospi(2.0 * v2, &sn2, &cs2);
  o.th1 = rad * cs2;
  o.th2 = rad * sn2;
  const bool zref = fabs(o.nz) <= 0.9;  // ref = z unless the normal is near z, then x
  o.rx = zref ? 0.0 : 1.0;
  o.rz = zref ? 1.0 : 0.0;
  const double t1x = o.ny * o.rz, t1y = o.nz * o.rx - o.nx * o.rz, t1z = -o.ny * o.rx;  // n x ref
  o.tn = sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
  o.t1x = t1x / o.tn;
  o.t1y = t1y / o.tn;
  o.t1z = t1z / o.tn;
  o.t2x = o.ny * o.t1z - o.nz * o.t1y;
  o.t2y = o.nz * o.t1x - o.nx * o.t1z;
  o.t2z = o.nx * o.t1y - o.ny * o.t1x;
}

__global__ void __launch_bounds__(256) k_sample(const SamplerK s, float* __restrict__ pts, float* __restrict__ nrm,
                                                float* __restrict__ dlt, float* __restrict__ wts) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)s.F * s.M) return;
  const int f = (int)(i / s.M), m = (int)(i - (long long)f * s.M);
  const Surf u = load_surface(s);
  SampleGeo o;
  sample_geo(s, u, f, m, o);
  pts[3 * i] = (float)o.x;
  pts[3 * i + 1] = (float)o.y;
  pts[3 * i + 2] = (float)o.z;
  nrm[3 * i] = (float)o.nx;
  nrm[3 * i + 1] = (float)o.ny;
  nrm[3 * i + 2] = (float)o.nz;
  dlt[3 * i] = (float)(o.th1 * o.t1x + o.th2 * o.t2x);
  dlt[3 * i + 1] = (float)(o.th1 * o.t1y + o.th2 * o.t2y);
  dlt[3 * i + 2] = (float)(o.th1 * o.t1z + o.th2 * o.t2z);
  wts[i] = (float)(o.nz / o.area * (double)s.M);  // core/integrators.py:124-127
}

// Surface parameter derivatives of S and S' = dS/dr2 at r2 (the closed forms
// of the conic part; S_a_i = r2^p, S'_a_i = p r2^(p-1), p = 2(i+1)):
//   S_c  = r2/(1+q) + (1+k) c^2 r2^2 / (q (1+q)^2),  S_k  = c^3 r2^2 / (2 q (1+q)^2)
//   S'_c = 1/(2q) + (1+k) c^2 r2 / (2 q^3),          S'_k = c^3 r2 / (4 q^3)
__device__ __forceinline__ void smp_sag_dtheta(const Surf& u, double r2, double* dS, double* dG) {
  const double al = (1.0 + u.k) * u.c * u.c;
  const double q = sqrt(1.0 - al * r2), op = 1.0 + q;
  dS[0] = r2 / op + al * r2 * r2 / (q * op * op);
  dS[1] = u.c * u.c * u.c * r2 * r2 / (2.0 * q * op * op);
  dG[0] = 1.0 / (2.0 * q) + al * r2 / (2.0 * q * q * q);
  dG[1] = u.c * u.c * u.c * r2 / (4.0 * q * q * q);
  double p = r2 * r2, pm1 = r2;
  for (int i = 0; i < IACT_MAX_ASPH; ++i) {
    dS[2 + i] = i < u.na ? p : 0.0;
    dG[2 + i] = i < u.na ? (double)(2 * (i + 1)) * pm1 : 0.0;
    p *= r2 * r2;
    pm1 *= r2 * r2;
  }
}

// Reverse of k_sample with respect to the surface: per sample, dL/dS' (the
// slope g drives the normal, and through it the tangent-plane delta and the
// weight) and dL/dz (the point's sag), contracted with the parameter
// derivatives of S and S'; CTA sums, then FP64 atomics.
__global__ void __launch_bounds__(256) k_sample_bwd(const SamplerK s, const float* __restrict__ gp,
                                                    const float* __restrict__ gn, const float* __restrict__ gd,
                                                    const float* __restrict__ gw, double* __restrict__ gth) {
  constexpr int NT = 2 + IACT_MAX_ASPH;
  __shared__ double red[NT][8];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[NT];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j] = 0.0;
  if (i < (long long)s.F * s.M) {
    const int f = (int)(i / s.M), m = (int)(i - (long long)f * s.M);
    const Surf u = load_surface(s);
    SampleGeo o;
    sample_geo(s, u, f, m, o);
    const double Gz = gp ? (double)gp[3 * i + 2] : 0.0;
    double Gn[3] = {0.0, 0.0, 0.0}, Gd[3] = {0.0, 0.0, 0.0};
    if (gn) { Gn[0] = gn[3 * i]; Gn[1] = gn[3 * i + 1]; Gn[2] = gn[3 * i + 2]; }
    if (gd) { Gd[0] = gd[3 * i]; Gd[1] = gd[3 * i + 1]; Gd[2] = gd[3 * i + 2]; }
    const double Gw = gw ? (double)gw[i] : 0.0;
    // dn/dg: N = (-2g xs, -2g ys, 1), n = N / |N|, dn = (dN - n (n . dN)) / |N|
    const double dNx = -2.0 * o.xs, dNy = -2.0 * o.ys;
    const double nd = o.nx * dNx + o.ny * dNy;
    const double vx = (dNx - o.nx * nd) / o.nn, vy = (dNy - o.ny * nd) / o.nn, vz = (-o.nz * nd) / o.nn;
    // delta = th1 t1 + th2 t2; t1 = (n x ref) / |n x ref|, t2 = n x t1
    const double cx = vy * o.rz, cy = vz * o.rx - vx * o.rz, cz = -vy * o.rx;  // d(n x ref)
    const double tc = o.t1x * cx + o.t1y * cy + o.t1z * cz;
    const double d1x = (cx - o.t1x * tc) / o.tn, d1y = (cy - o.t1y * tc) / o.tn, d1z = (cz - o.t1z * tc) / o.tn;
    const double d2x = (vy * o.t1z - vz * o.t1y) + (o.ny * d1z - o.nz * d1y);
    const double d2y = (vz * o.t1x - vx * o.t1z) + (o.nz * d1x - o.nx * d1z);
    const double d2z = (vx * o.t1y - vy * o.t1x) + (o.nx * d1y - o.ny * d1x);
    const double ddx = o.th1 * d1x + o.th2 * d2x, ddy = o.th1 * d1y + o.th2 * d2y, ddz = o.th1 * d1z + o.th2 * d2z;
    const double Gg = Gn[0] * vx + Gn[1] * vy + Gn[2] * vz + Gd[0] * ddx + Gd[1] * ddy + Gd[2] * ddz +
                      Gw * vz * (double)s.M / o.area;
    double dS[NT], dG[NT], dS0[NT], dG0[NT];
    smp_sag_dtheta(u, o.r2, dS, dG);
    smp_sag_dtheta(u, o.r02, dS0, dG0);
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j] = Gz * (dS[j] - dS0[j]) + Gg * dG[j];
  }
  // CTA reduction: warp shuffles, then one partial per warp in shared memory
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    double v = acc[j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    if (lane == 0) red[j][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < NT && threadIdx.x < 2 + s.n_asph) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
    if (v != 0.0) atomicAdd(gth + threadIdx.x, v);
  }
}

int sampler_params(const iact_sampler_t* s, SamplerK& k) {
  if (!s) return set_error(IACT_E_INVALID, "sampler is NULL");
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
  if ((long long)s->n_facets * s->n_samples > 0 && !s->offsets)
    return set_error(IACT_E_INVALID, "sampler: offsets is NULL");
  k.F = s->n_facets; k.M = s->n_samples; k.aperture = s->aperture; k.n_vert = s->n_vert; k.n_asph = s->n_asph;
  k.c = s->curvature; k.k = s->conic;
  for (int i = 0; i < IACT_MAX_ASPH; ++i) k.asph[i] = i < s->n_asph ? (double)s->asph[i] : 0.0;
  k.surface = s->surface;
  k.offsets = s->offsets; k.radii = s->radii; k.vertices = s->vertices; k.seed = s->seed;
  return IACT_OK;
}

}  // namespace iact

using namespace iact;

extern "C" int iact_sample_facets(const iact_sampler_t* s, float* points, float* normals, float* delta,
                                  float* weights, void* stream) {
  SamplerK k;
  int rc = sampler_params(s, k);
  if (rc) return rc;
  const long long n = (long long)k.F * k.M;
  if (n == 0) return IACT_OK;
  if (!points || !normals || !delta || !weights) return set_error(IACT_E_INVALID, "iact_sample_facets: NULL array");
  k_sample<<<(int)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(k, points, normals, delta, weights);
  return launched("k_sample launch");
}

extern "C" int iact_sample_facets_backward(const iact_sampler_t* s, const float* g_points, const float* g_normals,
                                           const float* g_delta, const float* g_weights, double* g_surface,
                                           void* stream) {
  SamplerK k;
  int rc = sampler_params(s, k);
  if (rc) return rc;
  if (!g_surface) return set_error(IACT_E_INVALID, "iact_sample_facets_backward: g_surface is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = check_cuda(cudaMemsetAsync(g_surface, 0, sizeof(double) * (2 + k.n_asph), st), "zero surface gradients");
  if (rc) return rc;
  const long long n = (long long)k.F * k.M;
  if (n == 0 || (!g_points && !g_normals && !g_delta && !g_weights)) return IACT_OK;
  k_sample_bwd<<<(int)((n + 255) / 256), 256, 0, st>>>(k, g_points, g_normals, g_delta, g_weights, g_surface);
  return launched("k_sample_bwd launch");
}
