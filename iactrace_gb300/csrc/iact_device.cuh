// Per-ray device math of the render path (sm_103a).
//
// Each function states the reference expression it evaluates
// (GerritRo/iactrace v0.4.0). The per-primitive and per-mirror constants the
// reference recomputes on every ray (cylinder axis and height, triangle
// edges, mirror rotation matrices, z0) are computed once per launch, with
// the same float32 operations, into compact shared-memory records.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/iactrace_gb300.h"

namespace iact {

constexpr float kBig = 1e10f;  // the reference's miss / shadow sentinel
constexpr float kEps = 1e-8f;
constexpr unsigned kFull = 0xffffffffu;

// ------------------------------------------- programmatic dependent launch
// A kernel launched with the programmatic stream serialization attribute
// (launch_after below) may be scheduled while its predecessor on the stream
// still runs; grid_dep_wait, before its first read of the predecessor's
// results, waits until that grid has completed and its writes are visible.
// For a kernel launched without the attribute both are no-ops.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// lets the stream's next kernel (launched with the attribute) be scheduled
// once every CTA of this grid has started; its grid_dep_wait still waits for
// this grid to complete
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// ------------------------------------------------------------ table records
// Sizes in floats; records are packed back to back in shared memory.
constexpr int kCylF = 8;    // p1(3) axis(3) height r*r
constexpr int kBoxF = 6;    // min(3) max(3)
constexpr int kSphF = 4;    // center(3) r*r
constexpr int kOboxF = 15;  // center(3) half(3) R(9) row-major local->world
constexpr int kTriF = 9;    // v0(3) e1(3) e2(3)
constexpr int kMirF = 52;   // see MirRec

// One stage >= 1 mirror, as laid out in shared memory (floats).
struct MirRec {
  float R[9];       // 0..8  local->world rotation
  float pos[3];     // 9..11
  float off[2];     // 12..13
  float unused14;   // 14
  float c;          // 15  curvature
  float kp1;        // 16  1 + conic (float32)
  float alpha;      // 17  (1+k) c c (float32)
  float r2ap;       // 18  disk radius^2
  float n_asph;     // 19
  float aperture;   // 20
  float n_vert;     // 21
  float stage;      // 22
  float k;          // 23  conic constant
  float asph[8];    // 24..31
  float vert[16];   // 32..47
  float z0_hi;      // 48  sag at the offset (FP64 value as a float pair hi + lo)
  float z0_lo;      // 49
  float alpha_hi;   // 50  (1+k) c c (FP64 value as a float pair)
  float alpha_lo;   // 51
};
static_assert(sizeof(MirRec) == kMirF * sizeof(float), "MirRec layout");

// ------------------------------------------------- double-float arithmetic
// A value hi + lo held as two float32 (|lo| <= ulp(hi) / 2): about 48
// significant bits, computed on the FP32 pipe. Error-free transformations
// (Knuth's two-sum, Dekker's fast two-sum, the FMA two-product) and the
// double-float add / multiply built on them (Dekker 1971; Hida, Li and
// Bailey, "Library for double-double and quad-double arithmetic", 2007:
// the "sloppy" add, whose error is about 2^-47 (|a| + |b|)). Written with
// round-to-nearest intrinsics so that no step is contracted or reordered.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a = 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ff_add_f(FF a, float b) {
  const FF s = ff_two_sum(a.hi, b);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
  const float p = __fmul_rn(a.hi, b);
  const float e = __fmaf_rn(a.hi, b, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a.lo, b, e));
}
__device__ __forceinline__ float ff_f(FF a) { return __fadd_rn(a.hi, a.lo); }

// Hardware approximations (PTX rcp.approx / sqrt.approx, <= 1 ulp-ish).
// Used where the value only feeds a hit/miss comparison or a sensor-plane
// coordinate whose error stays far inside the pixel-edge band.
__device__ __forceinline__ float rcp_a(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float sqrt_a(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }

// core/transforms.py:72-107 euler_to_matrix: R = (Rz @ Ry) @ Rx, degrees.
__device__ __forceinline__ void euler_to_matrix(float tip, float tilt, float rot, float* R) {
  const float k = 0.017453292519943295f;  // pi / 180
  float sx, cx, sy, cy, sz, cz;
  sincosf(tip * k, &sx, &cx);
  sincosf(tilt * k, &sy, &cy);
  sincosf(rot * k, &sz, &cz);
  // Rz @ Ry = [[cz*cy, -sz, cz*sy], [sz*cy, cz, sz*sy], [-sy, 0, cy]]
  float a00 = cz * cy, a01 = -sz, a02 = cz * sy;
  float a10 = sz * cy, a11 = cz, a12 = sz * sy;
  float a20 = -sy, a21 = 0.f, a22 = cy;
  // (Rz @ Ry) @ Rx, Rx = [[1,0,0],[0,cx,-sx],[0,sx,cx]]
  R[0] = a00; R[1] = a01 * cx + a02 * sx; R[2] = a02 * cx - a01 * sx;
  R[3] = a10; R[4] = a11 * cx + a12 * sx; R[5] = a12 * cx - a11 * sx;
  R[6] = a20; R[7] = a21 * cx + a22 * sx; R[8] = a22 * cx - a21 * sx;
}

__device__ __forceinline__ V3 rmul(const float* R, V3 v) {
  return {fmaf(R[2], v.z, fmaf(R[1], v.y, R[0] * v.x)), fmaf(R[5], v.z, fmaf(R[4], v.y, R[3] * v.x)),
          fmaf(R[8], v.z, fmaf(R[7], v.y, R[6] * v.x))};
}
__device__ __forceinline__ V3 rtmul(const float* R, V3 v) {
  return {fmaf(R[6], v.z, fmaf(R[3], v.y, R[0] * v.x)), fmaf(R[7], v.z, fmaf(R[4], v.y, R[1] * v.x)),
          fmaf(R[8], v.z, fmaf(R[5], v.y, R[2] * v.x))};
}

// ------------------------------------------------------------- primitives
// Each returns true when the primitive's t (as the reference computes it)
// is < 1e10, i.e. when it shadows the ray (core/render.py:40). The group
// minimum of the reference is never NaN (every t passes a jnp.where that
// maps NaN to inf), so "some member's t < 1e10" is the same test.

// core/intersections.py:44-87 intersect_cylinder
__device__ __forceinline__ bool cyl_shadows(const float* c, V3 o, V3 d) {
  V3 p1 = mk(c[0], c[1], c[2]), ax = mk(c[3], c[4], c[5]);
  float h = c[6], r2 = c[7];
  V3 oc = o - p1;
  float oca = dot(oc, ax), rda = dot(d, ax);
  V3 ocp = oc - oca * ax;
  V3 rdp = d - rda * ax;
  float a = dot(rdp, rdp);
  float b = 2.f * dot(ocp, rdp);
  float cc = dot(ocp, ocp) - r2;
  float disc = b * b - 4.f * a * cc;
  float sq = sqrt_a(fmaxf(disc, 0.f));
  float inv2a = rcp_a(2.f * a + kEps);
  float t1 = (-b - sq) * inv2a;
  float t2 = (-b + sq) * inv2a;
  float y1 = fmaf(t1, rda, oca), y2 = fmaf(t2, rda, oca);
  bool h1 = (t1 > kEps) & (y1 >= 0.f) & (y1 <= h) & (t1 < kBig);
  bool h2 = (t2 > kEps) & (y2 >= 0.f) & (y2 <= h) & (t2 < kBig);
  bool hit = (disc >= 0.f) & (h1 | h2);
  float invr = rcp_a(rda + kEps);
  float tb = -oca * invr;
  float tt = (h - oca) * invr;
  V3 pb = ocp + tb * rdp, pt = ocp + tt * rdp;
  hit |= (tb > kEps) & (dot(pb, pb) <= r2) & (tb < kBig);
  hit |= (tt > kEps) & (dot(pt, pt) <= r2) & (tt < kBig);
  return hit;
}

// core/intersections.py:90-110 intersect_box; jnp.minimum/maximum propagate
// NaN, so a NaN slab value means no hit.
__device__ __forceinline__ bool box_shadows(const float* bx, V3 o, V3 d) {
  float ix = rcp_a(d.x + kEps), iy = rcp_a(d.y + kEps), iz = rcp_a(d.z + kEps);
  float x1 = (bx[0] - o.x) * ix, x2 = (bx[3] - o.x) * ix;
  float y1 = (bx[1] - o.y) * iy, y2 = (bx[4] - o.y) * iy;
  float z1 = (bx[2] - o.z) * iz, z2 = (bx[5] - o.z) * iz;
  bool nan = isnan(x1) | isnan(x2) | isnan(y1) | isnan(y2) | isnan(z1) | isnan(z2);
  float tmin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fminf(z1, z2));
  float tmax = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fmaxf(z1, z2));
  float tr = (tmin > kEps) ? tmin : tmax;
  return (tmax >= tmin) & (tmax > kEps) & !nan & (tr < kBig);
}

// core/intersections.py:195-226 intersect_sphere
__device__ __forceinline__ bool sph_shadows(const float* s, V3 o, V3 d) {
  V3 oc = o - mk(s[0], s[1], s[2]);
  float a = dot(d, d);
  float b = 2.f * dot(oc, d);
  float c = dot(oc, oc) - s[3];
  float disc = b * b - 4.f * a * c;
  float sq = sqrt_a(fmaxf(disc, 0.f));
  float inv2a = rcp_a(2.f * a + kEps);
  float t1 = (-b - sq) * inv2a, t2 = (-b + sq) * inv2a;
  return (disc >= 0.f) & (((t1 > kEps) & (t1 < kBig)) | ((t2 > kEps) & (t2 < kBig)));
}

__device__ __forceinline__ float sgnf(float v) { return v > 0.f ? 1.f : (v < 0.f ? -1.f : 0.f); }

// core/intersections.py:113-149 intersect_oriented_box
__device__ __forceinline__ bool obox_shadows(const float* b, V3 o, V3 d) {
  const float* R = b + 6;
  V3 lo = rtmul(R, o - mk(b[0], b[1], b[2]));
  V3 ld = rtmul(R, d);
  float ix = rcp_a(ld.x + kEps * sgnf(ld.x + kEps));
  float iy = rcp_a(ld.y + kEps * sgnf(ld.y + kEps));
  float iz = rcp_a(ld.z + kEps * sgnf(ld.z + kEps));
  float x1 = (-b[3] - lo.x) * ix, x2 = (b[3] - lo.x) * ix;
  float y1 = (-b[4] - lo.y) * iy, y2 = (b[4] - lo.y) * iy;
  float z1 = (-b[5] - lo.z) * iz, z2 = (b[5] - lo.z) * iz;
  bool nan = isnan(x1) | isnan(x2) | isnan(y1) | isnan(y2) | isnan(z1) | isnan(z2);
  float tmin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fminf(z1, z2));
  float tmax = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fmaxf(z1, z2));
  float tr = (tmin > kEps) ? tmin : tmax;
  return (tmax >= tmin) & (tmax > kEps) & !nan & (tr > kEps) & (tr < kBig);
}

// core/intersections.py:152-192 intersect_triangle (Moller-Trumbore)
__device__ __forceinline__ bool tri_shadows(const float* t, V3 o, V3 d) {
  V3 v0 = mk(t[0], t[1], t[2]), e1 = mk(t[3], t[4], t[5]), e2 = mk(t[6], t[7], t[8]);
  V3 h = mk(d.y * e2.z - d.z * e2.y, d.z * e2.x - d.x * e2.z, d.x * e2.y - d.y * e2.x);
  float a = dot(e1, h);
  bool parallel = fabsf(a) < kEps;
  float f = rcp_a(a + kEps * sgnf(a + kEps));
  V3 s = o - v0;
  float u = f * dot(s, h);
  V3 q = mk(s.y * e1.z - s.z * e1.y, s.z * e1.x - s.x * e1.z, s.x * e1.y - s.y * e1.x);
  float v = f * dot(d, q);
  float tt = f * dot(e2, q);
  return !parallel & (u >= 0.f) & (u <= 1.f) & (v >= 0.f) & (u + v <= 1.f) & (tt > kEps) & (tt < kBig);
}

// Shadow-table view (shared memory). Counts are CTA-uniform.
struct Obst {
  const float* cyl;
  const float* box;
  const float* sph;
  const float* obox;
  const float* tri;
  int n_cyl, n_box, n_sph, n_obox, n_tri;
};

// core/render.py:21-41 _check_occlusions, for one ray: true = shadowed.
__device__ __forceinline__ bool occluded(const Obst& ob, V3 o, V3 d) {
  bool s = false;
#pragma unroll 1
  for (int i = 0; i < ob.n_cyl; ++i) s |= cyl_shadows(ob.cyl + i * kCylF, o, d);
#pragma unroll 1
  for (int i = 0; i < ob.n_box; ++i) s |= box_shadows(ob.box + i * kBoxF, o, d);
#pragma unroll 1
  for (int i = 0; i < ob.n_sph; ++i) s |= sph_shadows(ob.sph + i * kSphF, o, d);
#pragma unroll 1
  for (int i = 0; i < ob.n_obox; ++i) s |= obox_shadows(ob.obox + i * kOboxF, o, d);
#pragma unroll 1
  for (int i = 0; i < ob.n_tri; ++i) s |= tri_shadows(ob.tri + i * kTriF, o, d);
  return s;
}

// ------------------------------------------------------ bundle culling
// The 32 rays of a warp task leave one facet's 32-sample chunk towards one
// source: their shadow rays lie inside a "thick ray" around an axis ray
// c + t u (t >= 0), of radius R0 + t * dlt (R0 bounds |o_i - c|, dlt bounds
// |u_i - u|). A primitive whose bounding volume stays farther than that
// from the axis ray cannot shadow any ray of the bundle and is skipped; the
// others (the candidates) get the reference's per-ray test unchanged, so
// shadow masks are identical to testing every primitive. Bounding volumes:
// the cylinder's capsule, the box itself, the sphere itself, bounding
// spheres of oriented boxes and triangles. The reach adds 2 mm + 1e-4 of
// the distance for float32 rounding of the bundle and of the per-ray tests.
struct Bundle {
  V3 c, u;
  float R0, dlt;
};

// R0 + t dlt at the farthest distance t a hit on a volume of bounding
// radius `rad` around `q` can lie from a ray origin, plus the margin
__device__ __forceinline__ float bundle_reach(const Bundle& b, V3 q, float rad) {
  V3 w = q - b.c;
  const float T = sqrt_a(dot(w, w)) * 1.00001f + rad + b.R0;
  return b.R0 + T * b.dlt + 2e-3f + 1e-4f * T;
}

// squared distance from point p to the ray c + t u, t >= 0 (|u| = 1)
__device__ __forceinline__ float ray_point_d2(const Bundle& b, V3 p) {
  V3 w = p - b.c;
  const float t = fmaxf(dot(w, b.u), 0.f);
  V3 e = w - t * b.u;
  return dot(e, e);
}

__device__ __forceinline__ bool sphere_may_hit(const Bundle& b, V3 q, float rad) {
  const float lim = rad + bundle_reach(b, q, rad);
  return ray_point_d2(b, q) <= lim * lim;
}

// capsule (segment p1 + s ax, s in [0, h], radius r) vs the thick ray: the
// exact minimum distance between the ray and the segment is the smaller of
// the interior stationary point (if feasible) and the three edge minima
__device__ __forceinline__ bool capsule_may_hit(const Bundle& b, V3 p1, V3 ax, float h, float r) {
  const V3 mid = p1 + (0.5f * h) * ax;
  const float lim = r + bundle_reach(b, mid, 0.5f * h + r);
  const V3 w0 = b.c - p1;
  const float bb = dot(b.u, ax), d = dot(b.u, w0), e = dot(ax, w0);
  const float den = 1.f - bb * bb;
  if (den < 1e-2f) return true;  // ray within ~6 deg of the axis: always a candidate
  float best = fminf(ray_point_d2(b, p1), ray_point_d2(b, p1 + h * ax));
  {  // t = 0: the ray origin against the segment
    const float s = fminf(fmaxf(e, 0.f), h);
    V3 q = w0 - s * ax;
    best = fminf(best, dot(q, q));
  }
  const float t = (bb * e - d) * rcp_a(den), s = e + t * bb;
  if (t >= 0.f && s >= 0.f && s <= h) {
    V3 q = w0 + t * b.u - s * ax;
    best = fminf(best, dot(q, q));
  }
  return best <= lim * lim;
}

// axis ray against the box grown by the reach (slab test, t >= 0)
__device__ __forceinline__ bool aabb_may_hit(const Bundle& b, const float* bx) {
  const V3 lo = mk(bx[0], bx[1], bx[2]), hi = mk(bx[3], bx[4], bx[5]);
  const V3 ctr = 0.5f * (lo + hi), half = 0.5f * (hi - lo);
  const float g = bundle_reach(b, ctr, sqrt_a(dot(half, half)) * 1.00001f);
  float t0 = 0.f, t1 = 3.0e38f;
  const float cc[3] = {b.c.x, b.c.y, b.c.z}, uu[3] = {b.u.x, b.u.y, b.u.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float l = bx[a] - g, hgh = bx[3 + a] + g;
    if (fabsf(uu[a]) < 1e-20f) {
      if (cc[a] < l || cc[a] > hgh) return false;
    } else {
      const float inv = rcp_a(uu[a]);
      const float ta = (l - cc[a]) * inv, tb = (hgh - cc[a]) * inv;
      t0 = fmaxf(t0, fminf(ta, tb));
      t1 = fminf(t1, fmaxf(ta, tb));
    }
  }
  return t0 <= t1;
}

// primitive k of the unified index space (cylinders, boxes, spheres,
// oriented boxes, triangles) may shadow some ray of the bundle
__device__ __forceinline__ bool prim_may_hit(const Obst& ob, int k, const Bundle& b) {
  if (k < ob.n_cyl) {
    const float* c = ob.cyl + k * kCylF;
    return capsule_may_hit(b, mk(c[0], c[1], c[2]), mk(c[3], c[4], c[5]), c[6], sqrt_a(c[7]) * 1.00001f);
  }
  k -= ob.n_cyl;
  if (k < ob.n_box) return aabb_may_hit(b, ob.box + k * kBoxF);
  k -= ob.n_box;
  if (k < ob.n_sph) {
    const float* s = ob.sph + k * kSphF;
    return sphere_may_hit(b, mk(s[0], s[1], s[2]), sqrt_a(s[3]) * 1.00001f);
  }
  k -= ob.n_sph;
  if (k < ob.n_obox) {
    const float* o = ob.obox + k * kOboxF;
    return sphere_may_hit(b, mk(o[0], o[1], o[2]), sqrt_a(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]) * 1.00001f);
  }
  k -= ob.n_obox;
  const float* t = ob.tri + k * kTriF;
  const V3 v0 = mk(t[0], t[1], t[2]), e1 = mk(t[3], t[4], t[5]), e2 = mk(t[6], t[7], t[8]);
  const V3 g = v0 + (1.f / 3.f) * (e1 + e2);
  V3 a = v0 - g, bq = (v0 + e1) - g, cq = (v0 + e2) - g;
  const float rad = sqrt_a(fmaxf(fmaxf(dot(a, a), dot(bq, bq)), dot(cq, cq))) * 1.00001f;
  return sphere_may_hit(b, g, rad);
}

// core/render.py:21-41 for one ray, primitives restricted to the set bits
// of the bundle's candidate mask (n_words 32-bit words; 0 words: test all)
__device__ __forceinline__ bool occluded_mask(const Obst& ob, const uint32_t* mask, int n_words, V3 o, V3 d) {
  if (n_words <= 0) return occluded(ob, o, d);
  bool sh = false;
#pragma unroll 1
  for (int w = 0; w < n_words; ++w) {
    uint32_t m = mask[w];
#pragma unroll 1
    while (m) {
      int k = w * 32 + __ffs(m) - 1;
      m &= m - 1u;
      if (k < ob.n_cyl) {
        sh |= cyl_shadows(ob.cyl + k * kCylF, o, d);
        continue;
      }
      k -= ob.n_cyl;
      if (k < ob.n_box) {
        sh |= box_shadows(ob.box + k * kBoxF, o, d);
        continue;
      }
      k -= ob.n_box;
      if (k < ob.n_sph) {
        sh |= sph_shadows(ob.sph + k * kSphF, o, d);
        continue;
      }
      k -= ob.n_sph;
      if (k < ob.n_obox) {
        sh |= obox_shadows(ob.obox + k * kOboxF, o, d);
        continue;
      }
      k -= ob.n_obox;
      sh |= tri_shadows(ob.tri + k * kTriF, o, d);
    }
  }
  return sh;
}

// ----------------------------------------------------------------- sensor
struct SensorK {
  int type, n_pixels, width, height;
  float R[9];
  float pos[3];
  float x0, y0, dx, dy, edge_width;
  float inv_dx, inv_dy;               // 1/dx, 1/dy
  float hq_x, hq_y, hr_y, inv_inr;    // sqrt(3)/3/size, 1/(3 size), 2/(3 size), 1/inradius
  float hex_size, inradius, gc, gs, off_x, off_y, hex_sx, hex_sy, edge_threshold;
  int q_min, r_min, table_q, table_r;
  float sigma;
  int kernel_size;
  float hex_lim2;  // (inradius * edge_threshold - 1e-5)^2: points this close to a cell centre bin to that cell
  int axes;        // 1: the sensor's rotation is exactly the identity (local axes = world axes)
};

// core/intersections.py:6-41 intersect_plane -> local (x, y) or (1e10, 1e10).
// AX = true is the same computation for a sensor whose rotation is exactly
// the identity (s.axes): the dot products with the unit axes reduce to
// components. fmaf with exact zeros and ones returns the other operand, so
// both forms give the same floats (up to the sign of a zero result, which
// no binning distinguishes).
template <bool AX = false>
__device__ __forceinline__ void plane_hit(const SensorK& s, V3 o, V3 d, float& x, float& y) {
  V3 u1 = mk(s.R[0], s.R[3], s.R[6]), u2 = mk(s.R[1], s.R[4], s.R[7]), n = mk(s.R[2], s.R[5], s.R[8]);
  V3 c = mk(s.pos[0], s.pos[1], s.pos[2]);
  float ndotd = AX ? d.z : dot(d, n), ndoto = AX ? o.z : dot(o, n), ndotp = AX ? c.z : dot(n, c);
  bool parallel = fabsf(ndotd) < 1e-10f;
  float t = (ndotp - ndoto) * rcp_a(parallel ? 1.f : ndotd);
  V3 op = (o + t * d) - c;
  bool invalid = parallel || (t <= 0.f);
  x = invalid ? kBig : (AX ? op.x : dot(op, u1));
  y = invalid ? kBig : (AX ? op.y : dot(op, u2));
}

// sensors/square.py:66-91 SquareSensor.accumulate: pixel id or -1
__device__ __forceinline__ int bin_square(const SensorK& s, float x, float y) {
  // explicit roundings (no contraction): every kernel bins a point identically
  const float xc = __fmul_rn(__fsub_rn(x, s.x0), s.inv_dx), yc = __fmul_rn(__fsub_rn(y, s.y0), s.inv_dy);
  const float xf = floorf(xc), yf = floorf(yc);
  // compare in float: out-of-range and NaN fail, as the int32 cast would
  bool valid = (xf >= 0.f) && (xf < (float)s.width) && (yf >= 0.f) && (yf < (float)s.height);
  const float fx = __fsub_rn(xc, xf), fy = __fsub_rn(yc, yf);
  const float dist = fminf(__fmul_rn(fminf(fx, __fsub_rn(1.f, fx)), s.dx), __fmul_rn(fminf(fy, __fsub_rn(1.f, fy)), s.dy));
  valid = valid && !(dist < s.edge_width);
  return valid ? (int)yf * s.width + (int)xf : -1;
}

// sensors/hexagonal.py:16-23 _rotate and :26-29 _cartesian_to_axial, :32-39 _axial_round
__device__ __forceinline__ void hex_axial(const SensorK& s, float x, float y, float& xg, float& yg,
                                          float& qi, float& ri) {
  // explicit roundings (no contraction): every kernel bins a point identically
  const float xs = __fsub_rn(x, s.off_x), ys = __fsub_rn(y, s.off_y);
  xg = __fsub_rn(__fmul_rn(s.gc, xs), __fmul_rn(s.gs, ys));
  yg = __fadd_rn(__fmul_rn(s.gs, xs), __fmul_rn(s.gc, ys));
  const float q = __fsub_rn(__fmul_rn(s.hq_x, xg), __fmul_rn(s.hq_y, yg));  // (sqrt(3)/3 x - y/3) / size
  const float r = __fmul_rn(s.hr_y, yg);                                     // (2 y / 3) / size
  const float sv = __fsub_rn(-q, r);
  qi = rintf(q);
  ri = rintf(r);
  const float si = rintf(sv);
  const float dq = fabsf(__fsub_rn(qi, q)), dr = fabsf(__fsub_rn(ri, r)), ds = fabsf(__fsub_rn(si, sv));
  if ((dq > dr) && (dq > ds)) qi = __fsub_rn(-ri, si);
  if ((dr > dq) && (dr > ds)) ri = __fsub_rn(-qi, si);
}

// sensors/hexagonal.py:155-172 _lookup_pixels over a table in shared memory
template <typename TT>
__device__ __forceinline__ int hex_lookup(const SensorK& s, const TT* table, float qi, float ri) {
  float qx = qi - (float)s.q_min, rx = ri - (float)s.r_min;
  bool in = (qx >= 0.f) & (qx < (float)s.table_q) & (rx >= 0.f) & (rx < (float)s.table_r);
  int p = in ? (int)table[(int)qx * s.table_r + (int)rx] : -1;
  return p >= 0 ? p : -1;
}

// sensors/hexagonal.py:42-47 _hex_norm
__device__ __forceinline__ float hex_norm(float x, float y, float inv_inr) {
  const float ax = fabsf(x), ay = fabsf(y);
  return __fmul_rn(fmaxf(ax, __fadd_rn(__fmul_rn(0.5f, ax), __fmul_rn(0.8660254037844386f, ay))), inv_inr);
}

// lattice centre of axial cell (qi, ri) in the grid frame
__device__ __forceinline__ void hex_centre(const SensorK& s, float qi, float ri, float& cx, float& cy) {
  cx = __fmul_rn(s.hex_sx, __fadd_rn(qi, __fmul_rn(0.5f, ri)));
  cy = __fmul_rn(s.hex_sy, ri);
}

// sensors/hexagonal.py:174-194 HexagonalSensor.accumulate: pixel id or -1
template <typename TT>
__device__ __forceinline__ int bin_hex(const SensorK& s, const TT* table, float x, float y) {
  float xg, yg, qi, ri;
  hex_axial(s, x, y, xg, yg, qi, ri);
  int p = hex_lookup(s, table, qi, ri);
  float hcx, hcy;
  hex_centre(s, qi, ri, hcx, hcy);
  float hd = hex_norm(__fsub_rn(xg, hcx), __fsub_rn(yg, hcy), s.inv_inr);
  return (hd > s.edge_threshold) ? -1 : p;
}

// The last hexagon a lane binned into: its centre (sensor-plane frame) and
// pixel id.
struct HexCache {
  float cx, cy;
  int pid;
};

// bin_hex with a one-cell cache: a point within inradius * edge_threshold
// - 1e-5 m of the cached cell's centre lies inside that cell (the hexagonal
// norm never exceeds the Euclidean one over the inradius) and outside the
// edge band, so the reference's rounding, lookup and edge test give the
// cached id; the 1e-5 m margin covers their float32 rounding. The test runs
// in the sensor-plane frame (the grid frame is a rotation and a shift of
// it, which keep distances), with the centre mapped back from the grid
// frame on a miss (rounding ~1e-7 m, inside the margin). Otherwise the full
// path runs and refills the cache.
template <typename TT>
__device__ __forceinline__ int bin_hex_cached(const SensorK& s, const TT* table, float x, float y, HexCache& hc) {
  const float ex = x - hc.cx, ey = y - hc.cy;
  if (ex * ex + ey * ey < s.hex_lim2) return hc.pid;
  float xg2, yg2, qi, ri;
  hex_axial(s, x, y, xg2, yg2, qi, ri);
  const int p = hex_lookup(s, table, qi, ri);
  float hcx, hcy;
  hex_centre(s, qi, ri, hcx, hcy);
  const float hd = hex_norm(__fsub_rn(xg2, hcx), __fsub_rn(yg2, hcy), s.inv_inr);
  // grid -> sensor frame: x - off_x = gc xg + gs yg, y - off_y = -gs xg + gc yg
  hc.cx = s.off_x + (s.gc * hcx + s.gs * hcy);
  hc.cy = s.off_y + (s.gc * hcy - s.gs * hcx);
  hc.pid = p;
  return (hd > s.edge_threshold) ? -1 : p;
}

// ------------------------------------------------------- stage >= 1 mirrors
// core/surfaces.py:25-39 _sag_raw in FP64 (reference form; used once per
// mirror for z0): the sag root is the one place where the float32 chain
// cancels (ray origins several metres from the surface against a 1e-6
// residual tolerance).
__device__ __forceinline__ double sag_raw_d(const float* m, double r2) {
  double c = m[15], alpha = (1.0 + (double)m[23]) * c * c;
  double den = 1.0 + sqrt(1.0 - alpha * r2);
  double z = r2 * c / den;
  int na = (int)m[19];
  if (na > 0) {
    double r4 = r2 * r2, p = r4, sacc = 0.0;
    for (int i = 0; i < na; ++i) {  // a_i * r2^(2(i+1))
      sacc += (double)m[24 + i] * p;
      p *= r4;
    }
    z += sacc;
  }
  return z;
}
// core/surfaces.py:25-39 _sag_raw and its r2-derivatives. With
// q = sqrt(1 - alpha r2), alpha = (1+k) c^2:
//   S = c r2 / (1 + q) + sum_i a_i r2^(2(i+1)),  S' = c / (2q) + ...,  S'' = c alpha / (4 q^3) + ...
// float32 version: the first Newton phase of mirror_hit.
__device__ __forceinline__ float sag_f(const float* m, float r2, float& dS) {
  const float c = m[15];
  const float qq = fmaf(-m[17], r2, 1.f);
  const float rq = rsqrtf(qq);
  float S = c * r2 * rcp_a(fmaf(qq, rq, 1.f));
  float d = 0.5f * c * rq;
  const int na = (int)m[19];
  if (na > 0) {
    const float r4 = r2 * r2;
    float p = r4, pm1 = r2;
    for (int i = 0; i < na; ++i) {
      const float a = m[24 + i];
      S = fmaf(a, p, S);
      d = fmaf(a * (float)(2 * (i + 1)), pm1, d);
      p *= r4;
      pm1 *= r4;
    }
  }
  dS = d;
  return S;
}

// Double-float version: S to about 1e-13 relative (the square root and the
// reciprocal from the float32 approximations plus one Newton-Raphson
// correction each, y' = y + y (1 - x y) and q' = q + (x - q^2) / (2q): the
// error 2^-22 squares to 2^-44), S' and S'' in float32 from the same
// approximations (they scale the Newton step, bound its remainder and set
// the float32 normal). Outside the conic's domain (1 - alpha r2 < 0) S is
// NaN; at its edge q = 0.
__device__ __forceinline__ FF sag_ff(const float* m, FF r2, float& dS, float& Srr, float& qqf) {
  const float c = m[15];
  const FF qq = ff_add_f(ff_neg(ff_mul(FF{m[50], m[51]}, r2)), 1.f);
  qqf = ff_f(qq);
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(qq.hi));
  const bool pos = qq.hi > 0.f, zero = qq.hi == 0.f;
  // q = sqrt(qq): q0 = qq y, corrected by (qq - q0^2) y / 2
  const float q0 = __fmul_rn(qq.hi, y);
  const FF rsd = ff_add(qq, ff_neg(FF{__fmul_rn(q0, q0), __fmaf_rn(q0, q0, -__fmul_rn(q0, q0))}));
  FF q = ff_fast_two_sum(q0, __fmul_rn(ff_f(rsd), __fmul_rn(0.5f, y)));
  if (!pos) q = FF{zero ? 0.f : __int_as_float(0x7fc00000), 0.f};
  const float rq = pos ? y : (zero ? __int_as_float(0x7f800000) : __int_as_float(0x7fc00000));
  // id = 1 / (1 + q): z0 = rcp(op), corrected by z0 (1 - op z0)
  const FF op = ff_add_f(q, 1.f);
  const float z0 = rcp_a(op.hi);
  const float pz = __fmul_rn(op.hi, z0);
  const float ez = __fsub_rn(__fsub_rn(__fsub_rn(1.f, pz), __fmaf_rn(op.hi, z0, -pz)), __fmul_rn(op.lo, z0));
  const FF id = ff_fast_two_sum(z0, __fmul_rn(z0, ez));
  FF S = ff_mul(r2, ff_mul_f(id, c));
  float d = 0.5f * c * rq;
  float dd = 0.25f * c * m[17] * rq * rq * rq;
  const int na = (int)m[19];
  if (na > 0) {
    const FF r4 = ff_mul(r2, r2);
    const float r2f = ff_f(r2), r4f = r2f * r2f;
    FF p = r4;                    // r2^p, p = 2(i+1)
    float pm1 = r2f, pm2 = 1.f;   // r2^(p-1), r2^(p-2)
    for (int i = 0; i < na; ++i) {
      const float a = m[24 + i], pf = (float)(2 * (i + 1));
      S = ff_add(S, ff_mul_f(p, a));
      d = fmaf(a * pf, pm1, d);
      dd = fmaf(a * pf * (pf - 1.f), pm2, dd);
      p = ff_mul(p, r4);
      pm1 *= r4f;
      pm2 *= r4f;
    }
  }
  dS = d;
  Srr = dd;
  return S;
}

// core/intersections.py:229-285 intersect_conic on the raw-frame origin, in
// float32 by the cancellation-free form (q = -(B + sign(B) sqrt(disc)) / 2,
// roots q / A and C / q): the smallest root above 1e-8, +inf (or NaN) when
// the ray misses the conic.
__device__ __forceinline__ float conic_start(const float* m, float ox, float oy, float oz, V3 d) {
  const float inf = __int_as_float(0x7f800000);
  const float c = m[15], kp = m[16];
  if (fabsf(c) < 1e-12f) return (fabsf(d.z) > 1e-10f) ? -oz * rcp_a(d.z) : inf;  // plane
  const float A = c * (d.x * d.x + d.y * d.y + kp * d.z * d.z);
  const float B = 2.f * (c * (ox * d.x + oy * d.y + kp * oz * d.z) - d.z);
  const float C = c * (ox * ox + oy * oy + kp * oz * oz) - 2.f * oz;
  const float disc = B * B - 4.f * A * C;
  const float qv = -0.5f * (B + copysignf(sqrtf(fmaxf(disc, 0.f)), B));
  const float t1 = qv * rcp_a(A), t2 = C * rcp_a(qv);
  const bool v1 = t1 > 1e-8f, v2 = t2 > 1e-8f;
  return (disc < 0.f) ? inf : ((v1 && v2) ? fminf(t1, t2) : (v1 ? t1 : (v2 ? t2 : inf)));
}

// core/surfaces.py:67-108 AsphericSurface.intersect + core/intersections.py:290-367
// newton_raphson_intersect (conic start, 10 steps, tol 1e-8, valid if
// t > 1e-8 and |g| < 1e-6). Local frame in, local point and unit normal
// out; returns t or +inf when invalid or outside the aperture
// (core/render.py:100-101). g(t) = o_z + t d_z - sag(o_xy + t d_xy).
//   1. conic start and Newton steps in float32 while the steps exceed the
//      float32 resolution (1e-5): the conic root may lie on the quadric's
//      other sheet, metres from the surface, and these steps carry t across.
//   2. Newton steps in double-float arithmetic (the ray point, the sag and
//      the residual g as float pairs, about 2^-44 relative; g' in float32:
//      it only scales the step, the iteration still converges to the root
//      an FP64 evaluation gives), with the reference's test |g| < 1e-8
//      (the step at the first evaluation that passes it is still applied,
//      as in the reference).
//      Where a step from a failing evaluation leaves a residual
//      |g''| step^2 / 2 below 1e-9 |g'| (step below 1e-4, inside the domain),
//      the evaluation the reference makes next passes the test and moves t
//      by less than 1e-9: the iteration ends there.
//   3. After a final step below 1e-4 the sag and its slope at t are the last
//      evaluation's moved by Taylor steps in r2 (residual far below 1e-6:
//      valid); otherwise the surface is evaluated again at t.
// The float32 steps and the residual bound change t by far less than the
// float32 resolution of the outputs. A NaN residual stays NaN through every
// later step in the reference: the ray is invalid and the iteration stops.
__device__ __forceinline__ float mirror_hit(const float* m, V3 o, V3 d, V3& pl, V3& nl) {
  const float inf = __int_as_float(0x7f800000);
  // origin in the raw surface frame (core/surfaces.py:86-91)
  const float oxf = o.x + m[12], oyf = o.y + m[13], ozf = o.z + m[48];
  float tf = conic_start(m, oxf, oyf, ozf, d);
  bool live = fabsf(tf) < inf;
  int it = 0;
  if (live) {
    for (; it < 8; ++it) {
      const float xs = fmaf(tf, d.x, oxf), ys = fmaf(tf, d.y, oyf);
      float dSf;
      const float Sf = sag_f(m, fmaf(xs, xs, ys * ys), dSf);
      const float g = fmaf(tf, d.z, ozf) - Sf;
      const float gp = d.z - 2.f * dSf * (xs * d.x + ys * d.y);
      const float st = g * rcp_a((fabsf(gp) > 1e-12f) ? gp : 1e-12f);
      if (!(fabsf(st) < inf)) break;  // keep the last finite t: the double-float phase decides
      tf -= st;
      if (fabsf(st) < 1e-5f) {
        ++it;
        break;
      }
    }
  }
  // origin in the raw frame as exact float pairs
  const FF ox = ff_two_sum(o.x, m[12]), oy = ff_two_sum(o.y, m[13]);
  const FF oz = ff_add_f(FF{m[48], m[49]}, o.z);
  FF t = {tf, 0.f}, S = {0.f, 0.f}, xs = {0.f, 0.f}, ys = {0.f, 0.f};
  float dS = 0.f, Srr = 0.f, stepf = 0.f, w = 0.f;
  bool conv = false;
  for (; it < 10 && live && !conv; ++it) {
    xs = ff_add(ox, ff_mul_f(t, d.x));
    ys = ff_add(oy, ff_mul_f(t, d.y));
    float qqf;
    S = sag_ff(m, ff_add(ff_mul(xs, xs), ff_mul(ys, ys)), dS, Srr, qqf);
    const float g = ff_f(ff_add(ff_add(oz, ff_mul_f(t, d.z)), ff_neg(S)));
    w = xs.hi * d.x + ys.hi * d.y;
    const float gp = d.z - 2.f * dS * w;
    const float gs = (fabsf(gp) > 1e-12f) ? gp : 1e-12f;
    conv = fabsf(g) < 1e-8f;
    live = !isnan(g);
    stepf = g * rcp_a(gs);
    t = ff_add_f(t, -stepf);
    if (!conv) {
      const float gpp = fabsf(2.f * dS * (d.x * d.x + d.y * d.y) + 4.f * Srr * w * w);
      conv = (fabsf(stepf) < 1e-4f) && (qqf > 1e-2f) && (0.5f * gpp * stepf * stepf < 1e-9f * fabsf(gs));
    }
  }
  bool valid;
  float px, py, pz;
  if (!live) {
    valid = false;
    px = py = pz = 0.f;
  } else if (conv && fabsf(stepf) < 1e-4f) {
    // r2(t) - r2(t + step) for the last step, then Taylor steps of S and S'
    const float dr2 = stepf * (stepf * (d.x * d.x + d.y * d.y) - 2.f * w);
    S = ff_add_f(S, fmaf(0.5f * Srr, dr2, dS) * dr2);
    dS = fmaf(Srr, dr2, dS);
    px = fmaf(-stepf, d.x, ff_f(ff_add_f(xs, -m[12])));
    py = fmaf(-stepf, d.y, ff_f(ff_add_f(ys, -m[13])));
    valid = t.hi > 1e-8f;
  } else {
    xs = ff_add(ox, ff_mul_f(t, d.x));
    ys = ff_add(oy, ff_mul_f(t, d.y));
    float qqf;
    S = sag_ff(m, ff_add(ff_mul(xs, xs), ff_mul(ys, ys)), dS, Srr, qqf);
    const float g = ff_f(ff_add(ff_add(oz, ff_mul_f(t, d.z)), ff_neg(S)));
    px = ff_f(ff_add_f(xs, -m[12]));
    py = ff_f(ff_add_f(ys, -m[13]));
    valid = (t.hi > 1e-8f) && (fabsf(g) < 1e-6f);
  }
  pz = ff_f(ff_add(S, FF{-m[48], -m[49]}));
  const float xsf = px + m[12], ysf = py + m[13];
  const float nx = -2.f * dS * xsf, ny = -2.f * dS * ysf;
  const float inn = rsqrtf(fmaf(nx, nx, fmaf(ny, ny, 1.f)));
  pl = mk(px, py, pz);
  nl = mk(nx * inn, ny * inn, inn);
  // telescope/mirrors.py:147-149 disk, :209-220 polygon check_aperture
  bool in_ap;
  if ((int)m[20] == IACT_APERTURE_DISK) {
    in_ap = pl.x * pl.x + pl.y * pl.y <= m[18];
  } else {
    in_ap = true;
    int n = (int)m[21];
    for (int i = 0; i < n; ++i) {
      int j = (i + 1 == n) ? 0 : i + 1;
      float ax = m[32 + 2 * i], ay = m[33 + 2 * i], bx = m[32 + 2 * j], by = m[33 + 2 * j];
      float cr = (bx - ax) * (pl.y - ay) - (by - ay) * (pl.x - ax);
      in_ap = in_ap && (cr >= 0.f);
    }
  }
  return (valid && in_ap) ? ff_f(t) : inf;
}

// Offsets (floats) of the record groups inside the table region.
struct TableOffsets {
  int cyl, box, sph, obox, tri, mir, total;
};
__host__ __device__ inline TableOffsets table_offsets(int n_cyl, int n_box, int n_sph, int n_obox,
                                                      int n_tri, int n_mir) {
  TableOffsets t;
  t.cyl = 0;
  t.box = t.cyl + n_cyl * kCylF;
  t.sph = t.box + n_box * kBoxF;
  t.obox = t.sph + n_sph * kSphF;
  t.tri = t.obox + n_obox * kOboxF;
  t.mir = (t.tri + n_tri * kTriF + 3) & ~3;
  t.total = t.mir + n_mir * kMirF;
  return t;
}


// Obstruction view over the table region staged in shared memory.
__device__ __forceinline__ Obst make_obst(const float* tab, int n_cyl, int n_box, int n_sph, int n_obox, int n_tri) {
  const TableOffsets to = table_offsets(n_cyl, n_box, n_sph, n_obox, n_tri, 0);
  Obst ob;
  ob.cyl = tab + to.cyl; ob.box = tab + to.box; ob.sph = tab + to.sph; ob.obox = tab + to.obox; ob.tri = tab + to.tri;
  ob.n_cyl = n_cyl; ob.n_box = n_box; ob.n_sph = n_sph; ob.n_obox = n_obox; ob.n_tri = n_tri;
  return ob;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

}  // namespace iact

namespace iact {

// Sag derivatives of one stage mirror for the adjoint (core/surfaces.py:25-58).
// S(rho) = c rho / (1 + q) + sum_i a_i rho^(2(i+1)), q = sqrt(1 - (1+k) c^2 rho):
//   S_rho = c / (2q) + sum_i p_i a_i rho^(p_i - 1),  S_rhorho = c (1+k) c^2 / (4 q^3) + ...
//   S_c = rho/(1+q) + (1+k) c^2 rho^2 / (q (1+q)^2),  S_k = c^3 rho^2 / (2 q (1+q)^2)
//   S_rho,c = 1/(2q) + (1+k) c^2 rho / (2 q^3),       S_rho,k = c^3 rho / (4 q^3)
//   S_a_i = rho^p_i,  S_rho,a_i = p_i rho^(p_i - 1)  (formed by the caller)
// float32: these are derivatives at a known hit, sums of positive-scale
// terms without the cancellation of the root's residual (the root itself is
// found to about 1e-13, mirror_hit).
struct SagD {
  float S, Sr, Srr, Sc, Sk, Src, Srk;
};

__device__ __forceinline__ void sag_derivs(const float* m, float rho, SagD& o) {
  const float c = m[15], al = m[17];
  const float qq = fmaf(-al, rho, 1.f);
  const float iq = qq > 0.f ? rsqrtf(qq) : (qq == 0.f ? __int_as_float(0x7f800000) : __int_as_float(0x7fc00000));
  const float q = qq > 0.f ? qq * iq : (qq == 0.f ? 0.f : iq);
  const float iq3 = iq * iq * iq, iopq = 1.f / (1.f + q), iopq2 = iopq * iopq;
  o.S = c * rho * iopq;
  o.Sr = 0.5f * c * iq;
  o.Srr = 0.25f * c * al * iq3;
  o.Sc = rho * iopq + al * rho * rho * iq * iopq2;
  o.Sk = 0.5f * c * c * c * rho * rho * iq * iopq2;
  o.Src = 0.5f * iq + 0.5f * al * rho * iq3;
  o.Srk = 0.25f * c * c * c * rho * iq3;
  const int na = (int)m[19];
  float rp = rho * rho;  // rho^p, p = 2
  float rpm1 = rho;      // rho^(p-1)
  float rpm2 = 1.f;      // rho^(p-2)
  for (int i = 0; i < na; ++i) {
    const float p = 2.f * (i + 1), a = m[24 + i];
    o.S += a * rp;
    o.Sr += a * p * rpm1;
    o.Srr += a * p * (p - 1.f) * rpm2;
    rp *= rho * rho;
    rpm1 *= rho * rho;
    rpm2 *= rho * rho;
  }
}

}  // namespace iact

namespace iact {

// Counter-based generator for per-ray jitter: Philox4x32-10 (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011).
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint64_t p0 = (uint64_t)M0 * c[0], p1 = (uint64_t)M1 * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += W0;
    k1 += W1;
  }
}

// Two N(0,1) draws for ray (source s, facet f, sample m) by Box-Muller on
// the first two Philox words: u1 in (0, 1], u2 in [0, 1), 24-bit resolution.
__device__ __forceinline__ void ray_normals(uint32_t seed, int s, int f, int m, float& z0, float& z1) {
  uint32_t c[4] = {(uint32_t)m, (uint32_t)f, (uint32_t)s, 0x1ACE7u};
  philox4x32_10(c, seed, 0x5EEDu);
  const float u1 = (float)((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
  const float u2 = (float)(c[1] >> 8) * (1.0f / 16777216.0f);
  // hardware approximations (absolute error ~1e-6 in z0, z1: a jitter of
  // sigma * 1e-6 rad, far below the binning and parity tolerances)
  const float rad = sqrtf(-2.f * __logf(u1));
  float sn, cs;
  __sincosf(6.28318530717958647f * u2, &sn, &cs);
  z0 = rad * cs;
  z1 = rad * sn;
}

// Extended source: unit direction dh (normalised source direction) tilted by
// sigma * (z0 t1 + z1 t2) in its tangent plane, t1 = normalize(dh x ref),
// ref = x if |dh_z| > 0.9 else z (the basis of core/reflection.py:40-47), t2 = dh x t1.
// The basis depends on the source only (computed once per source run).
struct JBasis {
  V3 dh, t1, t2;
};
__device__ __forceinline__ JBasis jitter_basis(V3 src) {
  JBasis b;
  b.dh = rsqrtf(dot(src, src)) * src;
  const V3 dh = b.dh;
  const V3 ref = fabsf(dh.z) > 0.9f ? mk(1.f, 0.f, 0.f) : mk(0.f, 0.f, 1.f);
  V3 t1 = mk(dh.y * ref.z - dh.z * ref.y, dh.z * ref.x - dh.x * ref.z, dh.x * ref.y - dh.y * ref.x);
  t1 = rsqrtf(dot(t1, t1)) * t1;
  b.t1 = t1;
  b.t2 = mk(dh.y * t1.z - dh.z * t1.y, dh.z * t1.x - dh.x * t1.z, dh.x * t1.y - dh.y * t1.x);
  return b;
}
__device__ __forceinline__ V3 jitter_dir(const JBasis& b, float sigma, float z0, float z1) {
  const V3 d = b.dh + sigma * (z0 * b.t1 + z1 * b.t2);
  return rsqrtf(dot(d, d)) * d;
}

}  // namespace iact
