// ORACLE — test infrastructure only. Nothing in the iactrace_gb300 product
// path includes, links or calls this file; only tests/, the smoke check of
// __graft_entry__ and the cpu_baseline / reference arm of bench.py use it,
// as the oracle of the parity tests and as the timed CPU restatement.
//
// A CPU restatement of the render path of GerritRo/iactrace v0.4.0
// (JAX/Equinox), templated on the arithmetic type T:
//   T = double : the FP64 oracle the CUDA path is compared against,
//   T = float  : the FP32 restatement (same op order as the reference's
//                float32 JAX code) used for index parity and, multi-threaded,
//                as the timed CPU baseline.
// Every function cites the reference file:line it restates. Operation order
// follows the reference expression by expression; build with
// -ffp-contract=off so that no fused multiply-add changes the rounding.
//
// Parity pin: the reference cannot run unmodified here (JAX is absent), so
// its own Python source is executed on a numpy stand-in for jax/equinox
// (tests/golden/make_golden.py) and the outputs are committed as golden
// fixtures; tests/test_oracle_golden.py checks this restatement against them.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/iactrace_gb300.h"

namespace oracle {

template <typename T>
struct Vec3 {
  T x, y, z;
};

template <typename T>
inline T inf_v() {
  return std::numeric_limits<T>::infinity();
}

// jnp.minimum / jnp.maximum / jnp.min / jnp.max propagate NaN.
template <typename T>
inline T nmin(T a, T b) {
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<T>::quiet_NaN();
  return a < b ? a : b;
}
template <typename T>
inline T nmax(T a, T b) {
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<T>::quiet_NaN();
  return a > b ? a : b;
}

// jnp.sum(a * b, axis=-1) over three components: ((a0*b0 + a1*b1) + a2*b2)
template <typename T>
inline T dot3(const Vec3<T>& a, const Vec3<T>& b) {
  return (a.x * b.x + a.y * b.y) + a.z * b.z;
}
template <typename T>
inline Vec3<T> sub3(const Vec3<T>& a, const Vec3<T>& b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
inline Vec3<T> ld3(const float* p) {
  return {T(p[0]), T(p[1]), T(p[2])};
}
// jnp.linalg.norm over three components
template <typename T>
inline T norm3(const Vec3<T>& a) {
  return std::sqrt(dot3(a, a));
}
// jnp.cross
template <typename T>
inline Vec3<T> cross3(const Vec3<T>& a, const Vec3<T>& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
inline T sgn(T v) {
  return v > T(0) ? T(1) : (v < T(0) ? T(-1) : T(0));
}

template <typename T>
struct Mat3 {
  T m[3][3];
  // einsum('ij,nj->ni', R, v)
  Vec3<T> mul(const Vec3<T>& v) const {
    return {(m[0][0] * v.x + m[0][1] * v.y) + m[0][2] * v.z,
            (m[1][0] * v.x + m[1][1] * v.y) + m[1][2] * v.z,
            (m[2][0] * v.x + m[2][1] * v.y) + m[2][2] * v.z};
  }
  // einsum('ij,nj->ni', R.T, v)
  Vec3<T> tmul(const Vec3<T>& v) const {
    return {(m[0][0] * v.x + m[1][0] * v.y) + m[2][0] * v.z,
            (m[0][1] * v.x + m[1][1] * v.y) + m[2][1] * v.z,
            (m[0][2] * v.x + m[1][2] * v.y) + m[2][2] * v.z};
  }
};

template <typename T>
inline Mat3<T> matmul(const Mat3<T>& a, const Mat3<T>& b) {
  Mat3<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      r.m[i][j] = (a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j]) + a.m[i][2] * b.m[2][j];
  return r;
}

// core/transforms.py:72-107 euler_to_matrix: degrees -> Rz @ Ry @ Rx
template <typename T>
inline Mat3<T> euler_to_matrix(const float* deg) {
  const T k = T(M_PI / 180.0);
  T rx = T(deg[0]) * k, ry = T(deg[1]) * k, rz = T(deg[2]) * k;
  T cx = std::cos(rx), sx = std::sin(rx);
  T cy = std::cos(ry), sy = std::sin(ry);
  T cz = std::cos(rz), sz = std::sin(rz);
  Mat3<T> Rx = {{{1, 0, 0}, {0, cx, -sx}, {0, sx, cx}}};
  Mat3<T> Ry = {{{cy, 0, sy}, {0, 1, 0}, {-sy, 0, cy}}};
  Mat3<T> Rz = {{{cz, -sz, 0}, {sz, cz, 0}, {0, 0, 1}}};
  return matmul(matmul(Rz, Ry), Rx);  // (Rz @ Ry) @ Rx
}

// core/reflection.py:5-20 reflect: returns r and cos = -(d.n)
template <typename T>
inline Vec3<T> reflect(const Vec3<T>& d, const Vec3<T>& n, T* cos_out) {
  T c = dot3(d, n);
  T c2 = T(2) * c;
  *cos_out = -c;
  return {d.x - c2 * n.x, d.y - c2 * n.y, d.z - c2 * n.z};
}

// ---------------------------------------------------------------- primitives

// core/intersections.py:44-87 intersect_cylinder
template <typename T>
inline T intersect_cylinder(const Vec3<T>& o, const Vec3<T>& d, const float* cyl) {
  const T eps = T(1e-8);
  Vec3<T> p1 = ld3<T>(cyl), p2 = ld3<T>(cyl + 3);
  T radius = T(cyl[6]);
  Vec3<T> axis = sub3(p2, p1);
  T height = norm3(axis);
  axis = {axis.x / height, axis.y / height, axis.z / height};
  Vec3<T> oc = sub3(o, p1);
  T oc_axial = dot3(oc, axis);
  T rd_axial = dot3(d, axis);
  Vec3<T> oc_perp = {oc.x - oc_axial * axis.x, oc.y - oc_axial * axis.y, oc.z - oc_axial * axis.z};
  Vec3<T> rd_perp = {d.x - rd_axial * axis.x, d.y - rd_axial * axis.y, d.z - rd_axial * axis.z};
  T a = dot3(rd_perp, rd_perp);
  T b = T(2) * dot3(oc_perp, rd_perp);
  T c = dot3(oc_perp, oc_perp) - radius * radius;
  T disc = b * b - T(4) * a * c;
  T sq = std::sqrt(std::max(disc, T(0)));
  T t1 = (-b - sq) / (T(2) * a + eps);
  T t2 = (-b + sq) / (T(2) * a + eps);
  T y1 = oc_axial + t1 * rd_axial;
  T y2 = oc_axial + t2 * rd_axial;
  t1 = ((t1 > eps) && (y1 >= 0) && (y1 <= height) && (disc >= 0)) ? t1 : inf_v<T>();
  t2 = ((t2 > eps) && (y2 >= 0) && (y2 <= height) && (disc >= 0)) ? t2 : inf_v<T>();
  T t_bottom = -oc_axial / (rd_axial + eps);
  T t_top = (height - oc_axial) / (rd_axial + eps);
  Vec3<T> pb = {oc_perp.x + t_bottom * rd_perp.x, oc_perp.y + t_bottom * rd_perp.y,
                oc_perp.z + t_bottom * rd_perp.z};
  Vec3<T> pt = {oc_perp.x + t_top * rd_perp.x, oc_perp.y + t_top * rd_perp.y,
                oc_perp.z + t_top * rd_perp.z};
  T r2 = radius * radius;
  t_bottom = ((t_bottom > eps) && (dot3(pb, pb) <= r2)) ? t_bottom : inf_v<T>();
  t_top = ((t_top > eps) && (dot3(pt, pt) <= r2)) ? t_top : inf_v<T>();
  return nmin(nmin(nmin(t1, t2), t_bottom), t_top);
}

// core/intersections.py:90-110 intersect_box (axis aligned slab test)
template <typename T>
inline T intersect_box(const Vec3<T>& o, const Vec3<T>& d, const float* box) {
  const T eps = T(1e-8);
  T p1[3] = {T(box[0]), T(box[1]), T(box[2])};
  T p2[3] = {T(box[3]), T(box[4]), T(box[5])};
  T oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  T t_min = -inf_v<T>(), t_max = inf_v<T>();
  for (int i = 0; i < 3; ++i) {
    T bmin = nmin(p1[i], p2[i]), bmax = nmax(p1[i], p2[i]);
    T inv = T(1) / (dd[i] + eps);
    T t1 = (bmin - oo[i]) * inv;
    T t2 = (bmax - oo[i]) * inv;
    T tn = nmin(t1, t2), tf = nmax(t1, t2);
    t_min = (i == 0) ? tn : nmax(t_min, tn);
    t_max = (i == 0) ? tf : nmin(t_max, tf);
  }
  bool hit = (t_max >= t_min) && (t_max > eps);
  T tr = (t_min > eps) ? t_min : t_max;
  return hit ? tr : inf_v<T>();
}

// core/intersections.py:195-226 intersect_sphere
template <typename T>
inline T intersect_sphere(const Vec3<T>& o, const Vec3<T>& d, const float* sph) {
  const T eps = T(1e-8);
  Vec3<T> oc = sub3(o, ld3<T>(sph));
  T radius = T(sph[3]);
  T a = dot3(d, d);
  T b = T(2) * dot3(oc, d);
  T c = dot3(oc, oc) - radius * radius;
  T disc = b * b - T(4) * a * c;
  T sq = std::sqrt(std::max(disc, T(0)));
  T t1 = (-b - sq) / (T(2) * a + eps);
  T t2 = (-b + sq) / (T(2) * a + eps);
  T t1v = ((t1 > eps) && (disc >= 0)) ? t1 : inf_v<T>();
  T t2v = ((t2 > eps) && (disc >= 0)) ? t2 : inf_v<T>();
  return nmin(t1v, t2v);
}

// core/intersections.py:113-149 intersect_oriented_box; R row-major local->world
template <typename T>
inline T intersect_oriented_box(const Vec3<T>& o, const Vec3<T>& d, const float* ob) {
  const T eps = T(1e-8);
  Mat3<T> R;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R.m[i][j] = T(ob[6 + 3 * i + j]);
  Vec3<T> lo = R.tmul(sub3(o, ld3<T>(ob)));
  Vec3<T> ldr = R.tmul(d);
  T half[3] = {T(ob[3]), T(ob[4]), T(ob[5])};
  T ll[3] = {lo.x, lo.y, lo.z}, dd[3] = {ldr.x, ldr.y, ldr.z};
  T t_min = 0, t_max = 0;
  for (int i = 0; i < 3; ++i) {
    T inv = T(1) / (dd[i] + eps * sgn(dd[i] + eps));
    T t1 = (-half[i] - ll[i]) * inv;
    T t2 = (half[i] - ll[i]) * inv;
    T tn = nmin(t1, t2), tf = nmax(t1, t2);
    t_min = (i == 0) ? tn : nmax(t_min, tn);
    t_max = (i == 0) ? tf : nmin(t_max, tf);
  }
  bool hit = (t_max >= t_min) && (t_max > eps);
  T tr = (t_min > eps) ? t_min : t_max;
  return (hit && (tr > eps)) ? tr : inf_v<T>();
}

// core/intersections.py:152-192 intersect_triangle (Moller-Trumbore)
template <typename T>
inline T intersect_triangle(const Vec3<T>& o, const Vec3<T>& d, const float* tri) {
  const T eps = T(1e-8);
  Vec3<T> v0 = ld3<T>(tri), v1 = ld3<T>(tri + 3), v2 = ld3<T>(tri + 6);
  Vec3<T> e1 = sub3(v1, v0), e2 = sub3(v2, v0);
  Vec3<T> h = cross3(d, e2);
  T a = dot3(e1, h);
  bool parallel = std::fabs(a) < eps;
  T f = T(1) / (a + eps * sgn(a + eps));
  Vec3<T> s = sub3(o, v0);
  T u = f * dot3(s, h);
  Vec3<T> q = cross3(s, e1);
  T v = f * dot3(d, q);
  T t = f * dot3(e2, q);
  bool valid = !parallel && (u >= 0) && (u <= 1) && (v >= 0) && (u + v <= 1) && (t > eps);
  return valid ? t : inf_v<T>();
}

// core/render.py:21-41 _check_occlusions: 1 unless some group's min t < 1e10
template <typename T>
inline T shadow_mask(const iact_scene_t& sc, const Vec3<T>& o, const Vec3<T>& d) {
  const T big = T(1e10);
  // one group per kind (core/obstructions.py:258-277 group_obstructions);
  // a group shadows iff its min t (jnp.min, NaN-propagating) is < 1e10.
  auto group = [&](int n, const float* tab, int stride, auto fn) -> bool {
    if (n <= 0) return false;
    T m = fn(o, d, tab);
    for (int i = 1; i < n; ++i) m = nmin(m, fn(o, d, tab + (size_t)i * stride));
    return m < big;
  };
  T mask = T(1);
  if (group(sc.n_cyl, sc.cyl, 7, intersect_cylinder<T>)) mask = mask * T(0);
  if (group(sc.n_box, sc.box, 6, intersect_box<T>)) mask = mask * T(0);
  if (group(sc.n_sph, sc.sph, 4, intersect_sphere<T>)) mask = mask * T(0);
  if (group(sc.n_obox, sc.obox, 15, intersect_oriented_box<T>)) mask = mask * T(0);
  if (group(sc.n_tri, sc.tri, 9, intersect_triangle<T>)) mask = mask * T(0);
  return mask;
}

// ------------------------------------------------------------------ surfaces

// core/surfaces.py:25-39 _sag_raw; aspheric term i multiplies r2**(2(i+1))
template <typename T>
inline T sag_raw(const iact_mirror_t& mr, T x, T y) {
  T c = T(mr.curvature), k = T(mr.conic);
  T r2 = x * x + y * y;
  T denom = T(1) + std::sqrt(T(1) - (T(1) + k) * c * c * r2);
  T z = r2 * c / denom;
  if (mr.n_asph > 0) {
    T s = 0;
    for (int i = 0; i < mr.n_asph; ++i) s = s + T(mr.asph[i]) * std::pow(r2, T(2 * (i + 1)));
    z = z + s;
  }
  return z;
}

// d(_sag_raw)/dr2, the derivative jax.grad takes through r2 = x^2 + y^2
// (core/surfaces.py:51-58 normal, core/intersections.py:328-330 g_deriv)
template <typename T>
inline T sag_raw_dr2(const iact_mirror_t& mr, T r2) {
  T c = T(mr.curvature), k = T(mr.conic);
  T alpha = (T(1) + k) * c * c;
  T s = std::sqrt(T(1) - alpha * r2);
  T denom = T(1) + s;
  // z = r2*c/denom ; dz/dr2 = c/denom + r2*c*alpha/(2 s denom^2)
  T dz = c / denom + (r2 * c) * alpha / (T(2) * s * denom * denom);
  for (int i = 0; i < mr.n_asph; ++i) {
    T p = T(2 * (i + 1));
    dz = dz + T(mr.asph[i]) * p * std::pow(r2, p - T(1));
  }
  return dz;
}

// core/surfaces.py:41-45 sag (with the parent-surface offset)
template <typename T>
inline T sag(const iact_mirror_t& mr, T x, T y) {
  T x0 = T(mr.offset[0]), y0 = T(mr.offset[1]);
  T z0 = sag_raw<T>(mr, x0, y0);
  return sag_raw<T>(mr, x + x0, y + y0) - z0;
}

// core/surfaces.py:51-58 normal
template <typename T>
inline Vec3<T> surface_normal(const iact_mirror_t& mr, T x, T y) {
  T xs = x + T(mr.offset[0]), ys = y + T(mr.offset[1]);
  T r2 = xs * xs + ys * ys;
  T g = sag_raw_dr2<T>(mr, r2);
  T dzdx = g * (T(2) * xs), dzdy = g * (T(2) * ys);
  Vec3<T> n = {-dzdx, -dzdy, T(1)};
  T nn = norm3(n);
  return {n.x / nn, n.y / nn, n.z / nn};
}

// core/intersections.py:229-285 intersect_conic
template <typename T>
inline T intersect_conic(const Vec3<T>& o, const Vec3<T>& d, T c, T k) {
  T kp = T(1) + k;
  T A = c * (d.x * d.x + d.y * d.y + kp * d.z * d.z);
  T B = T(2) * (c * (o.x * d.x + o.y * d.y + kp * o.z * d.z) - d.z);
  T C = c * (o.x * o.x + o.y * o.y + kp * o.z * o.z) - T(2) * o.z;
  bool is_plane = std::fabs(c) < T(1e-12);
  T t_plane = (std::fabs(d.z) > T(1e-10)) ? -o.z / d.z : inf_v<T>();
  T disc = B * B - T(4) * A * C;
  bool no_int = disc < 0;
  T sq = std::sqrt(std::max(disc, T(0)));
  T t1 = (-B - sq) / (T(2) * A + T(1e-30));
  T t2 = (-B + sq) / (T(2) * A + T(1e-30));
  bool v1 = t1 > T(1e-8), v2 = t2 > T(1e-8);
  T tc = (v1 && v2) ? nmin(t1, t2) : (v1 ? t1 : (v2 ? t2 : inf_v<T>()));
  tc = no_int ? inf_v<T>() : tc;
  return is_plane ? t_plane : tc;
}

// core/surfaces.py:67-108 AsphericSurface.intersect with
// core/intersections.py:290-367 newton_raphson_intersect (max_iter 10, tol 1e-8)
template <typename T>
inline T surface_intersect(const iact_mirror_t& mr, const Vec3<T>& o, const Vec3<T>& d,
                           Vec3<T>* point, Vec3<T>* normal) {
  const T tol = T(1e-8);
  T x0 = T(mr.offset[0]), y0 = T(mr.offset[1]);
  T z0 = sag_raw<T>(mr, x0, y0);
  Vec3<T> oraw = {o.x + x0, o.y + y0, o.z + z0};
  T t = intersect_conic<T>(oraw, d, T(mr.curvature), T(mr.conic));
  auto g = [&](T tt) {
    T x = o.x + tt * d.x, y = o.y + tt * d.y, z = o.z + tt * d.z;
    return z - (sag_raw<T>(mr, x + x0, y + y0) - z0);
  };
  auto gp = [&](T tt) {
    T x = o.x + tt * d.x, y = o.y + tt * d.y;
    T xs = x + x0, ys = y + y0;
    T dr2 = sag_raw_dr2<T>(mr, xs * xs + ys * ys);
    return d.z - (dr2 * (T(2) * xs) * d.x + dr2 * (T(2) * ys) * d.y);
  };
  bool conv = false;
  for (int it = 0; it < 10; ++it) {  // lax.scan newton_step, length 10
    T gv = g(t);
    T gd = gp(t);
    T gs = (std::fabs(gd) > T(1e-12)) ? gd : T(1e-12);
    T tn = t - gv / gs;
    bool nc = conv || (std::fabs(gv) < tol);
    t = conv ? t : tn;
    conv = nc;
  }
  T xh = o.x + t * d.x, yh = o.y + t * d.y;
  T res = std::fabs(g(t));
  bool valid = (t > T(1e-8)) && (res < tol * T(100));
  *point = {xh, yh, sag<T>(mr, xh, yh)};
  *normal = surface_normal<T>(mr, xh, yh);
  return valid ? t : inf_v<T>();
}

// telescope/mirrors.py:147-149 (disk) and :209-220 (polygon) check_aperture
template <typename T>
inline bool check_aperture(const iact_mirror_t& mr, T x, T y) {
  if (mr.aperture == IACT_APERTURE_DISK) {
    T r = T(mr.radius);
    return x * x + y * y <= r * r;
  }
  bool inside = true;
  int n = mr.n_vert;
  for (int i = 0; i < n; ++i) {
    T ax = T(mr.vert[i][0]), ay = T(mr.vert[i][1]);
    T bx = T(mr.vert[(i + 1) % n][0]), by = T(mr.vert[(i + 1) % n][1]);
    T cr = (bx - ax) * (y - ay) - (by - ay) * (x - ax);
    inside = inside && (cr >= 0);
  }
  return inside;
}

// core/intersections.py:6-41 intersect_plane: local (x, y) or (1e10, 1e10)
template <typename T>
inline void intersect_plane(const Vec3<T>& o, const Vec3<T>& d, const Vec3<T>& center,
                            const Mat3<T>& R, T* xo, T* yo) {
  Vec3<T> u1 = {R.m[0][0], R.m[1][0], R.m[2][0]};
  Vec3<T> u2 = {R.m[0][1], R.m[1][1], R.m[2][1]};
  Vec3<T> n = {R.m[0][2], R.m[1][2], R.m[2][2]};
  T ndotd = dot3(d, n), ndoto = dot3(o, n), ndotp = dot3(n, center);
  bool parallel = std::fabs(ndotd) < T(1e-10);
  T safe = parallel ? T(1) : ndotd;
  T t = (ndotp - ndoto) / safe;
  Vec3<T> p = {o.x + t * d.x, o.y + t * d.y, o.z + t * d.z};
  Vec3<T> op = sub3(p, center);
  T x = dot3(op, u1), y = dot3(op, u2);
  bool invalid = parallel || (t <= 0);
  *xo = invalid ? T(1e10) : x;
  *yo = invalid ? T(1e10) : y;
}

// ------------------------------------------------------------------- sensors

// float -> int32 as numpy does on x86 (out of range / NaN -> INT_MIN);
// any such value lands outside the sensor, which is all the binning uses.
template <typename T>
inline int64_t f2i(T v) {
  if (!(v >= T(-2147483648.0) && v < T(2147483648.0))) return INT32_MIN;
  return (int64_t)v;
}

// sensors/square.py:66-91 SquareSensor.accumulate (per ray); margin = FP
// distance to the nearest pixel edge (or to the edge_width band).
template <typename T>
inline int32_t bin_square(const iact_sensor_t& s, T x, T y, T* margin) {
  T dx = T(s.dx), dy = T(s.dy);
  T xc = (x - T(s.x0)) / dx, yc = (y - T(s.y0)) / dy;
  int64_t xi = f2i(std::floor(xc)), yi = f2i(std::floor(yc));
  bool valid = (xi >= 0) && (xi < s.width) && (yi >= 0) && (yi < s.height);
  T xf = xc - T((int32_t)xi), yf = yc - T((int32_t)yi);
  T dist = std::min(std::min(xf, T(1) - xf) * dx, std::min(yf, T(1) - yf) * dy);
  bool on_edge = dist < T(s.edge_width);
  valid = valid && !on_edge;
  if (margin) {
    T m = dist;
    if (s.edge_width > 0) m = std::min(m, std::fabs(dist - T(s.edge_width)));
    *margin = m;
  }
  return valid ? (int32_t)(yi * s.width + xi) : -1;
}

template <typename T>
struct HexLocal {
  T xg, yg, qi, ri;
  int32_t pix;
};

// sensors/hexagonal.py:32-39 _axial_round (jnp.round = half to even)
template <typename T>
inline void axial_round(T q, T r, T* qo, T* ro) {
  T s = -q - r;
  T qi = std::nearbyint(q), ri = std::nearbyint(r), si = std::nearbyint(s);
  T dq = std::fabs(qi - q), dr = std::fabs(ri - r), ds = std::fabs(si - s);
  if ((dq > dr) && (dq > ds)) qi = -ri - si;
  if ((dr > dq) && (dr > ds)) ri = -qi - si;
  *qo = qi;
  *ro = ri;
}

// sensors/hexagonal.py:155-172 _lookup_pixels
template <typename T>
inline int32_t hex_lookup(const iact_sensor_t& s, T qi, T ri) {
  int64_t q = f2i(qi), r = f2i(ri);
  if (q == INT32_MIN || r == INT32_MIN) return -1;
  int64_t qx = q - s.q_min, rx = r - s.r_min;
  if (qx < 0 || qx >= s.table_q || rx < 0 || rx >= s.table_r) return -1;
  int32_t p = s.table[qx * s.table_r + rx];
  return p >= 0 ? p : -1;
}

// sensors/hexagonal.py:16-23,174-181 grid rotation and axial coordinates
template <typename T>
inline HexLocal<T> hex_locate(const iact_sensor_t& s, T x, T y) {
  const T SQRT3_3 = T(0.5773502691896257);
  T xs = x - T(s.off_x), ys = y - T(s.off_y);
  T c = T(s.grid_cos), sn = T(s.grid_sin);
  HexLocal<T> h;
  h.xg = c * xs - sn * ys;
  h.yg = sn * xs + c * ys;
  T size = T(s.hex_size);
  T q = (SQRT3_3 * h.xg - h.yg / T(3)) / size;
  T r = (T(2) * h.yg / T(3)) / size;
  axial_round(q, r, &h.qi, &h.ri);
  h.pix = hex_lookup(s, h.qi, h.ri);
  return h;
}

// sensors/hexagonal.py:42-47 _hex_norm
template <typename T>
inline T hex_norm(T x, T y, T inradius) {
  const T SQRT3_2 = T(0.8660254037844386);
  T ax = std::fabs(x), ay = std::fabs(y);
  return nmax(ax, T(0.5) * ax + SQRT3_2 * ay) / inradius;
}

// sensors/hexagonal.py:174-194 HexagonalSensor.accumulate (per ray)
template <typename T>
inline int32_t bin_hex(const iact_sensor_t& s, T x, T y, T* margin) {
  HexLocal<T> h = hex_locate(s, x, y);
  T hcx = T(s.hex_sx) * (h.qi + h.ri / T(2));
  T hcy = T(s.hex_sy) * h.ri;
  T inr = T(s.inradius);
  T hd = hex_norm(h.xg - hcx, h.yg - hcy, inr);
  bool on_edge = hd > T(s.edge_threshold);
  if (margin) {
    T m = (T(1) - hd) * inr;
    if (s.edge_threshold < 1.0f) m = std::min(m, std::fabs(hd - T(s.edge_threshold)) * inr);
    *margin = m;
  }
  if (on_edge) return -1;
  return h.pix;
}

template <typename T>
inline int32_t bin_hard(const iact_sensor_t& s, T x, T y, T* margin) {
  return s.type == IACT_SENSOR_SQUARE ? bin_square(s, x, y, margin) : bin_hex(s, x, y, margin);
}

// sensors/square.py:144-172 DifferentiableSquareSensor.accumulate: Gaussian
// over (2K+1)^2 taps normalised per ray, out-of-range taps dropped after.
// Rays whose plane hit is the (1e10, 1e10) sentinel deposit nothing (the
// reference's 0/0 normalisation would turn them into NaN).
template <typename T, typename F>
inline void splat_square(const iact_sensor_t& s, T x, T y, T v, F&& deposit) {
  if (!(x < T(1e9) && y < T(1e9))) return;
  T dx = T(s.dx), dy = T(s.dy);
  T xp = (x - T(s.x0)) / dx, yp = (y - T(s.y0)) / dy;
  T xb = std::floor(xp), yb = std::floor(yp);
  int64_t xi0 = f2i(xb), yi0 = f2i(yb);
  T xf = xp - T((int32_t)xi0), yf = yp - T((int32_t)yi0);
  int K = s.kernel_size, n = 2 * K + 1;
  T sig2 = T(s.sigma) * T(s.sigma);
  std::vector<T> w((size_t)n * n);
  T tot = 0;
  for (int i = 0; i < n; ++i)      // offset_y = i - K
    for (int j = 0; j < n; ++j) {  // offset_x = j - K (meshgrid indexing="xy")
      T ddx = xf - T(j - K), ddy = yf - T(i - K);
      T e = std::exp(T(-0.5) * (ddx * ddx + ddy * ddy) / sig2);
      w[(size_t)i * n + j] = e;
      tot = tot + e;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      int64_t xi = xi0 + (j - K), yi = yi0 + (i - K);
      if (xi < 0 || xi >= s.width || yi < 0 || yi >= s.height) continue;
      deposit((int32_t)(yi * s.width + xi), v * (w[(size_t)i * n + j] / tot));
    }
}

// sensors/hexagonal.py:264-315 DifferentiableHexagonalSensor.accumulate
// (rings = kernel_size; sigma in units of the inradius). Same sentinel rule.
template <typename T, typename F>
inline void splat_hex(const iact_sensor_t& s, T x, T y, T v, F&& deposit) {
  if (!(x < T(1e9) && y < T(1e9))) return;
  HexLocal<T> h = hex_locate(s, x, y);
  T bx = T(s.hex_sx) * (h.qi + h.ri / T(2));
  T by = T(s.hex_sy) * h.ri;
  T ddx = h.xg - bx, ddy = h.yg - by;
  int K = s.kernel_size;
  T inr = T(s.inradius), sg = T(s.sigma);
  struct Tap {
    int q, r;
    T w;
  };
  std::vector<Tap> taps;
  T tot = 0;
  for (int q = -K; q <= K; ++q)  // sensors/hexagonal.py:50-58 neighbour order
    for (int r = -K; r <= K; ++r) {
      if (std::max(std::max(std::abs(q), std::abs(r)), std::abs(-q - r)) > K) continue;
      T ox = T(s.hex_sx) * (T(q) + T(r) / T(2));
      T oy = T(s.hex_sy) * T(r);
      T hd = hex_norm(ddx - ox, ddy - oy, inr);
      T a = hd / sg;
      T e = std::exp(T(-0.5) * (a * a));
      taps.push_back({q, r, e});
      tot = tot + e;
    }
  for (const Tap& tp : taps) {
    int32_t p = hex_lookup(s, h.qi + T(tp.q), h.ri + T(tp.r));
    if (p < 0) continue;
    deposit(p, v * (tp.w / tot));
  }
}

// ------------------------------------------------------------------- render

template <typename T>
struct World {
  std::vector<Vec3<T>> tp, tn;  // [F*M]
  std::vector<T> tw;            // [F*M]
};

// telescope/mirrors.py:64-79 MirrorGroup.transform_to_world (all stage-0 groups)
template <typename T>
inline World<T> transform_to_world(const iact_scene_t& sc) {
  World<T> w;
  size_t F = (size_t)sc.n_facets, M = (size_t)sc.n_samples;
  w.tp.resize(F * M);
  w.tn.resize(F * M);
  w.tw.resize(F * M);
  for (size_t f = 0; f < F; ++f) {
    Mat3<T> R = euler_to_matrix<T>(sc.facet_rot + 3 * f);
    Vec3<T> pos = ld3<T>(sc.facet_pos + 3 * f);
    T scale = T(sc.facet_scale[f]);
    for (size_t m = 0; m < M; ++m) {
      size_t i = f * M + m;
      Vec3<T> p = R.mul(ld3<T>(sc.points + 3 * i));
      Vec3<T> n = R.mul(ld3<T>(sc.normals + 3 * i));
      Vec3<T> dl = R.mul(ld3<T>(sc.delta + 3 * i));
      w.tp[i] = {p.x + pos.x, p.y + pos.y, p.z + pos.z};
      Vec3<T> pe = {n.x + scale * dl.x, n.y + scale * dl.y, n.z + scale * dl.z};
      T nn = norm3(pe);
      w.tn[i] = {pe.x / nn, pe.y / nn, pe.z / nn};
      w.tw[i] = T(sc.weights[i]);
    }
  }
  return w;
}

// Philox4x32-10 (Salmon et al., SC 2011): the per-ray jitter stream of
// extended sources (include/iactrace_gb300.h, IACT_SRC_EXTENDED).
inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int i = 0; i < 10; ++i) {
    const uint64_t p0 = (uint64_t)M0 * c[0], p1 = (uint64_t)M1 * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += W0;
    k1 += W1;
  }
}

template <typename T>
inline void ray_normals(uint32_t seed, int s, int f, int m, T* z0, T* z1) {
  uint32_t c[4] = {(uint32_t)m, (uint32_t)f, (uint32_t)s, 0x1ACE7u};
  philox4x32_10(c, seed, 0x5EEDu);
  const T u1 = T((c[0] >> 8) + 1u) * T(1.0 / 16777216.0);
  const T u2 = T(c[1] >> 8) * T(1.0 / 16777216.0);
  const T rad = std::sqrt(T(-2) * std::log(u1));
  *z0 = rad * std::cos(T(2 * M_PI) * u2);
  *z1 = rad * std::sin(T(2 * M_PI) * u2);
}

// direction dh tilted by sigma (z0 t1 + z1 t2), tangent basis as
// core/reflection.py:40-47
template <typename T>
inline Vec3<T> jitter_dir(Vec3<T> dh, T sigma, T z0, T z1) {
  Vec3<T> ref = std::fabs(dh.z) > T(0.9) ? Vec3<T>{1, 0, 0} : Vec3<T>{0, 0, 1};
  Vec3<T> t1 = cross3(dh, ref);
  T n1 = norm3(t1);
  t1 = {t1.x / n1, t1.y / n1, t1.z / n1};
  Vec3<T> t2 = cross3(dh, t1);
  Vec3<T> d = {dh.x + sigma * (z0 * t1.x + z1 * t2.x), dh.y + sigma * (z0 * t1.y + z1 * t2.y),
               dh.z + sigma * (z0 * t1.z + z1 * t2.z)};
  T nd = norm3(d);
  return {d.x / nd, d.y / nd, d.z / nd};
}

template <typename T>
struct RayOut {
  T x, y, val;
  int32_t hit_mirror;  // index into sc.mirrors of the last stage hit, -1 if none
};

template <typename T>
struct Prepared {
  std::vector<Mat3<T>> mrot;  // stage-mirror rotations
  std::vector<int> stage_begin, stage_end;
  Mat3<T> srot;
  Vec3<T> spos;
};

template <typename T>
inline Prepared<T> prepare(const iact_scene_t& sc, const iact_sensor_t& sn) {
  Prepared<T> p;
  for (int i = 0; i < sc.n_mirrors; ++i) p.mrot.push_back(euler_to_matrix<T>(sc.mirrors[i].rot));
  int i = 0;
  while (i < sc.n_mirrors) {
    int j = i;
    while (j < sc.n_mirrors && sc.mirrors[j].stage == sc.mirrors[i].stage) ++j;
    p.stage_begin.push_back(i);
    p.stage_end.push_back(j);
    i = j;
  }
  p.srot = euler_to_matrix<T>(sn.rot);
  p.spos = ld3<T>(sn.pos);
  return p;
}

// core/render.py:118-157 _trace_single_mirror for one ray, with
// core/render.py:44-115 _reflect_at_stage / _intersect_group for stages >= 1
template <typename T>
inline RayOut<T> trace_ray(const iact_scene_t& sc, const Prepared<T>& pr, const World<T>& w,
                           size_t sample, int src_type, const float* src, T value, uint32_t seed = 0,
                           int s = 0) {
  Vec3<T> tp = w.tp[sample], tn = w.tn[sample];
  Vec3<T> d;
  if (src_type == IACT_SRC_POINT) {
    Vec3<T> dd = sub3(tp, ld3<T>(src));
    T nn = norm3(dd);
    d = {dd.x / nn, dd.y / nn, dd.z / nn};
  } else if (src_type == IACT_SRC_EXTENDED) {
    const int M = sc.n_samples;
    const int f = (int)(sample / (size_t)M), m = (int)(sample % (size_t)M);
    T z0, z1;
    ray_normals<T>(seed, s, f, m, &z0, &z1);
    Vec3<T> dh = ld3<T>(src);
    T nh = norm3(dh);
    d = jitter_dir<T>({dh.x / nh, dh.y / nh, dh.z / nh}, T(src[3]), z0, z1);
  } else {
    d = ld3<T>(src);
  }
  T shadow = shadow_mask(sc, tp, Vec3<T>{-d.x, -d.y, -d.z});
  T cosv;
  Vec3<T> r = reflect(d, tn, &cosv);
  T val = value * cosv / w.tw[sample] * shadow;
  Vec3<T> o = tp;
  int32_t last_hit = -1;
  for (size_t st = 0; st < pr.stage_begin.size(); ++st) {
    T best_t = inf_v<T>();
    Vec3<T> best_p = {0, 0, 0}, best_n = {0, 0, 0};
    int32_t best_i = -1;
    for (int mi = pr.stage_begin[st]; mi < pr.stage_end[st]; ++mi) {
      const iact_mirror_t& mr = sc.mirrors[mi];
      const Mat3<T>& R = pr.mrot[mi];
      Vec3<T> ol = R.tmul(sub3(o, ld3<T>(mr.pos)));
      Vec3<T> dl = R.tmul(r);
      Vec3<T> pl, nl;
      T t = surface_intersect<T>(mr, ol, dl, &pl, &nl);
      if (!check_aperture<T>(mr, pl.x, pl.y)) t = inf_v<T>();
      if (t < best_t) {  // strict: the first of equal minima wins (argmin)
        Vec3<T> pw = R.mul(pl);
        best_t = t;
        best_p = {pw.x + T(mr.pos[0]), pw.y + T(mr.pos[1]), pw.z + T(mr.pos[2])};
        best_n = R.mul(nl);
        best_i = mi;
      }
    }
    T c2;
    Vec3<T> rr = reflect(r, best_n, &c2);
    T hit = (best_t < T(1e10)) ? T(1) : T(0);
    T sh = shadow_mask(sc, o, r);
    val = val * hit * sh * std::fabs(c2);
    o = best_p;
    r = rr;
    last_hit = best_i;
  }
  RayOut<T> out;
  intersect_plane<T>(o, r, pr.spos, pr.srot, &out.x, &out.y);
  out.val = val;
  out.hit_mirror = last_hit;
  return out;
}

}  // namespace oracle
