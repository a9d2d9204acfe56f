// Device code shared by the single-scene render (iact_render.cu) and the
// batched persistent render (iact_batched.cu): per-launch parameters, the
// per-ray chain and the per-tile work.
#pragma once

#include "iact_device.cuh"

// Resident CTAs per SM the single-stage render kernels are compiled for
// (256 threads each): 5 caps them at 48 registers per thread.
#ifndef IACT_RENDER_MIN_CTAS
#define IACT_RENDER_MIN_CTAS 5
#endif

namespace iact {

struct PrepK {
  int F, M;
  const float* facet_pos;
  const float* facet_rot;
  const float* facet_scale;
  const float* points;
  const float* normals;
  const float* delta;
  const float* weights;
  float4* P4;
  float4* N4;
  float4* D4;  // optional: world delta / |n + scale delta| (roughness-scale gradients)
  float4* B4;  // optional (culling): per facet bundle centre and radius
  float* tables;
  const float* cyl;
  const float* box;
  const float* sph;
  const float* obox;
  const float* tri;
  const iact_mirror_t* mirrors;
  int n_cyl, n_box, n_sph, n_obox, n_tri, n_mir;
  uint4* zero;         // optional: region cleared by the prep launch (the accumulator)
  long long n_zero;    // its size in 16-byte words
  int* counter;        // optional: 16 ints cleared (tile counter, error word)
};

// Per-launch constant tables: telescope/mirrors.py and core/obstructions.py
// constants precomputed once (one CTA).
__device__ __forceinline__ void prep_tables(const PrepK& p) {
  TableOffsets to = table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir);
  for (int k = threadIdx.x; k < p.n_cyl; k += blockDim.x) {
    const float* c = p.cyl + 7 * k;
    float* o = p.tables + to.cyl + kCylF * k;
    // core/intersections.py:46-48 axis, height
    float ax = c[3] - c[0], ay = c[4] - c[1], az = c[5] - c[2];
    float h = sqrtf(ax * ax + ay * ay + az * az);
    o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
    o[3] = ax / h; o[4] = ay / h; o[5] = az / h;
    o[6] = h;
    o[7] = c[6] * c[6];
  }
  for (int k = threadIdx.x; k < p.n_box; k += blockDim.x) {
    const float* b = p.box + 6 * k;
    float* o = p.tables + to.box + kBoxF * k;
    for (int a = 0; a < 3; ++a) {  // core/intersections.py:94-95
      o[a] = fminf(b[a], b[3 + a]);
      o[3 + a] = fmaxf(b[a], b[3 + a]);
    }
  }
  for (int k = threadIdx.x; k < p.n_sph; k += blockDim.x) {
    const float* s = p.sph + 4 * k;
    float* o = p.tables + to.sph + kSphF * k;
    o[0] = s[0]; o[1] = s[1]; o[2] = s[2];
    o[3] = s[3] * s[3];
  }
  for (int k = threadIdx.x; k < p.n_obox * kOboxF; k += blockDim.x) p.tables[to.obox + k] = p.obox[k];
  for (int k = threadIdx.x; k < p.n_tri; k += blockDim.x) {
    const float* t = p.tri + 9 * k;
    float* o = p.tables + to.tri + kTriF * k;
    o[0] = t[0]; o[1] = t[1]; o[2] = t[2];
    for (int a = 0; a < 3; ++a) {  // core/intersections.py:166-167 edges
      o[3 + a] = t[3 + a] - t[a];
      o[6 + a] = t[6 + a] - t[a];
    }
  }
  for (int k = threadIdx.x; k < p.n_mir; k += blockDim.x) {
    const iact_mirror_t& m = p.mirrors[k];
    float* o = p.tables + to.mir + kMirF * k;
    euler_to_matrix(m.rot[0], m.rot[1], m.rot[2], o);
    o[9] = m.pos[0]; o[10] = m.pos[1]; o[11] = m.pos[2];
    o[12] = m.offset[0]; o[13] = m.offset[1];
    o[15] = m.curvature;
    o[16] = 1.f + m.conic;
    o[17] = (1.f + m.conic) * m.curvature * m.curvature;
    o[18] = m.radius * m.radius;
    o[19] = (float)m.n_asph;
    o[20] = (float)m.aperture;
    o[21] = (float)m.n_vert;
    o[22] = (float)m.stage;
    o[23] = m.conic;
    for (int a = 0; a < 8; ++a) o[24 + a] = a < m.n_asph ? m.asph[a] : 0.f;
    for (int a = 0; a < 8; ++a) {
      o[32 + 2 * a] = a < m.n_vert ? m.vert[a][0] : 0.f;
      o[33 + 2 * a] = a < m.n_vert ? m.vert[a][1] : 0.f;
    }
    // the sag at the offset (core/surfaces.py:41-45 z0) and (1+k) c^2, FP64,
    // stored as float pairs hi + lo
    o[14] = 0.f;
    const double z0 = sag_raw_d(o, (double)m.offset[0] * m.offset[0] + (double)m.offset[1] * m.offset[1]);
    const double al = (1.0 + (double)m.conic) * (double)m.curvature * (double)m.curvature;
    o[48] = (float)z0;
    o[49] = (float)(z0 - (double)o[48]);
    o[50] = (float)al;
    o[51] = (float)(al - (double)o[50]);
  }
}

// telescope/mirrors.py:64-79 transform_to_world for one (facet, sample);
// returns the world point.
__device__ __forceinline__ V3 prep_sample(const PrepK& p, long long i) {
  const int f = (int)(i / p.M);
  float R[9];
  euler_to_matrix(p.facet_rot[3 * f], p.facet_rot[3 * f + 1], p.facet_rot[3 * f + 2], R);
  V3 pl = mk(p.points[3 * i], p.points[3 * i + 1], p.points[3 * i + 2]);
  V3 nl = mk(p.normals[3 * i], p.normals[3 * i + 1], p.normals[3 * i + 2]);
  V3 dl = mk(p.delta[3 * i], p.delta[3 * i + 1], p.delta[3 * i + 2]);
  V3 pw = rmul(R, pl) + mk(p.facet_pos[3 * f], p.facet_pos[3 * f + 1], p.facet_pos[3 * f + 2]);
  V3 nw = rmul(R, nl), dw = rmul(R, dl);
  float sc = p.facet_scale[f];
  V3 pe = nw + sc * dw;  // perturbed = normals_world + scale * delta_world
  float nn = sqrtf(dot(pe, pe));
  p.P4[i] = make_float4(pw.x, pw.y, pw.z, 1.f / p.weights[i]);
  p.N4[i] = make_float4(pe.x / nn, pe.y / nn, pe.z / nn, 0.f);
  if (p.D4) p.D4[i] = make_float4(dw.x / nn, dw.y / nn, dw.z / nn, 0.f);
  return pw;
}

// Bundle bound of facet f for the candidate masks, one warp: B4[f] =
// (facet position, largest |p| of its local sample points). Every world
// point R p + pos lies within |p| of pos (rotations keep lengths), so the
// sphere bounds the facet's samples exactly, and no rotation is needed
// (this runs beside the sample warps of the same launch). The local origin
// is the facet's centre, so the sphere is nearly as tight as one about the
// points' centroid; Monte-Carlo samples cover a facet at random, so one
// mask per (source, facet) serves all of its 32-sample chunks.
__device__ __forceinline__ void facet_bound(const PrepK& p, int f) {
  const int lane = threadIdx.x & 31;
  const float* pts = p.points + (size_t)f * p.M * 3;
  float r2 = 0.f;
#pragma unroll 4
  for (int m = lane; m < p.M; m += 32) {
    const float x = __ldg(pts + 3 * m), y = __ldg(pts + 3 * m + 1), z = __ldg(pts + 3 * m + 2);
    r2 = fmaxf(r2, x * x + y * y + z * z);
  }
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) r2 = fmaxf(r2, __shfl_xor_sync(kFull, r2, k));
  if (lane == 0)
    p.B4[f] = make_float4(p.facet_pos[3 * f], p.facet_pos[3 * f + 1], p.facet_pos[3 * f + 2],
                          sqrtf(r2) * 1.0001f + 1e-6f);
}

// World samples of (facet, 32-sample chunk) units, one warp per unit, then
// (with culling) one warp per facet bound: warp `w0` of `nw` warps strides
// over both.
__device__ __forceinline__ void prep_units(const PrepK& p, long long w0, long long nw) {
  const int lane = threadIdx.x & 31;
  const int nch = (p.M + 31) >> 5;
  const long long units = (long long)p.F * nch;
  const long long total = units + (p.B4 ? p.F : 0);
  for (long long u = w0; u < total; u += nw) {
    if (u >= units) {
      facet_bound(p, (int)(u - units));
      continue;
    }
    const int f = (int)(u / nch), m = (int)(u - (long long)f * nch) * 32 + lane;
    if (m < p.M) prep_sample(p, (long long)f * p.M + m);
  }
}

struct RenderK {
  int F, M, S, P;
  const float4* P4;
  const float4* N4;
  const float* sources;
  const float* values;
  const float* tables;
  int n_table_floats;
  int n_cyl, n_box, n_sph, n_obox, n_tri, n_mir;
  const int* hex_table;
  int hex_in_smem;
  SensorK sn;
  double* acc;       // FP64 accumulator [rows_total * P] in the workspace
  int rows_in_smem;  // FP32 histogram rows held in shared memory per tile, 0 = add to `acc` directly
  int SB, FC, CC;    // tile: sources, facets, 32-sample chunks
  int n_fchunk, n_cchunk, n_tiles;
  int* counter;
  uint32_t seed;  // jitter stream of extended sources
  const float4* B4;  // per facet bundle bounds (culling on)
  int n_words;       // 32-bit candidate-mask words per task; 0 = no culling
  const uint32_t* gmask;  // k_render_hard: candidate word per (source, facet) pair [S * F], or null (no primitives)
  int flush_tiles;        // k_render_hard, IMAGE mode: tiles between flushes of the FP32 row
};

// candidate words of all (source, facet) pairs of p into out[S * F]
// (k_masks, iact_render.cu): the scene has 1..32 primitives, B4 and the
// tables are written
int launch_masks(int src_type, const RenderK& p, uint32_t* out, cudaStream_t st);

// Where hits go: FP32 shared-memory rows of the current tile, or the FP64
// global accumulator. The choice is uniform over the CTA.
struct Sink {
  float* sh;
  double* g;
  __device__ __forceinline__ void add(int key, float v) const {
    if (sh) atomicAdd(sh + key, v);
    else atomicAdd(g + key, (double)v);
  }
};

// Hits into FP32 shared-memory rows only (the soft-pixel kernel's sink).
struct RowSink {
  float* sh;
  __device__ __forceinline__ void add(int key, float v) const { atomicAdd(sh + key, v); }
};

// all 32 lanes call; key < 0 or v == 0 means nothing to add for this lane
template <typename SK>
__device__ __forceinline__ void warp_add(const SK& sink, int key, float v) {
  const int k0 = __shfl_sync(kFull, key, 0);
  if (__all_sync(kFull, key == k0)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && k0 >= 0 && v != 0.f) sink.add(k0, v);
  } else if (key >= 0 && v != 0.f) {
    sink.add(key, v);
  }
}

// Rows whose adds come from lanes on different sources' spots (the
// source-per-lane tile body): a lane's address rarely equals another
// lane's, so each lane adds on its own, without warp_add's vote.
struct SpreadSink {
  float* sh;
};
__device__ __forceinline__ void warp_add(const SpreadSink& sink, int key, float v) {
  if (key >= 0 && v != 0.f) atomicAdd(sink.sh + key, v);
}

// sensors/square.py:144-172 DifferentiableSquareSensor.accumulate, one ray
// (all lanes call; inactive lanes pass ok = false). Rays whose plane hit is
// the 1e10 sentinel deposit nothing.
template <typename SK>
__device__ __forceinline__ void splat_square(const SensorK& s, const SK& sink, int rowbase, bool ok,
                                             float x, float y, float v) {
  ok = ok && (x < 1e9f) && (y < 1e9f);
  float xp = (x - s.x0) * s.inv_dx, yp = (y - s.y0) * s.inv_dy;
  float xb = floorf(xp), yb = floorf(yp);
  float xf = xp - xb, yf = yp - yb;
  const int K = s.kernel_size, n = 2 * K + 1;
  const float inv2s = __fdiv_rn(-0.5f, s.sigma * s.sigma);
  float tot = 0.f;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      float ddx = xf - (float)(j - K), ddy = yf - (float)(i - K);
      tot += __expf(inv2s * (ddx * ddx + ddy * ddy));
    }
  const float scale = ok ? v / tot : 0.f;
  const int xi0 = ok ? (int)xb : 0, yi0 = ok ? (int)yb : 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      float ddx = xf - (float)(j - K), ddy = yf - (float)(i - K);
      float w = __expf(inv2s * (ddx * ddx + ddy * ddy)) * scale;
      int xi = xi0 + j - K, yi = yi0 + i - K;
      bool in = ok && xi >= 0 && xi < s.width && yi >= 0 && yi < s.height;
      warp_add(sink, in ? rowbase + yi * s.width + xi : -1, w);
    }
}

// sensors/hexagonal.py:264-315 DifferentiableHexagonalSensor.accumulate
// (all lanes call; inactive lanes pass ok = false). The tap weights of the
// one-ring kernel (kernel_size 1, the reference default) stay in registers
// between the normalisation and the deposit; larger kernels recompute them.
template <typename TT, typename SK>
__device__ __forceinline__ void splat_hex(const SensorK& s, const TT* table, const SK& sink,
                                          int rowbase, bool ok, float x, float y, float v) {
  ok = ok && (x < 1e9f) && (y < 1e9f);
  float xg, yg, qi, ri;
  hex_axial(s, ok ? x : 0.f, ok ? y : 0.f, xg, yg, qi, ri);
  float ddx = xg - s.hex_sx * (qi + 0.5f * ri), ddy = yg - s.hex_sy * ri;
  const int K = s.kernel_size;
  const float inv_sig = 1.f / s.sigma;
  if (K == 1) {
    constexpr int dq[7] = {-1, -1, 0, 0, 0, 1, 1}, dr[7] = {0, 1, -1, 0, 1, -1, 0};  // the ring in (q, r) order
    float w[7], tot = 0.f;
#pragma unroll
    for (int j = 0; j < 7; ++j) {
      const float a = hex_norm(ddx - s.hex_sx * ((float)dq[j] + 0.5f * (float)dr[j]),
                               ddy - s.hex_sy * (float)dr[j], s.inv_inr) * inv_sig;
      w[j] = __expf(-0.5f * (a * a));
      tot += w[j];
    }
    const float scale = ok ? v / tot : 0.f;
    // lookup-table index of the base hexagon; the ring is at fixed offsets
    const float qx = qi - (float)s.q_min, rx = ri - (float)s.r_min;
    const bool inner = ok && (qx >= 1.f) & (qx < (float)(s.table_q - 1)) & (rx >= 1.f) & (rx < (float)(s.table_r - 1));
    const int base = inner ? (int)qx * s.table_r + (int)rx : 0;
#pragma unroll
    for (int j = 0; j < 7; ++j) {
      int p;
      if (inner) {
        p = (int)table[base + dq[j] * s.table_r + dr[j]];
        p = p >= 0 ? p : -1;
      } else {
        p = ok ? hex_lookup(s, table, qi + (float)dq[j], ri + (float)dr[j]) : -1;
      }
      warp_add(sink, p >= 0 ? rowbase + p : -1, w[j] * scale);
    }
    return;
  }
  float tot = 0.f;
  for (int q = -K; q <= K; ++q)
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float a = hex_norm(ddx - s.hex_sx * ((float)q + 0.5f * (float)r), ddy - s.hex_sy * (float)r, s.inv_inr) *
                inv_sig;
      tot += __expf(-0.5f * (a * a));
    }
  const float scale = ok ? v / tot : 0.f;
  for (int q = -K; q <= K; ++q)
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float a = hex_norm(ddx - s.hex_sx * ((float)q + 0.5f * (float)r), ddy - s.hex_sy * (float)r, s.inv_inr) *
                inv_sig;
      float w = __expf(-0.5f * (a * a)) * scale;
      int p = ok ? hex_lookup(s, table, qi + (float)q, ri + (float)r) : -1;
      warp_add(sink, p >= 0 ? rowbase + p : -1, w);
    }
}

// core/render.py:118-157 for one ray; returns sensor-plane (x, y), value and
// the index of the last stage mirror hit (-1 if none).
// The primary shadow test covers the set bits of the warp bundle's
// candidate mask (n_words == 0: every primitive).
template <int SRC, bool STAGES, bool AX = false>
__device__ __forceinline__ void trace_ray(const RenderK& p, const Obst& ob, const float* mir, float4 P,
                                          float4 N, V3 src, const JBasis& jb, float sigma, float z0, float z1,
                                          float v, float& x,
                                          float& y, float& val, int& hit_mirror, const uint32_t* cmask,
                                          int n_words) {
  V3 tp = mk(P.x, P.y, P.z), tn = mk(N.x, N.y, N.z);
  V3 d;
  if (SRC == IACT_SRC_POINT) {
    V3 dd = tp - src;  // dirs = normalize(tp - src)
    d = rsqrtf(dot(dd, dd)) * dd;
  } else if (SRC == IACT_SRC_EXTENDED) {
    d = jitter_dir(jb, sigma, z0, z1);
  } else {
    d = src;  // parallel: the source entry is the direction, as given
  }
  const bool sh = occluded_mask(ob, cmask, n_words, tp, mk(-d.x, -d.y, -d.z));
  const float c = dot(d, tn);  // core/reflection.py:5-20
  V3 r = d - (2.f * c) * tn;
  val = (v * -c * P.w) * (sh ? 0.f : 1.f);  // values * cos / tw * shadow
  V3 o = tp;
  hit_mirror = -1;
  if (STAGES) {
    // core/render.py:44-79 _reflect_at_stage, one pass per stage
    int mi = 0;
    while (mi < p.n_mir) {
      const int stg = (int)mir[mi * kMirF + 22];
      float best_t = __int_as_float(0x7f800000);
      V3 bp = mk(0.f, 0.f, 0.f), bn = mk(0.f, 0.f, 0.f);
      int bi = -1;
      int mj = mi;
      for (; mj < p.n_mir && (int)mir[mj * kMirF + 22] == stg; ++mj) {
        const float* m = mir + mj * kMirF;
        V3 pos = mk(m[9], m[10], m[11]);
        V3 pl, nl;
        float t = mirror_hit(m, rtmul(m, o - pos), rtmul(m, r), pl, nl);
        if (t < best_t) {  // closest hit, first index on ties (argmin)
          best_t = t;
          bp = rmul(m, pl) + pos;
          bn = rmul(m, nl);
          bi = mj;
        }
      }
      const float c2 = dot(r, bn);
      V3 rr = r - (2.f * c2) * bn;
      const bool sh2 = occluded(ob, o, r);
      val = val * (best_t < kBig ? 1.f : 0.f) * (sh2 ? 0.f : 1.f) * fabsf(c2);
      o = bp;
      r = rr;
      hit_mirror = bi;
      mi = mj;
    }
  }
  plane_hit<AX>(p.sn, o, r, x, y);
}

// One work tile (source block, facet chunk, 32-sample chunk) of the forward
// render: every warp traces its share of the tile's warp tasks, then the
// tile's shared-memory rows go to the FP64 accumulator. All threads of the
// CTA call this; it ends after a __syncthreads.
// Axis and angular spread of a warp task's shadow rays (towards the
// source): point sources from the bundle centre c, parallel and extended
// sources along minus the given direction (jitter bounded by the largest
// Box-Muller radius, 5.8 sigma, of 24-bit uniforms).
template <int SRC>
__device__ __forceinline__ void bundle_axis(V3 src, float sigma, V3 c, float R0, V3& u, float& dlt) {
  // approximate square roots and reciprocals (relative error ~1e-7) stay far
  // inside the 2 mm + 1e-4 margin of the reach
  if (SRC == IACT_SRC_POINT) {
    V3 w = src - c;
    const float il = rsqrtf(dot(w, w)), L = dot(w, w) * il;
    u = il * w;
    dlt = L > 4.f * R0 ? 2.f * R0 * rcp_a(L - R0) * 1.00001f + 1e-6f : 2.f;
  } else {
    u = -rsqrtf(dot(src, src)) * src;
    dlt = (SRC == IACT_SRC_EXTENDED ? 6.f * fabsf(sigma) : 0.f) + 1e-6f;
  }
}

// Warp-collective: candidate masks of the warp's tasks [tb, te) (source sl,
// facet fl, chunk cl of a tile starting at (s0, f0, c0); chunk fastest) into
// mask[t * nw + w]. One lane per (task, 32-primitive word): the task's
// bundle is decoded once and its word assembled in a register; no
// CTA-wide barrier (each warp reads only its own tasks' masks).
// Candidate word w (primitives 32w..32w+31) of the pair (source s, facet f).
template <int SRC>
__device__ __forceinline__ uint32_t mask_word(const float4* B4, const float* sources, const Obst& ob, int s, int f,
                                              int w) {
  const int np = ob.n_cyl + ob.n_box + ob.n_sph + ob.n_obox + ob.n_tri;
  constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
  const float4 B = __ldg(B4 + f);
  Bundle bd;
  bd.c = mk(B.x, B.y, B.z);
  bd.R0 = B.w;
  const V3 src = mk(__ldg(sources + SS * s), __ldg(sources + SS * s + 1), __ldg(sources + SS * s + 2));
  bundle_axis<SRC>(src, SRC == IACT_SRC_EXTENDED ? __ldg(sources + SS * s + 3) : 0.f, bd.c, bd.R0, bd.u, bd.dlt);
  uint32_t word = 0u;
  const int k1 = min(np, 32 * w + 32);
  for (int k = 32 * w; k < k1; ++k)
    if (prim_may_hit(ob, k, bd)) word |= 1u << (k & 31);
  return word;
}

template <int SRC>
// Candidate masks of the (source, facet) pairs of this warp's tasks
// [tb, te) (tasks are ordered (source, facet, chunk): a pair's CCc chunk
// tasks share its mask): lane = (pair, 32-primitive word); mask index =
// pair * nw + word, pair = source_local * FCc + facet_local. Pairs at the
// ends of the range may also be computed by the neighbouring warp, which
// writes the same words.
__device__ __forceinline__ void warp_masks(const float4* B4, const float* sources, int nw, const Obst& ob,
                                           int s0, int f0, int FCc, int CCc, int tb, int te, uint32_t* mask) {
  const int pb = tb / CCc, pe = (te + CCc - 1) / CCc;
  for (int i = pb * nw + (threadIdx.x & 31); i < pe * nw; i += 32) {
    const int q = i / nw, w = i - q * nw;
    const int sl = q / FCc, fl = q - sl * FCc;
    mask[i] = mask_word<SRC>(B4, sources, ob, s0 + sl, f0 + fl, w);
  }
  __syncwarp();
}

template <int SRC, bool SOFT, int MODE, bool STAGES, bool AX = false>
__device__ __forceinline__ void render_tile(const RenderK& p, const Obst& ob, const float* mir, const short* htab,
                                            float* sh_hist, const Sink& sink, int tile, uint32_t* tmask) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5, nthr = blockDim.x;
  const int nch = (p.M + 31) >> 5;
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);

  int rl_key = -1;  // run-length merged hit of this lane (hard sensors)
  float rl_val = 0.f;
  HexCache hc = {3.0e38f, 3.0e38f, -1};  // last hexagon of this lane (hard hex sensors)
  JBasis jb;                             // tangent basis of the current source (extended sources)
  int jb_s = -1;
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  if (p.n_words) warp_masks<SRC>(p.B4, p.sources, p.n_words, ob, s0, f0, FCc, CCc, tb, te, tmask);
  // task t = (source sl, facet fl, chunk cl), chunk fastest; decoded once
  int sl = tb / (FCc * CCc);
  int fl = (tb - sl * FCc * CCc) / CCc;
  int cl = tb - sl * FCc * CCc - fl * CCc;
  for (int t = tb; t < te; ++t) {
    const int m = (c0 + cl) * 32 + lane;
    const int s = s0 + sl, f = f0 + fl;
    const bool act = m < p.M;
    constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
    const V3 src = mk(__ldg(p.sources + SS * s), __ldg(p.sources + SS * s + 1), __ldg(p.sources + SS * s + 2));
    const float sig = (SRC == IACT_SRC_EXTENDED) ? __ldg(p.sources + SS * s + 3) : 0.f;
    const float v = __ldg(p.values + s);
    if (SRC == IACT_SRC_EXTENDED && s != jb_s) {  // warp-uniform
      jb = jitter_basis(src);
      jb_s = s;
    }
    float x = 0.f, y = 0.f, val = 0.f;
    int hm;
    if (act) {
      const size_t si = (size_t)f * p.M + m;
      float z0 = 0.f, z1 = 0.f;
      if (SRC == IACT_SRC_EXTENDED) ray_normals(p.seed, s, f, m, z0, z1);
      trace_ray<SRC, STAGES, AX>(p, ob, mir, __ldg(p.P4 + si), __ldg(p.N4 + si), src, jb, sig, z0, z1, v, x, y, val,
                             hm, tmask + (sl * FCc + fl) * p.n_words, p.n_words);
    }
    int rowbase;
    if (MODE == IACT_MODE_RESPONSE) rowbase = (p.rows_in_smem ? sl : s) * p.P;
    else rowbase = 0;
    if (SOFT) {
      if (p.sn.type == IACT_SENSOR_SOFT_SQUARE) splat_square(p.sn, sink, rowbase, act, x, y, val);
      else if (p.hex_in_smem) splat_hex(p.sn, htab, sink, rowbase, act, x, y, val);
      else splat_hex(p.sn, p.hex_table, sink, rowbase, act, x, y, val);
    } else if (act) {
      const int pix = (p.sn.type == IACT_SENSOR_SQUARE)
                          ? bin_square(p.sn, x, y)
                          : (p.hex_in_smem ? bin_hex_cached(p.sn, htab, x, y, hc)
                                           : bin_hex_cached(p.sn, p.hex_table, x, y, hc));
      if ((pix >= 0) & (val != 0.f)) {
        const int key = rowbase + pix;
        if (key == rl_key) {
          rl_val += val;
        } else {
          if (rl_key >= 0) sink.add(rl_key, rl_val);
          rl_key = key;
          rl_val = val;
        }
      }
    }
    if (++cl == CCc) {
      cl = 0;
      if (++fl == FCc) {
        fl = 0;
        ++sl;
      }
    }
  }
  if (!SOFT && rl_key >= 0) sink.add(rl_key, rl_val);
  __syncthreads();
  if (p.rows_in_smem) {
    // this tile's FP32 rows -> FP64 accumulator, then clear for the next tile
    const int base = (MODE == IACT_MODE_RESPONSE) ? s0 : 0;
    const int nrows = (MODE == IACT_MODE_RESPONSE) ? SBc : 1;
    for (int i = threadIdx.x; i < nrows * p.P; i += nthr) {
      const float h = sh_hist[i];
      if (h != 0.f) {
        atomicAdd(p.acc + (size_t)base * p.P + i, (double)h);
        sh_hist[i] = 0.f;
      }
    }
  }

}

// FP32 shared-memory rows [nrows, P] -> FP64 accumulator rows from `base`,
// then cleared (all threads of the CTA, after a barrier).
__device__ __forceinline__ void flush_rows(const RenderK& p, float* sh_hist, int base, int nrows) {
  for (int i = threadIdx.x; i < nrows * p.P; i += blockDim.x) {
    const float h = sh_hist[i];
    if (h != 0.f) {
      atomicAdd(p.acc + (size_t)base * p.P + i, (double)h);
      sh_hist[i] = 0.f;
    }
  }
}

// Candidate words of the (source, facet) pairs i of a render [S * F], one
// thread per pair (the scene has at most 32 primitives): the bundle test of
// warp_masks, once per pair for the whole launch.
template <int SRC>
__device__ __forceinline__ void pair_masks(const RenderK& p, const Obst& ob, long long i0, long long stride,
                                           uint32_t* out) {
  const long long n = (long long)p.S * p.F;
  for (long long i = i0; i < n; i += stride) {
    const int s = (int)(i / p.F), f = (int)(i - (long long)s * p.F);
    out[i] = mask_word<SRC>(p.B4, p.sources, ob, s, f, 0);
  }
}

// core/render.py:21-41 for one ray against the set bits of one 32-bit
// candidate word (primitives 0..31 of the unified index space).
__device__ __forceinline__ bool shadow_word(const Obst& ob, uint32_t m, V3 o, V3 d) {
  bool sh = false;
#pragma unroll 1
  while (m) {
    int k = __ffs(m) - 1;
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
  return sh;
}

// Soft-pixel tile body of the common case (sensors/square.py:144-172,
// sensors/hexagonal.py:264-315 deposits): a single-stage scene, point,
// parallel or extended sources, a sensor whose rotation is the identity,
// the rows and (hexagons) the lookup table in shared memory, candidate
// words per (source, facet) pair from k_masks (or no primitives). The per-ray
// arithmetic is render_tile<SRC, true, MODE, false, AX>'s (the same trace,
// splat and warp-aggregated adds); the sensor kind and the row sink are
// compile-time, per-pair values (source, its jitter basis, value, candidate
// word) are loaded once per pair, and lanes past a facet's last sample
// trace its last sample with value 0. Response rows are flushed per tile,
// an image row as render_tile_hard's.
template <int SRC, int MODE, bool HEX>
__device__ __forceinline__ void render_tile_soft(const RenderK& p, const Obst& ob, const short* htab,
                                                 float* sh_hist, int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nch = (p.M + 31) >> 5;
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);
  const RowSink sink{sh_hist};
  constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  int q = tb / CCc;  // pair index sl * FCc + fl
  int sl = q / FCc, fl = q - sl * FCc;
  int cl = tb - q * CCc;
  const int mlast = p.M - 1;
  for (int t = tb; t < te;) {
    const int s = s0 + sl, f = f0 + fl;
    const int ce = min(CCc, cl + (te - t));
    t += ce - cl;
    const V3 src = mk(__ldg(p.sources + SS * s), __ldg(p.sources + SS * s + 1), __ldg(p.sources + SS * s + 2));
    const float sig = (SRC == IACT_SRC_EXTENDED) ? __ldg(p.sources + SS * s + 3) : 0.f;
    const float v = __ldg(p.values + s);
    const uint32_t word = p.gmask ? __ldg(p.gmask + (size_t)s * p.F + f) : 0u;  // pair's candidates (k_masks)
    const int rowbase = (MODE == IACT_MODE_RESPONSE) ? sl * p.P : 0;
    const int fbase = f * p.M;
    JBasis jb;
    if (SRC == IACT_SRC_EXTENDED) jb = jitter_basis(src);
    for (; cl < ce; ++cl) {
      const int m = (c0 + cl) * 32 + lane;
      const bool act = m < p.M;
      const float4 P = __ldg(p.P4 + fbase + (act ? m : mlast)), N = __ldg(p.N4 + fbase + (act ? m : mlast));
      const V3 tp = mk(P.x, P.y, P.z), tn = mk(N.x, N.y, N.z);
      V3 d;
      if (SRC == IACT_SRC_POINT) {
        V3 dd = tp - src;  // dirs = normalize(tp - src)
        d = rsqrtf(dot(dd, dd)) * dd;
      } else if (SRC == IACT_SRC_EXTENDED) {
        float z0, z1;
        ray_normals(p.seed, s, f, act ? m : mlast, z0, z1);
        d = jitter_dir(jb, sig, z0, z1);
      } else {
        d = src;
      }
      bool sh = false;
      if (word) sh = shadow_word(ob, word, tp, mk(-d.x, -d.y, -d.z));  // warp-uniform
      const float c = dot(d, tn);                                       // core/reflection.py:5-20
      const V3 r = d - (2.f * c) * tn;
      const float val = (v * -c * P.w) * (sh ? 0.f : 1.f);  // values * cos / tw * shadow
      float x, y;
      plane_hit<true>(p.sn, tp, r, x, y);
      if (HEX) splat_hex(p.sn, htab, sink, rowbase, act, x, y, val);
      else splat_square(p.sn, sink, rowbase, act, x, y, val);
    }
    cl = 0;
    ++q;
    if (++fl == FCc) {
      fl = 0;
      ++sl;
    }
  }
  if (MODE == IACT_MODE_RESPONSE) {
    __syncthreads();
    flush_rows(p, sh_hist, s0, SBc);
  }
}

// Soft-pixel image tile body with one source per lane (image renders of at
// least 32 sources, p.SB == 32). A warp task is one (facet, sample) traced
// towards the tile's 32 sources, so the 32 lanes' hits fall on 32 sources'
// spots instead of on one source's spot. A shared-memory float add is a
// compare-and-swap loop that runs once more for every lane sharing its
// address, and the taps of one source's rays pile onto a few pixels; the
// taps of different sources seldom meet. The sample point and normal are
// warp-uniform loads; a lane's source, value and jitter basis stay in
// registers for the whole tile; the candidate word of a facet is the OR of
// the lanes' pair words (a superset, so the shadow tests stay exact). Each
// ray runs the same floating-point operations as in render_tile_soft (the
// same Philox stream per (source, facet, sample)); only the order of the
// sums differs.
template <int SRC, bool HEX>
__device__ __forceinline__ void render_tile_soft_spread(const RenderK& p, const Obst& ob, const short* htab,
                                                        float* sh_hist, int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int f0 = fc * p.FC, m0 = cc * p.CC * 32;
  const int FCc = min(p.FC, p.F - f0);
  const int msz = min(p.CC * 32, p.M - m0);  // samples of each facet in this tile
  const int s_lane = sblk * 32 + lane;
  const bool sact = s_lane < p.S;
  const int s = sact ? s_lane : p.S - 1;
  constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
  const V3 src = mk(__ldg(p.sources + SS * s), __ldg(p.sources + SS * s + 1), __ldg(p.sources + SS * s + 2));
  const float sig = (SRC == IACT_SRC_EXTENDED) ? __ldg(p.sources + SS * s + 3) : 0.f;
  const float v = __ldg(p.values + s);
  JBasis jb;
  if (SRC == IACT_SRC_EXTENDED) jb = jitter_basis(src);
  const SpreadSink sink{sh_hist};
  const int T = FCc * msz;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  int fl = tb / msz, ml = tb - fl * msz;
  int wf = -1;
  uint32_t word = 0u;
  for (int t = tb; t < te; ++t) {
    const int f = f0 + fl, m = m0 + ml;
    if (p.gmask && f != wf) {  // the facet's candidates for any of the lanes' sources (k_masks)
      word = __reduce_or_sync(kFull, sact ? __ldg(p.gmask + (size_t)s * p.F + f) : 0u);
      wf = f;
    }
    const int mi = f * p.M + m;  // F * M < 2^30
    const float4 P = __ldg(p.P4 + mi), N = __ldg(p.N4 + mi);
    const V3 tp = mk(P.x, P.y, P.z), tn = mk(N.x, N.y, N.z);
    V3 d;
    if (SRC == IACT_SRC_POINT) {
      V3 dd = tp - src;  // dirs = normalize(tp - src)
      d = rsqrtf(dot(dd, dd)) * dd;
    } else if (SRC == IACT_SRC_EXTENDED) {
      float z0, z1;
      ray_normals(p.seed, s, f, m, z0, z1);
      d = jitter_dir(jb, sig, z0, z1);
    } else {
      d = src;
    }
    bool sh = false;
    if (word) sh = shadow_word(ob, word, tp, mk(-d.x, -d.y, -d.z));  // warp-uniform word
    const float c = dot(d, tn);                                       // core/reflection.py:5-20
    const V3 r = d - (2.f * c) * tn;
    const float val = (v * -c * P.w) * (sh ? 0.f : 1.f);  // values * cos / tw * shadow
    float x, y;
    plane_hit<true>(p.sn, tp, r, x, y);
    if (HEX) splat_hex(p.sn, htab, sink, 0, sact, x, y, val);
    else splat_square(p.sn, sink, 0, sact, x, y, val);
    if (++ml == msz) {
      ml = 0;
      ++fl;
    }
  }
}

// Hard-pixel tile body of the common case: a single-stage scene, point or
// parallel sources, a sensor whose rotation is the identity, histogram rows
// (and, for hexagons, the lookup table) in shared memory, and at most 32
// shadowing primitives (one candidate word per (source, facet) pair; no
// primitives at all also qualifies). It evaluates what render_tile<SRC,
// false, MODE, false, true> does with the same floating-point operations in
// the same order (core/render.py:118-157, sensors/square.py:66-91,
// sensors/hexagonal.py:174-194), so every ray bins to the same pixel with
// the same value. What differs is the control flow around them:
//   * the sensor kind and the placement of the table and the rows are
//     compile-time, not tested per ray;
//   * source, value, candidate word and sample pointers are loaded once per
//     (source, facet) pair, not per 32-ray task;
//   * lanes past the last sample trace the facet's last sample with value 0
//     instead of branching around the ray;
//   * the run-length merge of the hits keeps two keys per lane and is
//     selects plus one predicated shared-memory add, and the hexagon cell cache takes the full binning
//     when any lane of the warp misses it (a warp vote), without a divergent
//     branch.
template <int SRC, int MODE, bool HEX>
__device__ __forceinline__ void render_tile_hard(const RenderK& p, const Obst& ob, const short* htab,
                                                 float* sh_hist, int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nch = (p.M + 31) >> 5;
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);

  // run-length merged hits of this lane: two (key, value) slots, slot 0 the
  // newest key; a third key flushes slot 1 (a lane whose rays alternate
  // between two pixels adds nothing until a third appears)
  int rl_key = -1, rk1 = -1;
  float rl_val = 0.f, rv1 = 0.f;
  HexCache hc = {3.0e38f, 3.0e38f, -1};  // last hexagon of this lane
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  // tasks t = (pair q = (source sl, facet fl), chunk cl), chunk fastest
  int q = tb / CCc;
  int sl = q / FCc, fl = q - sl * FCc;
  int cl = tb - q * CCc;
  const int mlast = p.M - 1;
  for (int t = tb; t < te;) {
    const int s = s0 + sl, f = f0 + fl;
    const int ce = min(CCc, cl + (te - t));
    t += ce - cl;
    const V3 src = mk(__ldg(p.sources + 3 * s), __ldg(p.sources + 3 * s + 1), __ldg(p.sources + 3 * s + 2));
    const float v = __ldg(p.values + s);
    const uint32_t word = p.gmask ? __ldg(p.gmask + (size_t)s * p.F + f) : 0u;  // pair's candidates (k_masks)
    const int fbase = f * p.M;  // first sample of the facet (F * M < 2^30)
    const int rowbase = (MODE == IACT_MODE_RESPONSE) ? sl * p.P : 0;
    for (; cl < ce; ++cl) {
      const int m = (c0 + cl) * 32 + lane;
      const bool act = m < p.M;
      const int mi = fbase + (act ? m : mlast);
      const float4 P = __ldg(p.P4 + mi), N = __ldg(p.N4 + mi);
      const V3 tp = mk(P.x, P.y, P.z), tn = mk(N.x, N.y, N.z);
      V3 d;
      if (SRC == IACT_SRC_POINT) {
        V3 dd = tp - src;  // dirs = normalize(tp - src)
        d = rsqrtf(dot(dd, dd)) * dd;
      } else {
        d = src;
      }
      bool sh = false;
      if (word) sh = shadow_word(ob, word, tp, mk(-d.x, -d.y, -d.z));  // warp-uniform
      const float c = dot(d, tn);                                       // core/reflection.py:5-20
      const V3 r = d - (2.f * c) * tn;
      float val = (v * -c * P.w) * (sh ? 0.f : 1.f);  // values * cos / tw * shadow
      val = act ? val : 0.f;
      float x, y;
      plane_hit<true>(p.sn, tp, r, x, y);
      int pix;
      if (HEX) {
        const float ex = x - hc.cx, ey = y - hc.cy;
        const bool in = ex * ex + ey * ey < p.sn.hex_lim2;
        pix = hc.pid;
        if (__any_sync(kFull, !in)) {
          float xg, yg, qi, ri;
          hex_axial(p.sn, x, y, xg, yg, qi, ri);
          const int pf = hex_lookup(p.sn, htab, qi, ri);
          float hcx, hcy;
          hex_centre(p.sn, qi, ri, hcx, hcy);
          const float hd = hex_norm(__fsub_rn(xg, hcx), __fsub_rn(yg, hcy), p.sn.inv_inr);
          // grid -> sensor frame: x - off_x = gc xg + gs yg, y - off_y = -gs xg + gc yg
          const float ncx = p.sn.off_x + (p.sn.gc * hcx + p.sn.gs * hcy);
          const float ncy = p.sn.off_y + (p.sn.gc * hcy - p.sn.gs * hcx);
          hc.cx = in ? hc.cx : ncx;
          hc.cy = in ? hc.cy : ncy;
          hc.pid = in ? hc.pid : pf;
          pix = in ? pix : ((hd > p.sn.edge_threshold) ? -1 : pf);
        }
      } else {
        pix = bin_square(p.sn, x, y);
      }
      const bool dep = (pix >= 0) & (val != 0.f);
      const int key = rowbase + pix;
      const bool in0 = key == rl_key, in1 = key == rk1;
      const bool nk = dep & !in0 & !in1;
      if (nk & (rk1 >= 0)) atomicAdd(sh_hist + rk1, rv1);
      rl_val = (dep & in0) ? rl_val + val : rl_val;
      rv1 = (dep & in1) ? rv1 + val : rv1;
      rk1 = nk ? rl_key : rk1;
      rv1 = nk ? rl_val : rv1;
      rl_key = nk ? key : rl_key;
      rl_val = nk ? val : rl_val;
    }
    cl = 0;
    ++q;
    if (++fl == FCc) {
      fl = 0;
      ++sl;
    }
  }
  if (rl_key >= 0) atomicAdd(sh_hist + rl_key, rl_val);
  if (rk1 >= 0) atomicAdd(sh_hist + rk1, rv1);
  if (MODE == IACT_MODE_RESPONSE) {
    // this tile's FP32 rows -> FP64 accumulator, then clear for the next tile
    __syncthreads();
    flush_rows(p, sh_hist, s0, SBc);
  }
}

}  // namespace iact
