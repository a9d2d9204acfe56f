// Device code shared by the single-scene render (iact_render.cu) and the
// batched persistent render (iact_batched.cu): per-launch parameters, the
// per-ray chain and the per-tile work.
#pragma once

#include "iact_device.cuh"

namespace iact {

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
};

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

// all 32 lanes call; key < 0 or v == 0 means nothing to add for this lane
__device__ __forceinline__ void warp_add(const Sink& sink, int key, float v) {
  const int k0 = __shfl_sync(kFull, key, 0);
  if (__all_sync(kFull, key == k0)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && k0 >= 0 && v != 0.f) sink.add(k0, v);
  } else if (key >= 0 && v != 0.f) {
    sink.add(key, v);
  }
}

// sensors/square.py:144-172 DifferentiableSquareSensor.accumulate, one ray
// (all lanes call; inactive lanes pass ok = false). Rays whose plane hit is
// the 1e10 sentinel deposit nothing.
__device__ __forceinline__ void splat_square(const SensorK& s, const Sink& sink, int rowbase, bool ok,
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
      tot += expf(inv2s * (ddx * ddx + ddy * ddy));
    }
  const float scale = ok ? v / tot : 0.f;
  const int xi0 = ok ? (int)xb : 0, yi0 = ok ? (int)yb : 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      float ddx = xf - (float)(j - K), ddy = yf - (float)(i - K);
      float w = expf(inv2s * (ddx * ddx + ddy * ddy)) * scale;
      int xi = xi0 + j - K, yi = yi0 + i - K;
      bool in = ok && xi >= 0 && xi < s.width && yi >= 0 && yi < s.height;
      warp_add(sink, in ? rowbase + yi * s.width + xi : -1, w);
    }
}

// sensors/hexagonal.py:264-315 DifferentiableHexagonalSensor.accumulate
template <typename TT>
__device__ __forceinline__ void splat_hex(const SensorK& s, const TT* table, const Sink& sink,
                                          int rowbase, bool ok, float x, float y, float v) {
  ok = ok && (x < 1e9f) && (y < 1e9f);
  float xg, yg, qi, ri;
  hex_axial(s, ok ? x : 0.f, ok ? y : 0.f, xg, yg, qi, ri);
  float ddx = xg - s.hex_sx * (qi + 0.5f * ri), ddy = yg - s.hex_sy * ri;
  const int K = s.kernel_size;
  const float inv_sig = 1.f / s.sigma;
  float tot = 0.f;
  for (int q = -K; q <= K; ++q)
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float a = hex_norm(ddx - s.hex_sx * ((float)q + 0.5f * (float)r), ddy - s.hex_sy * (float)r, s.inv_inr) *
                inv_sig;
      tot += expf(-0.5f * (a * a));
    }
  const float scale = ok ? v / tot : 0.f;
  for (int q = -K; q <= K; ++q)
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float a = hex_norm(ddx - s.hex_sx * ((float)q + 0.5f * (float)r), ddy - s.hex_sy * (float)r, s.inv_inr) *
                inv_sig;
      float w = expf(-0.5f * (a * a)) * scale;
      int p = ok ? hex_lookup(s, table, qi + (float)q, ri + (float)r) : -1;
      warp_add(sink, p >= 0 ? rowbase + p : -1, w);
    }
}

// core/render.py:118-157 for one ray; returns sensor-plane (x, y), value and
// the index of the last stage mirror hit (-1 if none).
template <int SRC, bool STAGES>
__device__ __forceinline__ void trace_ray(const RenderK& p, const Obst& ob, const float* mir, float4 P,
                                          float4 N, V3 src, float sigma, float z0, float z1, float v, float& x,
                                          float& y, float& val, int& hit_mirror) {
  V3 tp = mk(P.x, P.y, P.z), tn = mk(N.x, N.y, N.z);
  V3 d;
  if (SRC == IACT_SRC_POINT) {
    V3 dd = tp - src;  // dirs = normalize(tp - src)
    d = rsqrtf(dot(dd, dd)) * dd;
  } else if (SRC == IACT_SRC_EXTENDED) {
    d = jitter_dir(rsqrtf(dot(src, src)) * src, sigma, z0, z1);
  } else {
    d = src;  // parallel: the source entry is the direction, as given
  }
  const bool sh = occluded(ob, tp, mk(-d.x, -d.y, -d.z));
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
  plane_hit(p.sn, o, r, x, y);
}

// One work tile (source block, facet chunk, 32-sample chunk) of the forward
// render: every warp traces its share of the tile's warp tasks, then the
// tile's shared-memory rows go to the FP64 accumulator. All threads of the
// CTA call this; it ends after a __syncthreads.
template <int SRC, bool SOFT, int MODE, bool STAGES>
__device__ __forceinline__ void render_tile(const RenderK& p, const Obst& ob, const float* mir, const short* htab,
                                            float* sh_hist, const Sink& sink, int tile) {
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
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
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
    float x = 0.f, y = 0.f, val = 0.f;
    int hm;
    if (act) {
      const size_t si = (size_t)f * p.M + m;
      float z0 = 0.f, z1 = 0.f;
      if (SRC == IACT_SRC_EXTENDED) ray_normals(p.seed, s, f, m, z0, z1);
      trace_ray<SRC, STAGES>(p, ob, mir, __ldg(p.P4 + si), __ldg(p.N4 + si), src, sig, z0, z1, v, x, y, val, hm);
    }
    int rowbase;
    if (MODE == IACT_MODE_RESPONSE) rowbase = (p.rows_in_smem ? sl : s) * p.P;
    else rowbase = 0;
    if (SOFT) {
      if (p.sn.type == IACT_SENSOR_SOFT_SQUARE) splat_square(p.sn, sink, rowbase, act, x, y, val);
      else if (p.hex_in_smem) splat_hex(p.sn, htab, sink, rowbase, act, x, y, val);
      else splat_hex(p.sn, p.hex_table, sink, rowbase, act, x, y, val);
    } else if (act) {
      const int pix = (p.sn.type == IACT_SENSOR_SQUARE) ? bin_square(p.sn, x, y)
                      : (p.hex_in_smem ? bin_hex(p.sn, htab, x, y) : bin_hex(p.sn, p.hex_table, x, y));
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

}  // namespace iact
