// Adjoint (reverse-mode) of the single-stage render path.
//
// The reference has no backward of its own; users differentiate `render`
// with jax.grad (core/render.py:118-171 through sensors/*.py accumulate).
// This kernel computes the same gradients for a given dL/d(image) or
// dL/d(response matrix) by re-tracing every ray (recompute, nothing stored)
// and running the reverse sweep of its chain:
//
//   tp = R p + pos, n' = R normalize(n + s delta)        (mirrors.py:64-79)
//   d  = normalize(tp - src)  |  d = src                  (render.py:129-133)
//   c = d.n', r = d - 2 c n', val = v (-c) / w * shadow   (render.py:138-141, reflection.py:5-20)
//   (x, y) = plane hit of (tp, r)                          (intersections.py:6-41)
//   hard bins: d img[pix] / d val = 1 (pixel ids carry no gradient)
//   soft bins: val * w_k(x, y) / sum_k w_k                 (square.py:144-172, hexagonal.py:264-315)
//
// Shadow and hit masks are piecewise constant and carry no gradient, as in
// jax.grad. Gradients reach facet rotations (Euler degrees), facet
// positions, facet roughness scales, source positions/directions and source
// values. Each lane keeps running sums for its current facet and source;
// when a warp moves to another facet or source it reduces them across the
// warp and adds them to FP64 buckets (per facet: dL/dR as the world-frame
// matrix H with dL/dR = H R, dL/dpos, dL/dscale). k_adjoint_finish turns H
// into Euler-angle gradients once per facet.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "iact_device.cuh"
#include "iact_internal.h"

namespace iact {

struct AdjK {
  int F, M, S, P;
  const float4* P4;
  const float4* N4;
  const float4* D4;
  const float* facet_pos;
  const float* sources;
  const float* values;
  const float* grad_out;  // [P] or [S, P]
  const float* tables;
  int n_table_floats;
  int n_cyl, n_box, n_sph, n_obox, n_tri;
  const int* hex_table;
  int hex_in_smem;
  SensorK sn;
  double* gfacet;  // [F, kFacetGrad]
  double* gsrc;    // [S, 4]: d/dsource (3), d/dvalue
  int SB, FC, CC, n_fchunk, n_cchunk, n_tiles;
  int* counter;
};

// Per-lane running sums of one (facet, source) stream of rays.
struct Acc {
  float H[9];
  float gp[3];
  float gs;
  float gsrc[3];
  float gv;
};

__device__ __forceinline__ void acc_zero_facet(Acc& a) {
#pragma unroll
  for (int i = 0; i < 9; ++i) a.H[i] = 0.f;
  a.gp[0] = a.gp[1] = a.gp[2] = 0.f;
  a.gs = 0.f;
}
__device__ __forceinline__ void acc_zero_src(Acc& a) {
  a.gsrc[0] = a.gsrc[1] = a.gsrc[2] = 0.f;
  a.gv = 0.f;
}

// all lanes of the warp call with the same f
__device__ __forceinline__ void flush_facet(Acc& a, double* gfacet, int f) {
  double* dst = gfacet + (size_t)f * kFacetGrad;
  float v[kFacetGrad];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = a.H[i];
  v[9] = a.gp[0]; v[10] = a.gp[1]; v[11] = a.gp[2];
  v[12] = a.gs;
#pragma unroll
  for (int i = 0; i < kFacetGrad; ++i) {
    const float t = warp_sum(v[i]);
    if ((threadIdx.x & 31) == 0 && t != 0.f) atomicAdd(dst + i, (double)t);
  }
  acc_zero_facet(a);
}
__device__ __forceinline__ void flush_src(Acc& a, double* gsrc, int s) {
  double* dst = gsrc + (size_t)s * 4;
  float v[4] = {a.gsrc[0], a.gsrc[1], a.gsrc[2], a.gv};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float t = warp_sum(v[i]);
    if ((threadIdx.x & 31) == 0 && t != 0.f) atomicAdd(dst + i, (double)t);
  }
  acc_zero_src(a);
}

// dL/dval and dL/d(x, y) of one ray's deposit (sensors/square.py:144-172).
// Soft square: w_k = exp(-0.5 (dx_k^2 + dy_k^2)/sigma^2) over the pixel
// offsets; L = sum_k g_k val w_k / W. dL/dx = val/W sum_k (g_k - gbar) dw_k/dx.
__device__ __forceinline__ void soft_square_bwd(const SensorK& s, const float* g, int rowbase, float x, float y,
                                                float val, float& gval, float& gx, float& gy) {
  gval = gx = gy = 0.f;
  if (!((x < 1e9f) && (y < 1e9f))) return;
  float xp = (x - s.x0) * s.inv_dx, yp = (y - s.y0) * s.inv_dy;
  float xb = floorf(xp), yb = floorf(yp);
  float xf = xp - xb, yf = yp - yb;
  const int K = s.kernel_size, n = 2 * K + 1;
  const float is2 = 1.f / (s.sigma * s.sigma);
  const int xi0 = (int)xb, yi0 = (int)yb;
  float W = 0.f, sgw = 0.f, dWx = 0.f, dWy = 0.f, sgdx = 0.f, sgdy = 0.f;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      float ddx = xf - (float)(j - K), ddy = yf - (float)(i - K);
      float w = expf(-0.5f * is2 * (ddx * ddx + ddy * ddy));
      float wx = -w * ddx * is2 * s.inv_dx, wy = -w * ddy * is2 * s.inv_dy;  // dw/dx, dw/dy
      int xi = xi0 + j - K, yi = yi0 + i - K;
      float gk = (xi >= 0 && xi < s.width && yi >= 0 && yi < s.height) ? g[rowbase + yi * s.width + xi] : 0.f;
      W += w; sgw += gk * w; dWx += wx; dWy += wy; sgdx += gk * wx; sgdy += gk * wy;
    }
  const float iW = 1.f / W;
  gval = sgw * iW;
  gx = val * iW * (sgdx - gval * dWx);
  gy = val * iW * (sgdy - gval * dWy);
}

// sensors/hexagonal.py:264-315 soft hex deposit, reverse.
template <typename TT>
__device__ __forceinline__ void soft_hex_bwd(const SensorK& s, const TT* table, const float* g, int rowbase, float x,
                                             float y, float val, float& gval, float& gx, float& gy) {
  gval = gx = gy = 0.f;
  if (!((x < 1e9f) && (y < 1e9f))) return;
  float xg, yg, qi, ri;
  hex_axial(s, x, y, xg, yg, qi, ri);
  float ddx = xg - s.hex_sx * (qi + 0.5f * ri), ddy = yg - s.hex_sy * ri;
  const int K = s.kernel_size;
  const float isg = 1.f / s.sigma;
  float W = 0.f, sgw = 0.f, dWx = 0.f, dWy = 0.f, sgdx = 0.f, sgdy = 0.f;  // d/d(grid x, grid y)
  for (int q = -K; q <= K; ++q)
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float ux = ddx - s.hex_sx * ((float)q + 0.5f * (float)r), uy = ddy - s.hex_sy * (float)r;
      float ax = fabsf(ux), ay = fabsf(uy);
      float m2 = 0.5f * ax + 0.8660254037844386f * ay;
      bool first = ax >= m2;  // hex norm = max(|ux|, |ux|/2 + sqrt(3)/2 |uy|) / inradius
      float hd = (first ? ax : m2) * s.inv_inr;
      float a = hd * isg;
      float w = expf(-0.5f * a * a);
      float dhx = (first ? 1.f : 0.5f) * (ux >= 0.f ? 1.f : -1.f) * s.inv_inr;
      float dhy = (first ? 0.f : 0.8660254037844386f) * (uy >= 0.f ? 1.f : -1.f) * s.inv_inr;
      float dwda = -w * a * isg;  // dw/dhd
      float wx = dwda * dhx, wy = dwda * dhy;
      int p = hex_lookup(s, table, qi + (float)q, ri + (float)r);
      float gk = p >= 0 ? g[rowbase + p] : 0.f;
      W += w; sgw += gk * w; dWx += wx; dWy += wy; sgdx += gk * wx; sgdy += gk * wy;
    }
  const float iW = 1.f / W;
  gval = sgw * iW;
  const float gxg = val * iW * (sgdx - gval * dWx), gyg = val * iW * (sgdy - gval * dWy);
  // grid = rotate(x - off, -rot): xg = gc x' - gs y', yg = gs x' + gc y'
  gx = s.gc * gxg + s.gs * gyg;
  gy = -s.gs * gxg + s.gc * gyg;
}

template <int SRC, bool SOFT, int MODE>
__global__ void __launch_bounds__(256) k_adjoint(const AdjK p) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_tile;
  const int tab_n = (p.n_table_floats + 3) & ~3;
  const int htab_n = p.hex_in_smem ? ((p.sn.table_q * p.sn.table_r + 7) & ~7) : 0;
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + tab_n);
  const int nthr = blockDim.x;
  for (int i = threadIdx.x; i < p.n_table_floats; i += nthr) tab[i] = p.tables[i];
  for (int i = threadIdx.x; i < htab_n; i += nthr)
    htab[i] = (short)(i < p.sn.table_q * p.sn.table_r ? p.hex_table[i] : -1);
  const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  const SensorK& sn = p.sn;
  // sensor plane frame (intersections.py:19-21)
  const V3 u1 = mk(sn.R[0], sn.R[3], sn.R[6]), u2 = mk(sn.R[1], sn.R[4], sn.R[7]), ns = mk(sn.R[2], sn.R[5], sn.R[8]);
  const V3 C = mk(sn.pos[0], sn.pos[1], sn.pos[2]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = nthr >> 5;
  const int nch = (p.M + 31) >> 5;
  Acc acc;
  acc_zero_facet(acc);
  acc_zero_src(acc);
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(p.counter, 1);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= p.n_tiles) break;
    const int per_s = p.n_fchunk * p.n_cchunk;
    const int sblk = tile / per_s;
    const int fc = (tile - sblk * per_s) / p.n_cchunk;
    const int cc = tile - sblk * per_s - fc * p.n_cchunk;
    const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
    const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);
    const int T = SBc * FCc * CCc;
    const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
    int sl = tb / (FCc * CCc);
    int fl = (tb - sl * FCc * CCc) / CCc;
    int cl = tb - sl * FCc * CCc - fl * CCc;
    int cur_f = -1, cur_s = -1;
    for (int t = tb; t < te; ++t) {
      const int s = s0 + sl, f = f0 + fl;
      if (f != cur_f) {
        if (cur_f >= 0) flush_facet(acc, p.gfacet, cur_f);
        cur_f = f;
      }
      if (s != cur_s) {
        if (cur_s >= 0) flush_src(acc, p.gsrc, cur_s);
        cur_s = s;
      }
      const int m = (c0 + cl) * 32 + lane;
      const V3 src = mk(__ldg(p.sources + 3 * s), __ldg(p.sources + 3 * s + 1), __ldg(p.sources + 3 * s + 2));
      const float v = __ldg(p.values + s);
      const V3 fpos = mk(__ldg(p.facet_pos + 3 * f), __ldg(p.facet_pos + 3 * f + 1), __ldg(p.facet_pos + 3 * f + 2));
      const int rowbase = (MODE == IACT_MODE_RESPONSE) ? s * p.P : 0;
      if (m < p.M) {
        const size_t si = (size_t)f * p.M + m;
        const float4 P4 = __ldg(p.P4 + si), N4 = __ldg(p.N4 + si);
        const V3 tp = mk(P4.x, P4.y, P4.z), nn = mk(N4.x, N4.y, N4.z);
        const float iw = P4.w;
        // ---- forward re-trace
        V3 d, w;
        float inv_len = 0.f;
        if (SRC == IACT_SRC_POINT) {
          w = tp - src;
          inv_len = rsqrtf(dot(w, w));
          d = inv_len * w;
        } else {
          d = src;
        }
        const bool shadowed = occluded(ob, tp, mk(-d.x, -d.y, -d.z));
        const float c = dot(d, nn);
        const V3 r = d - (2.f * c) * nn;
        const float val = v * -c * iw;
        const float ndotd = dot(r, ns);
        const bool parallel = fabsf(ndotd) < 1e-10f;
        const float inv_nd = rcp_a(parallel ? 1.f : ndotd);
        const float tpl = (dot(ns, C) - dot(tp, ns)) * inv_nd;
        const V3 op = (tp + tpl * r) - C;
        const bool hit_plane = !parallel && (tpl > 0.f);
        const float x = hit_plane ? dot(op, u1) : kBig, y = hit_plane ? dot(op, u2) : kBig;
        // ---- reverse of the deposit
        float gval = 0.f, gx = 0.f, gy = 0.f;
        if (!shadowed) {
          if (SOFT) {
            if (sn.type == IACT_SENSOR_SOFT_SQUARE) soft_square_bwd(sn, p.grad_out, rowbase, x, y, val, gval, gx, gy);
            else if (p.hex_in_smem) soft_hex_bwd(sn, htab, p.grad_out, rowbase, x, y, val, gval, gx, gy);
            else soft_hex_bwd(sn, p.hex_table, p.grad_out, rowbase, x, y, val, gval, gx, gy);
          } else {
            const int pix = (sn.type == IACT_SENSOR_SQUARE) ? bin_square(sn, x, y)
                            : (p.hex_in_smem ? bin_hex(sn, htab, x, y) : bin_hex(sn, p.hex_table, x, y));
            gval = pix >= 0 ? __ldg(p.grad_out + rowbase + pix) : 0.f;
          }
        }
        if ((gval != 0.f) | (gx != 0.f) | (gy != 0.f)) {
          // plane (intersections.py:23-35): p = tp + t r, t = ns.(C - tp) / ns.r
          V3 gpl = gx * u1 + gy * u2;  // dL/dp
          const float dLdt = dot(gpl, r);
          V3 a = gpl - (dLdt * inv_nd) * ns;            // dL/dtp through the plane
          V3 gr = tpl * gpl - (dLdt * tpl * inv_nd) * ns;  // dL/dr through the plane
          // val = v (-c) iw ; r = d - 2 c n'
          const float dLdc = -gval * v * iw - 2.f * dot(gr, nn);
          const V3 b = (-2.f * c) * gr + dLdc * d;  // dL/dn'
          const V3 gd = gr + dLdc * nn;             // dL/dd
          V3 gsrc;
          if (SRC == IACT_SRC_POINT) {
            const V3 gw = inv_len * (gd - dot(d, gd) * d);  // d = w/|w|
            a = a + gw;
            gsrc = mk(-gw.x, -gw.y, -gw.z);
          } else {
            gsrc = gd;
          }
          // facet buckets: H += a (tp - pos)^T + b n'^T ; dL/dpos = a
          const V3 pr = tp - fpos;
          acc.H[0] += a.x * pr.x + b.x * nn.x; acc.H[1] += a.x * pr.y + b.x * nn.y; acc.H[2] += a.x * pr.z + b.x * nn.z;
          acc.H[3] += a.y * pr.x + b.y * nn.x; acc.H[4] += a.y * pr.y + b.y * nn.y; acc.H[5] += a.y * pr.z + b.y * nn.z;
          acc.H[6] += a.z * pr.x + b.z * nn.x; acc.H[7] += a.z * pr.y + b.z * nn.y; acc.H[8] += a.z * pr.z + b.z * nn.z;
          acc.gp[0] += a.x; acc.gp[1] += a.y; acc.gp[2] += a.z;
          if (p.D4) {  // n' = normalize(n + s delta): dn'/ds = (I - n'n'^T) delta_w / |m|
            const float4 D4 = __ldg(p.D4 + si);
            const V3 dw = mk(D4.x, D4.y, D4.z);
            acc.gs += dot(b, dw) - dot(b, nn) * dot(nn, dw);
          }
          acc.gsrc[0] += gsrc.x; acc.gsrc[1] += gsrc.y; acc.gsrc[2] += gsrc.z;
          acc.gv += gval * -c * iw;
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
    // warp-uniform: every lane ran the same task range
    if (cur_f >= 0) flush_facet(acc, p.gfacet, cur_f);
    if (cur_s >= 0) flush_src(acc, p.gsrc, cur_s);
  }
}

// Per facet: dL/dR = H R, then dL/d(tip, tilt, rot) in degrees with
// R = Rz(rot) Ry(tilt) Rx(tip) (core/transforms.py:72-107); per source the
// FP64 sums to float.
__global__ void k_adjoint_finish(const double* gfacet, const double* gsrc, const float* facet_rot, int F, int S,
                                 float* g_rot, float* g_pos, float* g_scale, float* g_src, float* g_val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < F) {
    const double* h = gfacet + (size_t)i * kFacetGrad;
    const double k = 0.017453292519943295;
    const double a = facet_rot[3 * i] * k, b = facet_rot[3 * i + 1] * k, c = facet_rot[3 * i + 2] * k;
    const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cc = cos(c), sc = sin(c);
    const double Rx[9] = {1, 0, 0, 0, ca, -sa, 0, sa, ca}, dRx[9] = {0, 0, 0, 0, -sa, -ca, 0, ca, -sa};
    const double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb}, dRy[9] = {-sb, 0, cb, 0, 0, 0, -cb, 0, -sb};
    const double Rz[9] = {cc, -sc, 0, sc, cc, 0, 0, 0, 1}, dRz[9] = {-sc, -cc, 0, cc, -sc, 0, 0, 0, 0};
    auto mm = [](const double* A, const double* B, double* Cm) {
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) Cm[3 * r + q] = A[3 * r] * B[q] + A[3 * r + 1] * B[3 + q] + A[3 * r + 2] * B[6 + q];
    };
    double ZY[9], R[9], G[9], T1[9], D[9];
    mm(Rz, Ry, ZY);
    mm(ZY, Rx, R);
    mm(h, R, G);  // dL/dR = H R
    double out[3];
    mm(ZY, dRx, D);  // dR/dtip
    out[0] = 0;
    for (int j = 0; j < 9; ++j) out[0] += G[j] * D[j];
    mm(Rz, dRy, T1);  // dR/dtilt
    mm(T1, Rx, D);
    out[1] = 0;
    for (int j = 0; j < 9; ++j) out[1] += G[j] * D[j];
    mm(dRz, Ry, T1);  // dR/drot
    mm(T1, Rx, D);
    out[2] = 0;
    for (int j = 0; j < 9; ++j) out[2] += G[j] * D[j];
    if (g_rot)
      for (int j = 0; j < 3; ++j) g_rot[3 * i + j] = (float)(out[j] * k);
    if (g_pos)
      for (int j = 0; j < 3; ++j) g_pos[3 * i + j] = (float)h[9 + j];
    if (g_scale) g_scale[i] = (float)h[12];
  }
  if (i < S) {
    if (g_src)
      for (int j = 0; j < 3; ++j) g_src[3 * i + j] = (float)gsrc[4 * i + j];
    if (g_val) g_val[i] = (float)gsrc[4 * i + 3];
  }
}

namespace {

template <int SRC, bool SOFT, int MODE>
int run_adjoint(const AdjK& p, int block, size_t smem, cudaStream_t st) {
  auto kern = k_adjoint<SRC, SOFT, MODE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_adjoint smem)");
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
  if (e != cudaSuccess) return check_cuda(e, "occupancy query");
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "adjoint kernel does not fit on an SM");
  const int grid = std::max(1, std::min(p.n_tiles, per_sm * device_info().sm_count));
  kern<<<grid, block, smem, st>>>(p);
  return check_cuda(cudaGetLastError(), "k_adjoint launch");
}

template <int SRC, bool SOFT>
int adj_mode(int mode, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  return mode == IACT_MODE_RESPONSE ? run_adjoint<SRC, SOFT, IACT_MODE_RESPONSE>(p, block, smem, st)
                                    : run_adjoint<SRC, SOFT, IACT_MODE_IMAGE>(p, block, smem, st);
}

}  // namespace

int launch_backward(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                    const float* values, int S, int mode, const float* grad_out, float* g_rot, float* g_pos,
                    float* g_scale, float* g_src, float* g_val, void* ws, size_t ws_bytes, const iact_opts_t* opts,
                    cudaStream_t st) {
  (void)ws_bytes;
  const int F = sc->n_facets;
  const WsLayout L = workspace_for(sc, sn, S, IACT_MODE_BACKWARD);
  char* w = static_cast<char*>(ws);
  double* gfacet = reinterpret_cast<double*>(w + L.acc);
  double* gsrc = gfacet + (size_t)F * kFacetGrad;
  const size_t nacc = (size_t)F * kFacetGrad + (size_t)S * 4;
  int rc = check_cuda(cudaMemsetAsync(gfacet, 0, nacc * sizeof(double), st), "zero gradient buckets");
  if (rc) return rc;
  if (S > 0 && F > 0 && sc->n_samples > 0) {
    rc = check_cuda(cudaMemsetAsync(w + L.counter, 0, 64, st), "reset tile counter");
    if (rc) return rc;
    rc = launch_prep(sc, L, w, st, g_scale != nullptr);
    if (rc) return rc;
    AdjK p;
    memset(&p, 0, sizeof(p));
    p.F = F; p.M = sc->n_samples; p.S = S; p.P = sn->n_pixels;
    p.P4 = reinterpret_cast<const float4*>(w + L.p4);
    p.N4 = reinterpret_cast<const float4*>(w + L.n4);
    p.D4 = g_scale ? reinterpret_cast<const float4*>(w + L.d4) : nullptr;
    p.facet_pos = sc->facet_pos;
    p.sources = sources; p.values = values; p.grad_out = grad_out;
    p.tables = reinterpret_cast<const float*>(w + L.tables);
    p.n_table_floats = L.n_table_floats;
    p.n_cyl = sc->n_cyl; p.n_box = sc->n_box; p.n_sph = sc->n_sph; p.n_obox = sc->n_obox; p.n_tri = sc->n_tri;
    p.hex_table = sn->table;
    p.sn = make_sensor(sn);
    p.gfacet = gfacet;
    p.gsrc = gsrc;
    p.counter = reinterpret_cast<int*>(w + L.counter);
    const int block = (opts && opts->block_threads > 0) ? opts->block_threads : 256;
    const int nw = block / 32;
    const int nch = (p.M + 31) / 32;
    p.SB = std::min(S, nw);
    const int target = nw * 48;
    p.CC = std::min(nch, std::max(1, target / p.SB));
    p.FC = std::min(F, std::max(1, target / (p.SB * p.CC)));
    p.n_fchunk = (F + p.FC - 1) / p.FC;
    p.n_cchunk = (nch + p.CC - 1) / p.CC;
    const long long tiles = (long long)((S + p.SB - 1) / p.SB) * p.n_fchunk * p.n_cchunk;
    if (tiles > 0x7fffffffLL) return set_error(IACT_E_UNSUPPORTED, "too many work tiles");
    p.n_tiles = (int)tiles;
    const size_t tab_bytes = sizeof(float) * (size_t)((L.n_table_floats + 3) & ~3);
    const bool hex = (sn->type == IACT_SENSOR_HEX || sn->type == IACT_SENSOR_SOFT_HEX);
    const size_t htab = hex ? (size_t)sn->table_q * sn->table_r : 0;
    const size_t htab_bytes = sizeof(short) * ((htab + 7) & ~(size_t)7);
    p.hex_in_smem = (hex && sn->n_pixels < 32768 && tab_bytes + htab_bytes <= 96 * 1024) ? 1 : 0;
    const size_t smem = tab_bytes + (p.hex_in_smem ? htab_bytes : 0);
    const bool soft = sn->type == IACT_SENSOR_SOFT_SQUARE || sn->type == IACT_SENSOR_SOFT_HEX;
    void* const* ev = opts ? opts->kernel_events : nullptr;
    if (ev && ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
    if (src_type == IACT_SRC_POINT)
      rc = soft ? adj_mode<IACT_SRC_POINT, true>(mode, p, block, smem, st)
                : adj_mode<IACT_SRC_POINT, false>(mode, p, block, smem, st);
    else
      rc = soft ? adj_mode<IACT_SRC_PARALLEL, true>(mode, p, block, smem, st)
                : adj_mode<IACT_SRC_PARALLEL, false>(mode, p, block, smem, st);
    if (rc) return rc;
    if (ev && ev[1]) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), st);
  }
  const int n = std::max(F, S);
  if (n > 0) {
    k_adjoint_finish<<<(n + 255) / 256, 256, 0, st>>>(gfacet, gsrc, sc->facet_rot, F, S, g_rot, g_pos, g_scale,
                                                        g_src, g_val);
    rc = check_cuda(cudaGetLastError(), "k_adjoint_finish launch");
  }
  return rc;
}

}  // namespace iact
