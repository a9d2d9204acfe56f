// Device code of the adjoint shared by the single-scene backward
// (iact_adjoint.cu) and the batched backward (iact_batched_adjoint.cu):
// launch parameters, per-lane sums, the reverse sweeps and one work tile.
#pragma once

#include "iact_device.cuh"
#include "iact_internal.h"
#include "iact_render_impl.cuh"

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
  double* gmir;    // [n_mir, kMirGrad]: dL/dR (9), dL/dpos (3), dL/dc, dL/dk, dL/da (8)
  int n_mir;
  int SB, FC, CC, n_fchunk, n_cchunk, n_tiles;
  int* counter;
  uint32_t seed;  // jitter stream of extended sources
  const float4* B4;  // per facet bundle bounds (culling on)
  int n_words;       // 32-bit candidate-mask words per task; 0 = no culling
  float* gsamp;      // optional [F*M, 7]: per sample dL/d(world point, perturbed normal, 1/weight)
  int want_mgrad;    // stage-mirror parameter gradients requested (gmir)
  const uint32_t* gmask;  // k_adjoint_hard: candidate word per (source, facet) pair [S * F], or null
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
// offsets; L = sum_k g_k val w_k / W, so dL/dval = gbar = sum_k g_k w_k / W
// and dL/dx = val/W sum_k (g_k - gbar) dw_k/dx. The sums run on g_k - g_0
// (g_0: the centre tap), which is exact for the dominant tap: the direct
// form cancels catastrophically in float32 when one tap carries the ray.
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
  const bool c_in = xi0 >= 0 && xi0 < s.width && yi0 >= 0 && yi0 < s.height;
  const float g0 = c_in ? g[rowbase + yi0 * s.width + xi0] : 0.f;
  float W = 0.f, sgw = 0.f, dWx = 0.f, dWy = 0.f, sgdx = 0.f, sgdy = 0.f;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      float ddx = xf - (float)(j - K), ddy = yf - (float)(i - K);
      float w = __expf(-0.5f * is2 * (ddx * ddx + ddy * ddy));
      float wx = -w * ddx * is2 * s.inv_dx, wy = -w * ddy * is2 * s.inv_dy;  // dw/dx, dw/dy
      int xi = xi0 + j - K, yi = yi0 + i - K;
      float gk = (xi >= 0 && xi < s.width && yi >= 0 && yi < s.height) ? g[rowbase + yi * s.width + xi] : 0.f;
      const float dg = gk - g0;
      W += w; sgw += dg * w; dWx += wx; dWy += wy; sgdx += dg * wx; sgdy += dg * wy;
    }
  const float iW = 1.f / W;
  const float dbar = sgw * iW;  // gbar - g0
  gval = g0 + dbar;
  gx = val * iW * (sgdx - dbar * dWx);
  gy = val * iW * (sgdy - dbar * dWy);
}

// sensors/hexagonal.py:264-315 soft hex deposit, reverse (same centred sums
// as soft_square_bwd, centred on the base hexagon's gradient).
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
  const int p0 = hex_lookup(s, table, qi, ri);
  const float g0 = p0 >= 0 ? g[rowbase + p0] : 0.f;
  float W = 0.f, sgw = 0.f, dWx = 0.f, dWy = 0.f, sgdx = 0.f, sgdy = 0.f;  // d/d(grid x, grid y)
  // lookup-table index of the base hexagon; interior rings are at fixed offsets
  const float qx = qi - (float)s.q_min, rx = ri - (float)s.r_min;
  const bool inner = (qx >= (float)K) & (qx < (float)(s.table_q - K)) & (rx >= (float)K) & (rx < (float)(s.table_r - K));
  const int base = inner ? (int)qx * s.table_r + (int)rx : 0;
#pragma unroll 3
  for (int q = -K; q <= K; ++q)
#pragma unroll 3
    for (int r = -K; r <= K; ++r) {
      if (max(max(abs(q), abs(r)), abs(q + r)) > K) continue;
      float ux = ddx - s.hex_sx * ((float)q + 0.5f * (float)r), uy = ddy - s.hex_sy * (float)r;
      float ax = fabsf(ux), ay = fabsf(uy);
      float m2 = 0.5f * ax + 0.8660254037844386f * ay;
      bool first = ax >= m2;  // hex norm = max(|ux|, |ux|/2 + sqrt(3)/2 |uy|) / inradius
      float hd = (first ? ax : m2) * s.inv_inr;
      float a = hd * isg;
      float w = __expf(-0.5f * a * a);
      float dhx = (first ? 1.f : 0.5f) * (ux >= 0.f ? 1.f : -1.f) * s.inv_inr;
      float dhy = (first ? 0.f : 0.8660254037844386f) * (uy >= 0.f ? 1.f : -1.f) * s.inv_inr;
      float dwda = -w * a * isg;  // dw/dhd
      float wx = dwda * dhx, wy = dwda * dhy;
      int p;
      if (inner) {
        p = (int)table[base + q * s.table_r + r];
        p = p >= 0 ? p : -1;
      } else {
        p = hex_lookup(s, table, qi + (float)q, ri + (float)r);
      }
      float dg = (p >= 0 ? g[rowbase + p] : 0.f) - g0;
      W += w; sgw += dg * w; dWx += wx; dWy += wy; sgdx += dg * wx; sgdy += dg * wy;
    }
  const float iW = 1.f / W;
  const float dbar = sgw * iW;
  gval = g0 + dbar;
  const float gxg = val * iW * (sgdx - dbar * dWx), gyg = val * iW * (sgdy - dbar * dWy);
  // grid = rotate(x - off, -rot): xg = gc x' - gs y', yg = gs x' + gc y'
  gx = s.gc * gxg + s.gs * gyg;
  gy = -s.gs * gxg + s.gc * gyg;
}


// Adds each lane's stage-mirror gradient terms g (mirror j; j < 0: none)
// into the CTA's shared sums. Warp-collective (all 32 lanes). When every
// contributing lane hit the same mirror, a butterfly reduce-scatter over the
// 32 lanes (31 shuffles) leaves lane i with the warp's sum of term i and
// lanes 0..kMirGrad-1 add one term each (distinct addresses); otherwise
// each lane adds its own terms.
__device__ __forceinline__ void warp_add_mirror_grads(float* mgrad, int j, const float (&g)[kMirGrad], int lane) {
  const unsigned any = __ballot_sync(kFull, j >= 0);
  if (any == 0u) return;
  const int j0 = __shfl_sync(kFull, j, __ffs(any) - 1);
  if (__all_sync(kFull, j < 0 || j == j0)) {
    float v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = (i < kMirGrad && j >= 0) ? g[i] : 0.f;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const bool hi = (lane & off) != 0;
#pragma unroll
      for (int i = 0; i < off; ++i) {
        const float send = hi ? v[i] : v[i + off];
        const float keep = hi ? v[i + off] : v[i];
        v[i] = keep + __shfl_xor_sync(kFull, send, off);
      }
    }
    if (lane < kMirGrad && v[0] != 0.f) atomicAdd(mgrad + j0 * kMirGrad + lane, v[0]);
  } else if (j >= 0) {
#pragma unroll
    for (int i = 0; i < kMirGrad; ++i)
      if (g[i] != 0.f) atomicAdd(mgrad + j * kMirGrad + i, g[i]);
  }
}

// One stage >= 1 reflection as recorded by the forward re-trace.
struct StageRec {
  V3 o, r;      // incoming ray (world)
  float val;    // value before this stage
  int j;        // mirror index (scene order)
  float t;      // Newton root
  V3 pl, nl;    // local hit point and unit normal
  float c2;     // r . n_world
};

// Forward of one later stage (core/render.py:44-115): the closest hit
// (first index on ties, as argmin) over the mirrors of the stage that starts
// at table index mi, for the ray (o, r) carrying val. Returns the table index
// past the stage; hit tells whether any mirror of the stage was hit, and R
// then holds the record of the reflection.
__device__ __forceinline__ int stage_fwd(const float* mir, int n_mir, int mi, V3 o, V3 r, float val, StageRec& R,
                                         bool& hit) {
  const int stg = (int)mir[mi * kMirF + 22];
  float best_t = __int_as_float(0x7f800000);
  V3 bpl = mk(0.f, 0.f, 0.f), bnl = mk(0.f, 0.f, 0.f);
  int bi = -1;
  int mj = mi;
  for (; mj < n_mir && (int)mir[mj * kMirF + 22] == stg; ++mj) {
    const float* mm = mir + mj * kMirF;
    const V3 pos = mk(mm[9], mm[10], mm[11]);
    V3 pl, nl;
    const float tt = mirror_hit(mm, rtmul(mm, o - pos), rtmul(mm, r), pl, nl);
    if (tt < best_t) {
      best_t = tt; bpl = pl; bnl = nl; bi = mj;
    }
  }
  hit = best_t < kBig;
  if (hit) {
    R.o = o; R.r = r; R.val = val; R.j = bi; R.t = best_t; R.pl = bpl; R.nl = bnl;
    R.c2 = dot(r, rmul(mir + bi * kMirF, bnl));
  }
  return mj;
}

// The ray after the reflection R records: o' = Rj pl + Pj, r' = r - 2 c2 n_w,
// val' = val |c2|.
__device__ __forceinline__ void stage_apply(const float* mir, const StageRec& R, V3& o, V3& r, float& val) {
  const float* mm = mir + R.j * kMirF;
  const V3 nw = rmul(mm, R.nl);
  val = val * fabsf(R.c2);
  o = rmul(mm, R.pl) + mk(mm[9], mm[10], mm[11]);
  r = r - (2.f * R.c2) * nw;
}

// The record of later stage k of a ray that hit every stage, re-traced from
// the primary reflection (o0, r0, val0): the reverse sweep's source for
// stages that left the ring (scenes with more than kAdjRing stages).
__device__ __forceinline__ void stage_retrace(const float* mir, int n_mir, int k, V3 o0, V3 r0, float val0,
                                           StageRec& out) {
  V3 o = o0, r = r0;
  float val = val0;
  int mi = 0;
  for (int kk = 0; mi < n_mir; ++kk) {
    bool hit;
    mi = stage_fwd(mir, n_mir, mi, o, r, val, out, hit);
    if (kk == k || !hit) return;
    stage_apply(mir, out, o, r, val);
  }
}

// Reverse of core/render.py:44-115 for one ray at one stage: from dL/d(o',
// r', val') after the reflection to dL/d(o, r, val) before it, adding the
// mirror's parameter gradients into g (kMirGrad floats). The hit t(o, r,
// theta) is the Newton root of g(t) = o_z + t d_z - sag(o_xy + t d_xy) = 0,
// differentiated implicitly (dt = -(dG) / G_t with G_t = N . d_local,
// N = (-sag_x, -sag_y, 1)); the reference unrolls its 10 Newton steps, which
// agrees to the root's residual.
// PARAMS: also form the mirror's parameter gradients g (else g is untouched
// and only the chain through the stage is reversed).
template <bool PARAMS>
__device__ __forceinline__ void stage_bwd(const float* m, const StageRec& R, V3& go, V3& gr, float& gv,
                                          float* g) {
  const float* Rj = m;
  const V3 Pj = mk(m[9], m[10], m[11]);
  const V3 nw = rmul(Rj, R.nl);
  // val' = val |c2|
  const float sgn = R.c2 >= 0.f ? 1.f : -1.f;
  float gc2 = gv * R.val * sgn;
  const float gval_in = gv * fabsf(R.c2);
  // r' = r - 2 c2 nw, c2 = r . nw
  gc2 += -2.f * dot(gr, nw);
  V3 gnw = (-2.f * R.c2) * gr;
  V3 gr_in = gr + gc2 * nw;
  gnw = gnw + gc2 * R.r;
  // o' = Rj pl + Pj, nw = Rj nl
  const V3 gpl = rtmul(Rj, go);
  const V3 gnl = rtmul(Rj, gnw);
  float gR[9];
  gR[0] = go.x * R.pl.x + gnw.x * R.nl.x; gR[1] = go.x * R.pl.y + gnw.x * R.nl.y; gR[2] = go.x * R.pl.z + gnw.x * R.nl.z;
  gR[3] = go.y * R.pl.x + gnw.y * R.nl.x; gR[4] = go.y * R.pl.y + gnw.y * R.nl.y; gR[5] = go.y * R.pl.z + gnw.y * R.nl.z;
  gR[6] = go.z * R.pl.x + gnw.z * R.nl.x; gR[7] = go.z * R.pl.y + gnw.z * R.nl.y; gR[8] = go.z * R.pl.z + gnw.z * R.nl.z;
  V3 gP = go;
  // nl = N/|N|, |N| = 1/nl_z
  const float ndg = dot(R.nl, gnl);
  const V3 gN = R.nl.z * (gnl - ndg * R.nl);
  // surface derivatives at the hit and at the facet offset (z0)
  const float x0 = m[12], y0 = m[13];
  const float Xs = R.pl.x + x0, Ys = R.pl.y + y0;
  SagD D, D0;
  sag_derivs(m, Xs * Xs + Ys * Ys, D);
  if (x0 != 0.f || y0 != 0.f) {
    sag_derivs(m, x0 * x0 + y0 * y0, D0);
  } else {  // no offset: z0 = 0 for every parameter value
    D0.S = D0.Sr = D0.Srr = D0.Sc = D0.Sk = D0.Src = D0.Srk = 0.f;
  }
  const float sX = 2.f * Xs * D.Sr, sY = 2.f * Ys * D.Sr;
  const float sXX = 2.f * D.Sr + 4.f * Xs * Xs * D.Srr, sXY = 4.f * Xs * Ys * D.Srr, sYY = 2.f * D.Sr + 4.f * Ys * Ys * D.Srr;
  float gX = -(gN.x * sXX + gN.y * sXY), gY = -(gN.x * sXY + gN.y * sYY);
  const float wN = -(2.f * Xs * gN.x + 2.f * Ys * gN.y);  // dL/dS_rho through the normal
  float gth_c = wN * D.Src, gth_k = wN * D.Srk;
  // pl = (X, Y, S(rho) - S(rho0))
  gX += gpl.x + gpl.z * sX;
  gY += gpl.y + gpl.z * sY;
  gth_c += gpl.z * (D.Sc - D0.Sc);
  gth_k += gpl.z * (D.Sk - D0.Sk);
  // X = ol_x + t dl_x, Y = ol_y + t dl_y ; t implicit
  const V3 ol = rtmul(Rj, R.o - Pj), dl = rtmul(Rj, R.r);
  V3 gol = mk(gX, gY, 0.f);
  V3 gdl = mk(R.t * gX, R.t * gY, 0.f);
  const float gt = gX * dl.x + gY * dl.y;
  const float Gt = -sX * dl.x - sY * dl.y + dl.z;
  const float lam = gt / Gt;
  const V3 Nv = mk(-sX, -sY, 1.f);
  gol = gol - lam * Nv;
  gdl = gdl - (lam * R.t) * Nv;
  gth_c += lam * (D.Sc - D0.Sc);
  gth_k += lam * (D.Sk - D0.Sk);
  // aspheric terms: dS/da_i = rho^p - rho0^p, dS_rho/da_i = p rho^(p-1), p = 2(i+1)
  float gth_a[8];
  {
    const int na = (int)m[19];
    const float rho = Xs * Xs + Ys * Ys, rho0 = x0 * x0 + y0 * y0, kz = gpl.z + lam;
    float rp = rho * rho, rpm1 = rho, rp0 = rho0 * rho0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      gth_a[i] = 0.f;
      if (i < na) {
        gth_a[i] = wN * (2.f * (i + 1)) * rpm1 + kz * (rp - rp0);
        rp *= rho * rho;
        rpm1 *= rho * rho;
        rp0 *= rho0 * rho0;
      }
    }
  }
  (void)ol;
  // ol = Rj^T (o - Pj), dl = Rj^T r
  const V3 Rg_ol = rmul(Rj, gol), Rg_dl = rmul(Rj, gdl);
  go = Rg_ol;
  gP = gP - Rg_ol;
  const V3 op = R.o - Pj;
  gR[0] += op.x * gol.x + R.r.x * gdl.x; gR[1] += op.x * gol.y + R.r.x * gdl.y; gR[2] += op.x * gol.z + R.r.x * gdl.z;
  gR[3] += op.y * gol.x + R.r.y * gdl.x; gR[4] += op.y * gol.y + R.r.y * gdl.y; gR[5] += op.y * gol.z + R.r.y * gdl.z;
  gR[6] += op.z * gol.x + R.r.z * gdl.x; gR[7] += op.z * gol.y + R.r.z * gdl.y; gR[8] += op.z * gol.z + R.r.z * gdl.z;
  gr = gr_in + Rg_dl;
  gv = gval_in;
  if (PARAMS) {
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i] = gR[i];
    g[9] = gP.x; g[10] = gP.y; g[11] = gP.z;
    g[12] = gth_c;
    g[13] = gth_k;
#pragma unroll
    for (int i = 0; i < 8; ++i) g[14 + i] = gth_a[i];
  }
}

// One work tile (source block, facet chunk, 32-sample chunk) of the
// adjoint: candidate masks, then every warp re-traces and reverses its share
// of the tasks; per-lane (facet, source) sums are flushed by the end of the
// tile. CTA-collective (contains __syncthreads).
// AX: the sensor's rotation is exactly the identity (p.sn.axes): the plane
// hit takes components instead of dot products with the unit axes (the same
// floats, as plane_hit<true>).
// DEEP: the scene has more than kAdjRing later stages; the reverse of a
// stage that left the ring re-traces it (stage_retrace). Scenes with at most
// kAdjRing stages take the kernels without that path.
template <int SRC, bool SOFT, int MODE, bool STAGES, bool AX = false, bool DEEP = false>
__device__ __forceinline__ void adjoint_tile(const AdjK& p, const Obst& ob, const float* mir, const short* htab,
                                             float* mgrad, uint32_t* tmask, int tile) {
  const SensorK& sn = p.sn;
  // sensor plane frame (intersections.py:19-21)
  const V3 u1 = mk(sn.R[0], sn.R[3], sn.R[6]), u2 = mk(sn.R[1], sn.R[4], sn.R[7]), ns = mk(sn.R[2], sn.R[5], sn.R[8]);
  const V3 C = mk(sn.pos[0], sn.pos[1], sn.pos[2]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nch = (p.M + 31) >> 5;
  Acc acc;
  acc_zero_facet(acc);
  acc_zero_src(acc);
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  if (p.n_words) warp_masks<SRC>(p.B4, p.sources, p.n_words, ob, s0, f0, FCc, CCc, tb, te, tmask);
  int sl = tb / (FCc * CCc);
  int fl = (tb - sl * FCc * CCc) / CCc;
  int cl = tb - sl * FCc * CCc - fl * CCc;
  int cur_f = -1, cur_s = -1;
  JBasis jb;  // tangent basis of the current source (extended sources)
  int jb_s = -1;
  HexCache hc = {3.0e38f, 3.0e38f, -1};  // last hexagon of this lane (hard hex sensors)
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
    constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
    const V3 src = mk(__ldg(p.sources + SS * s), __ldg(p.sources + SS * s + 1), __ldg(p.sources + SS * s + 2));
    const float v = __ldg(p.values + s);
    const V3 fpos = mk(__ldg(p.facet_pos + 3 * f), __ldg(p.facet_pos + 3 * f + 1), __ldg(p.facet_pos + 3 * f + 2));
    const int rowbase = (MODE == IACT_MODE_RESPONSE) ? s * p.P : 0;
    // with stage mirrors, lanes past the chunk's last sample run the body on
    // a clamped sample with no contribution, so the warp stays converged for
    // the collective stage-mirror sums
    const bool ok = m < p.M;
    const int mc = ok ? m : p.M - 1;
    if (STAGES || ok) {
      const size_t si = (size_t)f * p.M + mc;
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
      } else if (SRC == IACT_SRC_EXTENDED) {  // jitter regenerated from its counter
        float z0, z1;
        ray_normals(p.seed, s, f, mc, z0, z1);
        if (s != jb_s) {  // warp-uniform
          jb = jitter_basis(src);
          jb_s = s;
        }
        d = jitter_dir(jb, __ldg(p.sources + SS * s + 3), z0, z1);
      } else {
        d = src;
      }
      const bool shadowed = occluded_mask(ob, tmask + (sl * FCc + fl) * p.n_words, p.n_words, tp,
                                          mk(-d.x, -d.y, -d.z));
      const float c = dot(d, nn);
      const V3 r0 = d - (2.f * c) * nn;
      const float val0 = v * -c * iw;
      // later stages, recorded for the reverse sweep (core/render.py:44-79):
      // stage k's record in rec[k % kAdjRing]; the reverse sweep runs k
      // downwards and overwrites a slot only after its stage is reversed
      StageRec rec[kAdjRing];
      int nst = 0;
      bool alive = ok && !shadowed;
      V3 o = tp, r = r0;
      float val = val0;
      if (STAGES) {
        int mi = 0;
        while (mi < p.n_mir) {
          StageRec& R = rec[nst & (kAdjRing - 1)];
          bool hit;
          mi = stage_fwd(mir, p.n_mir, mi, o, r, val, R, hit);
          alive = alive && hit && !occluded(ob, o, r);
          if (hit) {
            ++nst;
            stage_apply(mir, R, o, r, val);
          } else {
            alive = false;
          }
        }
      }
      const float ndotd = AX ? r.z : dot(r, ns);
      const bool parallel = fabsf(ndotd) < 1e-10f;
      const float inv_nd = rcp_a(parallel ? 1.f : ndotd);
      const float tpl = ((AX ? C.z : dot(ns, C)) - (AX ? o.z : dot(o, ns))) * inv_nd;
      const V3 op = (o + tpl * r) - C;
      const bool hit_plane = !parallel && (tpl > 0.f);
      const float x = hit_plane ? (AX ? op.x : dot(op, u1)) : kBig;
      const float y = hit_plane ? (AX ? op.y : dot(op, u2)) : kBig;
      // ---- reverse of the deposit
      float gval = 0.f, gx = 0.f, gy = 0.f;
      if (alive) {
        if (SOFT) {
          if (sn.type == IACT_SENSOR_SOFT_SQUARE) soft_square_bwd(sn, p.grad_out, rowbase, x, y, val, gval, gx, gy);
          else if (p.hex_in_smem) soft_hex_bwd(sn, htab, p.grad_out, rowbase, x, y, val, gval, gx, gy);
          else soft_hex_bwd(sn, p.hex_table, p.grad_out, rowbase, x, y, val, gval, gx, gy);
        } else {
          const int pix = (sn.type == IACT_SENSOR_SQUARE) ? bin_square(sn, x, y)
                          : (p.hex_in_smem ? bin_hex_cached(sn, htab, x, y, hc)
                                           : bin_hex_cached(sn, p.hex_table, x, y, hc));
          gval = pix >= 0 ? __ldg(p.grad_out + rowbase + pix) : 0.f;
        }
      }
      const bool act = (gval != 0.f) | (gx != 0.f) | (gy != 0.f);
      V3 a = mk(0.f, 0.f, 0.f), gr = mk(0.f, 0.f, 0.f);
      float gv0 = gval;
      if (SOFT && act) {  // hard pixels are constants: nothing flows back through the hit point
        // plane (intersections.py:23-35): p = o + t r, t = ns.(C - o) / ns.r
        V3 gpl = gx * u1 + gy * u2;  // dL/dp
        const float dLdt = dot(gpl, r);
        a = gpl - (dLdt * inv_nd) * ns;               // dL/do through the plane
        gr = tpl * gpl - (dLdt * tpl * inv_nd) * ns;  // dL/dr through the plane
      }
      if (STAGES && !p.want_mgrad && act) {  // the chain through the stages only
        for (int k = nst - 1; k >= 0; --k) {
          float gm[kMirGrad];
          StageRec& Rk = rec[k & (kAdjRing - 1)];
          if (DEEP && k < nst - kAdjRing) stage_retrace(mir, p.n_mir, k, tp, r0, val0, Rk);  // left the ring
          stage_bwd<false>(mir + Rk.j * kMirF, Rk, a, gr, gv0, gm);
        }
      }
      if (STAGES && p.want_mgrad) {  // warp-converged: the mirror sums are warp-collective
        const int kmax = __reduce_max_sync(kFull, act ? nst : 0);
        for (int k = kmax - 1; k >= 0; --k) {
          float gm[kMirGrad];
          int j = -1;
          if (act && k < nst) {
            StageRec& Rk = rec[k & (kAdjRing - 1)];
            if (DEEP && k < nst - kAdjRing) stage_retrace(mir, p.n_mir, k, tp, r0, val0, Rk);  // left the ring
            stage_bwd<true>(mir + Rk.j * kMirF, Rk, a, gr, gv0, gm);
            j = Rk.j;
          } else {
#pragma unroll
            for (int i = 0; i < kMirGrad; ++i) gm[i] = 0.f;
          }
          warp_add_mirror_grads(mgrad, j, gm, lane);
        }
      }
      if (act) {
        // val = v (-c) iw ; r = d - 2 c n'. With hard pixels and no later
        // stage, a = dL/do and gr = dL/dr are exactly zero here (kHit false).
        constexpr bool kHit = SOFT || STAGES;
        const float dLdc = kHit ? -gv0 * v * iw - 2.f * dot(gr, nn) : -gv0 * v * iw;
        const V3 b = kHit ? (-2.f * c) * gr + dLdc * d : dLdc * d;  // dL/dn'
        const V3 gd = kHit ? gr + dLdc * nn : dLdc * nn;            // dL/dd
        V3 gsrc;
        if (SRC == IACT_SRC_POINT) {
          const V3 gw = inv_len * (gd - dot(d, gd) * d);  // d = w/|w|
          a = kHit ? a + gw : gw;
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
        acc.gv += gv0 * -c * iw;
        if (p.gsamp) {  // per-sample sums over the sources (resampling gradients)
          float* gs = p.gsamp + si * 7;
          atomicAdd(gs + 0, a.x); atomicAdd(gs + 1, a.y); atomicAdd(gs + 2, a.z);
          atomicAdd(gs + 3, b.x); atomicAdd(gs + 4, b.y); atomicAdd(gs + 5, b.z);
          atomicAdd(gs + 6, gv0 * v * -c);
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
  // warp-uniform: every lane ran the same task range
  if (cur_f >= 0) flush_facet(acc, p.gfacet, cur_f);
  if (cur_s >= 0) flush_src(acc, p.gsrc, cur_s);
}

// flush_facet without the roughness-scale sum (hard-pixel adjoint, no D4)
__device__ __forceinline__ void flush_facet_hard(Acc& a, double* gfacet, int f) {
  double* dst = gfacet + (size_t)f * kFacetGrad;
  float v[12];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = a.H[i];
  v[9] = a.gp[0]; v[10] = a.gp[1]; v[11] = a.gp[2];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const float t = warp_sum(v[i]);
    if ((threadIdx.x & 31) == 0 && t != 0.f) atomicAdd(dst + i, (double)t);
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) a.H[i] = 0.f;
  a.gp[0] = a.gp[1] = a.gp[2] = 0.f;
}

// Hard-pixel adjoint tile of the common case: a single-stage scene, point or
// parallel sources, a sensor whose rotation is the identity, the hexagon
// table in shared memory, candidate words per (source, facet) pair from
// k_masks, and no roughness-scale or per-sample gradients. The arithmetic is
// adjoint_tile<SRC, false, MODE, false, true>'s (pixel ids are constants, so
// only the value path carries gradient back to the reflection and the
// direction); the sensor kind and table placement are compile-time, lanes
// past the last sample run the facet's last sample with no contribution,
// per-pair values are loaded once per pair, and a warp's tasks run facet by
// facet (source next, chunk fastest): the per-source sums (4 values) are
// reduced at every pair change and the per-facet sums (13 values) only when
// the facet changes.
template <int SRC, int MODE, bool HEX>
__device__ __forceinline__ void adjoint_tile_hard(const AdjK& p, const Obst& ob, const short* htab, int tile) {
  const SensorK& sn = p.sn;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nch = (p.M + 31) >> 5;
  Acc acc;
  acc_zero_facet(acc);
  acc_zero_src(acc);
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  // tasks t = (facet fl, source sl, chunk cl), chunk fastest
  int q = tb / CCc;  // pair index fl * SBc + sl
  int fl = q / SBc, sl = q - fl * SBc;
  int cl = tb - q * CCc;
  int cur_f = -1;
  HexCache hc = {3.0e38f, 3.0e38f, -1};  // last hexagon of this lane
  const int mlast = p.M - 1;
  for (int t = tb; t < te;) {
    const int s = s0 + sl, f = f0 + fl;
    const int ce = min(CCc, cl + (te - t));
    t += ce - cl;
    if (f != cur_f) {
      if (cur_f >= 0) flush_facet_hard(acc, p.gfacet, cur_f);
      cur_f = f;
    }
    const V3 src = mk(__ldg(p.sources + 3 * s), __ldg(p.sources + 3 * s + 1), __ldg(p.sources + 3 * s + 2));
    const float v = __ldg(p.values + s);
    const V3 fpos = mk(__ldg(p.facet_pos + 3 * f), __ldg(p.facet_pos + 3 * f + 1), __ldg(p.facet_pos + 3 * f + 2));
    const uint32_t word = p.gmask ? __ldg(p.gmask + (size_t)s * p.F + f) : 0u;
    const int rowbase = (MODE == IACT_MODE_RESPONSE) ? s * p.P : 0;
    const int fbase = f * p.M;
    for (; cl < ce; ++cl) {
      const int m = (c0 + cl) * 32 + lane;
      const bool ok = m < p.M;
      const int si = fbase + (ok ? m : mlast);
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
      bool shadowed = false;
      if (word) shadowed = shadow_word(ob, word, tp, mk(-d.x, -d.y, -d.z));  // warp-uniform
      const float c = dot(d, nn);
      const V3 r = d - (2.f * c) * nn;
      const float ndotd = r.z;
      const bool parallel = fabsf(ndotd) < 1e-10f;
      const float inv_nd = rcp_a(parallel ? 1.f : ndotd);
      const float tpl = (sn.pos[2] - tp.z) * inv_nd;
      const bool hit_plane = !parallel && (tpl > 0.f);
      const float x = hit_plane ? (tp.x + tpl * r.x) - sn.pos[0] : kBig;
      const float y = hit_plane ? (tp.y + tpl * r.y) - sn.pos[1] : kBig;
      // ---- reverse of the deposit: d img[pix] / d val = 1
      int pix;
      if (HEX) {
        const float ex = x - hc.cx, ey = y - hc.cy;
        const bool in = ex * ex + ey * ey < sn.hex_lim2;
        pix = hc.pid;
        if (__any_sync(kFull, !in)) {
          float xg, yg, qi, ri;
          hex_axial(sn, x, y, xg, yg, qi, ri);
          const int pf = hex_lookup(sn, htab, qi, ri);
          float hcx, hcy;
          hex_centre(sn, qi, ri, hcx, hcy);
          const float hd = hex_norm(__fsub_rn(xg, hcx), __fsub_rn(yg, hcy), sn.inv_inr);
          const float ncx = sn.off_x + (sn.gc * hcx + sn.gs * hcy);
          const float ncy = sn.off_y + (sn.gc * hcy - sn.gs * hcx);
          hc.cx = in ? hc.cx : ncx;
          hc.cy = in ? hc.cy : ncy;
          hc.pid = in ? hc.pid : pf;
          pix = in ? pix : ((hd > sn.edge_threshold) ? -1 : pf);
        }
      } else {
        pix = bin_square(sn, x, y);
      }
      const bool alive = ok && !shadowed && (pix >= 0);
      const float gv0 = alive ? __ldg(p.grad_out + rowbase + pix) : 0.f;
      if (gv0 == 0.f) continue;
      // val = v (-c) iw ; r = d - 2 c n' (nothing flows back through the hit point)
      const float dLdc = -gv0 * v * iw;
      const V3 b = dLdc * d;    // dL/dn'
      const V3 gd = dLdc * nn;  // dL/dd
      V3 a, gs;
      if (SRC == IACT_SRC_POINT) {
        const V3 gw = inv_len * (gd - dot(d, gd) * d);  // d = w/|w|
        a = gw;
        gs = mk(-gw.x, -gw.y, -gw.z);
      } else {
        a = mk(0.f, 0.f, 0.f);
        gs = gd;
      }
      // facet buckets: H += a (tp - pos)^T + b n'^T ; dL/dpos = a
      const V3 pr = tp - fpos;
      acc.H[0] += a.x * pr.x + b.x * nn.x; acc.H[1] += a.x * pr.y + b.x * nn.y; acc.H[2] += a.x * pr.z + b.x * nn.z;
      acc.H[3] += a.y * pr.x + b.y * nn.x; acc.H[4] += a.y * pr.y + b.y * nn.y; acc.H[5] += a.y * pr.z + b.y * nn.z;
      acc.H[6] += a.z * pr.x + b.z * nn.x; acc.H[7] += a.z * pr.y + b.z * nn.y; acc.H[8] += a.z * pr.z + b.z * nn.z;
      acc.gp[0] += a.x; acc.gp[1] += a.y; acc.gp[2] += a.z;
      acc.gsrc[0] += gs.x; acc.gsrc[1] += gs.y; acc.gsrc[2] += gs.z;
      acc.gv += gv0 * -c * iw;
    }
    flush_src(acc, p.gsrc, s);  // the next pair has another source (or this warp ends)
    cl = 0;
    ++q;
    if (++sl == SBc) {
      sl = 0;
      ++fl;
    }
  }
  if (cur_f >= 0) flush_facet_hard(acc, p.gfacet, cur_f);
}

// Soft-pixel adjoint tile of the common case: a single-stage scene, point,
// parallel or extended sources, a sensor whose rotation is the identity,
// the hexagon table in shared memory, candidate words per (source, facet)
// pair from k_masks, and no roughness-scale or per-sample gradients. The
// arithmetic is adjoint_tile<SRC, true, MODE, false, true>'s: the reverse of
// the soft deposit (soft_square_bwd / soft_hex_bwd), of the sensor-plane hit
// and of the reflection; the sensor kind is compile-time, per-pair values
// (source, jitter basis, value, facet position, candidate word) are loaded
// once per pair, and a warp's tasks run facet by facet (source next, chunk
// fastest) as in adjoint_tile_hard.
template <int SRC, int MODE, bool HEX>
__device__ __forceinline__ void adjoint_tile_soft(const AdjK& p, const Obst& ob, const short* htab, int tile) {
  const SensorK& sn = p.sn;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nch = (p.M + 31) >> 5;
  Acc acc;
  acc_zero_facet(acc);
  acc_zero_src(acc);
  const int per_s = p.n_fchunk * p.n_cchunk;
  const int sblk = tile / per_s;
  const int fc = (tile - sblk * per_s) / p.n_cchunk;
  const int cc = tile - sblk * per_s - fc * p.n_cchunk;
  const int s0 = sblk * p.SB, f0 = fc * p.FC, c0 = cc * p.CC;
  const int SBc = min(p.SB, p.S - s0), FCc = min(p.FC, p.F - f0), CCc = min(p.CC, nch - c0);
  const int T = SBc * FCc * CCc;
  const int tb = (warp * T) / nw, te = ((warp + 1) * T) / nw;
  constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
  // tasks t = (facet fl, source sl, chunk cl), chunk fastest
  int q = tb / CCc;  // pair index fl * SBc + sl
  int fl = q / SBc, sl = q - fl * SBc;
  int cl = tb - q * CCc;
  int cur_f = -1;
  const int mlast = p.M - 1;
  for (int t = tb; t < te;) {
    const int s = s0 + sl, f = f0 + fl;
    const int ce = min(CCc, cl + (te - t));
    t += ce - cl;
    if (f != cur_f) {
      if (cur_f >= 0) flush_facet_hard(acc, p.gfacet, cur_f);
      cur_f = f;
    }
    const V3 src = mk(__ldg(p.sources + SS * s), __ldg(p.sources + SS * s + 1), __ldg(p.sources + SS * s + 2));
    const float sig = (SRC == IACT_SRC_EXTENDED) ? __ldg(p.sources + SS * s + 3) : 0.f;
    const float v = __ldg(p.values + s);
    const V3 fpos = mk(__ldg(p.facet_pos + 3 * f), __ldg(p.facet_pos + 3 * f + 1), __ldg(p.facet_pos + 3 * f + 2));
    const uint32_t word = p.gmask ? __ldg(p.gmask + (size_t)s * p.F + f) : 0u;
    const int rowbase = (MODE == IACT_MODE_RESPONSE) ? s * p.P : 0;
    const int fbase = f * p.M;
    JBasis jb;
    if (SRC == IACT_SRC_EXTENDED) jb = jitter_basis(src);
    for (; cl < ce; ++cl) {
      const int m = (c0 + cl) * 32 + lane;
      const bool ok = m < p.M;
      const int mc = ok ? m : mlast;
      const float4 P4 = __ldg(p.P4 + fbase + mc), N4 = __ldg(p.N4 + fbase + mc);
      const V3 tp = mk(P4.x, P4.y, P4.z), nn = mk(N4.x, N4.y, N4.z);
      const float iw = P4.w;
      // ---- forward re-trace
      V3 d, w;
      float inv_len = 0.f;
      if (SRC == IACT_SRC_POINT) {
        w = tp - src;
        inv_len = rsqrtf(dot(w, w));
        d = inv_len * w;
      } else if (SRC == IACT_SRC_EXTENDED) {  // jitter regenerated from its counter
        float z0, z1;
        ray_normals(p.seed, s, f, mc, z0, z1);
        d = jitter_dir(jb, sig, z0, z1);
      } else {
        d = src;
      }
      bool shadowed = false;
      if (word) shadowed = shadow_word(ob, word, tp, mk(-d.x, -d.y, -d.z));  // warp-uniform
      const float c = dot(d, nn);
      const V3 r = d - (2.f * c) * nn;
      const float val = v * -c * iw;
      const bool parallel = fabsf(r.z) < 1e-10f;
      const float inv_nd = rcp_a(parallel ? 1.f : r.z);
      const float tpl = (sn.pos[2] - tp.z) * inv_nd;
      const bool hit_plane = !parallel && (tpl > 0.f);
      const float x = hit_plane ? (tp.x + tpl * r.x) - sn.pos[0] : kBig;
      const float y = hit_plane ? (tp.y + tpl * r.y) - sn.pos[1] : kBig;
      // ---- reverse of the soft deposit
      float gval = 0.f, gx = 0.f, gy = 0.f;
      if (ok && !shadowed) {
        if (HEX) soft_hex_bwd(sn, htab, p.grad_out, rowbase, x, y, val, gval, gx, gy);
        else soft_square_bwd(sn, p.grad_out, rowbase, x, y, val, gval, gx, gy);
      }
      if ((gval == 0.f) & (gx == 0.f) & (gy == 0.f)) continue;
      // plane (intersections.py:23-35): p = o + t r, t = ns.(C - o) / ns.r, ns = z
      const V3 gpl = mk(gx, gy, 0.f);  // dL/dp
      const float dLdt = dot(gpl, r);
      V3 a = mk(gpl.x, gpl.y, -(dLdt * inv_nd));                   // dL/do through the plane
      const V3 gr = mk(tpl * gpl.x, tpl * gpl.y, -(dLdt * tpl * inv_nd));  // dL/dr through the plane
      // val = v (-c) iw ; r = d - 2 c n'
      const float dLdc = -gval * v * iw - 2.f * dot(gr, nn);
      const V3 b = (-2.f * c) * gr + dLdc * d;  // dL/dn'
      const V3 gd = gr + dLdc * nn;             // dL/dd
      V3 gs;
      if (SRC == IACT_SRC_POINT) {
        const V3 gw = inv_len * (gd - dot(d, gd) * d);  // d = w/|w|
        a = a + gw;
        gs = mk(-gw.x, -gw.y, -gw.z);
      } else {
        gs = gd;
      }
      // facet buckets: H += a (tp - pos)^T + b n'^T ; dL/dpos = a
      const V3 pr = tp - fpos;
      acc.H[0] += a.x * pr.x + b.x * nn.x; acc.H[1] += a.x * pr.y + b.x * nn.y; acc.H[2] += a.x * pr.z + b.x * nn.z;
      acc.H[3] += a.y * pr.x + b.y * nn.x; acc.H[4] += a.y * pr.y + b.y * nn.y; acc.H[5] += a.y * pr.z + b.y * nn.z;
      acc.H[6] += a.z * pr.x + b.z * nn.x; acc.H[7] += a.z * pr.y + b.z * nn.y; acc.H[8] += a.z * pr.z + b.z * nn.z;
      acc.gp[0] += a.x; acc.gp[1] += a.y; acc.gp[2] += a.z;
      acc.gsrc[0] += gs.x; acc.gsrc[1] += gs.y; acc.gsrc[2] += gs.z;
      acc.gv += gval * -c * iw;
    }
    flush_src(acc, p.gsrc, s);  // the next pair has another source (or this warp ends)
    cl = 0;
    ++q;
    if (++sl == SBc) {
      sl = 0;
      ++fl;
    }
  }
  if (cur_f >= 0) flush_facet_hard(acc, p.gfacet, cur_f);
}

// Per facet: dL/dR = H R, then dL/d(tip, tilt, rot) in degrees with// Per facet: dL/dR = H R, then dL/d(tip, tilt, rot) in degrees with
// R = Rz(rot) Ry(tilt) Rx(tip) (core/transforms.py:72-107); per source the
// FP64 sums to float.
// cs = (cos, sin) of tip, tilt and rot in radians
__device__ __forceinline__ void euler_grads_cs(const double* G, const double* cs, double* out) {
  // dL/d(tip, tilt, rot) per degree from dL/dR, R = Rz(rot) Ry(tilt) Rx(tip)
  const double k = 0.017453292519943295;
  const double ca = cs[0], sa = cs[1], cb = cs[2], sb = cs[3], cc = cs[4], sc = cs[5];
  const double Rx[9] = {1, 0, 0, 0, ca, -sa, 0, sa, ca}, dRx[9] = {0, 0, 0, 0, -sa, -ca, 0, ca, -sa};
  const double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb}, dRy[9] = {-sb, 0, cb, 0, 0, 0, -cb, 0, -sb};
  const double Rz[9] = {cc, -sc, 0, sc, cc, 0, 0, 0, 1}, dRz[9] = {-sc, -cc, 0, cc, -sc, 0, 0, 0, 0};
  auto mm = [](const double* A, const double* B, double* Cm) {
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) Cm[3 * r + q] = A[3 * r] * B[q] + A[3 * r + 1] * B[3 + q] + A[3 * r + 2] * B[6 + q];
  };
  double ZY[9], T1[9], D[9];
  mm(Rz, Ry, ZY);
  mm(ZY, dRx, D);
  out[0] = 0;
  for (int j = 0; j < 9; ++j) out[0] += G[j] * D[j];
  mm(Rz, dRy, T1);
  mm(T1, Rx, D);
  out[1] = 0;
  for (int j = 0; j < 9; ++j) out[1] += G[j] * D[j];
  mm(dRz, Ry, T1);
  mm(T1, Rx, D);
  out[2] = 0;
  for (int j = 0; j < 9; ++j) out[2] += G[j] * D[j];
  for (int j = 0; j < 3; ++j) out[j] *= k;
}
__device__ __forceinline__ void euler_cs(const float* deg, double* cs) {
  const double k = 0.017453292519943295;
  for (int j = 0; j < 3; ++j) sincos(deg[j] * k, &cs[2 * j + 1], &cs[2 * j]);
}
__device__ __forceinline__ void euler_grads(const double* G, const float* deg, double* out) {
  double cs[6];
  euler_cs(deg, cs);
  euler_grads_cs(G, cs, out);
}

__device__ __forceinline__ void adjoint_mirror_item(int i, const double* gmir, const iact_mirror_t* mirrors,
                                                    float* g_rot, float* g_pos, float* g_surf) {
  const double* h = gmir + (size_t)i * kMirGrad;
  double out[3];
  euler_grads(h, mirrors[i].rot, out);
  if (g_rot)
    for (int j = 0; j < 3; ++j) g_rot[3 * i + j] = (float)out[j];
  if (g_pos)
    for (int j = 0; j < 3; ++j) g_pos[3 * i + j] = (float)h[9 + j];
  if (g_surf)
    for (int j = 0; j < 2 + IACT_MAX_ASPH; ++j) g_surf[(2 + IACT_MAX_ASPH) * i + j] = (float)h[12 + j];
}

__device__ __forceinline__ void adjoint_finish_item(int i, const double* gfacet, const double* gsrc,
                                                    const float* facet_rot, int F, int S, float* g_rot, float* g_pos,
                                                    float* g_scale, float* g_src, float* g_val) {
  if (i < F) {
    const double* h = gfacet + (size_t)i * kFacetGrad;
    // dL/dR = H R with R the facet rotation
    double cs[6];
    euler_cs(facet_rot + 3 * i, cs);
    const double ca = cs[0], sa = cs[1], cb = cs[2], sb = cs[3], cc = cs[4], sc = cs[5];
    const double R[9] = {cc * cb, cc * sb * sa - sc * ca, cc * sb * ca + sc * sa,
                         sc * cb, sc * sb * sa + cc * ca, sc * sb * ca - cc * sa,
                         -sb, cb * sa, cb * ca};
    double G[9];
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) G[3 * r + q] = h[3 * r] * R[q] + h[3 * r + 1] * R[3 + q] + h[3 * r + 2] * R[6 + q];
    double out[3];
    euler_grads_cs(G, cs, out);
    if (g_rot)
      for (int j = 0; j < 3; ++j) g_rot[3 * i + j] = (float)out[j];
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

// host: launch parameters of one backward over a workspace laid out by
// workspace_for(..., IACT_MODE_BACKWARD) at `w`, and its tile / shared-memory
// plan for `block` threads (smem: tables, int16 hex table, stage-mirror
// partial sums, candidate masks); tiles shrink until there are `min_tiles`
AdjK adjoint_params(const iact_scene_t* sc, const iact_sensor_t* sn, const WsLayout& L, char* w,
                    const float* sources, const float* values, const float* grad_out, int S, bool with_scale,
                    const iact_opts_t* opts);
int plan_adjoint(AdjK& p, const iact_sensor_t* sn, int block, size_t& smem, long long min_tiles,
                 const iact_opts_t* opts = nullptr, int default_tpw = 48);

}  // namespace iact
