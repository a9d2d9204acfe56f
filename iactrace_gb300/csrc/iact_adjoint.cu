// Adjoint (reverse-mode) of the render path.
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
// Later mirror stages (core/render.py:44-115, any number) are recorded
// during the re-trace (the last kAdjRing of them; earlier ones are re-traced
// again when the reverse sweep reaches them) and reversed with the
// implicit-function derivative of their Newton root (stage_bwd). Shadow and hit masks are
// piecewise constant and carry no gradient, as in jax.grad. Gradients reach facet rotations (Euler degrees), facet
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

#include "iact_adjoint_impl.cuh"
#include "iact_device.cuh"
#include "iact_internal.h"

namespace iact {

template <int SRC, bool SOFT, int MODE, bool STAGES, bool AX = false, bool DEEP = false>
__global__ void __launch_bounds__(256, STAGES ? 2 : (SOFT ? 3 : 4)) k_adjoint(const AdjK p) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_tile;
  grid_dep_wait();  // the prep launch's tables, samples and zeroed buckets
  grid_dep_launch();
  const int tab_n = (p.n_table_floats + 3) & ~3;
  const int htab_n = p.hex_in_smem ? ((p.sn.table_q * p.sn.table_r + 7) & ~7) : 0;
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + tab_n);
  const int nthr = blockDim.x;
  for (int i = threadIdx.x; i < p.n_table_floats; i += nthr) tab[i] = p.tables[i];
  for (int i = threadIdx.x; i < htab_n; i += nthr)
    htab[i] = (short)(i < p.sn.table_q * p.sn.table_r ? p.hex_table[i] : -1);
  float* mgrad = reinterpret_cast<float*>(htab + htab_n);  // [n_mir, kMirGrad] CTA partial sums
  uint32_t* tmask = reinterpret_cast<uint32_t*>(mgrad + (STAGES ? p.n_mir * kMirGrad : 0));  // tile's candidate masks
  for (int i = threadIdx.x; i < (STAGES ? p.n_mir * kMirGrad : 0); i += nthr) mgrad[i] = 0.f;
  const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  const float* mir = tab + table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir).mir;
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(p.counter, 1);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= p.n_tiles) break;
    adjoint_tile<SRC, SOFT, MODE, STAGES, AX, DEEP>(p, ob, mir, htab, mgrad, tmask, tile);
  }
  if (STAGES) {
    __syncthreads();
    for (int i = threadIdx.x; i < p.n_mir * kMirGrad; i += nthr)
      if (mgrad[i] != 0.f) atomicAdd(p.gmir + i, (double)mgrad[i]);
  }
}

// Shared-memory layout (tables, hexagon table) and persistent tile loop of
// the specialised adjoints (k_adjoint_hard, k_adjoint_soft). Tiles end
// without a barrier, so the tile index is double-buffered.
template <bool HEX, typename Body>
__device__ __forceinline__ void adj_tile_loop(const AdjK& p, Body body) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_tile[2];
  const int tab_n = (p.n_table_floats + 3) & ~3;
  const int htab_n = HEX ? ((p.sn.table_q * p.sn.table_r + 7) & ~7) : 0;
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + tab_n);
  const int nthr = blockDim.x;
  grid_dep_wait();  // the prep and mask launches' results
  grid_dep_launch();
  for (int i = threadIdx.x; i < p.n_table_floats; i += nthr) tab[i] = p.tables[i];
  for (int i = threadIdx.x; i < htab_n; i += nthr)
    htab[i] = (short)(i < p.sn.table_q * p.sn.table_r ? p.hex_table[i] : -1);
  const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  __syncthreads();
  for (int it = 0;; ++it) {
    if (threadIdx.x == 0) s_tile[it & 1] = atomicAdd(p.counter, 1);
    __syncthreads();
    const int tile = s_tile[it & 1];
    if (tile >= p.n_tiles) break;
    body(ob, htab, tile);
  }
}

// k_adjoint for the common hard-pixel case (adjoint_tile_hard): the host
// picks it when the backward qualifies.
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, 4) k_adjoint_hard(const AdjK p) {
  adj_tile_loop<HEX>(p, [&](const Obst& ob, const short* htab, int tile) {
    adjoint_tile_hard<SRC, MODE, HEX>(p, ob, htab, tile);
  });
}

// k_adjoint for the common soft-pixel case (adjoint_tile_soft).
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, 3) k_adjoint_soft(const AdjK p) {
  adj_tile_loop<HEX>(p, [&](const Obst& ob, const short* htab, int tile) {
    adjoint_tile_soft<SRC, MODE, HEX>(p, ob, htab, tile);
  });
}

__global__ void k_adjoint_mirrors(const double* gmir, const iact_mirror_t* mirrors, int n_mir, float* g_rot,
                                  float* g_pos, float* g_surf) {
  grid_dep_wait();  // the adjoint's buckets
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_mir) adjoint_mirror_item(i, gmir, mirrors, g_rot, g_pos, g_surf);
}

__global__ void k_adjoint_finish(const double* gfacet, const double* gsrc, const float* facet_rot, int F, int S,
                                 float* g_rot, float* g_pos, float* g_scale, float* g_src, float* g_val) {
  grid_dep_wait();  // the adjoint's buckets
  grid_dep_launch();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  adjoint_finish_item(i, gfacet, gsrc, facet_rot, F, S, g_rot, g_pos, g_scale, g_src, g_val);
}

namespace {

template <int SRC, bool SOFT, int MODE, bool STAGES, bool DEEP = false>
int run_adjoint(const AdjK& p, int block, size_t smem, cudaStream_t st) {
  auto kern = k_adjoint<SRC, SOFT, MODE, STAGES, false, DEEP>;
  // hard pixels, single stage, axis-aligned sensor: a kernel whose plane hit
  // takes components instead of dot products with the sensor axes
  if constexpr (!SOFT && !STAGES && SRC != IACT_SRC_EXTENDED)
    if (p.sn.axes) kern = k_adjoint<SRC, SOFT, MODE, STAGES, true>;
  int per_sm = 0;
  const int rc = resident_ctas(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "adjoint kernel does not fit on an SM");
  const int grid = std::max(1, std::min(p.n_tiles, per_sm * device_info().sm_count));
  return check_cuda(launch_after(kern, dim3(grid), dim3(block), smem, st, p), "k_adjoint launch");
}

template <int SRC, bool SOFT, bool STAGES, bool DEEP = false>
int adj_mode(int mode, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  return mode == IACT_MODE_RESPONSE ? run_adjoint<SRC, SOFT, IACT_MODE_RESPONSE, STAGES, DEEP>(p, block, smem, st)
                                    : run_adjoint<SRC, SOFT, IACT_MODE_IMAGE, STAGES, DEEP>(p, block, smem, st);
}
// n_stages: later stages of the scene (0: primary only; above kAdjRing: the
// kernels that re-trace stages which left the record ring)
template <int SRC, bool SOFT>
int adj_stages(int n_stages, int mode, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  if (n_stages > kAdjRing) return adj_mode<SRC, SOFT, true, true>(mode, p, block, smem, st);
  return n_stages > 0 ? adj_mode<SRC, SOFT, true>(mode, p, block, smem, st)
                      : adj_mode<SRC, SOFT, false>(mode, p, block, smem, st);
}

// the common hard-pixel case (k_adjoint_hard)
int run_adjoint_hard(int src_type, int mode, bool hex, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  void (*kern)(const AdjK);
  if (src_type == IACT_SRC_POINT) {
    if (mode == IACT_MODE_RESPONSE)
      kern = hex ? k_adjoint_hard<IACT_SRC_POINT, IACT_MODE_RESPONSE, true> : k_adjoint_hard<IACT_SRC_POINT, IACT_MODE_RESPONSE, false>;
    else
      kern = hex ? k_adjoint_hard<IACT_SRC_POINT, IACT_MODE_IMAGE, true> : k_adjoint_hard<IACT_SRC_POINT, IACT_MODE_IMAGE, false>;
  } else {
    if (mode == IACT_MODE_RESPONSE)
      kern = hex ? k_adjoint_hard<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE, true>
                 : k_adjoint_hard<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE, false>;
    else
      kern = hex ? k_adjoint_hard<IACT_SRC_PARALLEL, IACT_MODE_IMAGE, true>
                 : k_adjoint_hard<IACT_SRC_PARALLEL, IACT_MODE_IMAGE, false>;
  }
  int per_sm = 0;
  const int rc = resident_ctas(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "adjoint kernel does not fit on an SM");
  const int grid = std::max(1, std::min(p.n_tiles, per_sm * device_info().sm_count));
  return check_cuda(launch_after(kern, dim3(grid), dim3(block), smem, st, p), "k_adjoint launch");
}

// the common soft-pixel case (k_adjoint_soft)
template <int SRC>
int run_adjoint_soft_src(int mode, bool hex, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  void (*kern)(const AdjK);
  if (mode == IACT_MODE_RESPONSE)
    kern = hex ? k_adjoint_soft<SRC, IACT_MODE_RESPONSE, true> : k_adjoint_soft<SRC, IACT_MODE_RESPONSE, false>;
  else
    kern = hex ? k_adjoint_soft<SRC, IACT_MODE_IMAGE, true> : k_adjoint_soft<SRC, IACT_MODE_IMAGE, false>;
  int per_sm = 0;
  const int rc = resident_ctas(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "adjoint kernel does not fit on an SM");
  const int grid = std::max(1, std::min(p.n_tiles, per_sm * device_info().sm_count));
  return check_cuda(launch_after(kern, dim3(grid), dim3(block), smem, st, p), "k_adjoint launch");
}
int run_adjoint_soft(int src_type, int mode, bool hex, const AdjK& p, int block, size_t smem, cudaStream_t st) {
  if (src_type == IACT_SRC_POINT) return run_adjoint_soft_src<IACT_SRC_POINT>(mode, hex, p, block, smem, st);
  if (src_type == IACT_SRC_EXTENDED) return run_adjoint_soft_src<IACT_SRC_EXTENDED>(mode, hex, p, block, smem, st);
  return run_adjoint_soft_src<IACT_SRC_PARALLEL>(mode, hex, p, block, smem, st);
}

// the render parameters k_masks reads, from the adjoint's
RenderK mask_params(const AdjK& a) {
  RenderK r;
  memset(&r, 0, sizeof(r));
  r.S = a.S; r.F = a.F; r.M = a.M; r.P = a.P;
  r.sources = a.sources; r.values = a.values;
  r.tables = a.tables; r.n_table_floats = a.n_table_floats;
  r.n_cyl = a.n_cyl; r.n_box = a.n_box; r.n_sph = a.n_sph; r.n_obox = a.n_obox; r.n_tri = a.n_tri;
  r.B4 = a.B4;
  r.n_words = a.n_words;
  return r;
}

}  // namespace

AdjK adjoint_params(const iact_scene_t* sc, const iact_sensor_t* sn, const WsLayout& L, char* w,
                    const float* sources, const float* values, const float* grad_out, int S, bool with_scale,
                    const iact_opts_t* opts) {
  AdjK p;
  memset(&p, 0, sizeof(p));
  const int F = sc->n_facets;
  p.F = F; p.M = sc->n_samples; p.S = S; p.P = sn->n_pixels;
  p.P4 = reinterpret_cast<const float4*>(w + L.p4);
  p.N4 = reinterpret_cast<const float4*>(w + L.n4);
  p.D4 = with_scale ? reinterpret_cast<const float4*>(w + L.d4) : nullptr;
  p.facet_pos = sc->facet_pos;
  p.sources = sources; p.values = values; p.grad_out = grad_out;
  p.tables = reinterpret_cast<const float*>(w + L.tables);
  p.n_table_floats = L.n_table_floats;
  p.n_cyl = sc->n_cyl; p.n_box = sc->n_box; p.n_sph = sc->n_sph; p.n_obox = sc->n_obox; p.n_tri = sc->n_tri;
  p.hex_table = sn->table;
  p.sn = make_sensor(sn);
  p.gfacet = reinterpret_cast<double*>(w + L.acc);
  p.gsrc = p.gfacet + (size_t)F * kFacetGrad;
  p.gmir = p.gsrc + (size_t)S * 4;
  p.n_mir = sc->n_mirrors;
  p.counter = reinterpret_cast<int*>(w + L.counter);
  p.B4 = L.n_b4 ? reinterpret_cast<const float4*>(w + L.b4) : nullptr;
  p.n_words = (L.n_b4 && !(opts && (opts->flags & IACT_FLAG_NO_CULL))) ? (n_primitives(sc) + 31) / 32 : 0;
  p.seed = opts ? opts->seed : 0u;
  return p;
}

int plan_adjoint(AdjK& p, const iact_sensor_t* sn, int block, size_t& smem, long long min_tiles,
                 const iact_opts_t* opts, int default_tpw) {
  const int nw = block / 32;
  const int nch = (p.M + 31) / 32;
  // opts: sources per tile and 32-ray tasks per warp per tile, as for the forward render
  p.SB = std::max(1, std::min(p.S, (opts && opts->sources_per_cta > 0) ? opts->sources_per_cta : nw));
  const int tpw = (opts && opts->tasks_per_warp > 0) ? opts->tasks_per_warp : default_tpw;
  int target = std::max(1, std::min(nw * tpw, p.n_words ? 4096 / p.n_words : 1 << 30));
  for (;;) {
    p.CC = std::max(1, std::min(nch, std::max(1, target / p.SB)));
    p.FC = std::max(1, std::min(p.F, std::max(1, target / (p.SB * p.CC))));
    p.n_fchunk = (p.F + p.FC - 1) / p.FC;
    p.n_cchunk = (nch + p.CC - 1) / p.CC;
    const long long tiles =
        (p.S > 0 && p.F > 0 && p.M > 0) ? (long long)((p.S + p.SB - 1) / p.SB) * p.n_fchunk * p.n_cchunk : 0;
    if (tiles > 0x7fffffffLL) return set_error(IACT_E_UNSUPPORTED, "too many work tiles");
    p.n_tiles = (int)tiles;
    // small launches: halve the tile until the GPU holds enough of them to balance
    if (tiles == 0 || tiles >= min_tiles || target <= nw) break;
    target = std::max(nw, target / 2);
  }
  const size_t tab_bytes = sizeof(float) * (size_t)((p.n_table_floats + 3) & ~3);
  const bool hex = (sn->type == IACT_SENSOR_HEX || sn->type == IACT_SENSOR_SOFT_HEX);
  const size_t htab = hex ? (size_t)sn->table_q * sn->table_r : 0;
  const size_t htab_bytes = sizeof(short) * ((htab + 7) & ~(size_t)7);
  p.hex_in_smem = (hex && sn->n_pixels < 32768 && tab_bytes + htab_bytes <= 96 * 1024) ? 1 : 0;
  smem = tab_bytes + (p.hex_in_smem ? htab_bytes : 0) + sizeof(float) * (size_t)p.n_mir * kMirGrad +
         sizeof(uint32_t) * (size_t)p.n_words * p.SB * p.FC;
  return IACT_OK;
}

int launch_backward(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                    const float* values, int S, int mode, const float* grad_out, float* g_rot, float* g_pos,
                    float* g_scale, float* g_src, float* g_val, float* g_mrot, float* g_mpos, float* g_msurf,
                    float* g_samples, void* ws, size_t ws_bytes, const iact_opts_t* opts, cudaStream_t st) {
  (void)ws_bytes;
  const int F = sc->n_facets;
  const WsLayout L = workspace_for(sc, sn, S, IACT_MODE_BACKWARD);
  char* w = static_cast<char*>(ws);
  double* gfacet = reinterpret_cast<double*>(w + L.acc);
  double* gsrc = gfacet + (size_t)F * kFacetGrad;
  double* gmir = gsrc + (size_t)S * 4;
  const int n_mir = sc->n_mirrors;
  const size_t nacc = (size_t)F * kFacetGrad + (size_t)S * 4 + (size_t)n_mir * kMirGrad;
  const bool work = S > 0 && F > 0 && sc->n_samples > 0;
  int rc = IACT_OK;
  if (!work) {  // the finish kernels still read the (empty) buckets
    rc = check_cuda(cudaMemsetAsync(gfacet, 0, nacc * sizeof(double), st), "zero gradient buckets");
    if (rc) return rc;
  }
  const size_t nsamp = (size_t)F * std::max(sc->n_samples, 0) * 7;
  if (g_samples && nsamp) {
    rc = check_cuda(cudaMemsetAsync(g_samples, 0, nsamp * sizeof(float), st), "zero sample gradients");
    if (rc) return rc;
  }
  if (work) {
    // the prep launch also clears the gradient buckets and the tile counter
    rc = launch_prep(sc, L, w, st, g_scale != nullptr, gfacet, nacc * sizeof(double),
                     reinterpret_cast<int*>(w + L.counter));
    if (rc) return rc;
    AdjK p = adjoint_params(sc, sn, L, w, sources, values, grad_out, S, g_scale != nullptr, opts);
    p.gsamp = g_samples;
    p.want_mgrad = (g_mrot || g_mpos || g_msurf) ? 1 : 0;
    const int block = (opts && opts->block_threads > 0) ? opts->block_threads : 256;
    size_t smem = 0;
    // larger tiles for response adjoints (4096 sources: 192 tasks per warp
    // 4.18 ms, 48: 4.34 ms)
    rc = plan_adjoint(p, sn, block, smem, 8LL * std::max(device_info().sm_count, 1), opts,
                      mode == IACT_MODE_RESPONSE ? 192 : 48);
    if (rc) return rc;
    const bool soft = sn->type == IACT_SENSOR_SOFT_SQUARE || sn->type == IACT_SENSOR_SOFT_HEX;
    void* const* ev = opts ? opts->kernel_events : nullptr;
    if (ev && ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
    const int stages = n_mir > 0 ? std::max(sc->n_stages, 1) : 0;
    // the common hard-pixel case: k_adjoint_hard with the candidate word of
    // every (source, facet) pair from k_masks (inside the kernel events)
    // (soft pixels: k_adjoint_soft, also for extended sources)
    const bool hex_kind = sn->type == IACT_SENSOR_HEX || sn->type == IACT_SENSOR_SOFT_HEX;
    const bool hard = n_mir == 0 && (soft || src_type == IACT_SRC_POINT || src_type == IACT_SRC_PARALLEL) &&
                      p.sn.axes && !g_scale && !g_samples && (!hex_kind || p.hex_in_smem) &&
                      ((p.n_words == 1 && L.n_masks > 0) || n_primitives(sc) == 0);
    if (hard) {
      if (p.n_words) {
        p.gmask = reinterpret_cast<const uint32_t*>(w + L.masks);
        rc = launch_masks(src_type, mask_params(p), reinterpret_cast<uint32_t*>(w + L.masks), st);
        if (rc) return rc;
      }
      const size_t hsmem = sizeof(float) * (size_t)((p.n_table_floats + 3) & ~3) +
                           (hex_kind ? sizeof(short) * (((size_t)sn->table_q * sn->table_r + 7) & ~(size_t)7) : 0);
      if (soft) rc = run_adjoint_soft(src_type, mode, hex_kind, p, block, hsmem, st);
      else rc = run_adjoint_hard(src_type, mode, hex_kind, p, block, hsmem, st);
    } else if (src_type == IACT_SRC_POINT)
      rc = soft ? adj_stages<IACT_SRC_POINT, true>(stages, mode, p, block, smem, st)
                : adj_stages<IACT_SRC_POINT, false>(stages, mode, p, block, smem, st);
    else if (src_type == IACT_SRC_EXTENDED)
      rc = soft ? adj_stages<IACT_SRC_EXTENDED, true>(stages, mode, p, block, smem, st)
                : adj_stages<IACT_SRC_EXTENDED, false>(stages, mode, p, block, smem, st);
    else
      rc = soft ? adj_stages<IACT_SRC_PARALLEL, true>(stages, mode, p, block, smem, st)
                : adj_stages<IACT_SRC_PARALLEL, false>(stages, mode, p, block, smem, st);
    if (rc) return rc;
    if (ev && ev[1]) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), st);
  }
  const int n = std::max(F, S);
  if (n > 0) {
    // FP64 trigonometry per facet (GB300: 2 FP64 FMAs per clock per SM):
    // one warp per block spreads the facets over the SMs
    rc = check_cuda(launch_after(k_adjoint_finish, dim3((n + 31) / 32), dim3(32), 0, st, gfacet, gsrc,
                                 sc->facet_rot, F, S, g_rot, g_pos, g_scale, g_src, g_val),
                    "k_adjoint_finish launch");
    if (rc) return rc;
  }
  if (n_mir > 0 && (g_mrot || g_mpos || g_msurf)) {
    rc = check_cuda(launch_after(k_adjoint_mirrors, dim3((n_mir + 63) / 64), dim3(64), 0, st, gmir, sc->mirrors,
                                 n_mir, g_mrot, g_mpos, g_msurf),
                    "k_adjoint_mirrors launch");
  }
  return rc;
}

}  // namespace iact
