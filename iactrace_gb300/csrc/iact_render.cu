// Forward render kernels of the GB300 render path.
//
//   k_prep    : telescope/mirrors.py:64-79 transform_to_world for every
//               (facet, sample) once per call, into float4 world samples,
//               plus the per-launch constant tables (obstruction records,
//               stage-mirror records) the render kernel stages in shared
//               memory.
//   k_render  : core/render.py:118-171 for every ray (source, facet, sample):
//               one lane owns one ray through the fused chain (direction,
//               shadow, reflect, later stages, sensor plane, pixel bin).
//               Persistent CTAs pull (source block, facet chunk, sample
//               chunk) tiles from an atomic queue. Pixel hits are run-length
//               merged per lane in registers, then added into shared-memory
//               histogram rows (one row for an image, one row per source of
//               the block for a response matrix) that are flushed to global
//               memory with one atomic per non-zero bin.
//   k_debug   : core/render.py:223-268 render_debug, one thread per ray.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>

#include "iact_device.cuh"
#include "iact_internal.h"
#include "iact_render_impl.cuh"

namespace iact {

__global__ void __launch_bounds__(256) k_prep(const PrepK p) {
  grid_dep_launch();
  if (blockIdx.x == 0) prep_tables(p);
  if (p.counter && blockIdx.x == 0 && threadIdx.x < 16) p.counter[threadIdx.x] = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_zero;
       i += (long long)gridDim.x * blockDim.x)
    p.zero[i] = make_uint4(0u, 0u, 0u, 0u);
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  prep_units(p, w, ((long long)gridDim.x * blockDim.x) >> 5);
}

template <int SRC, bool SOFT, int MODE, bool STAGES>
__global__ void __launch_bounds__(256, STAGES ? 3 : IACT_RENDER_MIN_CTAS) k_render(const RenderK p) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_tile;
  grid_dep_wait();  // the prep launch's tables, samples and zeroed accumulator
  grid_dep_launch();
  const int tab_n = (p.n_table_floats + 3) & ~3;
  const int htab_n = p.hex_in_smem ? ((p.sn.table_q * p.sn.table_r + 7) & ~7) : 0;  // int16 entries
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + tab_n);
  float* sh_hist = smem + tab_n + htab_n / 2;
  const int hist_n = p.rows_in_smem * p.P;
  uint32_t* tmask = reinterpret_cast<uint32_t*>(sh_hist + hist_n);  // candidate masks of a tile's tasks
  const int nthr = blockDim.x;

  for (int i = threadIdx.x; i < p.n_table_floats; i += nthr) tab[i] = p.tables[i];
  for (int i = threadIdx.x; i < htab_n; i += nthr)
    htab[i] = (short)(i < p.sn.table_q * p.sn.table_r ? p.hex_table[i] : -1);
  for (int i = threadIdx.x; i < hist_n; i += nthr) sh_hist[i] = 0.f;

  const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  const float* mir = tab + table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir).mir;
  Sink sink;
  sink.sh = p.rows_in_smem ? sh_hist : nullptr;
  sink.g = p.acc;

  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(p.counter, 1);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= p.n_tiles) break;
    // single-stage scenes with an axis-aligned sensor (the common case) take
    // the plane hit without the frame's dot products; p.sn.axes is uniform.
    // Not for extended sources, whose kernels would spill with two tile bodies.
    if (!STAGES && SRC != IACT_SRC_EXTENDED && p.sn.axes) render_tile<SRC, SOFT, MODE, STAGES, true>(p, ob, mir, htab, sh_hist, sink, tile, tmask);
    else render_tile<SRC, SOFT, MODE, STAGES>(p, ob, mir, htab, sh_hist, sink, tile, tmask);
  }
}

// Candidate word of every (source, facet) pair of a render (scenes of 1..32
// primitives) for k_render_hard, after the prep launch wrote the facet
// bounds and the tables.
template <int SRC>
__global__ void __launch_bounds__(256) k_masks(const RenderK p, uint32_t* out) {
  extern __shared__ __align__(16) float smem[];
  grid_dep_wait();  // the prep launch's facet bounds and tables
  grid_dep_launch();
  for (int i = threadIdx.x; i < p.n_table_floats; i += blockDim.x) smem[i] = p.tables[i];
  __syncthreads();
  const Obst ob = make_obst(smem, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  pair_masks<SRC>(p, ob, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, out);
}

// Shared-memory layout and persistent tile loop of the specialised kernels
// (k_render_hard, k_render_soft): tables, hexagon table, FP32 rows. A
// response tile flushes its rows itself; an image's one row is flushed
// every p.flush_tiles tiles and when the CTA runs out of tiles. The tile
// index is double-buffered: an image tile ends without a barrier, so thread
// 0 may fetch the next index while a slow warp still reads this one.
template <int MODE, bool HEX, typename Body>
__device__ __forceinline__ void rows_tile_loop(const RenderK& p, Body body) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_tile[2];
  const int tab_n = (p.n_table_floats + 3) & ~3;
  const int htab_n = HEX ? ((p.sn.table_q * p.sn.table_r + 7) & ~7) : 0;  // int16 entries
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + tab_n);
  float* sh_hist = smem + tab_n + htab_n / 2;
  const int hist_n = p.rows_in_smem * p.P;
  const int nthr = blockDim.x;
  grid_dep_wait();  // the prep and mask launches' results
  grid_dep_launch();

  for (int i = threadIdx.x; i < p.n_table_floats; i += nthr) tab[i] = p.tables[i];
  for (int i = threadIdx.x; i < htab_n; i += nthr)
    htab[i] = (short)(i < p.sn.table_q * p.sn.table_r ? p.hex_table[i] : -1);
  for (int i = threadIdx.x; i < hist_n; i += nthr) sh_hist[i] = 0.f;
  const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  __syncthreads();
  for (int it = 0;; ++it) {  // it = tiles this CTA has rendered
    if (threadIdx.x == 0) s_tile[it & 1] = atomicAdd(p.counter, 1);
    __syncthreads();
    const int tile = s_tile[it & 1];
    if (MODE == IACT_MODE_IMAGE && it > 0 && (tile >= p.n_tiles || it % p.flush_tiles == 0)) {
      flush_rows(p, sh_hist, 0, 1);
      __syncthreads();
    }
    if (tile >= p.n_tiles) break;
    body(ob, htab, sh_hist, tile);
  }
}

// k_render for the common hard-pixel case (render_tile_hard): the host picks
// it when the launch qualifies (single stage, point or parallel sources,
// axis-aligned sensor, rows and hexagon table in shared memory, candidate
// words per pair from k_masks).
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, IACT_RENDER_MIN_CTAS) k_render_hard(const RenderK p) {
  rows_tile_loop<MODE, HEX>(p, [&](const Obst& ob, const short* htab, float* rows, int tile) {
    render_tile_hard<SRC, MODE, HEX>(p, ob, htab, rows, tile);
  });
}

// k_render for the common soft-pixel case (render_tile_soft): as
// k_render_hard, also for extended sources.
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, IACT_RENDER_MIN_CTAS) k_render_soft(const RenderK p) {
  rows_tile_loop<MODE, HEX>(p, [&](const Obst& ob, const short* htab, float* rows, int tile) {
    render_tile_soft<SRC, MODE, HEX>(p, ob, htab, rows, tile);
  });
}

// k_render_soft for image renders of at least 32 sources, one source per
// lane (render_tile_soft_spread).
template <int SRC, bool HEX>
__global__ void __launch_bounds__(256, IACT_RENDER_MIN_CTAS) k_render_soft_spread(const RenderK p) {
  rows_tile_loop<IACT_MODE_IMAGE, HEX>(p, [&](const Obst& ob, const short* htab, float* rows, int tile) {
    render_tile_soft_spread<SRC, HEX>(p, ob, htab, rows, tile);
  });
}

// FP64 accumulator -> FP32 output
__global__ void __launch_bounds__(256) k_finish(const double* __restrict__ acc, float* __restrict__ out, size_t n) {
  grid_dep_wait();  // the render's accumulator
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)acc[i];
}

template <int SRC, bool STAGES>
__global__ void __launch_bounds__(256) k_debug(const RenderK p, float* pts, float* vals, int32_t* pix,
                                               int32_t* hit_mirror) {
  extern __shared__ __align__(16) float smem[];
  const int tab_n = (p.n_table_floats + 3) & ~3;
  for (int i = threadIdx.x; i < p.n_table_floats; i += blockDim.x) smem[i] = p.tables[i];
  (void)tab_n;
  __syncthreads();
  const TableOffsets to = table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir);
  Obst ob;
  ob.cyl = smem + to.cyl; ob.box = smem + to.box; ob.sph = smem + to.sph;
  ob.obox = smem + to.obox; ob.tri = smem + to.tri;
  ob.n_cyl = p.n_cyl; ob.n_box = p.n_box; ob.n_sph = p.n_sph; ob.n_obox = p.n_obox; ob.n_tri = p.n_tri;
  const float* mir = smem + to.mir;
  const long long n = (long long)p.F * p.S * p.M;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(i % p.M);
    const long long fs = i / p.M;
    const int s = (int)(fs % p.S), f = (int)(fs / p.S);
    const size_t si = (size_t)f * p.M + m;
    float x, y, val;
    int hm;
    constexpr int SS = (SRC == IACT_SRC_EXTENDED) ? 4 : 3;
    float z0 = 0.f, z1 = 0.f;
    if (SRC == IACT_SRC_EXTENDED) ray_normals(p.seed, s, f, m, z0, z1);
    const V3 src = mk(p.sources[SS * s], p.sources[SS * s + 1], p.sources[SS * s + 2]);
    const JBasis jb = jitter_basis(src);
    trace_ray<SRC, STAGES>(p, ob, mir, p.P4[si], p.N4[si], src, jb,
                           SRC == IACT_SRC_EXTENDED ? p.sources[SS * s + 3] : 0.f, z0, z1, p.values[s], x, y, val, hm,
                           nullptr, 0);
    pts[2 * i] = x;
    pts[2 * i + 1] = y;
    vals[i] = val;
    if (pix) {
      int q;
      if (p.sn.type == IACT_SENSOR_SQUARE || p.sn.type == IACT_SENSOR_SOFT_SQUARE) q = bin_square(p.sn, x, y);
      else q = bin_hex(p.sn, p.hex_table, x, y);
      pix[i] = q;
    }
    if (hit_mirror) hit_mirror[i] = hm;
  }
}

// ------------------------------------------------------------------ host side

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

DevInfo device_info() {
  static std::mutex mu;
  static DevInfo cache[64];
  static bool have[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(mu);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!have[dev]) {
    cudaDeviceGetAttribute(&cache[dev].sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&cache[dev].smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    have[dev] = true;
  }
  return cache[dev];
}

void host_euler(const float* deg, float* R) {
  const double k = M_PI / 180.0;
  double cx = cos(deg[0] * k), sx = sin(deg[0] * k);
  double cy = cos(deg[1] * k), sy = sin(deg[1] * k);
  double cz = cos(deg[2] * k), sz = sin(deg[2] * k);
  double a00 = cz * cy, a01 = -sz, a02 = cz * sy, a10 = sz * cy, a11 = cz, a12 = sz * sy, a20 = -sy, a21 = 0,
         a22 = cy;
  double r[9] = {a00, a01 * cx + a02 * sx, a02 * cx - a01 * sx, a10, a11 * cx + a12 * sx, a12 * cx - a11 * sx,
                 a20, a21 * cx + a22 * sx, a22 * cx - a21 * sx};
  for (int i = 0; i < 9; ++i) R[i] = (float)r[i];
}

SensorK make_sensor(const iact_sensor_t* s) {
  SensorK k;
  memset(&k, 0, sizeof(k));
  k.type = s->type;
  k.n_pixels = s->n_pixels;
  k.width = s->width;
  k.height = s->height;
  host_euler(s->rot, k.R);
  for (int i = 0; i < 3; ++i) k.pos[i] = s->pos[i];
  k.x0 = s->x0; k.y0 = s->y0; k.dx = s->dx; k.dy = s->dy; k.edge_width = s->edge_width;
  k.hex_size = s->hex_size; k.inradius = s->inradius; k.gc = s->grid_cos; k.gs = s->grid_sin;
  k.off_x = s->off_x; k.off_y = s->off_y; k.hex_sx = s->hex_sx; k.hex_sy = s->hex_sy;
  k.edge_threshold = s->edge_threshold;
  k.q_min = s->q_min; k.r_min = s->r_min; k.table_q = s->table_q; k.table_r = s->table_r;
  k.sigma = s->sigma;
  k.kernel_size = s->kernel_size;
  k.inv_dx = s->dx > 0.f ? (float)(1.0 / (double)s->dx) : 0.f;
  k.inv_dy = s->dy > 0.f ? (float)(1.0 / (double)s->dy) : 0.f;
  if (s->hex_size > 0.f) {
    const double sz = s->hex_size;
    k.hq_x = (float)(0.5773502691896257 / sz);
    k.hq_y = (float)(1.0 / (3.0 * sz));
    k.hr_y = (float)(2.0 / (3.0 * sz));
  }
  k.inv_inr = s->inradius > 0.f ? (float)(1.0 / (double)s->inradius) : 0.f;
  // cached-cell radius: inside the cell's inscribed circle and the edge
  // threshold, less a rounding margin (-1: the cache never hits)
  const double lim = (double)s->inradius * std::min((double)s->edge_threshold, 1.0) - 1e-5;
  k.hex_lim2 = lim > 0.0 ? (float)(lim * lim) : -1.f;
  k.axes = (k.R[0] == 1.f && k.R[4] == 1.f && k.R[8] == 1.f && k.R[1] == 0.f && k.R[2] == 0.f && k.R[3] == 0.f &&
            k.R[5] == 0.f && k.R[6] == 0.f && k.R[7] == 0.f) ? 1 : 0;
  return k;
}

int n_primitives(const iact_scene_t* sc) { return sc->n_cyl + sc->n_box + sc->n_sph + sc->n_obox + sc->n_tri; }

PrepK prep_params(const iact_scene_t* sc, const WsLayout& L, char* ws, bool with_delta) {
  PrepK p;
  memset(&p, 0, sizeof(p));
  p.F = sc->n_facets; p.M = sc->n_samples;
  p.facet_pos = sc->facet_pos; p.facet_rot = sc->facet_rot; p.facet_scale = sc->facet_scale;
  p.points = sc->points; p.normals = sc->normals; p.delta = sc->delta; p.weights = sc->weights;
  p.P4 = reinterpret_cast<float4*>(ws + L.p4);
  p.N4 = reinterpret_cast<float4*>(ws + L.n4);
  p.D4 = with_delta ? reinterpret_cast<float4*>(ws + L.d4) : nullptr;
  p.B4 = L.n_b4 ? reinterpret_cast<float4*>(ws + L.b4) : nullptr;
  p.tables = reinterpret_cast<float*>(ws + L.tables);
  p.cyl = sc->cyl; p.box = sc->box; p.sph = sc->sph; p.obox = sc->obox; p.tri = sc->tri;
  p.mirrors = sc->mirrors;
  p.n_cyl = sc->n_cyl; p.n_box = sc->n_box; p.n_sph = sc->n_sph; p.n_obox = sc->n_obox; p.n_tri = sc->n_tri;
  p.n_mir = sc->n_mirrors;
  return p;
}

int launch_prep(const iact_scene_t* sc, const WsLayout& L, char* ws, cudaStream_t st, bool with_delta, void* zero,
                size_t zero_bytes, int* counter) {
  PrepK p = prep_params(sc, L, ws, with_delta);
  p.zero = static_cast<uint4*>(zero);
  p.n_zero = zero ? (long long)((zero_bytes + 15) / 16) : 0;
  p.counter = counter;
  // one warp per (facet, 32-sample chunk), plus one per facet bound with culling
  const long long units = (long long)p.F * ((p.M + 31) / 32) + (p.B4 ? p.F : 0);
  const long long zb = (p.n_zero + 256LL * 8 - 1) / (256LL * 8);  // about 8 words per thread
  const int blocks = (int)std::min<long long>(std::max<long long>({1LL, (units + 7) / 8, zb}), 65535);
  k_prep<<<blocks, 256, 0, st>>>(p);
  return launched("k_prep launch");
}

RenderK base_params(const iact_scene_t* sc, const iact_sensor_t* sn, const WsLayout& L, char* ws,
                    const float* sources, const float* values, int S) {
  RenderK p;
  memset(&p, 0, sizeof(p));
  p.F = sc->n_facets; p.M = sc->n_samples; p.S = S; p.P = sn->n_pixels;
  p.P4 = reinterpret_cast<const float4*>(ws + L.p4);
  p.N4 = reinterpret_cast<const float4*>(ws + L.n4);
  p.sources = sources; p.values = values;
  p.tables = reinterpret_cast<const float*>(ws + L.tables);
  p.n_table_floats = L.n_table_floats;
  p.n_cyl = sc->n_cyl; p.n_box = sc->n_box; p.n_sph = sc->n_sph; p.n_obox = sc->n_obox; p.n_tri = sc->n_tri;
  p.n_mir = sc->n_mirrors;
  p.hex_table = sn->table;
  p.sn = make_sensor(sn);
  p.counter = reinterpret_cast<int*>(ws + L.counter);
  p.B4 = L.n_b4 ? reinterpret_cast<const float4*>(ws + L.b4) : nullptr;
  p.n_words = L.n_b4 ? (n_primitives(sc) + 31) / 32 : 0;
  return p;
}

int resident_ctas(const void* kern, int block, size_t smem, int* per_sm) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> smem_set;              // per (device, kernel)
  static std::map<std::tuple<int, const void*, int, size_t>, int> occ_cache;  // per launch shape
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(mu);
  const auto okey = std::make_tuple(dev, kern, block, smem);
  auto it = occ_cache.find(okey);
  if (it != occ_cache.end()) {
    *per_sm = it->second;
    return IACT_OK;
  }
  size_t& have = smem_set[std::make_pair(dev, kern)];
  if (smem > 48 * 1024 && smem > have) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(dynamic shared memory)");
    have = smem;
  }
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, block, smem);
  if (e != cudaSuccess) return check_cuda(e, "occupancy query");
  occ_cache[okey] = *per_sm;
  return IACT_OK;
}

// candidate words of all (source, facet) pairs (k_masks), tables staged in
// shared memory
int launch_masks(int src_type, const RenderK& p, uint32_t* out, cudaStream_t st) {
  const long long n = (long long)p.S * p.F;
  if (n <= 0) return IACT_OK;
  const size_t smem = sizeof(float) * (size_t)std::max(p.n_table_floats, 1);
  void (*kern)(const RenderK, uint32_t*) =
      src_type == IACT_SRC_POINT      ? k_masks<IACT_SRC_POINT>
      : src_type == IACT_SRC_EXTENDED ? k_masks<IACT_SRC_EXTENDED>
                                      : k_masks<IACT_SRC_PARALLEL>;
  int per_sm = 0;
  int rc = resident_ctas(reinterpret_cast<const void*>(kern), 256, smem, &per_sm);
  if (rc) return rc;
  const int grid = (int)std::min<long long>((n + 255) / 256, 65535);
  return check_cuda(launch_after(kern, dim3(grid), dim3(256), smem, st, p, out), "k_masks launch");
}

// one persistent launch of a render kernel: as many CTAs as are resident
int run_persistent(void (*kern)(const RenderK), RenderK p, int block, size_t smem, cudaStream_t st,
                   void* const* ev) {
  int per_sm = 0;
  int rc = resident_ctas(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "render kernel does not fit on an SM with this configuration");
  DevInfo di = device_info();
  int grid = std::min(p.n_tiles, per_sm * di.sm_count);
  grid = std::max(grid, 1);
  if (ev && ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
  rc = check_cuda(launch_after(kern, dim3(grid), dim3(block), smem, st, p), "k_render launch");
  if (ev && ev[1]) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), st);
  return rc;
}

template <int SRC, bool SOFT, int MODE, bool STAGES>
int run_render(RenderK p, int block, size_t smem, cudaStream_t st, void* const* ev) {
  return run_persistent(k_render<SRC, SOFT, MODE, STAGES>, p, block, smem, st, ev);
}

// the common hard-pixel case (k_render_hard)
int run_render_hard(int src_type, int mode, bool hex, RenderK p, int block, size_t smem, cudaStream_t st,
                    void* const* ev) {
  void (*kern)(const RenderK);
  if (src_type == IACT_SRC_POINT) {
    if (mode == IACT_MODE_RESPONSE)
      kern = hex ? k_render_hard<IACT_SRC_POINT, IACT_MODE_RESPONSE, true> : k_render_hard<IACT_SRC_POINT, IACT_MODE_RESPONSE, false>;
    else
      kern = hex ? k_render_hard<IACT_SRC_POINT, IACT_MODE_IMAGE, true> : k_render_hard<IACT_SRC_POINT, IACT_MODE_IMAGE, false>;
  } else {
    if (mode == IACT_MODE_RESPONSE)
      kern = hex ? k_render_hard<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE, true>
                 : k_render_hard<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE, false>;
    else
      kern = hex ? k_render_hard<IACT_SRC_PARALLEL, IACT_MODE_IMAGE, true> : k_render_hard<IACT_SRC_PARALLEL, IACT_MODE_IMAGE, false>;
  }
  return run_persistent(kern, p, block, smem, st, ev);
}

// the common soft-pixel case (k_render_soft)
template <int SRC>
int run_render_soft_src(int mode, bool hex, RenderK p, int block, size_t smem, cudaStream_t st, void* const* ev) {
  void (*kern)(const RenderK);
  if (mode == IACT_MODE_RESPONSE)
    kern = hex ? k_render_soft<SRC, IACT_MODE_RESPONSE, true> : k_render_soft<SRC, IACT_MODE_RESPONSE, false>;
  else
    kern = hex ? k_render_soft<SRC, IACT_MODE_IMAGE, true> : k_render_soft<SRC, IACT_MODE_IMAGE, false>;
  return run_persistent(kern, p, block, smem, st, ev);
}
int run_render_soft(int src_type, int mode, bool hex, RenderK p, int block, size_t smem, cudaStream_t st,
                    void* const* ev) {
  if (src_type == IACT_SRC_POINT) return run_render_soft_src<IACT_SRC_POINT>(mode, hex, p, block, smem, st, ev);
  if (src_type == IACT_SRC_EXTENDED) return run_render_soft_src<IACT_SRC_EXTENDED>(mode, hex, p, block, smem, st, ev);
  return run_render_soft_src<IACT_SRC_PARALLEL>(mode, hex, p, block, smem, st, ev);
}
// image renders of at least 32 sources (k_render_soft_spread)
int run_render_soft_spread(int src_type, bool hex, RenderK p, int block, size_t smem, cudaStream_t st,
                           void* const* ev) {
  void (*kern)(const RenderK);
  if (src_type == IACT_SRC_POINT)
    kern = hex ? k_render_soft_spread<IACT_SRC_POINT, true> : k_render_soft_spread<IACT_SRC_POINT, false>;
  else if (src_type == IACT_SRC_EXTENDED)
    kern = hex ? k_render_soft_spread<IACT_SRC_EXTENDED, true> : k_render_soft_spread<IACT_SRC_EXTENDED, false>;
  else
    kern = hex ? k_render_soft_spread<IACT_SRC_PARALLEL, true> : k_render_soft_spread<IACT_SRC_PARALLEL, false>;
  return run_persistent(kern, p, block, smem, st, ev);
}

template <int SRC, bool SOFT, int MODE>
int dispatch_stages(bool stages, RenderK p, int block, size_t smem, cudaStream_t st, void* const* ev) {
  return stages ? run_render<SRC, SOFT, MODE, true>(p, block, smem, st, ev)
                : run_render<SRC, SOFT, MODE, false>(p, block, smem, st, ev);
}
template <int SRC, bool SOFT>
int dispatch_mode(int mode, bool stages, RenderK p, int block, size_t smem, cudaStream_t st, void* const* ev) {
  return mode == IACT_MODE_RESPONSE ? dispatch_stages<SRC, SOFT, IACT_MODE_RESPONSE>(stages, p, block, smem, st, ev)
                                    : dispatch_stages<SRC, SOFT, IACT_MODE_IMAGE>(stages, p, block, smem, st, ev);
}
template <int SRC>
int dispatch_soft(bool soft, int mode, bool stages, RenderK p, int block, size_t smem, cudaStream_t st,
                  void* const* ev) {
  return soft ? dispatch_mode<SRC, true>(mode, stages, p, block, smem, st, ev)
              : dispatch_mode<SRC, false>(mode, stages, p, block, smem, st, ev);
}

size_t pair_mask_words(const iact_scene_t* sc, int S) {
  const int np = n_primitives(sc);
  const size_t n = (size_t)std::max(S, 0) * (size_t)std::max(sc->n_facets, 0);
  // at most 2^26 words (256 MiB): larger renders keep per-tile masks (k_render)
  return (np > 0 && np <= 32 && n <= ((size_t)1 << 26)) ? n : 0;
}

WsLayout workspace_layout(const iact_scene_t* sc, size_t acc_elems, bool with_delta, size_t mask_words) {
  WsLayout L;
  TableOffsets to = table_offsets(sc->n_cyl, sc->n_box, sc->n_sph, sc->n_obox, sc->n_tri, sc->n_mirrors);
  L.n_table_floats = to.total;
  size_t off = 0;
  L.counter = off;
  off = align256(off + 64);
  L.tables = off;
  off = align256(off + sizeof(float) * (size_t)std::max(to.total, 1));
  size_t n = (size_t)std::max(sc->n_facets, 0) * (size_t)std::max(sc->n_samples, 0);
  L.p4 = off;
  off = align256(off + sizeof(float4) * n);
  L.n4 = off;
  off = align256(off + sizeof(float4) * n);
  L.d4 = off;
  if (with_delta) off = align256(off + sizeof(float4) * n);
  L.b4 = off;  // bundle bounds, only for scenes with obstructions
  L.n_b4 = n_primitives(sc) > 0 ? (size_t)std::max(sc->n_facets, 0) : 0;
  off = align256(off + sizeof(float4) * L.n_b4);
  L.acc = off;
  off = align256(off + sizeof(double) * acc_elems);
  L.masks = off;
  L.n_masks = mask_words;
  off = align256(off + sizeof(uint32_t) * mask_words);
  L.total = off;
  return L;
}

size_t acc_elems(const iact_sensor_t* sn, int S, int mode) {
  if (mode == IACT_MODE_RESPONSE) return (size_t)std::max(S, 0) * (size_t)sn->n_pixels;
  if (mode == IACT_MODE_IMAGE) return (size_t)sn->n_pixels;
  return 0;
}

WsLayout workspace_for(const iact_scene_t* sc, const iact_sensor_t* sn, int S, int mode) {
  if (mode == IACT_MODE_BACKWARD)
    return workspace_layout(sc, (size_t)std::max(sc->n_facets, 0) * kFacetGrad + (size_t)std::max(S, 0) * 4 +
                                    (size_t)std::max(sc->n_mirrors, 0) * kMirGrad, true, pair_mask_words(sc, S));
  return workspace_layout(sc, acc_elems(sn, S, mode), false, pair_mask_words(sc, S));
}

int plan_tiles(RenderK& p, int mode, int block, const iact_opts_t* opts, long long min_tiles, int sb_fixed) {
  const int nw = block / 32;
  const int nch = (p.M + 31) / 32;
  const int S = p.S;
  // a response tile keeps one FP32 shared-memory row per source: two warps per
  // source halves that footprint and doubles the CTAs an SM holds
  int SB = (opts && opts->sources_per_cta > 0) ? opts->sources_per_cta
                                               : std::min(S, mode == IACT_MODE_RESPONSE ? std::max(1, nw / 2) : nw);
  SB = sb_fixed > 0 ? sb_fixed : std::max(1, std::min(SB, S));
  const bool fixed = opts && (opts->tasks_per_warp > 0 || opts->facets_per_tile > 0);
  // response tiles flush SB full rows each: larger tiles flush less often
  // (4096-source hard-hexagon response: 192 tasks per warp 3.23 ms, 96: 3.27,
  // 48: 3.46). Hard pixels only: a soft sensor's FP32 shared-memory rows
  // would then sum ~4x more ray taps per entry before each FP64 flush
  // (rows-vs-image agreement 3e-6 instead of < 1e-6 on the 256-source
  // soft-hexagon response).
  const bool soft = p.sn.type == IACT_SENSOR_SOFT_SQUARE || p.sn.type == IACT_SENSOR_SOFT_HEX;
  const int tpw = (opts && opts->tasks_per_warp > 0) ? opts->tasks_per_warp
                                                     : ((mode == IACT_MODE_RESPONSE && !soft) ? 192 : 48);
  // warp tasks (32 rays each) per tile; candidate masks stay within 16 KiB
  int target = std::max(1, std::min(nw * tpw, p.n_words ? 4096 / p.n_words : 1 << 30));
  for (;;) {
    int CC = std::max(1, std::min(nch, std::max(1, target / SB)));
    // split a facet's chunks evenly between its tiles (8 chunks in tiles of
    // 6: 4 + 4, not 6 + 2; a 276-primitive scene 281 -> 250 us)
    CC = (nch + (nch + CC - 1) / CC - 1) / ((nch + CC - 1) / CC);
    int FC = (opts && opts->facets_per_tile > 0) ? opts->facets_per_tile : std::max(1, target / (SB * CC));
    FC = std::max(1, std::min(FC, p.F));
    p.SB = SB; p.FC = FC; p.CC = CC;
    p.n_fchunk = (p.F + FC - 1) / FC;
    p.n_cchunk = (nch + CC - 1) / CC;
    const long long tiles =
        (S > 0 && p.F > 0 && p.M > 0) ? (long long)((S + SB - 1) / SB) * p.n_fchunk * p.n_cchunk : 0;
    if (tiles > 0x7fffffffLL) return set_error(IACT_E_UNSUPPORTED, "too many work tiles");
    p.n_tiles = (int)tiles;
    // small launches: halve the tile until the GPU holds enough of them to balance
    if (fixed || tiles == 0 || tiles >= min_tiles || target <= nw) break;
    target = std::max(nw, target / 2);
  }
  return IACT_OK;
}

int plan_smem(const iact_sensor_t* sn, int n_table_floats, int SB, int mode, int hist_mode, size_t budget,
              size_t tab_floor, size_t htab_floor, SmemPlan& sp) {
  const size_t P = (size_t)sn->n_pixels;
  sp.tab_bytes = std::max(tab_floor, sizeof(float) * (size_t)((n_table_floats + 3) & ~3));
  const bool hex = (sn->type == IACT_SENSOR_HEX || sn->type == IACT_SENSOR_SOFT_HEX);
  const size_t htab_elems = hex ? (size_t)sn->table_q * sn->table_r : 0;
  size_t htab_bytes = sizeof(short) * ((htab_elems + 7) & ~(size_t)7);
  sp.hex_in_smem = (hex && sn->n_pixels < 32768 && sp.tab_bytes + std::max(htab_bytes, htab_floor) <= budget / 2) ? 1 : 0;
  sp.htab_bytes = sp.hex_in_smem ? std::max(htab_bytes, htab_floor) : htab_floor;
  if (sp.tab_bytes + sp.htab_bytes > budget) return set_error(IACT_E_UNSUPPORTED, "scene tables exceed shared memory");
  const int rows = (mode == IACT_MODE_RESPONSE) ? SB : 1;
  const size_t hist_bytes = sizeof(float) * (size_t)rows * P;
  const bool use_smem = (hist_mode != 2) && (sp.tab_bytes + sp.htab_bytes + hist_bytes <= budget);
  if (hist_mode == 1 && !use_smem) return set_error(IACT_E_UNSUPPORTED, "histogram rows do not fit in shared memory");
  sp.rows_in_smem = use_smem ? rows : 0;
  sp.hist_bytes = use_smem ? hist_bytes : 0;
  return IACT_OK;
}

int launch_render(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                  const float* values, int S, int mode, float* out, void* ws, size_t ws_bytes,
                  const iact_opts_t* opts, cudaStream_t st) {
  (void)ws_bytes;
  const size_t n_acc = acc_elems(sn, S, mode);
  const WsLayout L = workspace_layout(sc, n_acc, false, pair_mask_words(sc, S));
  char* w = static_cast<char*>(ws);
  int rc;
  if (S == 0 || sc->n_facets == 0 || sc->n_samples == 0) {
    if (n_acc) return check_cuda(cudaMemsetAsync(out, 0, n_acc * sizeof(float), st), "zero output");
    return IACT_OK;
  }
  // the prep launch also clears the tile counter and the accumulator
  rc = launch_prep(sc, L, w, st, false, w + L.acc, n_acc * sizeof(double), reinterpret_cast<int*>(w + L.counter));
  if (rc) return rc;

  RenderK p = base_params(sc, sn, L, w, sources, values, S);
  p.acc = reinterpret_cast<double*>(w + L.acc);
  if (opts && (opts->flags & IACT_FLAG_NO_CULL)) p.n_words = 0;
  int block = (opts && opts->block_threads > 0) ? opts->block_threads : 256;
  if (block % 32 || block > 256) return set_error(IACT_E_INVALID, "opts.block_threads must be a multiple of 32, <= 256");
  DevInfo di = device_info();
  // tiles per SM below which small launches shrink their tiles: each tile
  // recomputes its candidate masks and ends with a barrier and a flush of
  // its histogram rows, so cheap rays
  // (single-stage scenes with few primitives) want fewer, larger tiles, and
  // costly or uneven rays (stage mirrors, many shadowing primitives) a finer
  // balance (measured: 1000-sample plain forward 7 % faster at 4 than at 8
  // per SM, the Cassegrain forward 13 % slower; 276-primitive scene 320 us
  // at 5 tiles per SM, 256 us at 10)
  const bool soft = (sn->type == IACT_SENSOR_SOFT_SQUARE || sn->type == IACT_SENSOR_SOFT_HEX);
  const bool stages = sc->n_mirrors > 0;
  // the common cases run k_render_hard (hard pixels, point or parallel
  // sources) or k_render_soft (soft pixels, also extended sources), with the
  // candidate word of every (source, facet) pair from k_masks
  const bool hard = !stages && p.sn.axes &&
                    (soft || src_type == IACT_SRC_POINT || src_type == IACT_SRC_PARALLEL) &&
                    ((p.n_words == 1 && L.n_masks > 0) || n_primitives(sc) == 0) &&
                    !(opts && opts->hist_mode == 2);
  // image renders of k_render_hard keep their FP32 row across tiles and need
  // no masks per tile, so their tiles are smaller (balance at the end of a
  // launch: 1000-sample plain forward 51.5 us at 12 tiles per SM vs 57.4 at
  // 16 and 56.2 at 4)
  const long long tiles_per_sm =
      (hard && !soft && mode == IACT_MODE_IMAGE) ? 12 : (sc->n_mirrors > 0 ? 8 : (n_primitives(sc) > 32 ? 10 : 4));
  const long long min_tiles = tiles_per_sm * std::max(di.sm_count, 1);
  // soft-pixel images of at least 32 sources trace one source per lane
  // (k_render_soft_spread) when full 32-source blocks fill at least 3/4 of
  // the lanes (alignment render, 256 extended sources: the taps of one
  // add instruction then seldom share an address)
  bool spread = hard && soft && mode == IACT_MODE_IMAGE && S >= 32 && 4LL * S >= 3LL * 32 * ((S + 31) / 32) &&
                !(opts && opts->sources_per_cta > 0);
  rc = plan_tiles(p, mode, block, opts, min_tiles, spread ? 32 : 0);
  if (rc) return rc;
  const size_t smem_max = (size_t)std::min(di.smem_optin > 0 ? di.smem_optin : 49152, 200 * 1024);
  SmemPlan sp;
  bool use_hard = false;
  size_t smem = 0;
  if (hard) {
    rc = plan_smem(sn, L.n_table_floats, p.SB, mode, opts ? opts->hist_mode : 0, smem_max, 0, 0, sp);
    if (rc) return rc;
    use_hard = sp.rows_in_smem > 0 &&
               (sn->type == IACT_SENSOR_SQUARE || sn->type == IACT_SENSOR_SOFT_SQUARE || sp.hex_in_smem);
    smem = sp.tab_bytes + sp.htab_bytes + sp.hist_bytes;
  }
  if (spread && !use_hard) {  // the generic kernel keeps its own tile shape
    spread = false;
    rc = plan_tiles(p, mode, block, opts, min_tiles, 0);
    if (rc) return rc;
  }
  if (!use_hard) {  // k_render: candidate masks of a tile's tasks in shared memory
    const size_t mask_bytes = sizeof(uint32_t) * (size_t)p.n_words * p.SB * p.FC;
    rc = plan_smem(sn, L.n_table_floats, p.SB, mode, opts ? opts->hist_mode : 0, smem_max - mask_bytes, 0, 0, sp);
    if (rc) return rc;
    smem = sp.tab_bytes + sp.htab_bytes + sp.hist_bytes + mask_bytes;
  }
  p.hex_in_smem = sp.hex_in_smem;
  p.rows_in_smem = sp.rows_in_smem;

  void* const* ev = opts ? opts->kernel_events : nullptr;
  p.seed = opts ? opts->seed : 0u;
  if (use_hard) {
    // the kernel events (profiling) bracket the masks and the render
    if (ev && ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
    if (p.n_words) {
      p.gmask = reinterpret_cast<const uint32_t*>(w + L.masks);
      rc = launch_masks(src_type, p, reinterpret_cast<uint32_t*>(w + L.masks), st);
      if (rc) return rc;
    }
    // an image row sums about 16k rays (hard pixels) or 12k rays of taps
    // (soft pixels, as many as a tile of the generic kernel) between flushes
    // to the FP64 accumulator
    const int tile_tasks = p.SB * p.FC * p.CC;
    p.flush_tiles = std::max(1, (soft ? 384 : 512) / std::max(tile_tasks, 1));
    void* const ev_end[2] = {nullptr, ev ? ev[1] : nullptr};
    if (spread) rc = run_render_soft_spread(src_type, sn->type == IACT_SENSOR_SOFT_HEX, p, block, smem, st, ev_end);
    else if (soft) rc = run_render_soft(src_type, mode, sn->type == IACT_SENSOR_SOFT_HEX, p, block, smem, st, ev_end);
    else rc = run_render_hard(src_type, mode, sn->type == IACT_SENSOR_HEX, p, block, smem, st, ev_end);
  } else if (src_type == IACT_SRC_POINT) {
    rc = dispatch_soft<IACT_SRC_POINT>(soft, mode, stages, p, block, smem, st, ev);
  } else if (src_type == IACT_SRC_EXTENDED) {
    rc = dispatch_soft<IACT_SRC_EXTENDED>(soft, mode, stages, p, block, smem, st, ev);
  } else {
    rc = dispatch_soft<IACT_SRC_PARALLEL>(soft, mode, stages, p, block, smem, st, ev);
  }
  if (rc) return rc;
  const int fb = (int)std::min<size_t>((n_acc + 255) / 256, 4096);
  return check_cuda(launch_after(k_finish, dim3(std::max(fb, 1)), dim3(256), 0, st, p.acc, out, n_acc),
                    "k_finish launch");
}

int launch_debug(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                 const float* values, int S, float* pts, float* vals, int32_t* pix, int32_t* hit_mirror,
                 void* ws, size_t ws_bytes, uint32_t seed, cudaStream_t st) {
  (void)ws_bytes;
  if (S == 0 || sc->n_facets == 0 || sc->n_samples == 0) return IACT_OK;
  const WsLayout L = workspace_layout(sc, 0, false);
  char* w = static_cast<char*>(ws);
  int rc = launch_prep(sc, L, w, st, false);
  if (rc) return rc;
  RenderK p = base_params(sc, sn, L, w, sources, values, S);
  const size_t smem = sizeof(float) * (size_t)((L.n_table_floats + 3) & ~3);
  const long long n = (long long)p.F * p.S * p.M;
  const int block = 256;
  const int grid = (int)std::min<long long>((n + block - 1) / block, 1 << 20);
  const bool stages = sc->n_mirrors > 0;
  const DevInfo di = device_info();
  // tables of up to IACT_MAX_OBSTRUCTIONS primitives exceed the 48 KiB a
  // kernel gets without opting in; resident_ctas opts in
  if (smem > (size_t)std::max(di.smem_optin, 48 * 1024))
    return set_error(IACT_E_UNSUPPORTED, "scene tables exceed the shared memory of an SM");
  p.seed = seed;
  void (*kern)(const RenderK, float*, float*, int32_t*, int32_t*);
  if (src_type == IACT_SRC_POINT) kern = stages ? k_debug<IACT_SRC_POINT, true> : k_debug<IACT_SRC_POINT, false>;
  else if (src_type == IACT_SRC_EXTENDED)
    kern = stages ? k_debug<IACT_SRC_EXTENDED, true> : k_debug<IACT_SRC_EXTENDED, false>;
  else kern = stages ? k_debug<IACT_SRC_PARALLEL, true> : k_debug<IACT_SRC_PARALLEL, false>;
  int per_sm = 0;
  rc = resident_ctas(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "debug kernel does not fit on an SM with these tables");
  kern<<<grid, block, smem, st>>>(p, pts, vals, pix, hit_mirror);
  return launched("k_debug launch");
}

__global__ void __launch_bounds__(256) k_probe_fma(float* out, int iters) {
  // 8 independent FMA chains per thread keep the FP32 pipe saturated
  float a[8];
  const float m = 1.0000001f, c = 1e-7f;
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 1e-3f + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int launch_probe_fma(float* out, int blocks, int iters, cudaStream_t st) {
  k_probe_fma<<<blocks, 256, 0, st>>>(out, iters);
  return launched("k_probe_fma launch");
}

}  // namespace iact
