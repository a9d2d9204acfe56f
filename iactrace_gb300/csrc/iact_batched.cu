// Batched persistent render: many telescope variants (jobs) in one launch.
//
//   k_batch_prep    : k_prep for every job at once (grid.y = job).
//   k_batch_render  : one persistent kernel per template class (source type,
//                     hard/soft sensor, mode, later stages). CTAs pull tiles
//                     from one queue over all jobs of the class; jobs are
//                     queued largest first, each job's tiles contiguous.
//                     When a CTA's next tile belongs to another job it
//                     copies that job's launch parameters and tables into
//                     shared memory, then runs the same tile body as
//                     k_render (render_tile).
//   k_batch_finish  : FP64 accumulators -> every job's FP32 output.
//
// Shared memory has one layout per class, sized for the largest tables,
// hexagon lookup table and histogram rows among its jobs, so the histogram
// area never moves and stays zero between tiles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "iact_batch.h"
#include "iact_device.cuh"
#include "iact_internal.h"
#include "iact_render_impl.cuh"

namespace iact {

// backward != 0: the backward prep (with roughness deltas where asked) and
// zeroed gradient buckets
__global__ void __launch_bounds__(256) k_batch_prep(const BatchJob* __restrict__ jobs, int backward) {
  const BatchJob& J = jobs[blockIdx.y];
  const PrepK& p = backward ? J.pkb : J.pk;
  if (blockIdx.x == 0) prep_tables(p);
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  prep_units(p, w, ((long long)gridDim.x * blockDim.x) >> 5);
  if (backward)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < J.gr.n_bucket;
         i += (long long)gridDim.x * blockDim.x)
      J.ak.gfacet[i] = 0.0;
}

int launch_batch_prep(const BatchJob* jobs, int n_jobs, int gx, int backward, cudaStream_t st) {
  k_batch_prep<<<dim3(gx, n_jobs), 256, 0, st>>>(jobs, backward);
  return launched("k_batch_prep launch");
}

// AX: every job of the launch has an axis-aligned sensor (plane hit without
// the frame's dot products, as in k_render)
template <int SRC, bool SOFT, int MODE, bool STAGES, bool AX = false>
__global__ void __launch_bounds__(256, STAGES ? 3 : IACT_RENDER_MIN_CTAS) k_batch_render(const BatchK b) {
  extern __shared__ __align__(16) float smem[];
  __shared__ __align__(16) RenderK s_p;
  __shared__ int s_tile, s_job, s_begin;
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + b.tab_floats);
  float* sh_hist = smem + b.tab_floats + b.htab_elems / 2;
  uint32_t* tmask = reinterpret_cast<uint32_t*>(sh_hist + b.hist_floats);
  const int nthr = blockDim.x;
  for (int i = threadIdx.x; i < b.hist_floats; i += nthr) sh_hist[i] = 0.f;
  int cur = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = atomicAdd(b.counter, 1);
      s_tile = t;
      if (t < b.n_tiles) {
        int lo = 0, hi = b.n_jobs - 1;  // last job whose first tile is <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.jobs[mid].tile_begin <= t) lo = mid;
          else hi = mid - 1;
        }
        s_job = lo;
        s_begin = b.jobs[lo].tile_begin;
      }
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= b.n_tiles) break;
    const int j = s_job;
    if (j != cur) {
      // every thread is past the previous tile's last use of s_p and the tables
      const int* src = reinterpret_cast<const int*>(&b.jobs[j].rk);
      int* dst = reinterpret_cast<int*>(&s_p);
      for (int i = threadIdx.x; i < (int)(sizeof(RenderK) / 4); i += nthr) dst[i] = src[i];
      __syncthreads();
      for (int i = threadIdx.x; i < s_p.n_table_floats; i += nthr) tab[i] = s_p.tables[i];
      if (s_p.hex_in_smem) {
        const int nq = s_p.sn.table_q * s_p.sn.table_r;
        const int n8 = (nq + 7) & ~7;
        for (int i = threadIdx.x; i < n8; i += nthr) htab[i] = (short)(i < nq ? s_p.hex_table[i] : -1);
      }
      __syncthreads();
      cur = j;
    }
    const RenderK& p = s_p;
    const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
    const float* mir = tab + table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir).mir;
    Sink sink;
    sink.sh = p.rows_in_smem ? sh_hist : nullptr;
    sink.g = p.acc;
    render_tile<SRC, SOFT, MODE, STAGES, AX>(p, ob, mir, htab, sh_hist, sink, tile - s_begin, tmask);
  }
}

// Candidate word of every (source, facet) pair of the jobs that render with
// k_batch_render_hard (grid.y = job; jobs without a mask area skip).
template <int SRC>
__global__ void __launch_bounds__(256) k_batch_masks(const BatchJob* __restrict__ jobs) {
  extern __shared__ __align__(16) float smem[];
  const RenderK& p = jobs[blockIdx.y].rk;
  if (!p.gmask) return;  // uniform over the CTA
  for (int i = threadIdx.x; i < p.n_table_floats; i += blockDim.x) smem[i] = p.tables[i];
  __syncthreads();
  const Obst ob = make_obst(smem, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
  pair_masks<SRC>(p, ob, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x,
                  const_cast<uint32_t*>(p.gmask));
}

// k_batch_render for a class whose jobs all take the hard-pixel tile body
// (render_tile_hard: single stage, point or parallel sources, axis-aligned
// sensors of one kind, rows and hexagon tables in shared memory, candidate
// words per pair from k_batch_masks). An image job's row is flushed when the
// CTA moves to another job, every flush_tiles tiles and at the end; the tile
// index is double-buffered because image tiles end without a barrier.
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, IACT_RENDER_MIN_CTAS) k_batch_render_hard(const BatchK b) {
  extern __shared__ __align__(16) float smem[];
  __shared__ __align__(16) RenderK s_p;
  __shared__ int s_tile[2], s_job[2], s_begin[2];
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + b.tab_floats);
  float* sh_hist = smem + b.tab_floats + b.htab_elems / 2;
  const int nthr = blockDim.x;
  for (int i = threadIdx.x; i < b.hist_floats; i += nthr) sh_hist[i] = 0.f;
  int cur = -1, since = 0;
  for (int it = 0;; ++it) {
    const int k = it & 1;
    if (threadIdx.x == 0) {
      const int t = atomicAdd(b.counter, 1);
      s_tile[k] = t;
      if (t < b.n_tiles) {
        int lo = 0, hi = b.n_jobs - 1;  // last job whose first tile is <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.jobs[mid].tile_begin <= t) lo = mid;
          else hi = mid - 1;
        }
        s_job[k] = lo;
        s_begin[k] = b.jobs[lo].tile_begin;
      }
    }
    __syncthreads();  // every warp is past its previous tile
    const int tile = s_tile[k];
    const int j = tile < b.n_tiles ? s_job[k] : -1;
    if (MODE == IACT_MODE_IMAGE && since > 0 && (j != cur || since >= s_p.flush_tiles)) {
      flush_rows(s_p, sh_hist, 0, 1);
      since = 0;
      __syncthreads();
    }
    if (tile >= b.n_tiles) break;
    if (j != cur) {
      const int* src = reinterpret_cast<const int*>(&b.jobs[j].rk);
      int* dst = reinterpret_cast<int*>(&s_p);
      for (int i = threadIdx.x; i < (int)(sizeof(RenderK) / 4); i += nthr) dst[i] = src[i];
      __syncthreads();
      for (int i = threadIdx.x; i < s_p.n_table_floats; i += nthr) tab[i] = s_p.tables[i];
      if (HEX) {
        const int nq = s_p.sn.table_q * s_p.sn.table_r;
        const int n8 = (nq + 7) & ~7;
        for (int i = threadIdx.x; i < n8; i += nthr) htab[i] = (short)(i < nq ? s_p.hex_table[i] : -1);
      }
      __syncthreads();
      cur = j;
    }
    const Obst ob = make_obst(tab, s_p.n_cyl, s_p.n_box, s_p.n_sph, s_p.n_obox, s_p.n_tri);
    render_tile_hard<SRC, MODE, HEX>(s_p, ob, htab, sh_hist, tile - s_begin[k]);
    ++since;
  }
}

__global__ void __launch_bounds__(256) k_batch_finish(const BatchJob* __restrict__ jobs) {
  const BatchJob& J = jobs[blockIdx.y];
  const double* acc = J.rk.acc;
  float* out = J.out;
  const long long n = J.n_out;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)acc[i];
}

namespace {

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

using BatchKernel = void (*)(BatchK);

template <int SRC, bool SOFT, int MODE>
BatchKernel pick_stages(bool stages, bool axes) {
  if constexpr (SRC != IACT_SRC_EXTENDED)
    if (!stages && axes) return k_batch_render<SRC, SOFT, MODE, false, true>;
  return stages ? k_batch_render<SRC, SOFT, MODE, true> : k_batch_render<SRC, SOFT, MODE, false>;
}
template <int SRC, bool SOFT>
BatchKernel pick_mode(int mode, bool stages, bool axes) {
  return mode == IACT_MODE_RESPONSE ? pick_stages<SRC, SOFT, IACT_MODE_RESPONSE>(stages, axes)
                                    : pick_stages<SRC, SOFT, IACT_MODE_IMAGE>(stages, axes);
}
template <int SRC>
BatchKernel pick_soft(bool soft, int mode, bool stages, bool axes) {
  return soft ? pick_mode<SRC, true>(mode, stages, axes) : pick_mode<SRC, false>(mode, stages, axes);
}
BatchKernel pick_kernel(int src_type, bool soft, int mode, bool stages, bool axes) {
  if (src_type == IACT_SRC_POINT) return pick_soft<IACT_SRC_POINT>(soft, mode, stages, axes);
  if (src_type == IACT_SRC_EXTENDED) return pick_soft<IACT_SRC_EXTENDED>(soft, mode, stages, axes);
  return pick_soft<IACT_SRC_PARALLEL>(soft, mode, stages, axes);
}

bool is_soft(const iact_sensor_t& s) { return s.type == IACT_SENSOR_SOFT_SQUARE || s.type == IACT_SENSOR_SOFT_HEX; }

template <int SRC, int MODE>
BatchKernel pick_hard_hex(bool hex) {
  return hex ? k_batch_render_hard<SRC, MODE, true> : k_batch_render_hard<SRC, MODE, false>;
}
// the class kernel: k_batch_render_hard for hard classes (hard = 1 square,
// 2 hexagonal sensors), else k_batch_render
BatchKernel class_kernel(int src_type, int mode, const iact_batch::Class& C) {
  if (C.hard) {
    const bool hex = C.hard == 2;
    if (src_type == IACT_SRC_POINT)
      return mode == IACT_MODE_RESPONSE ? pick_hard_hex<IACT_SRC_POINT, IACT_MODE_RESPONSE>(hex)
                                        : pick_hard_hex<IACT_SRC_POINT, IACT_MODE_IMAGE>(hex);
    return mode == IACT_MODE_RESPONSE ? pick_hard_hex<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE>(hex)
                                      : pick_hard_hex<IACT_SRC_PARALLEL, IACT_MODE_IMAGE>(hex);
  }
  return pick_kernel(src_type, C.soft, mode, C.stages, C.axes);
}

}  // namespace
}  // namespace iact

using namespace iact;

int iact::launch_batch_masks(const iact_batch* b, const BatchJob* jobs, int n_jobs, cudaStream_t st) {
  if (b->src_type == IACT_SRC_POINT)
    k_batch_masks<IACT_SRC_POINT><<<dim3(b->mask_gx, n_jobs), 256, b->mask_smem, st>>>(jobs);
  else
    k_batch_masks<IACT_SRC_PARALLEL><<<dim3(b->mask_gx, n_jobs), 256, b->mask_smem, st>>>(jobs);
  return launched("k_batch_masks launch");
}

extern "C" {

int iact_batch_create(const iact_job_t* jobs, int32_t n_jobs, int32_t source_type, int32_t mode,
                      const iact_opts_t* opts, iact_batch** out) {
  if (!out) return set_error(IACT_E_INVALID, "iact_batch_create: out is NULL");
  *out = nullptr;
  if (n_jobs < 0 || (n_jobs > 0 && !jobs)) return set_error(IACT_E_INVALID, "iact_batch_create: bad job list");
  if (n_jobs > 65535) return set_error(IACT_E_UNSUPPORTED, "iact_batch_create: more than 65535 jobs");
  if (mode != IACT_MODE_IMAGE && mode != IACT_MODE_RESPONSE)
    return set_error(IACT_E_INVALID, "mode must be IACT_MODE_IMAGE or IACT_MODE_RESPONSE");
  if (source_type != IACT_SRC_POINT && source_type != IACT_SRC_PARALLEL && source_type != IACT_SRC_EXTENDED)
    return set_error(IACT_E_INVALID, "source_type must be IACT_SRC_POINT, IACT_SRC_PARALLEL or IACT_SRC_EXTENDED");
  const int block = (opts && opts->block_threads > 0) ? opts->block_threads : 256;
  if (block % 32 || block > 256) return set_error(IACT_E_INVALID, "opts.block_threads must be a multiple of 32, <= 256");
  for (int i = 0; i < n_jobs; ++i) {
    const iact_job_t& J = jobs[i];
    const std::string at = "job " + std::to_string(i) + ": ";
    int rc = validate_scene(J.scene);
    if (!rc) rc = validate_sensor(J.sensor);
    if (rc) return set_error(rc, at + iact_last_error());
    if (J.n_sources < 0) return set_error(IACT_E_INVALID, at + "negative source count");
    if (J.n_sources > 0 && (!J.sources || !J.values)) return set_error(IACT_E_INVALID, at + "sources/values are NULL");
    if (mode == IACT_MODE_RESPONSE && (long long)J.n_sources * J.sensor->n_pixels > 0x7fffffffLL)
      return set_error(IACT_E_UNSUPPORTED, at + "response matrix larger than 2^31 entries");
    if (!J.out && acc_elems(J.sensor, J.n_sources, mode) > 0) return set_error(IACT_E_INVALID, at + "out is NULL");
    if (opts && (opts->flags & IACT_FLAG_BATCH_BACKWARD)) {
      if (J.scene->n_stages > kAdjRing)
        return set_error(IACT_E_UNSUPPORTED, at + "backward: at most 2 mirror stages after the primary in a batch "
                                                  "(iact_render_backward takes any number)");
      if (source_type == IACT_SRC_EXTENDED && J.g_sources)
        return set_error(IACT_E_UNSUPPORTED, at + "backward: no source gradients for extended sources");
      if (!J.grad_out && acc_elems(J.sensor, J.n_sources, mode) > 0)
        return set_error(IACT_E_INVALID, at + "backward: grad_out is NULL");
    }
  }
  const bool backward = opts && (opts->flags & IACT_FLAG_BATCH_BACKWARD);

  iact_batch* b = new (std::nothrow) iact_batch();
  if (!b) return set_error(IACT_E_INVALID, "iact_batch_create: out of host memory");
  b->src_type = source_type;
  b->mode = mode;
  b->block = block;
  b->backward = backward;
  memset(&b->opts, 0, sizeof(b->opts));
  if (opts) b->opts = *opts;
  b->scenes.resize(n_jobs);
  b->sensors.resize(n_jobs);
  b->jobs.assign(jobs, jobs + n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    b->scenes[i] = *jobs[i].scene;
    b->sensors[i] = *jobs[i].sensor;
    b->jobs[i].scene = &b->scenes[i];
    b->jobs[i].sensor = &b->sensors[i];
  }

  // per-job tiles (workspace pointers relative to a zero base for now)
  std::vector<RenderK> rk(n_jobs);
  std::vector<AdjK> ak(backward ? n_jobs : 0);
  std::vector<size_t> a_smem(backward ? n_jobs : 0);
  std::vector<WsLayout> lay(n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    // the backward layout holds the forward's arrays too (plus deltas and buckets)
    lay[i] = backward ? workspace_for(&b->scenes[i], &b->sensors[i], jobs[i].n_sources, IACT_MODE_BACKWARD)
                      : workspace_layout(&b->scenes[i], 0, false, pair_mask_words(&b->scenes[i], jobs[i].n_sources));
    rk[i] = base_params(&b->scenes[i], &b->sensors[i], lay[i], nullptr, jobs[i].sources, jobs[i].values,
                        jobs[i].n_sources);
    rk[i].seed = jobs[i].seed;
    if (opts && (opts->flags & IACT_FLAG_NO_CULL)) rk[i].n_words = 0;
    int rc = plan_tiles(rk[i], mode, block, opts, 0);
    if (!rc && backward) {
      iact_opts_t o;
      memset(&o, 0, sizeof(o));
      if (opts) o = *opts;
      o.seed = jobs[i].seed;
      ak[i] = adjoint_params(&b->scenes[i], &b->sensors[i], lay[i], nullptr, jobs[i].sources, jobs[i].values,
                             jobs[i].grad_out, jobs[i].n_sources, jobs[i].g_facet_scale != nullptr, &o);
      rc = plan_adjoint(ak[i], &b->sensors[i], block, a_smem[i], 0);
    }
    if (rc) {
      delete b;
      return rc;
    }
  }

  // template classes (soft, stages) in a fixed order, largest jobs first
  const DevInfo di = device_info();
  const size_t budget = (size_t)std::min(di.smem_optin > 0 ? di.smem_optin : 49152, 200 * 1024);
  const int hist_mode = opts ? opts->hist_mode : 0;
  for (int cls = 0; cls < 4; ++cls) {
    const int soft = cls >> 1, stages = cls & 1;
    std::vector<int> mem;
    for (int i = 0; i < n_jobs; ++i)
      if ((int)is_soft(b->sensors[i]) == soft && (int)(b->scenes[i].n_mirrors > 0) == stages) mem.push_back(i);
    if (mem.empty()) continue;
    std::stable_sort(mem.begin(), mem.end(), [&](int x, int y) { return rk[x].n_tiles > rk[y].n_tiles; });
    iact_batch::Class C;
    C.soft = soft;
    C.stages = stages;
    C.axes = 1;
    for (int i : mem) C.axes &= rk[i].sn.axes;
    C.jb = (int)b->order.size();
    C.nj = (int)mem.size();
    // table and hexagon-table floors: the largest of the class
    size_t tab_floor = 0, htab_floor = 0;
    for (int i : mem) tab_floor = std::max(tab_floor, sizeof(float) * (size_t)((lay[i].n_table_floats + 3) & ~3));
    for (int i : mem) {
      SmemPlan sp;
      if (plan_smem(&b->sensors[i], lay[i].n_table_floats, rk[i].SB, mode, 2, budget, tab_floor, 0, sp) == IACT_OK &&
          sp.hex_in_smem)
        htab_floor = std::max(htab_floor, sp.htab_bytes);
    }
    size_t masks = 0;  // candidate masks of one tile, largest over the class
    for (int i : mem) masks = std::max(masks, sizeof(uint32_t) * (size_t)rk[i].n_words * rk[i].SB * rk[i].FC);
    size_t hist = 0;
    long long tile = 0;
    for (int i : mem) {
      SmemPlan sp;
      int rc = plan_smem(&b->sensors[i], lay[i].n_table_floats, rk[i].SB, mode, hist_mode, budget - masks, tab_floor,
                         htab_floor, sp);
      if (rc) {
        delete b;
        return set_error(rc, "job " + std::to_string(i) + ": " + iact_last_error());
      }
      rk[i].hex_in_smem = sp.hex_in_smem;
      rk[i].rows_in_smem = sp.rows_in_smem;
      hist = std::max(hist, sp.hist_bytes);
      b->order.push_back(i);
      tile += rk[i].n_tiles;
    }
    if (tile > 0x7fffffffLL) {
      delete b;
      return set_error(IACT_E_UNSUPPORTED, "iact_batch_create: more than 2^31 tiles in one class");
    }
    C.n_tiles = (int)tile;
    // the hard-pixel tile body when every job of the class qualifies
    {
      const int kind = b->sensors[mem[0]].type;
      bool hard = !soft && !stages && (source_type == IACT_SRC_POINT || source_type == IACT_SRC_PARALLEL) &&
                  (kind == IACT_SENSOR_SQUARE || kind == IACT_SENSOR_HEX);
      for (int i : mem)
        hard = hard && b->sensors[i].type == kind && rk[i].sn.axes && rk[i].rows_in_smem > 0 &&
               (kind == IACT_SENSOR_SQUARE || rk[i].hex_in_smem) &&
               ((rk[i].n_words == 1 && lay[i].n_masks > 0) || n_primitives(&b->scenes[i]) == 0);
      C.hard = hard ? (kind == IACT_SENSOR_HEX ? 2 : 1) : 0;
      bool a_hard = hard && backward;
      for (int i : mem) a_hard = a_hard && !jobs[i].g_facet_scale;
      C.a_hard = a_hard ? 1 : 0;
      if (hard)  // an image row sums about 16k rays between flushes
        for (int i : mem) rk[i].flush_tiles = std::max(1, 512 / std::max(rk[i].SB * rk[i].FC * rk[i].CC, 1));
    }
    C.tab_floats = (int)(tab_floor / sizeof(float));
    C.htab_elems = (int)(htab_floor / sizeof(short));
    C.hist_floats = (int)(hist / sizeof(float));
    C.smem = tab_floor + htab_floor + hist + masks;
    if (backward) {  // adjoint layout: tables | int16 hex table | stage-mirror sums | masks
      size_t atab = 0, ahtab = 0, amir = 0, amask = 0;
      long long at = 0;
      for (int i : mem) {
        const AdjK& a = ak[i];
        atab = std::max(atab, sizeof(float) * (size_t)((a.n_table_floats + 3) & ~3));
        if (a.hex_in_smem)
          ahtab = std::max(ahtab, sizeof(short) * (((size_t)a.sn.table_q * a.sn.table_r + 7) & ~(size_t)7));
        amir = std::max(amir, sizeof(float) * (size_t)a.n_mir * kMirGrad);
        amask = std::max(amask, sizeof(uint32_t) * (size_t)a.n_words * a.SB * a.FC);
        at += a.n_tiles;
      }
      if (at > 0x7fffffffLL || atab + ahtab + amir + amask > budget) {
        delete b;
        return set_error(IACT_E_UNSUPPORTED, "iact_batch_create: backward plan does not fit");
      }
      C.a_tiles = (int)at;
      C.a_tab_floats = (int)(atab / sizeof(float));
      C.a_htab_elems = (int)(ahtab / sizeof(short));
      C.a_mgrad_floats = (int)(amir / sizeof(float));
      C.a_smem = atab + ahtab + amir + amask;
    }
    b->classes.push_back(C);
  }

  // workspace: counters, job table, per-job tables and samples, accumulators
  size_t off = 0;
  b->off_counter = off;  // 64 B per class: 4 forward, 4 backward
  off = a256(off + 64 * 8);
  b->off_jobs = off;
  off = a256(off + sizeof(BatchJob) * (size_t)std::max(n_jobs, 1));
  b->region.assign(n_jobs, 0);
  for (int pos = 0; pos < n_jobs; ++pos) {
    const int i = b->order[pos];
    b->region[pos] = off;
    off = a256(off + lay[i].total);
  }
  b->off_acc = off;
  b->acc_off.assign(n_jobs, 0);
  size_t acc = 0;
  for (int pos = 0; pos < n_jobs; ++pos) {
    const int i = b->order[pos];
    b->acc_off[pos] = acc;
    acc = a256(acc + sizeof(double) * acc_elems(&b->sensors[i], jobs[i].n_sources, mode));
  }
  b->acc_bytes = acc;
  b->total = a256(off + acc);
  for (int i = 0; i < n_jobs; ++i) {
    b->tiles += rk[i].n_tiles;
    if (backward) b->a_tiles += ak[i].n_tiles;
    b->rays += (long long)rk[i].S * rk[i].F * rk[i].M;
    b->max_fm = std::max(b->max_fm, (long long)rk[i].F * ((rk[i].M + 31) / 32));  // (facet, chunk) units
    b->max_out = std::max(b->max_out, (long long)acc_elems(&b->sensors[i], jobs[i].n_sources, mode));
    b->max_fs = std::max(b->max_fs, (long long)std::max(std::max(rk[i].F, rk[i].S), b->scenes[i].n_mirrors));
  }
  b->rk = std::move(rk);
  b->ak = std::move(ak);
  b->lay = std::move(lay);
  *out = b;
  return IACT_OK;
}

int iact_batch_workspace_size(const iact_batch* b, size_t* bytes) {
  if (!b || !bytes) return set_error(IACT_E_INVALID, "iact_batch_workspace_size: NULL argument");
  *bytes = b->total;
  return IACT_OK;
}

int iact_batch_prepare(iact_batch* b, void* workspace, size_t workspace_bytes, void* stream) {
  if (!b) return set_error(IACT_E_INVALID, "iact_batch_prepare: batch is NULL");
  if (!workspace) return set_error(IACT_E_WORKSPACE, "workspace is NULL");
  if (reinterpret_cast<uintptr_t>(workspace) % 256) return set_error(IACT_E_WORKSPACE, "workspace must be 256-byte aligned");
  if (workspace_bytes < b->total)
    return set_error(IACT_E_WORKSPACE, "workspace too small: need " + std::to_string(b->total) + " bytes");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  const int n_jobs = (int)b->jobs.size();
  std::vector<BatchJob> table(n_jobs);
  b->max_pairs = 0;
  b->mask_smem = 0;
  for (int ci = 0; ci < (int)b->classes.size(); ++ci) {
    const iact_batch::Class& C = b->classes[ci];
    int tile = 0, atile = 0;
    for (int pos = C.jb; pos < C.jb + C.nj; ++pos) {
      const int i = b->order[pos];
      char* base = ws + b->region[pos];
      BatchJob& J = table[pos];
      memset(&J, 0, sizeof(J));
      J.rk = b->rk[i];
      J.rk.P4 = reinterpret_cast<const float4*>(base + b->lay[i].p4);
      J.rk.N4 = reinterpret_cast<const float4*>(base + b->lay[i].n4);
      J.rk.tables = reinterpret_cast<const float*>(base + b->lay[i].tables);
      J.rk.counter = reinterpret_cast<int*>(base + b->lay[i].counter);
      J.rk.acc = reinterpret_cast<double*>(ws + b->off_acc + b->acc_off[pos]);
      J.rk.B4 = b->lay[i].n_b4 ? reinterpret_cast<const float4*>(base + b->lay[i].b4) : nullptr;
      if (C.hard && J.rk.n_words) {  // candidate words per pair (k_batch_masks)
        J.rk.gmask = reinterpret_cast<const uint32_t*>(base + b->lay[i].masks);
        b->max_pairs = std::max(b->max_pairs, (long long)J.rk.S * J.rk.F);
        b->mask_smem = std::max(b->mask_smem, sizeof(float) * (size_t)std::max(J.rk.n_table_floats, 1));
      }
      J.pk = prep_params(&b->scenes[i], b->lay[i], base, false);
      J.out = b->jobs[i].out;
      J.n_out = (long long)acc_elems(&b->sensors[i], b->jobs[i].n_sources, b->mode);
      J.tile_begin = tile;
      tile += J.rk.n_tiles;
      if (b->backward) {
        const iact_job_t& U = b->jobs[i];
        const AdjK& a0 = b->ak[i];
        AdjK& a = J.ak;
        a = a0;
        a.P4 = reinterpret_cast<const float4*>(base + b->lay[i].p4);
        a.N4 = reinterpret_cast<const float4*>(base + b->lay[i].n4);
        a.D4 = U.g_facet_scale ? reinterpret_cast<const float4*>(base + b->lay[i].d4) : nullptr;
        a.B4 = b->lay[i].n_b4 ? reinterpret_cast<const float4*>(base + b->lay[i].b4) : nullptr;
        a.tables = reinterpret_cast<const float*>(base + b->lay[i].tables);
        a.counter = reinterpret_cast<int*>(base + b->lay[i].counter);
        a.gfacet = reinterpret_cast<double*>(base + b->lay[i].acc);
        a.gsrc = a.gfacet + (size_t)a.F * kFacetGrad;
        a.gmir = a.gsrc + (size_t)a.S * 4;
        a.want_mgrad = (U.g_mirror_rot || U.g_mirror_pos || U.g_mirror_surface) ? 1 : 0;
        a.gmask = C.a_hard ? J.rk.gmask : nullptr;  // the forward's candidate words (k_batch_masks)
        J.pkb = prep_params(&b->scenes[i], b->lay[i], base, U.g_facet_scale != nullptr);
        J.gr.g_rot = U.g_facet_rot; J.gr.g_pos = U.g_facet_pos; J.gr.g_scale = U.g_facet_scale;
        J.gr.g_src = U.g_sources; J.gr.g_val = U.g_values;
        J.gr.g_mrot = U.g_mirror_rot; J.gr.g_mpos = U.g_mirror_pos; J.gr.g_msurf = U.g_mirror_surface;
        J.gr.facet_rot = b->scenes[i].facet_rot;
        J.gr.mirrors = b->scenes[i].mirrors;
        J.gr.F = a.F; J.gr.S = a.S; J.gr.n_mir = a.n_mir;
        J.gr.n_bucket = (long long)a.F * kFacetGrad + (long long)a.S * 4 + (long long)a.n_mir * kMirGrad;
        J.atile_begin = atile;
        atile += a.n_tiles;
      }
    }
  }
  int rc = IACT_OK;
  if (n_jobs > 0)
    rc = check_cuda(cudaMemcpyAsync(ws + b->off_jobs, table.data(), sizeof(BatchJob) * (size_t)n_jobs,
                                    cudaMemcpyHostToDevice, st),
                    "upload job table");
  if (rc) return rc;
  const DevInfo di = device_info();
  if (b->max_pairs > 0) {
    int per_sm = 0;
    rc = resident_ctas(reinterpret_cast<const void*>(b->src_type == IACT_SRC_POINT ? k_batch_masks<IACT_SRC_POINT>
                                                                                    : k_batch_masks<IACT_SRC_PARALLEL>),
                       256, b->mask_smem, &per_sm);
    if (rc) return rc;
    b->mask_gx = (int)std::max<long long>(1, std::min<long long>((b->max_pairs + 255) / 256, 1024));
  }
  for (iact_batch::Class& C : b->classes) {
    BatchKernel kern = class_kernel(b->src_type, b->mode, C);
    int per_sm = 0;
    rc = resident_ctas(reinterpret_cast<const void*>(kern), b->block, C.smem, &per_sm);
    if (rc) return rc;
    if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "batched render kernel does not fit on an SM");
    C.grid = std::max(1, std::min(C.n_tiles, per_sm * di.sm_count));
    if (b->backward) {
      per_sm = 0;
      rc = resident_ctas(batch_adjoint_kernel(b->src_type, b->mode, C), b->block, C.a_smem, &per_sm);
      if (rc) return rc;
      if (per_sm < 1) return set_error(IACT_E_UNSUPPORTED, "batched adjoint kernel does not fit on an SM");
      C.a_grid = std::max(1, std::min(C.a_tiles, per_sm * di.sm_count));
    }
  }
  b->afin_gx = (int)std::max<long long>(1, std::min<long long>((b->max_fs + 31) / 32, 1024));
  b->prep_gx = (int)std::max<long long>(1, std::min<long long>((b->max_fm + 7) / 8, 1024));  // 8 warps per block
  b->fin_gx = (int)std::max<long long>(1, std::min<long long>((b->max_out + 255) / 256, 1024));
  b->table = std::move(table);
  b->ws = ws;
  return IACT_OK;
}

int iact_batch_render(iact_batch* b, void* stream) {
  if (!b) return set_error(IACT_E_INVALID, "iact_batch_render: batch is NULL");
  if (!b->ws) return set_error(IACT_E_INVALID, "iact_batch_render: call iact_batch_prepare first");
  const int n_jobs = (int)b->jobs.size();
  if (n_jobs == 0) return IACT_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = b->ws;
  const BatchJob* jobs = reinterpret_cast<const BatchJob*>(ws + b->off_jobs);
  int rc = check_cuda(cudaMemsetAsync(ws + b->off_counter, 0, 64 * 4, st), "reset tile counters");
  if (rc) return rc;
  if (b->acc_bytes) {
    rc = check_cuda(cudaMemsetAsync(ws + b->off_acc, 0, b->acc_bytes, st), "zero accumulators");
    if (rc) return rc;
  }
  if (b->max_fm > 0) {
    rc = launch_batch_prep(jobs, n_jobs, b->prep_gx, 0, st);
    if (rc) return rc;
  }
  void* const* ev = b->opts.kernel_events;
  if (ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
  if (b->max_pairs > 0) {  // candidate words of the hard classes' jobs (inside the kernel events)
    rc = launch_batch_masks(b, jobs, n_jobs, st);
    if (rc) return rc;
  }
  for (int ci = 0; ci < (int)b->classes.size(); ++ci) {
    const iact_batch::Class& C = b->classes[ci];
    if (C.n_tiles == 0) continue;
    BatchK k;
    k.jobs = jobs + C.jb;
    k.n_jobs = C.nj;
    k.n_tiles = C.n_tiles;
    k.counter = reinterpret_cast<int*>(ws + b->off_counter + 64 * ci);
    k.tab_floats = C.tab_floats;
    k.htab_elems = C.htab_elems;
    k.hist_floats = C.hist_floats;
    class_kernel(b->src_type, b->mode, C)<<<C.grid, b->block, C.smem, st>>>(k);
    rc = launched("k_batch_render launch");
    if (rc) return rc;
  }
  if (ev[1]) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), st);
  if (b->max_out > 0) {
    k_batch_finish<<<dim3(b->fin_gx, n_jobs), 256, 0, st>>>(jobs);
    rc = launched("k_batch_finish launch");
  }
  return rc;
}

int iact_batch_info(const iact_batch* b, int64_t* out, int32_t n) {
  if (!b || !out) return set_error(IACT_E_INVALID, "iact_batch_info: NULL argument");
  int launches = (b->max_fm > 0 ? 1 : 0) + (b->max_out > 0 ? 1 : 0) + (b->max_pairs > 0 ? 1 : 0), alaunches = 0;
  for (const auto& C : b->classes) launches += C.n_tiles > 0 ? 1 : 0;
  if (b->backward) {
    alaunches = 2;  // prep (+ bucket zeroing), finish
    for (const auto& C : b->classes) alaunches += C.a_tiles > 0 ? 1 : 0;
  }
  const int64_t v[7] = {(int64_t)b->jobs.size(), b->tiles, b->rays, launches, (int64_t)b->classes.size(),
                        b->a_tiles, alaunches};
  for (int i = 0; i < n && i < 7; ++i) out[i] = v[i];
  return IACT_OK;
}

void iact_batch_destroy(iact_batch* b) { delete b; }

}  // extern "C"
