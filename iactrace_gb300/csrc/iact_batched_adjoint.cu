// Batched adjoint: the backward of iact_batch_render for every job at once.
//
//   k_batch_prep(backward)   world samples (+ roughness deltas), bundle
//                            bounds, tables, and zeroed gradient buckets of
//                            every job (iact_batched.cu)
//   k_batch_adjoint          one persistent kernel per template class over
//                            the adjoint tiles of all its jobs (largest
//                            first); a CTA restages the job's tables when its
//                            next tile belongs to another job, flushing its
//                            stage-mirror partial sums to the previous job,
//                            then runs the single-scene tile body
//                            (adjoint_tile)
//   k_batch_adjoint_finish   Euler-angle and output conversion per job
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "iact_adjoint_impl.cuh"
#include "iact_batch.h"
#include "iact_internal.h"

namespace iact {

template <int SRC, bool SOFT, int MODE, bool STAGES>
__global__ void __launch_bounds__(256, STAGES ? 2 : (SOFT ? 3 : 4)) k_batch_adjoint(const BatchK b) {
  extern __shared__ __align__(16) float smem[];
  __shared__ __align__(16) AdjK s_a;
  __shared__ int s_tile, s_job, s_begin;
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + b.tab_floats);
  float* mgrad = reinterpret_cast<float*>(htab + b.htab_elems);  // stage-mirror partial sums
  uint32_t* tmask = reinterpret_cast<uint32_t*>(mgrad + b.hist_floats);
  const int nthr = blockDim.x;
  for (int i = threadIdx.x; i < b.hist_floats; i += nthr) mgrad[i] = 0.f;
  int cur = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = atomicAdd(b.counter, 1);
      s_tile = t;
      if (t < b.n_tiles) {
        int lo = 0, hi = b.n_jobs - 1;  // last job whose first adjoint tile is <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.jobs[mid].atile_begin <= t) lo = mid;
          else hi = mid - 1;
        }
        s_job = lo;
        s_begin = b.jobs[lo].atile_begin;
      }
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= b.n_tiles) break;
    const int j = s_job;
    if (j != cur) {
      // every thread is past the previous tile: its mirror sums go to that job
      if (STAGES && cur >= 0) {
        for (int i = threadIdx.x; i < s_a.n_mir * kMirGrad; i += nthr)
          if (mgrad[i] != 0.f) {
            atomicAdd(s_a.gmir + i, (double)mgrad[i]);
            mgrad[i] = 0.f;
          }
        __syncthreads();
      }
      const int* src = reinterpret_cast<const int*>(&b.jobs[j].ak);
      int* dst = reinterpret_cast<int*>(&s_a);
      for (int i = threadIdx.x; i < (int)(sizeof(AdjK) / 4); i += nthr) dst[i] = src[i];
      __syncthreads();
      for (int i = threadIdx.x; i < s_a.n_table_floats; i += nthr) tab[i] = s_a.tables[i];
      if (s_a.hex_in_smem) {
        const int nq = s_a.sn.table_q * s_a.sn.table_r;
        const int n8 = (nq + 7) & ~7;
        for (int i = threadIdx.x; i < n8; i += nthr) htab[i] = (short)(i < nq ? s_a.hex_table[i] : -1);
      }
      __syncthreads();
      cur = j;
    }
    const AdjK& p = s_a;
    const Obst ob = make_obst(tab, p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri);
    const float* mir = tab + table_offsets(p.n_cyl, p.n_box, p.n_sph, p.n_obox, p.n_tri, p.n_mir).mir;
    adjoint_tile<SRC, SOFT, MODE, STAGES>(p, ob, mir, htab, mgrad, tmask, tile - s_begin);
  }
  if (STAGES && cur >= 0) {
    __syncthreads();
    for (int i = threadIdx.x; i < s_a.n_mir * kMirGrad; i += nthr)
      if (mgrad[i] != 0.f) atomicAdd(s_a.gmir + i, (double)mgrad[i]);
  }
}

__global__ void __launch_bounds__(256) k_batch_adjoint_finish(const BatchJob* __restrict__ jobs) {
  const BatchJob& J = jobs[blockIdx.y];
  const BatchGrad& g = J.gr;
  const int n = max(max(g.F, g.S), g.n_mir);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    adjoint_finish_item(i, J.ak.gfacet, J.ak.gsrc, g.facet_rot, g.F, g.S, g.g_rot, g.g_pos, g.g_scale, g.g_src,
                        g.g_val);
    if (i < g.n_mir && (g.g_mrot || g.g_mpos || g.g_msurf))
      adjoint_mirror_item(i, J.ak.gmir, g.mirrors, g.g_mrot, g.g_mpos, g.g_msurf);
  }
}

// k_batch_adjoint for a class whose jobs all take the hard-pixel adjoint
// body (adjoint_tile_hard; the class renders with k_batch_render_hard and no
// job asks for roughness-scale gradients): candidate words per pair from
// k_batch_masks. Tiles end without a barrier, so the tile index is
// double-buffered.
template <int SRC, int MODE, bool HEX>
__global__ void __launch_bounds__(256, 4) k_batch_adjoint_hard(const BatchK b) {
  extern __shared__ __align__(16) float smem[];
  __shared__ __align__(16) AdjK s_a;
  __shared__ int s_tile[2], s_job[2], s_begin[2];
  float* tab = smem;
  short* htab = reinterpret_cast<short*>(smem + b.tab_floats);
  const int nthr = blockDim.x;
  int cur = -1;
  for (int it = 0;; ++it) {
    const int k = it & 1;
    if (threadIdx.x == 0) {
      const int t = atomicAdd(b.counter, 1);
      s_tile[k] = t;
      if (t < b.n_tiles) {
        int lo = 0, hi = b.n_jobs - 1;  // last job whose first adjoint tile is <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.jobs[mid].atile_begin <= t) lo = mid;
          else hi = mid - 1;
        }
        s_job[k] = lo;
        s_begin[k] = b.jobs[lo].atile_begin;
      }
    }
    __syncthreads();  // every warp is past its previous tile
    const int tile = s_tile[k];
    if (tile >= b.n_tiles) break;
    const int j = s_job[k];
    if (j != cur) {
      const int* src = reinterpret_cast<const int*>(&b.jobs[j].ak);
      int* dst = reinterpret_cast<int*>(&s_a);
      for (int i = threadIdx.x; i < (int)(sizeof(AdjK) / 4); i += nthr) dst[i] = src[i];
      __syncthreads();
      for (int i = threadIdx.x; i < s_a.n_table_floats; i += nthr) tab[i] = s_a.tables[i];
      if (HEX) {
        const int nq = s_a.sn.table_q * s_a.sn.table_r;
        const int n8 = (nq + 7) & ~7;
        for (int i = threadIdx.x; i < n8; i += nthr) htab[i] = (short)(i < nq ? s_a.hex_table[i] : -1);
      }
      __syncthreads();
      cur = j;
    }
    const Obst ob = make_obst(tab, s_a.n_cyl, s_a.n_box, s_a.n_sph, s_a.n_obox, s_a.n_tri);
    adjoint_tile_hard<SRC, MODE, HEX>(s_a, ob, htab, tile - s_begin[k]);
  }
}

namespace {

using AdjKernel = void (*)(BatchK);

template <int SRC, int MODE>
AdjKernel pick_a_hard_hex(bool hex) {
  return hex ? k_batch_adjoint_hard<SRC, MODE, true> : k_batch_adjoint_hard<SRC, MODE, false>;
}
AdjKernel pick_adjoint_hard(int src_type, int mode, bool hex) {
  if (src_type == IACT_SRC_POINT)
    return mode == IACT_MODE_RESPONSE ? pick_a_hard_hex<IACT_SRC_POINT, IACT_MODE_RESPONSE>(hex)
                                      : pick_a_hard_hex<IACT_SRC_POINT, IACT_MODE_IMAGE>(hex);
  return mode == IACT_MODE_RESPONSE ? pick_a_hard_hex<IACT_SRC_PARALLEL, IACT_MODE_RESPONSE>(hex)
                                    : pick_a_hard_hex<IACT_SRC_PARALLEL, IACT_MODE_IMAGE>(hex);
}

template <int SRC, bool SOFT, int MODE>
AdjKernel pick_a_stages(bool stages) {
  return stages ? k_batch_adjoint<SRC, SOFT, MODE, true> : k_batch_adjoint<SRC, SOFT, MODE, false>;
}
template <int SRC, bool SOFT>
AdjKernel pick_a_mode(int mode, bool stages) {
  return mode == IACT_MODE_RESPONSE ? pick_a_stages<SRC, SOFT, IACT_MODE_RESPONSE>(stages)
                                    : pick_a_stages<SRC, SOFT, IACT_MODE_IMAGE>(stages);
}
template <int SRC>
AdjKernel pick_a_soft(bool soft, int mode, bool stages) {
  return soft ? pick_a_mode<SRC, true>(mode, stages) : pick_a_mode<SRC, false>(mode, stages);
}
AdjKernel pick_adjoint(int src_type, bool soft, int mode, bool stages) {
  if (src_type == IACT_SRC_POINT) return pick_a_soft<IACT_SRC_POINT>(soft, mode, stages);
  if (src_type == IACT_SRC_EXTENDED) return pick_a_soft<IACT_SRC_EXTENDED>(soft, mode, stages);
  return pick_a_soft<IACT_SRC_PARALLEL>(soft, mode, stages);
}

}  // namespace

const void* batch_adjoint_kernel(int src_type, int mode, const iact_batch::Class& C) {
  if (C.a_hard) return reinterpret_cast<const void*>(pick_adjoint_hard(src_type, mode, C.hard == 2));
  return reinterpret_cast<const void*>(pick_adjoint(src_type, C.soft, mode, C.stages));
}

}  // namespace iact

using namespace iact;

extern "C" int iact_batch_backward(iact_batch* b, void* stream) {
  if (!b) return set_error(IACT_E_INVALID, "iact_batch_backward: batch is NULL");
  if (!b->backward)
    return set_error(IACT_E_INVALID, "iact_batch_backward: create the batch with IACT_FLAG_BATCH_BACKWARD");
  if (!b->ws) return set_error(IACT_E_INVALID, "iact_batch_backward: call iact_batch_prepare first");
  const int n_jobs = (int)b->jobs.size();
  if (n_jobs == 0) return IACT_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = b->ws;
  const BatchJob* jobs = reinterpret_cast<const BatchJob*>(ws + b->off_jobs);
  int rc = check_cuda(cudaMemsetAsync(ws + b->off_counter + 64 * 4, 0, 64 * 4, st), "reset adjoint tile counters");
  if (rc) return rc;
  rc = launch_batch_prep(jobs, n_jobs, b->prep_gx, 1, st);
  if (rc) return rc;
  void* const* ev = b->opts.kernel_events;
  if (ev[0]) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), st);
  if (b->max_pairs > 0) {  // candidate words of the hard classes' jobs (the sources may have changed)
    rc = launch_batch_masks(b, jobs, n_jobs, st);
    if (rc) return rc;
  }
  for (int ci = 0; ci < (int)b->classes.size(); ++ci) {
    const iact_batch::Class& C = b->classes[ci];
    if (C.a_tiles == 0) continue;
    BatchK k;
    k.jobs = jobs + C.jb;
    k.n_jobs = C.nj;
    k.n_tiles = C.a_tiles;
    k.counter = reinterpret_cast<int*>(ws + b->off_counter + 64 * (4 + ci));
    k.tab_floats = C.a_tab_floats;
    k.htab_elems = C.a_htab_elems;
    k.hist_floats = C.a_mgrad_floats;
    reinterpret_cast<AdjKernel>(const_cast<void*>(batch_adjoint_kernel(b->src_type, b->mode, C)))
        <<<C.a_grid, b->block, C.a_smem, st>>>(k);
    rc = launched("k_batch_adjoint launch");
    if (rc) return rc;
  }
  if (ev[1]) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), st);
  k_batch_adjoint_finish<<<dim3(b->afin_gx, n_jobs), 32, 0, st>>>(jobs);  // one warp per block (FP64 trigonometry)
  return launched("k_batch_adjoint_finish launch");
}
