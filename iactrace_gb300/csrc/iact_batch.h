// Internals of the batched render shared by its translation units
// (iact_batched.cu: plan, forward; iact_batched_adjoint.cu: backward).
#pragma once

#include <vector>

#include "iact_adjoint_impl.cuh"
#include "iact_internal.h"
#include "iact_render_impl.cuh"

namespace iact {

// Gradient outputs of one job and what their finish needs.
struct BatchGrad {
  float *g_rot, *g_pos, *g_scale, *g_src, *g_val, *g_mrot, *g_mpos, *g_msurf;
  const float* facet_rot;
  const iact_mirror_t* mirrors;
  int F, S, n_mir, pad_;
  long long n_bucket;  // FP64 bucket entries (facets, sources, stage mirrors)
};

// One job of the device job table (pointers resolved into the workspace).
struct BatchJob {
  RenderK rk;
  PrepK pk;          // forward prep
  AdjK ak;           // backward (batches created with IACT_FLAG_BATCH_BACKWARD)
  PrepK pkb;         // backward prep (+ roughness deltas when requested)
  BatchGrad gr;
  float* out;
  long long n_out;   // out entries (P, or S*P)
  int tile_begin;    // first forward tile of this job in its class's queue
  int atile_begin;   // first adjoint tile of this job in its class's queue
};

struct BatchK {
  const BatchJob* jobs;  // this class's jobs (largest first)
  int n_jobs;
  int n_tiles;
  int* counter;
  int tab_floats;   // table area (floats, multiple of 4)
  int htab_elems;   // int16 hexagon lookup area (multiple of 8)
  int hist_floats;  // FP32 histogram area (forward) or stage-mirror partial sums (backward);
                    // the tile's candidate masks follow it
};

// k_batch_prep over every job (backward: the backward prep and zeroed
// gradient buckets) (iact_batched.cu)
int launch_batch_prep(const BatchJob* jobs, int n_jobs, int gx, int backward, cudaStream_t st);

}  // namespace iact

struct iact_batch {
  int src_type = 0, mode = 0, block = 256;
  bool backward = false;
  iact_opts_t opts;
  std::vector<iact_scene_t> scenes;
  std::vector<iact_sensor_t> sensors;
  std::vector<iact_job_t> jobs;
  // plan: job table position -> user's job index, per-position layout
  std::vector<int> order;
  std::vector<iact::RenderK> rk;  // workspace offsets still relative (base 0)
  std::vector<iact::AdjK> ak;     // idem, backward
  std::vector<iact::WsLayout> lay;
  std::vector<size_t> region, acc_off;
  struct Class {
    int soft = 0, stages = 0;
    int axes = 0;  // every job's sensor is axis-aligned
    int hard = 0;    // k_batch_render_hard: 1 square, 2 hexagonal sensors; 0 k_batch_render
    int a_hard = 0;  // k_batch_adjoint_hard (hard class, no roughness-scale gradients)
    int jb = 0, nj = 0, n_tiles = 0;
    int tab_floats = 0, htab_elems = 0, hist_floats = 0;
    size_t smem = 0;
    int grid = 0;
    // backward
    int a_tiles = 0, a_tab_floats = 0, a_htab_elems = 0, a_mgrad_floats = 0;
    size_t a_smem = 0;
    int a_grid = 0;
  };
  std::vector<Class> classes;
  size_t off_counter = 0, off_jobs = 0, off_acc = 0, acc_bytes = 0, total = 0;
  long long tiles = 0, a_tiles = 0, rays = 0, max_fm = 0, max_out = 0, max_fs = 0;  // max_fm: (facet, chunk) units
  long long max_pairs = 0;  // largest S * F among jobs with candidate words (k_batch_masks), 0: none
  size_t mask_smem = 0;     // k_batch_masks: largest table of those jobs (bytes)
  int mask_gx = 1;
  // prepare
  char* ws = nullptr;
  std::vector<iact::BatchJob> table;
  int prep_gx = 1, fin_gx = 1, afin_gx = 1;
};

namespace iact {
// the batched adjoint kernel of a template class (iact_batched_adjoint.cu)
const void* batch_adjoint_kernel(int src_type, int mode, const iact_batch::Class& C);
// k_batch_masks over the jobs of the hard classes (iact_batched.cu)
int launch_batch_masks(const iact_batch* b, const BatchJob* jobs, int n_jobs, cudaStream_t st);
}  // namespace iact
