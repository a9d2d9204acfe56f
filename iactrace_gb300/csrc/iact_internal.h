// Host-side internals shared by the translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/iactrace_gb300.h"
#include "iact_device.cuh"
#include "iact_render_impl.cuh"

namespace iact {

// thread-local message behind iact_last_error(); returns `code`
int set_error(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

// one more kernel queued by the library (process-wide count behind
// iact_kernel_launches); every launch site calls it after its launch
void count_launch();

// status of the `<<<...>>>` launch just made on this thread: counted when it
// was queued, IACT_E_CUDA with `what` in the message when it was not
inline int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) count_launch();
  return check_cuda(e, what);
}

// Launch of a kernel that follows another kernel of the same chain on
// `st` (prep -> masks -> render -> finish; prep -> masks -> adjoint ->
// finish) with programmatic stream serialization: it may be scheduled while
// its predecessor runs and waits in grid_dep_wait for the predecessor's
// results, so the launch gap between the two overlaps the predecessor.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_after(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, static_cast<Args&&>(args)...);
  if (e == cudaSuccess) count_launch();
  return e;
}

// validation of the descriptors shared by every entry point
int validate_scene(const iact_scene_t* sc);
int validate_sensor(const iact_sensor_t* sn);

// workspace layout (bytes from the workspace base, all 256-byte aligned)
struct WsLayout {
  size_t counter;  // int32 tile counter + int32 error word
  size_t tables;   // processed obstruction/mirror/sensor records (floats)
  size_t p4;       // float4 [F*M] world point, 1/weight
  size_t n4;       // float4 [F*M] perturbed world normal
  size_t d4;       // float4 [F*M] world delta / |n + scale delta| (backward only)
  size_t b4;       // float4 [F] facet bundle centre, radius (scenes with obstructions)
  size_t n_b4;     // entries of b4 (0: no obstructions, no culling)
  size_t acc;      // double: [rows * P] render accumulator, or the gradient buckets
  size_t masks;    // uint32 [S * F] candidate word per (source, facet) pair (renders of <= 32 primitives)
  size_t n_masks;  // entries of masks (0: none)
  size_t total;
  int n_table_floats;
};
constexpr int kFacetGrad = 13;  // per facet: dL/dR world-frame H (9), dL/dpos (3), dL/dscale (1)
constexpr int kMirGrad = 22;    // per stage mirror: dL/dR (9), dL/dpos (3), dL/dc, dL/dk, dL/da (8)
// Later-stage reflections the adjoint keeps per ray for its reverse sweep:
// the last kAdjRing (a ring, a power of two); the reverse of an earlier
// stage re-traces the ray from the primary to that stage. The batched
// adjoint takes scenes of at most kAdjRing later stages.
constexpr int kAdjRing = 2;
WsLayout workspace_layout(const iact_scene_t* sc, size_t acc_elems, bool with_delta, size_t mask_words = 0);
// candidate words a render of S sources keeps per (source, facet) pair:
// S * F for scenes of 1..32 shadowing primitives while that is at most 2^26,
// else 0 (the render then keeps per-tile masks)
size_t pair_mask_words(const iact_scene_t* sc, int S);
size_t acc_elems(const iact_sensor_t* sn, int S, int mode);  // 0 for DEBUG
WsLayout workspace_for(const iact_scene_t* sc, const iact_sensor_t* sn, int S, int mode);

struct DevInfo {
  int sm_count = 0;
  int smem_optin = 0;
};
DevInfo device_info();
// CTAs of `kern` an SM holds at (block, smem), cached per device and launch
// shape; raises the kernel's dynamic shared-memory limit when smem > 48 KiB.
int resident_ctas(const void* kern, int block, size_t smem, int* per_sm);
// zero / zero_bytes: a region the prep launch clears; counter: 16 ints it clears
int launch_prep(const iact_scene_t* sc, const WsLayout& L, char* ws, cudaStream_t st, bool with_delta,
                void* zero = nullptr, size_t zero_bytes = 0, int* counter = nullptr);
void host_euler(const float* deg, float* R);
SensorK make_sensor(const iact_sensor_t* s);

// Work-tile shape (sources x facets x 32-sample chunks) for a block of
// `block` threads: fills p.SB, FC, CC, n_fchunk, n_cchunk, n_tiles from
// p.F, p.M, p.S and the opts knobs; without explicit knobs the tile shrinks
// (down to one task per warp) until there are at least `min_tiles`.
// sb_fixed > 0 fixes the sources per tile (32 for the source-per-lane body).
int plan_tiles(RenderK& p, int mode, int block, const iact_opts_t* opts, long long min_tiles,
               int sb_fixed = 0);
// Shared-memory plan of one render: tables, int16 hex lookup table (if it
// fits in half the budget) and FP32 histogram rows (if they fit). Floors let
// a batch reserve the largest table sizes of all its jobs.
struct SmemPlan {
  size_t tab_bytes = 0, htab_bytes = 0, hist_bytes = 0;
  int hex_in_smem = 0, rows_in_smem = 0;
};
int plan_smem(const iact_sensor_t* sn, int n_table_floats, int SB, int mode, int hist_mode, size_t budget,
              size_t tab_floor, size_t htab_floor, SmemPlan& sp);
RenderK base_params(const iact_scene_t* sc, const iact_sensor_t* sn, const WsLayout& L, char* ws,
                    const float* sources, const float* values, int S);
PrepK prep_params(const iact_scene_t* sc, const WsLayout& L, char* ws, bool with_delta);
int n_primitives(const iact_scene_t* sc);  // obstruction primitives of all kinds

int launch_render(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                  const float* sources, const float* values, int S, int mode, float* out,
                  void* ws, size_t ws_bytes, const iact_opts_t* opts, cudaStream_t stream);
int launch_debug(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                 const float* sources, const float* values, int S, float* pts, float* vals,
                 int32_t* pix, int32_t* hit_mirror, void* ws, size_t ws_bytes, uint32_t seed,
                 cudaStream_t stream);

int launch_probe_fma(float* out, int blocks, int iters, cudaStream_t stream);
int launch_backward(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type, const float* sources,
                    const float* values, int S, int mode, const float* grad_out, float* g_rot, float* g_pos,
                    float* g_scale, float* g_src, float* g_val, float* g_mrot, float* g_mpos, float* g_msurf,
                    float* g_samples, void* ws, size_t ws_bytes, const iact_opts_t* opts, cudaStream_t stream);

}  // namespace iact
