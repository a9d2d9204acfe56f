// Host-side internals shared by the translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/iactrace_gb300.h"

namespace iact {

// thread-local message behind iact_last_error(); returns `code`
int set_error(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

// validation of the descriptors shared by every entry point
int validate_scene(const iact_scene_t* sc);
int validate_sensor(const iact_sensor_t* sn);

// workspace layout (bytes from the workspace base, all 256-byte aligned)
struct WsLayout {
  size_t counter;  // int32 tile counter + int32 error word
  size_t tables;   // processed obstruction/mirror/sensor records (floats)
  size_t p4;       // float4 [F*M] world point, 1/weight
  size_t n4;       // float4 [F*M] perturbed world normal
  size_t acc;      // double [rows * P] FP64 accumulator of the render
  size_t total;
  int n_table_floats;
};
WsLayout workspace_layout(const iact_scene_t* sc, size_t acc_elems);
size_t acc_elems(const iact_sensor_t* sn, int S, int mode);  // mode < 0: debug (none)

int launch_render(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                  const float* sources, const float* values, int S, int mode, float* out,
                  void* ws, size_t ws_bytes, const iact_opts_t* opts, cudaStream_t stream);
int launch_debug(const iact_scene_t* sc, const iact_sensor_t* sn, int src_type,
                 const float* sources, const float* values, int S, float* pts, float* vals,
                 int32_t* pix, int32_t* hit_mirror, void* ws, size_t ws_bytes,
                 cudaStream_t stream);

int launch_probe_fma(float* out, int blocks, int iters, cudaStream_t stream);

}  // namespace iact
