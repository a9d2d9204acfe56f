// C ABI entry points (include/iactrace_gb300.h): argument validation,
// thread-local error messages, workspace sizing and dispatch.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <string>

#include "iact_device.cuh"
#include "iact_internal.h"

namespace iact {

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return IACT_OK;
  return set_error(IACT_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int validate_scene(const iact_scene_t* sc) {
  if (!sc) return set_error(IACT_E_INVALID, "scene is NULL");
  if (sc->n_facets < 0 || sc->n_samples < 0) return set_error(IACT_E_INVALID, "negative facet or sample count");
  if ((long long)sc->n_facets * sc->n_samples > (1LL << 30))
    return set_error(IACT_E_UNSUPPORTED, "more than 2^30 primary samples");
  if (sc->n_facets > 0 && sc->n_samples > 0) {
    if (!sc->facet_pos || !sc->facet_rot || !sc->facet_scale || !sc->points || !sc->normals || !sc->delta ||
        !sc->weights)
      return set_error(IACT_E_INVALID, "primary sample arrays must be non-NULL");
  }
  if (sc->n_mirrors < 0 || sc->n_mirrors > IACT_MAX_STAGE_MIRRORS)
    return set_error(IACT_E_UNSUPPORTED, "stage-mirror count outside [0, IACT_MAX_STAGE_MIRRORS]");
  if (sc->n_mirrors > 0 && !sc->mirrors) return set_error(IACT_E_INVALID, "mirrors is NULL");
  if (sc->n_stages < 0 || sc->n_stages > sc->n_mirrors || (sc->n_mirrors > 0 && sc->n_stages == 0))
    return set_error(IACT_E_INVALID, "n_stages must count the distinct stages of the mirror table");
  const int counts[5] = {sc->n_cyl, sc->n_box, sc->n_sph, sc->n_obox, sc->n_tri};
  const void* ptrs[5] = {sc->cyl, sc->box, sc->sph, sc->obox, sc->tri};
  long long total = 0;
  for (int i = 0; i < 5; ++i) {
    if (counts[i] < 0) return set_error(IACT_E_INVALID, "negative obstruction count");
    if (counts[i] > 0 && !ptrs[i]) return set_error(IACT_E_INVALID, "obstruction table is NULL");
    total += counts[i];
  }
  if (total > IACT_MAX_OBSTRUCTIONS) return set_error(IACT_E_UNSUPPORTED, "more than IACT_MAX_OBSTRUCTIONS primitives");
  return IACT_OK;
}

int validate_sensor(const iact_sensor_t* sn) {
  if (!sn) return set_error(IACT_E_INVALID, "sensor is NULL");
  if (sn->type < IACT_SENSOR_SQUARE || sn->type > IACT_SENSOR_SOFT_HEX)
    return set_error(IACT_E_INVALID, "unknown sensor type");
  if (sn->n_pixels <= 0) return set_error(IACT_E_INVALID, "sensor has no pixels");
  const bool square = sn->type == IACT_SENSOR_SQUARE || sn->type == IACT_SENSOR_SOFT_SQUARE;
  if (square) {
    if (sn->width <= 0 || sn->height <= 0 || (long long)sn->width * sn->height != sn->n_pixels)
      return set_error(IACT_E_INVALID, "square sensor: n_pixels != width * height");
    if (!(sn->dx > 0.f) || !(sn->dy > 0.f)) return set_error(IACT_E_INVALID, "square sensor: pixel pitch must be > 0");
  } else {
    if (!sn->table || sn->table_q <= 0 || sn->table_r <= 0)
      return set_error(IACT_E_INVALID, "hex sensor: lookup table missing");
    if ((long long)sn->table_q * sn->table_r > (1LL << 24))
      return set_error(IACT_E_UNSUPPORTED, "hex sensor: lookup table too large");
    if (!(sn->hex_size > 0.f) || !(sn->inradius > 0.f)) return set_error(IACT_E_INVALID, "hex sensor: bad hex size");
  }
  if (sn->type == IACT_SENSOR_SOFT_SQUARE || sn->type == IACT_SENSOR_SOFT_HEX) {
    if (!(sn->sigma > 0.f)) return set_error(IACT_E_INVALID, "soft sensor: sigma must be > 0");
    if (sn->kernel_size < 0 || sn->kernel_size > 4) return set_error(IACT_E_UNSUPPORTED, "soft sensor: kernel_size outside [0, 4]");
  }
  return IACT_OK;
}

namespace {

int check_common(const iact_scene_t* sc, const iact_sensor_t* sn, int32_t src_type, const float* sources,
                 const float* values, int32_t S, int mode, void* ws, size_t ws_bytes) {
  int rc = validate_scene(sc);
  if (rc) return rc;
  rc = validate_sensor(sn);
  if (rc) return rc;
  if (src_type != IACT_SRC_POINT && src_type != IACT_SRC_PARALLEL && src_type != IACT_SRC_EXTENDED)
    return set_error(IACT_E_INVALID, "source_type must be IACT_SRC_POINT, IACT_SRC_PARALLEL or IACT_SRC_EXTENDED");
  if (S < 0) return set_error(IACT_E_INVALID, "negative source count");
  if (S > 0 && (!sources || !values)) return set_error(IACT_E_INVALID, "sources/values are NULL");
  const WsLayout L = workspace_for(sc, sn, S, mode);
  if (!ws) return set_error(IACT_E_WORKSPACE, "workspace is NULL");
  if (reinterpret_cast<uintptr_t>(ws) % 256) return set_error(IACT_E_WORKSPACE, "workspace must be 256-byte aligned");
  if (ws_bytes < L.total)
    return set_error(IACT_E_WORKSPACE, "workspace too small: need " + std::to_string(L.total) + " bytes");
  return IACT_OK;
}

}  // namespace
}  // namespace iact

using namespace iact;

extern "C" {

int iact_abi_version(void) { return IACT_ABI_VERSION; }

const char* iact_last_error(void) { return g_last_error.c_str(); }

int64_t iact_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

// sizes of the ABI structs as this library sees them (bindings check theirs);
// a fifth slot receives sizeof(iact_job_t), a sixth sizeof(iact_sampler_t)
int iact_abi_layout(size_t* out, int n) {
  if (!out || n < 4) return set_error(IACT_E_INVALID, "iact_abi_layout needs room for 4 sizes");
  out[0] = sizeof(iact_scene_t);
  out[1] = sizeof(iact_sensor_t);
  out[2] = sizeof(iact_mirror_t);
  out[3] = sizeof(iact_opts_t);
  if (n >= 5) out[4] = sizeof(iact_job_t);
  if (n >= 6) out[5] = sizeof(iact_sampler_t);
  return IACT_OK;
}

int iact_probe_fma(float* out, int32_t blocks, int32_t iters, void* stream) {
  if (!out || blocks <= 0 || iters <= 0) return set_error(IACT_E_INVALID, "iact_probe_fma: bad arguments");
  return launch_probe_fma(out, blocks, iters, static_cast<cudaStream_t>(stream));
}

int iact_workspace_size(const iact_scene_t* scene, const iact_sensor_t* sensor, int32_t n_sources, int32_t mode,
                        size_t* bytes) {
  int rc = validate_scene(scene);
  if (rc) return rc;
  rc = validate_sensor(sensor);
  if (rc) return rc;
  if (!bytes) return set_error(IACT_E_INVALID, "bytes is NULL");
  if (n_sources < 0) return set_error(IACT_E_INVALID, "negative source count");
  if (mode != IACT_MODE_IMAGE && mode != IACT_MODE_RESPONSE && mode != IACT_MODE_DEBUG && mode != IACT_MODE_BACKWARD)
    return set_error(IACT_E_INVALID, "unknown mode");
  *bytes = workspace_for(scene, sensor, n_sources, mode).total;
  return IACT_OK;
}

int iact_render(const iact_scene_t* scene, const iact_sensor_t* sensor, int32_t source_type,
                const float* sources, const float* values, int32_t n_sources, int32_t mode, float* out,
                void* workspace, size_t workspace_bytes, const iact_opts_t* opts, void* stream) {
  if (mode != IACT_MODE_IMAGE && mode != IACT_MODE_RESPONSE)
    return set_error(IACT_E_INVALID, "mode must be IACT_MODE_IMAGE or IACT_MODE_RESPONSE");
  int rc = check_common(scene, sensor, source_type, sources, values, n_sources, mode, workspace, workspace_bytes);
  if (rc) return rc;
  if (!out && acc_elems(sensor, n_sources, mode) > 0) return set_error(IACT_E_INVALID, "out is NULL");
  if (mode == IACT_MODE_RESPONSE && (long long)n_sources * sensor->n_pixels > 0x7fffffffLL)
    return set_error(IACT_E_UNSUPPORTED, "response matrix larger than 2^31 entries");
  return launch_render(scene, sensor, source_type, sources, values, n_sources, mode, out, workspace,
                       workspace_bytes, opts, static_cast<cudaStream_t>(stream));
}

int iact_render_debug(const iact_scene_t* scene, const iact_sensor_t* sensor, int32_t source_type,
                      const float* sources, const float* values, int32_t n_sources, float* pts, float* vals,
                      int32_t* pix, int32_t* hit_mirror, void* workspace, size_t workspace_bytes, uint32_t seed,
                      void* stream) {
  int rc = check_common(scene, sensor, source_type, sources, values, n_sources, IACT_MODE_DEBUG, workspace,
                        workspace_bytes);
  if (rc) return rc;
  const long long n = (long long)scene->n_facets * n_sources * scene->n_samples;
  if (n > 0 && (!pts || !vals)) return set_error(IACT_E_INVALID, "pts/vals are NULL");
  return launch_debug(scene, sensor, source_type, sources, values, n_sources, pts, vals, pix, hit_mirror,
                      workspace, workspace_bytes, seed, static_cast<cudaStream_t>(stream));
}

int iact_render_backward(const iact_scene_t* scene, const iact_sensor_t* sensor, int32_t source_type,
                         const float* sources, const float* values, int32_t n_sources, int32_t mode,
                         const float* grad_out, float* g_facet_rot, float* g_facet_pos, float* g_facet_scale,
                         float* g_sources, float* g_values, float* g_mirror_rot, float* g_mirror_pos,
                         float* g_mirror_surface, float* g_samples, void* workspace, size_t workspace_bytes,
                         const iact_opts_t* opts, void* stream) {
  if (mode != IACT_MODE_IMAGE && mode != IACT_MODE_RESPONSE)
    return set_error(IACT_E_INVALID, "mode must be IACT_MODE_IMAGE or IACT_MODE_RESPONSE");
  int rc = check_common(scene, sensor, source_type, sources, values, n_sources, IACT_MODE_BACKWARD, workspace,
                        workspace_bytes);
  if (rc) return rc;
  if (source_type == IACT_SRC_EXTENDED && g_sources)
    return set_error(IACT_E_UNSUPPORTED, "iact_render_backward: no source gradients for extended sources");
  if (!grad_out && acc_elems(sensor, n_sources, mode) > 0) return set_error(IACT_E_INVALID, "grad_out is NULL");
  return launch_backward(scene, sensor, source_type, sources, values, n_sources, mode, grad_out, g_facet_rot,
                         g_facet_pos, g_facet_scale, g_sources, g_values, g_mirror_rot, g_mirror_pos,
                         g_mirror_surface, g_samples, workspace, workspace_bytes, opts,
                         static_cast<cudaStream_t>(stream));
}

}  // extern "C"
