/*
 * iactrace_gb300 — C ABI of the GB300 (sm_103a) render path of IACTrace.
 *
 * One call traces Monte-Carlo rays (source s, primary facet f, sample m)
 * from the sampled primary-mirror points through obstruction shadowing,
 * reflection, optional later mirror stages and the sensor plane, and bins
 * them into a square or hexagonal pixel image.
 *
 * Conventions
 *   - Every pointer inside iact_scene_t / iact_sensor_t and every array
 *     argument is a DEVICE pointer (caller-owned, e.g. torch CUDA tensors),
 *     except the descriptor structs themselves, which live in host memory
 *     and are read only during the call.
 *   - Calls are stream-ordered on `stream` (a cudaStream_t passed as void*;
 *     NULL = legacy default stream). They never synchronise the device.
 *   - The callee allocates nothing: scratch memory is the caller's
 *     `workspace` of at least iact_workspace_size() bytes.
 *   - Return value: IACT_OK (0) or a negative IACT_E_* status. The message
 *     of the last failure on the calling thread is iact_last_error().
 *   - Layout: float32 everywhere, row-major, xyz innermost. Angles are
 *     Euler degrees (tip, tilt, rotation), R = Rz * Ry * Rx.
 *
 * Reference interface replaced (GerritRo/iactrace v0.4.0, JAX):
 *   iact_render(IMAGE)     <- core/render.py:174-220  render()
 *                             (telescope/telescope.py:56-83 Telescope.__call__)
 *   iact_render(RESPONSE)  <- core/render.py:271-324  render_response_matrix()
 *   iact_render_debug      <- core/render.py:223-268  render_debug()
 *   iact_render_backward   <- jax.grad of render() / render_response_matrix()
 *                             (no dedicated reference function)
 *   iact_batch_*           <- a Python loop (or jax.vmap) of Telescope.__call__
 *                             over telescope variants (no reference function)
 *   iact_sample_facets     <- core/integrators.py:97-187 MCIntegrator.sample_group
 *                             (counter-based streams instead of threefry)
 */
#ifndef IACTRACE_GB300_H
#define IACTRACE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IACT_ABI_VERSION 3

/* status codes */
#define IACT_OK 0
#define IACT_E_INVALID (-1)     /* bad argument (null pointer, size, enum)  */
#define IACT_E_UNSUPPORTED (-2) /* valid request the library cannot serve   */
#define IACT_E_CUDA (-3)        /* CUDA runtime error (launch/config)       */
#define IACT_E_WORKSPACE (-4)   /* workspace missing, too small, misaligned */
#define IACT_E_DEVICE (-5)      /* a kernel-side check failed (see message) */

/* limits of the packed tables */
#define IACT_MAX_ASPH 8          /* aspheric coefficients per surface      */
#define IACT_MAX_POLY 8          /* polygon aperture vertices              */
#define IACT_MAX_STAGE_MIRRORS 64 /* mirrors over all stages >= 1          */
#define IACT_MAX_OBSTRUCTIONS 2048 /* primitives over all obstruction kinds */

/* EXTENDED: a parallel source with a Gaussian angular profile; sources are
 * [S,4] = (direction xyz, sigma in radians); each ray's direction is the
 * normalised direction tilted by sigma * (z0, z1) in its tangent plane, with
 * (z0, z1) ~ N(0,1) from Philox4x32-10 keyed on (opts->seed, s, f, m). */
enum { IACT_SRC_POINT = 0, IACT_SRC_PARALLEL = 1, IACT_SRC_EXTENDED = 2 };
enum { IACT_MODE_IMAGE = 0, IACT_MODE_RESPONSE = 1, IACT_MODE_DEBUG = 2, IACT_MODE_BACKWARD = 3 };
enum {
  IACT_SENSOR_SQUARE = 0,      /* sensors/square.py:28-91     SquareSensor */
  IACT_SENSOR_HEX = 1,         /* sensors/hexagonal.py:104-194 HexagonalSensor */
  IACT_SENSOR_SOFT_SQUARE = 2, /* sensors/square.py:94-172 DifferentiableSquareSensor */
  IACT_SENSOR_SOFT_HEX = 3     /* sensors/hexagonal.py:197-315 DifferentiableHexagonalSensor */
};
enum { IACT_APERTURE_DISK = 0, IACT_APERTURE_POLYGON = 1 };

/* One mirror of an optical stage >= 1 (telescope/mirrors.py:101-229). */
typedef struct {
  int32_t stage;    /* optical stage, >= 1; the table is sorted by stage  */
  int32_t aperture; /* IACT_APERTURE_*                                     */
  int32_t n_asph;   /* aspheric coefficients in use (<= IACT_MAX_ASPH)     */
  int32_t n_vert;   /* polygon vertices in use (<= IACT_MAX_POLY)          */
  float pos[3];
  float rot[3];     /* Euler degrees */
  float offset[2];  /* (x0, y0) on the parent surface */
  float curvature, conic;
  float asph[IACT_MAX_ASPH]; /* coefficient i multiplies r^(4(i+1)) */
  float radius;              /* disk aperture radius */
  float vert[IACT_MAX_POLY][2];
  float pad_[5];
} iact_mirror_t; /* 176 bytes */

/* Scene: primary samples, later stages, obstructions. */
typedef struct {
  /* stage-0 facets, all primary groups concatenated (core/render.py:202-205) */
  int32_t n_facets;  /* F */
  int32_t n_samples; /* M (same for every facet) */
  const float* facet_pos;   /* [F,3] */
  const float* facet_rot;   /* [F,3] Euler degrees */
  const float* facet_scale; /* [F]   perturbation scale, radians */
  const float* points;      /* [F,M,3] local sample points */
  const float* normals;     /* [F,M,3] local unit normals */
  const float* delta;       /* [F,M,3] local unit-sigma perturbation deltas */
  const float* weights;     /* [F,M]   sample weights */
  /* stages >= 1, flattened in (stage, group, mirror) order */
  int32_t n_mirrors;
  int32_t n_stages; /* distinct stage values among the mirrors */
  const iact_mirror_t* mirrors; /* [n_mirrors] */
  /* obstructions (core/obstructions.py) */
  int32_t n_cyl, n_box, n_sph, n_obox, n_tri;
  const float* cyl;  /* [n_cyl,7]  p1(3) p2(3) r          */
  const float* box;  /* [n_box,6]  p1(3) p2(3)            */
  const float* sph;  /* [n_sph,4]  center(3) r            */
  const float* obox; /* [n_obox,15] center(3) half(3) R(9), R row-major local->world */
  const float* tri;  /* [n_tri,9]  v0(3) v1(3) v2(3)      */
} iact_scene_t;

/* Sensor plane + pixelisation. Constants are the float32 values the
 * reference computes at sensor construction. */
typedef struct {
  int32_t type;     /* IACT_SENSOR_* */
  int32_t n_pixels; /* accumulator size: width*height or hex pixel count */
  int32_t width, height;
  float pos[3];
  float rot[3]; /* Euler degrees */
  /* square (both kinds) */
  float x0, y0, dx, dy, edge_width;
  /* hexagonal (both kinds) */
  float hex_size, inradius, grid_cos, grid_sin, off_x, off_y;
  float hex_sx, hex_sy; /* size*sqrt(3) and size*1.5 (axial -> Cartesian) */
  float edge_threshold; /* 1 - edge_width / inradius */
  int32_t q_min, r_min, table_q, table_r;
  const int32_t* table; /* [table_q, table_r] pixel id or -1 */
  /* soft deposition (Differentiable* sensors) */
  float sigma;
  int32_t kernel_size;
} iact_sensor_t;

/* Shadow tests of a warp's 32 rays are restricted to the primitives whose
 * bounding volume comes near the rays' common bundle (exact: identical
 * shadow masks); this flag tests every primitive on every ray instead. */
#define IACT_FLAG_NO_CULL 1
/* iact_batch_create: also plan iact_batch_backward (workspace for the
 * gradient buckets of every job) */
#define IACT_FLAG_BATCH_BACKWARD 2

/* Optional launch knobs; NULL or zeros select the built-in defaults. */
typedef struct {
  int32_t block_threads;    /* threads per CTA (multiple of 32)           */
  int32_t sources_per_cta;  /* sources per work tile (0: half the warps of a
                               CTA for RESPONSE renders, else all)       */
  int32_t facets_per_tile;  /* primary facets per work tile               */
  int32_t hist_mode;        /* 0 auto, 1 shared-memory rows, 2 global     */
  int32_t tasks_per_warp;   /* 32-ray tasks per warp per work tile (0: 192 for
                               hard-pixel RESPONSE renders and RESPONSE
                               adjoints, else 48, halved for small launches
                               down to 4 tiles per SM, 12 for hard-pixel
                               IMAGE renders of at most 32 primitives)   */
  int32_t flags;            /* IACT_FLAG_* bits                           */
  uint32_t seed;            /* jitter stream of EXTENDED sources            */
  /* optional cudaEvent_t pair recorded on `stream` right before and after
   * the render kernel (profiling; for hard-pixel renders of at most 32
   * primitives the window also holds the candidate-mask launch before it);
   * NULL to skip */
  void* kernel_events[2];
} iact_opts_t;

int iact_abi_version(void);
const char* iact_last_error(void);
/* sizeof(iact_scene_t), sizeof(iact_sensor_t), sizeof(iact_mirror_t),
 * sizeof(iact_opts_t) and, if n >= 5, sizeof(iact_job_t), if n >= 6,
 * sizeof(iact_sampler_t) as compiled into the library (binding self-check). */
int iact_abi_layout(size_t* out, int n);

/* Diagnostics: runs `iters` dependent FP32 FMAs per thread over
 * `blocks` x 256 threads (a throughput probe of the FP32 pipe) and writes
 * one float per thread to out[blocks*256]. */
int iact_probe_fma(float* out, int32_t blocks, int32_t iters, void* stream);

/* Diagnostics: kernels this library has queued, on any stream and thread,
 * since it was loaded. Launches made while a stream is being captured into
 * a CUDA graph are counted once, at capture; the graph's replays are not. */
int64_t iact_kernel_launches(void);

/* Bytes of scratch needed by a call of the given mode (IMAGE / RESPONSE:
 * iact_render, DEBUG: iact_render_debug) on this scene, sensor and source
 * count. Holds the world-space samples, the per-launch tables and the FP64
 * accumulator of the image or matrix. */
int iact_workspace_size(const iact_scene_t* scene, const iact_sensor_t* sensor,
                        int32_t n_sources, int32_t mode, size_t* bytes);

/* Forward render.
 *   mode IMAGE:    out[n_pixels]            (fully written by the callee)
 *   mode RESPONSE: out[n_sources, n_pixels] (fully written by the callee)
 * Hits are summed per work tile in FP32 shared memory, across tiles in an
 * FP64 accumulator, and rounded to FP32 once at the end.
 * sources [S,3]: positions (POINT) or propagation directions (PARALLEL,
 * used as given, not normalised); values [S]. */
int iact_render(const iact_scene_t* scene, const iact_sensor_t* sensor,
                int32_t source_type, const float* sources, const float* values,
                int32_t n_sources, int32_t mode, float* out, void* workspace,
                size_t workspace_bytes, const iact_opts_t* opts, void* stream);

/* Forward render without a caller workspace; it has no counterpart in the
 * reference (JAX allocates internally). For callers that cannot allocate
 * device memory (device memory owned by another framework's pool, real-time
 * acquisition loops that must not allocate): the scratch is a fixed
 * IACT_NOALLOC_SCRATCH_BYTES array inside the library, held by every GPU
 * that loads it until exit. Larger requests fail with IACT_E_UNSUPPORTED.
 * The first call per device resolves the array's address (make it before
 * any stream capture) and keeps it for the process: after a
 * cudaDeviceReset of that device this entry point must not be called on it
 * again. Calls overlapping on the GPU race on the shared array. Arguments
 * and results as iact_render. */
#define IACT_NOALLOC_SCRATCH_BYTES (16u << 20)
int iact_render_noalloc(const iact_scene_t* scene, const iact_sensor_t* sensor,
                        int32_t source_type, const float* sources,
                        const float* values, int32_t n_sources, int32_t mode,
                        float* out, const iact_opts_t* opts, void* stream);

/* Per-ray hits in the reference's order, ray = (f*S + s)*M + m:
 *   pts [F*S*M,2] sensor-plane (x, y) or (1e10, 1e10); vals [F*S*M];
 *   pix [F*S*M] hard pixel id or -1 (may be NULL);
 *   hit_mirror [F*S*M] index into scene->mirrors of the last stage's hit,
 *   -1 for a miss or a single-stage scene (may be NULL). */
int iact_render_debug(const iact_scene_t* scene, const iact_sensor_t* sensor,
                      int32_t source_type, const float* sources,
                      const float* values, int32_t n_sources, float* pts,
                      float* vals, int32_t* pix, int32_t* hit_mirror,
                      void* workspace, size_t workspace_bytes, uint32_t seed,
                      void* stream);

/* Adjoint of iact_render (mode IMAGE or RESPONSE), through any number of
 * mirror stages after the primary: given grad_out = dL/d(out), writes
 * dL/d(facet rotations) [F,3] (per degree), dL/d(facet positions) [F,3],
 * dL/d(facet perturbation scales) [F], dL/d(sources) [S,3], dL/d(values)
 * [S], per stage mirror dL/d(rotation) [n_mirrors,3], dL/d(position)
 * [n_mirrors,3] and dL/d(curvature, conic, aspheric[8]) [n_mirrors,10], and
 * per primary sample (g_samples [F*M,7]) dL/d(world point) (3), dL/d(unit
 * perturbed world normal) (3) and dL/d(1/weight) (1), summed over the
 * sources, for gradients that flow through the sample arrays (primary
 * surface parameters via resampling); any output may be NULL. Each
 * ray's forward path is recomputed, nothing is stored between the calls.
 * Pixel ids and shadow masks carry no gradient (as under jax.grad); soft
 * sensors also pass gradients through the sensor-plane position. Workspace:
 * iact_workspace_size(..., IACT_MODE_BACKWARD, ...). Replaces jax.grad of
 * core/render.py:174-220 / :271-324 (no dedicated reference function). */
int iact_render_backward(const iact_scene_t* scene, const iact_sensor_t* sensor,
                         int32_t source_type, const float* sources,
                         const float* values, int32_t n_sources, int32_t mode,
                         const float* grad_out, float* g_facet_rot,
                         float* g_facet_pos, float* g_facet_scale,
                         float* g_sources, float* g_values,
                         float* g_mirror_rot, float* g_mirror_pos,
                         float* g_mirror_surface, float* g_samples,
                         void* workspace, size_t workspace_bytes,
                         const iact_opts_t* opts, void* stream);

/* ---- Batched persistent render -------------------------------------------
 * Many telescope variants and source sets of uneven size in one persistent
 * launch. A batch is a fixed list of jobs, each one iact_render call (own
 * scene, sensor, source count and output); all jobs share source_type and
 * mode. One persistent kernel per template class (hard/soft sensor x
 * with/without later mirror stages) walks a global queue of (job, source
 * block, facet chunk, 32-sample chunk) tiles, largest jobs first; a CTA
 * restages the job's tables in shared memory when its next tile belongs to
 * another job. Results equal iact_render's per job up to FP64 summation order.
 * No reference counterpart: the reference renders variants by a Python loop
 * (or jax.vmap) over Telescope.__call__ (telescope/telescope.py:56-83). */
typedef struct {
  const iact_scene_t* scene;   /* host descriptor of device arrays          */
  const iact_sensor_t* sensor; /* host descriptor of a device lookup table  */
  const float* sources;        /* device [S,3] ([S,4] for EXTENDED)         */
  const float* values;         /* device [S]                                */
  int32_t n_sources;
  uint32_t seed;               /* jitter stream of EXTENDED sources         */
  float* out;                  /* device [P] (IMAGE) or [S,P] (RESPONSE)    */
  /* iact_batch_backward only (batches created with IACT_FLAG_BATCH_BACKWARD):
   * dL/d(out) in, gradients out as in iact_render_backward; outputs may be
   * NULL */
  const float* grad_out;
  float* g_facet_rot;
  float* g_facet_pos;
  float* g_facet_scale;
  float* g_sources;
  float* g_values;
  float* g_mirror_rot;
  float* g_mirror_pos;
  float* g_mirror_surface;
} iact_job_t;

typedef struct iact_batch iact_batch;

/* Validates every job and plans tiles and shared memory from opts
 * (block_threads, tasks_per_warp, hist_mode, kernel_events; the per-call
 * sources_per_cta, facets_per_tile and seed are not used). Copies the
 * descriptors: the device arrays they name must outlive the batch. Host
 * only, no CUDA call. */
int iact_batch_create(const iact_job_t* jobs, int32_t n_jobs, int32_t source_type,
                      int32_t mode, const iact_opts_t* opts, iact_batch** out);
int iact_batch_workspace_size(const iact_batch* batch, size_t* bytes);
/* Binds the workspace (256-byte aligned) and queues the upload of the job
 * table on `stream`; sets the kernels' shared-memory limits and grids. */
int iact_batch_prepare(iact_batch* batch, void* workspace, size_t workspace_bytes,
                       void* stream);
/* Renders every job into its out: memsets and kernel launches on `stream`
 * only (no allocation, no host synchronisation), so the call can be
 * captured in a CUDA graph and replayed. Job arrays (samples, facet
 * parameters, sources, values) are read when the kernels run. */
int iact_batch_render(iact_batch* batch, void* stream);
/* Adjoint of iact_batch_render for every job of a batch created with
 * IACT_FLAG_BATCH_BACKWARD: reads each job's grad_out, writes its gradient
 * outputs (as iact_render_backward, same limits). Recomputes the forward
 * paths; one persistent launch per template class over all jobs' adjoint
 * tiles; capture-safe like iact_batch_render. */
int iact_batch_backward(iact_batch* batch, void* stream);
/* out[0] jobs, out[1] work tiles, out[2] rays, out[3] kernel launches per
 * iact_batch_render, out[4] template classes used, out[5] adjoint tiles,
 * out[6] kernel launches per iact_batch_backward */
int iact_batch_info(const iact_batch* batch, int64_t* out, int32_t n);
void iact_batch_destroy(iact_batch* batch);

/* ---- Monte-Carlo facet sampling on the device -----------------------------
 * One stage-0 mirror group (shared aspheric surface, per-facet disk radius or
 * convex polygon and offset) sampled as core/integrators.py:97-187
 * MCIntegrator.sample_group does: uniform points on the aperture
 * (utils/sampling.py:8-67: r = sqrt(u) disk, or an area-weighted fan
 * triangle of the polygon), lifted to the surface (core/surfaces.py:41-65),
 * unit normals, unit-sigma roughness deltas in the tangent plane
 * (core/reflection.py:22-49) and weights cos_z / area * n_samples. The
 * variates come from Philox4x32-10 keyed by (seed, facet, sample), so any
 * host can replay them; the arithmetic is FP64, stored as float32. */
typedef struct {
  int32_t n_facets, n_samples;
  int32_t aperture;           /* IACT_APERTURE_DISK or IACT_APERTURE_POLYGON */
  int32_t n_vert;             /* polygon vertices, 3..IACT_MAX_POLY          */
  float curvature, conic;
  int32_t n_asph;
  float asph[IACT_MAX_ASPH];
  const float* offsets;       /* device [F,2]                                */
  const float* radii;         /* device [F] (disk)                           */
  const float* vertices;      /* device [F, n_vert, 2] (polygon, convex)     */
  uint32_t seed;
  const float* surface;       /* optional device [2 + n_asph]: curvature,
                                 conic, aspheric coefficients, read on the
                                 device instead of the values above (a
                                 captured launch then follows updates)      */
} iact_sampler_t;

/* points, normals, delta: device [F, M, 3]; weights: device [F, M] */
int iact_sample_facets(const iact_sampler_t* sampler, float* points, float* normals,
                       float* delta, float* weights, void* stream);

/* Reverse of iact_sample_facets with respect to the shared surface: given
 * dL/d(points, normals, delta, weights) of the sampled arrays (device, same
 * shapes; any may be NULL = zero), writes dL/d(curvature, conic, aspheric
 * coefficients) to g_surface (device, 2 + n_asph doubles). The aperture
 * positions and roughness coefficients are the forward's (same seed); the
 * surface enters through the points' sag, the normals, the tangent-plane
 * deltas and the weights (core/surfaces.py:25-65, core/reflection.py:22-49,
 * core/integrators.py:124-127). Replaces the reference's autodiff of
 * MCIntegrator.sample_group (core/integrators.py:97-187). */
int iact_sample_facets_backward(const iact_sampler_t* sampler, const float* g_points,
                                const float* g_normals, const float* g_delta,
                                const float* g_weights, double* g_surface, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* IACTRACE_GB300_H */
