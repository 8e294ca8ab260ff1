/*
 * muon_gpu.h — C ABI of the GB300 rendering library (libmuon_gpu.so).
 *
 * The library replaces the body of the reference renderer's sample loop
 * (muon/renderer.cc:41-76: per sample Camera::CastRay -> Integrator::Trace ->
 * Film::SetPixel) with one call that renders a whole film on one GPU, and it
 * exposes the reference's acceleration-structure seam
 * (acceleration::Structure::Intersect / HasIntersection, muon/acceleration.h:
 * 44-49) as batched ray queries. Host code above this ABI (the `.muon` parser,
 * the `muon` CLI, film output) lives in the same library.
 *
 * Conventions
 *   - Every entry point returns an int status: MUON_OK (0) or a MUON_ERR_*
 *     code; muon_gpu_last_error() returns a thread-local message for the last
 *     failure on the calling thread. No C++ exception crosses the ABI.
 *   - Host arrays passed in are only read during the call; the library keeps
 *     its own copies. Arrays passed out are caller-allocated.
 *   - All vectors are float[3] in world space unless noted; matrices are
 *     column-major float[16] (column c occupies m[4c..4c+3]).
 *   - There is no CPU fallback: without a usable CUDA device the GPU entry
 *     points fail with MUON_ERR_CUDA.
 *   - Calls on one MuonScene are serialised by the caller; distinct scenes may
 *     be used from different host threads. Each scene owns one CUDA stream.
 */
#ifndef MUON_GPU_H_
#define MUON_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define MUON_OK 0
#define MUON_ERR_INVALID_ARG 1 /* bad handle, pointer, size or enum          */
#define MUON_ERR_OOM 2         /* host or device allocation failed           */
#define MUON_ERR_CUDA 3        /* CUDA runtime error / no device             */
#define MUON_ERR_TIMEOUT 4     /* a bounded device wait gave up              */
#define MUON_ERR_PARSE 5       /* scene file unreadable or unusable          */
#define MUON_ERR_IO 6          /* output file could not be written           */

/* ---- enums (values follow the reference's enum order) ----------------- */
/* Integrator types selected by the `integrator` scene command
 * (muon/parser.cc:330-355, classes in muon/integration.h:51-176). */
#define MUON_INTEGRATOR_NORMALS 0
#define MUON_INTEGRATOR_ALBEDO 1
#define MUON_INTEGRATOR_DEPTH 2
#define MUON_INTEGRATOR_RAYTRACER 3
#define MUON_INTEGRATOR_ANALYTIC_DIRECT 4
#define MUON_INTEGRATOR_PATHTRACER 5
/* muon/nee.h:7-14 */
#define MUON_NEE_OFF 0
#define MUON_NEE_ON 1
#define MUON_NEE_MIS 2
/* muon/importance_sampling.h:7-14 */
#define MUON_IS_HEMISPHERE 0
#define MUON_IS_COSINE 1
#define MUON_IS_BRDF 2
/* muon/brdf_type.h:7-14 */
#define MUON_BRDF_LAMBERTIAN 0
#define MUON_BRDF_PHONG 1
#define MUON_BRDF_GGX 2
/* muon/lighting.h:49-83 */
#define MUON_LIGHT_DIRECTIONAL 0
#define MUON_LIGHT_POINT 1
#define MUON_LIGHT_QUAD 2
/* muon/acceleration_type.h:11-28 */
#define MUON_ACCEL_LINEAR 0
#define MUON_ACCEL_BVH 1
#define MUON_PARTITION_UNIFORM 0
#define MUON_PARTITION_MIDPOINT 1
#define MUON_PARTITION_SAH 2
/* Primitive intersection arithmetic of the traversal kernels.
 *   FAST        the reference's triangle test (plane + three edge functions,
 *               muon/objects.cc:58-175) and sphere test on world-space data,
 *               with fused multiply-adds; hits equal the reference's except at
 *               rounding edges.
 *   WATERTIGHT  the watertight ray/triangle test of Woop, Benthin and Wald
 *               (JCGT 2013); spheres as FAST.
 *   EXACT       the reference's arithmetic bit for bit: each primitive is
 *               tested in its object space with the ray carried by the inverse
 *               transform and its direction re-normalised (muon/objects.cc:
 *               29-46, muon/transform.h:13-18), no fused multiply-adds, the
 *               distance measured back in world space. Slower for transformed
 *               primitives. */
#define MUON_ISECT_FAST 0
#define MUON_ISECT_WATERTIGHT 1
#define MUON_ISECT_EXACT 2

/* BVH builders (MuonSceneDesc.builder). HOST_SAH: binned SAH on the host
 * threads (acceleration and partition_strategy apply). GPU_LBVH: linear BVH
 * over Morton-sorted centroids on the device (Karras 2012), leaves of at most
 * 4 primitives; much faster to build, somewhat slower to traverse. GPU_SAH:
 * the host builder's binned SAH run on the device, with the same split
 * decisions and so the same nodes and boxes (references inside a leaf keep
 * their input order, nodes are numbered differently); partition_strategy
 * must be SAH, max_leaf_size applies. */
#define MUON_BUILDER_HOST_SAH 0
#define MUON_BUILDER_GPU_LBVH 1
#define MUON_BUILDER_GPU_SAH 2

/* render flags */
#define MUON_RENDER_STATS 1u      /* count bounds/object tests (slower)        */
#define MUON_RENDER_ACCUMULATE 2u /* add into the caller's film, do not zero   */
#define MUON_RENDER_TIMING 4u     /* time every kernel with CUDA events (the   */
                                  /* wavefronts then run one at a time)         */
#define MUON_RENDER_NO_GRAPH 8u   /* launch kernel by kernel, no CUDA graph    */

/* ---- scene description (flattened muon::Scene, muon/scene.h:22-95) ---- */
typedef struct MuonTransformDesc {
  float object_to_world[16]; /* Primitive::transform                     */
  float world_to_object[16]; /* Primitive::inv_transform                 */
  float normal_to_world[16]; /* Primitive::inv_transpose_transform       */
} MuonTransformDesc;

typedef struct MuonMaterialDesc { /* muon::Material, muon/materials.h:125-148 */
  float ambient[3];
  float diffuse[3];
  float specular[3];
  float emission[3];
  float shininess;
  float roughness;
  int32_t brdf; /* MUON_BRDF_*: the BRDF actually instantiated */
  int32_t pad;
} MuonMaterialDesc;

typedef struct MuonLightDesc { /* muon/lighting.h:36-83 */
  int32_t type;                /* MUON_LIGHT_*                             */
  float color[3];
  float p0[3]; /* quad: corner | point: position | directional: direction */
  float p1[3]; /* quad: edge0  | point: attenuation (const, lin, quad)    */
  float p2[3]; /* quad: edge1                                             */
} MuonLightDesc;

typedef struct MuonTriangleDesc { /* muon::Tri, muon/objects.h:62-86 */
  float v[3][3];      /* object-space vertex positions                 */
  float n[3][3];      /* vertex normals, used when smooth != 0         */
  int32_t transform;  /* index into transforms; -1 = identity          */
  int32_t material;   /* index into materials                          */
  int32_t light;      /* quad light this triangle represents; -1 = none */
  int32_t smooth;     /* interpolate vertex normals                    */
  int32_t prim_id;    /* primitive index in scene-file (parse) order   */
  int32_t pad;
} MuonTriangleDesc;

typedef struct MuonSphereDesc { /* muon::Sphere, muon/objects.h:89-98 */
  float center[3];
  float radius;
  int32_t transform;
  int32_t material;
  int32_t prim_id;
  int32_t pad;
} MuonSphereDesc;

typedef struct MuonCameraDesc { /* muon::Camera, muon/camera.h:9-32 */
  float eye[3];
  float look_at[3];
  float up[3];
  float fov_y_degrees;
  int32_t width; /* the film size in effect when the camera was declared */
  int32_t height;
} MuonCameraDesc;

typedef struct MuonSceneDesc {
  int32_t width, height; /* film size */
  MuonCameraDesc camera;
  const MuonTransformDesc *transforms;
  int32_t num_transforms;
  const MuonMaterialDesc *materials;
  int32_t num_materials;
  const MuonLightDesc *lights;
  int32_t num_lights;
  const MuonTriangleDesc *triangles;
  int64_t num_triangles;
  const MuonSphereDesc *spheres;
  int64_t num_spheres;
  int32_t acceleration;       /* MUON_ACCEL_*                       */
  int32_t partition_strategy; /* MUON_PARTITION_*                   */
  int32_t max_leaf_size;      /* 0 = default (4)                    */
  int32_t builder;            /* MUON_BUILDER_*                     */
} MuonSceneDesc;

/* Render settings: the integrator properties of muon::Scene
 * (muon/scene.h:32-47) plus GPU-only knobs. */
typedef struct MuonRenderParams {
  int32_t integrator; /* MUON_INTEGRATOR_* */
  int32_t pixel_samples;
  int32_t light_samples;
  int32_t light_stratify;
  int32_t next_event_estimation; /* MUON_NEE_* */
  int32_t russian_roulette;
  int32_t importance_sampling; /* MUON_IS_* */
  int32_t min_depth;
  int32_t max_depth; /* -1 = unbounded */
  int32_t sample_offset; /* index of the first sample (progressive runs) */
  uint64_t seed;
  int32_t intersect_mode; /* MUON_ISECT_* */
  int32_t wave_paths;    /* paths per wavefront (0 = 2^24); a render     */
                         /* keeps two wavefronts in flight, each with  */
                         /* about 200 + 36 x shadow slots bytes a path */
  uint32_t flags;        /* MUON_RENDER_*                               */
  int32_t pad;
} MuonRenderParams;

/* FP64 film: per pixel (row-major, y outer) the sum and sum of squares of the
 * sample radiances (RGB) and the sample count. Caller-allocated, 3*W*H
 * doubles for sum/sum_sq and W*H uint32 for count. */
typedef struct MuonFilm {
  int32_t width, height;
  double *sum;
  double *sum_sq;
  uint32_t *count;
} MuonFilm;

typedef struct MuonRay {
  float origin[3];
  float direction[3]; /* unit length */
} MuonRay;

typedef struct MuonHit {
  float distance;  /* world distance; +inf on a miss                 */
  int32_t prim_id; /* parse-order primitive id; -1 on a miss         */
  float position[3];
  float normal[3];
} MuonHit;

/* muon::TraceStats (muon/stats.h:11-44) for the last render, plus the
 * shadow rays the reference does not count as rays. */
typedef struct MuonStats {
  uint64_t primary_rays;
  uint64_t secondary_rays;
  uint64_t shadow_rays;
  uint64_t object_tests; /* filled only with MUON_RENDER_STATS */
  uint64_t object_hits;
  uint64_t bounds_tests;
  uint64_t bounds_hits;
  uint64_t paths;
  double render_ms;      /* device time of the last render               */
  double extend_ms;      /* closest-hit traversal kernels (MUON_RENDER_TIMING) */
  double occlude_ms;     /* any-hit traversal kernels (MUON_RENDER_TIMING)     */
  double shade_ms;       /* shading kernels (MUON_RENDER_TIMING)               */
  double fold_ms;        /* radiance fold kernels (MUON_RENDER_TIMING)         */
  uint64_t kernel_launches;
  uint64_t bvh_nodes;
  uint64_t primitives;
  /* traversal work split by kernel class, for roofline accounting; the test
   * counts are filled only with MUON_RENDER_STATS (box tests count the two
   * child boxes of every node visited) */
  uint64_t extend_rays;
  uint64_t extend_launches;
  uint64_t extend_box_tests;
  uint64_t extend_prim_tests;
  uint64_t occlude_rays;
  uint64_t occlude_launches;
  uint64_t occlude_box_tests;
  uint64_t occlude_prim_tests;
} MuonStats;

/* ---- host side: scene files (muon/parser.{h,cc}) ---------------------- */
typedef struct MuonParsedScene MuonParsedScene;

/* Parses a .muon file with the reference parser's semantics
 * (muon/parser.cc:230-880, Parser::Parse). Malformed lines are skipped with a
 * warning, as in the reference. */
int muon_parse_scene_file(const char *path, MuonParsedScene **out);
/* Same, from an in-memory string; relative `load` paths resolve against
 * base_dir (may be NULL). */
int muon_parse_scene_string(const char *text, const char *base_dir, MuonParsedScene **out);
/* Borrowed view of the parsed scene and its render settings; valid until
 * muon_parsed_scene_free. */
int muon_parsed_scene_desc(const MuonParsedScene *scene, MuonSceneDesc *desc, MuonRenderParams *params);
/* Film post-process settings from the file: gamma (muon/film.cc:29-33) and
 * the `output` path (NULL if none was given). */
float muon_parsed_scene_gamma(const MuonParsedScene *scene);
const char *muon_parsed_scene_output(const MuonParsedScene *scene);
int32_t muon_parsed_scene_warnings(const MuonParsedScene *scene);
void muon_parsed_scene_free(MuonParsedScene *scene);

/* Tone-maps a film like Film::WriteOutput (muon/film.cc:21-43: mean over
 * `count`, gamma, clamp to [0,1], x255 truncated) into 8-bit RGB (row-major,
 * 3*W*H bytes) and optionally writes it as PNG (.png) or binary PPM. */
int muon_film_tonemap(const MuonFilm *film, float gamma, uint8_t *rgb_out);
int muon_film_write(const MuonFilm *film, float gamma, const char *path);

/* ---- device side ------------------------------------------------------ */
typedef struct MuonScene MuonScene;

/* Builds the BVH on the host (muon/acceleration.cc:204-458 replaced by a
 * binned-SAH builder) and uploads the scene to the current CUDA device once.
 * Replaces Structure::AddPrimitive + Structure::Init (muon/acceleration.h:
 * 30-35). */
int muon_gpu_scene_create(const MuonSceneDesc *desc, MuonScene **out);
/* Frees the scene. Its large work arrays stay cached in the process for the
 * next scene on the same device (at most 1/8 of the device's memory; no
 * counterpart in the reference, whose scenes live in host memory). */
void muon_gpu_scene_destroy(MuonScene *scene);
/* Frees every cached work array on every device. */
void muon_gpu_release_cached(void);

/* Renders the whole film: replaces the per-thread sample loop of
 * Renderer::Render (muon/renderer.cc:41-76). Host film in, host film out. */
int muon_gpu_render(MuonScene *scene, const MuonRenderParams *params, MuonFilm *film);
/* Same with the film in device memory (pointers from cudaMalloc: 3*W*H
 * doubles each for sum/sum_sq, W*H uint32 for count). */
int muon_gpu_render_device(MuonScene *scene, const MuonRenderParams *params, double *d_sum,
                           double *d_sum_sq, uint32_t *d_count);

/* Batched ray queries mirroring Structure::Intersect and
 * Structure::HasIntersection (muon/acceleration.h:44-49) on host arrays. */
int muon_gpu_intersect(MuonScene *scene, const MuonRay *rays, int64_t n, int32_t intersect_mode,
                       MuonHit *hits);
int muon_gpu_occluded(MuonScene *scene, const MuonRay *rays, const float *max_distance, int64_t n,
                      int32_t intersect_mode, uint8_t *occluded);

/* No counterpart in the reference. For callers that must not allocate device
 * memory while rendering — a host application whose own allocator reserves
 * the GPU's memory at start-up, or a real-time loop that allocates nothing
 * after initialisation: renders like muon_gpu_render_device (path tracer or
 * normals/albedo/depth; same film layout and flags) but takes every byte of
 * working memory from one fixed buffer of MUON_NOALLOC_SCRATCH_BYTES that the
 * library declares statically, and calls no cudaMalloc/cudaFree, pinned-host
 * allocation, CUDA graph or event API. The scene must already exist
 * (muon_gpu_scene_create, which does allocate). The buffer is placed on a GPU
 * when the first scene is created there (CUDA loads the library's modules
 * lazily; scene creation loads this one) and stays until the process exits;
 * every call looks up its device address with the scene's device current.
 * Paths in flight per wavefront are limited to what fits in the buffer
 * (about MUON_NOALLOC_SCRATCH_BYTES / (196 + 36 * shadow slots per path));
 * a larger wave_paths is rejected with MUON_ERR_INVALID_ARG. All calls share
 * the one buffer and find the previous call's data in it: calls whose GPU
 * work overlaps (other streams, scenes or threads) race and corrupt each
 * other's results. muon_gpu_stats is not updated. */
#define MUON_NOALLOC_SCRATCH_BYTES (64u << 20)
int muon_gpu_render_noalloc(MuonScene *scene, const MuonRenderParams *params, double *d_sum, double *d_sum_sq,
                            uint32_t *d_count);

/* Counters and device timings of the last render (muon/stats.h:11-44). */
int muon_gpu_stats(const MuonScene *scene, MuonStats *stats);

/* ---- traversal work measured on the host ------------------------------------
 * What the reference's TraceStats counts (bounds tests and object tests,
 * muon/stats.h:11-44, incremented in muon/acceleration.cc:65-202), counted by
 * walking the flattened BVH that the GPU traverses on the host, in the GPU's
 * visiting order (nearer hit child first, farther one deferred). These counts
 * are the measure of work behind a roofline's algorithmic bytes, independent
 * of the GPU kernels' own counters. */
typedef struct MuonWalkCounts {
  uint64_t rays;
  uint64_t box_tests;  /* child boxes tested: 2 per interior node visited */
  uint64_t prim_tests; /* primitive records tested                        */
  uint64_t hits;       /* rays that hit something                         */
} MuonWalkCounts;

/* Walks n rays (tmax per ray, or NULL for no limit) through the BVH that
 * muon_gpu_scene_create builds from desc with the host builder: closest hit
 * (any_hit 0) or any hit. hit_ids (optional) receives per ray the parse-order
 * id of the primitive hit, or -1. intersect_mode: MUON_ISECT_EXACT or
 * MUON_ISECT_FAST. Host only: needs no GPU. */
int muon_walk_rays(const MuonSceneDesc *desc, const MuonRay *rays, const float *tmax, int64_t n, int32_t any_hit,
                   int32_t intersect_mode, int32_t *hit_ids, MuonWalkCounts *out);

typedef struct MuonTraversalProbe {
  MuonWalkCounts extend_walked;  /* host walk of the sampled closest-hit rays  */
  MuonWalkCounts occlude_walked; /* host walk of the sampled shadow rays       */
  uint64_t extend_rays;          /* rays in every extend queue of the render   */
  uint64_t occlude_rays;         /* rays in every shadow queue of the render   */
  /* Estimates for all rays of the render: per (wavefront, bounce) queue, its
   * length times the mean count of its walked sample. */
  double extend_box_tests, extend_prim_tests;
  double occlude_box_tests, occlude_prim_tests;
} MuonTraversalProbe;

/* Renders as muon_gpu_render does (film discarded, MUON_RENDER_STATS on,
 * kernel by kernel), copies up to rays_per_queue evenly spaced rays out of
 * every closest-hit and shadow queue of the render as the traversal kernels
 * receive them, and walks them on the host through the scene's own BVH and
 * primitive records (the arrays on the device). Afterwards muon_gpu_stats
 * holds the GPU kernels' counters of the same render, for comparison.
 * Path tracer with bounded depth; exact or fast intersection mode. */
int muon_gpu_probe_traversal(MuonScene *scene, const MuonRenderParams *params, int32_t rays_per_queue,
                             MuonTraversalProbe *out);

/* Read-bandwidth ceilings of the current device for a roofline, measured by
 * one kernel: level 0 reads a buffer of `bytes` (at most 64 KiB) from every
 * block through L1; level 1 reads a buffer of `bytes` that fits in L2 across
 * the grid, bypassing L1; level 2 reads a buffer larger than L2 across the
 * grid (DRAM). `passes` repeats inside the launch; GB/s of bytes delivered. */
int muon_gpu_measure_read_bandwidth(int32_t level, int64_t bytes, int32_t passes, double *gb_per_s);

/* ---- batched rendering -------------------------------------------------
 * Many scenes of uneven size, resolution and sample count rendered by one
 * wavefront: every kernel launch covers paths of all the scenes at once, and
 * the whole batch is replayed as one CUDA graph. This generalises the thread
 * pool of Renderer::Render (muon/renderer.cc:31-77) from one scene to many;
 * the reference itself renders one scene per process. Path tracer only. */
typedef struct MuonBatch MuonBatch;

typedef struct MuonBatchSceneStats {
  uint64_t primary_rays;
  double done_ms; /* from the start of the batch until this scene's film was complete */
} MuonBatchSceneStats;

/* Launch configuration chosen by muon_gpu_batch_autotune. */
typedef struct MuonBatchTuning {
  int32_t wave_paths;              /* paths per wavefront                        */
  int32_t traversal_blocks_per_sm; /* resident blocks of the traversal kernels   */
  int32_t candidates;              /* configurations timed                       */
  int32_t pad;
  double best_ms;                  /* time of the chosen configuration's trial   */
} MuonBatchTuning;

/* Copies the scenes (created on the current device by muon_gpu_scene_create;
 * they stay usable and unchanged) into one device image: their BVHs side by
 * side under separate roots, their materials, transforms and lights
 * concatenated. Scenes are scheduled shortest first. */
int muon_gpu_batch_create(MuonScene *const *scenes, int32_t n, MuonBatch **out);
void muon_gpu_batch_destroy(MuonBatch *batch);
/* Renders scene i with params[i] into film i (n entries each), like
 * muon_gpu_render_device / muon_gpu_render per scene. params[i].wave_paths is
 * ignored: the wavefront size is the batch's (autotuned or default). Every
 * max_depth must be >= 0. */
int muon_gpu_batch_render_device(MuonBatch *batch, const MuonRenderParams *params, double *const *d_sum,
                                 double *const *d_sum_sq, uint32_t *const *d_count);
int muon_gpu_batch_render(MuonBatch *batch, const MuonRenderParams *params, MuonFilm *films);
/* Times candidate launch configurations (wavefront size x traversal grid) on
 * a reduced-sample pass of the batch with these params, keeps the fastest for
 * later renders of this batch and reports it. */
int muon_gpu_batch_autotune(MuonBatch *batch, const MuonRenderParams *params, MuonBatchTuning *out);
/* Totals of the last batched render and, if per_scene is not NULL, one entry
 * per scene (in the order given to muon_gpu_batch_create). */
int muon_gpu_batch_stats(const MuonBatch *batch, MuonStats *total, MuonBatchSceneStats *per_scene);
/* One-shot form: create, render into host films, destroy. */
int muon_gpu_render_batch(MuonScene *const *scenes, const MuonRenderParams *params, int32_t n, MuonFilm *films);

/* The CUDA stream (cudaStream_t) all of this scene's work is launched on, for
 * callers that time or order work around it with CUDA events. */
int muon_gpu_scene_stream(const MuonScene *scene, void **stream);

/* The scene's BVH as its kernels read it, with the build's statistics
 * (the BVH of Structure::Init, muon/acceleration.cc:204-458). */
typedef struct MuonBvhInfo {
  int64_t nodes;     /* 64-byte nodes (two child boxes and links; node 0 is the root) */
  int64_t slots;     /* primitive records, in leaf order */
  int64_t leaves;
  int32_t max_depth; /* deepest node, the root at depth 0 (leaves included) */
  int32_t max_leaf;  /* most primitives in one leaf */
} MuonBvhInfo;
/* Fills *info; then, where not null, copies info->nodes nodes into `nodes`
 * (the device layout: per node the child boxes (c0.lo.x, c0.hi.x, c0.lo.y,
 * c0.hi.y), (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y), (c0.lo.z, c0.hi.z, c1.lo.z,
 * c1.hi.z) as floats, then the links (link0, link1, 0, 0) as int32: >= 0 an
 * interior node, < 0 a leaf whose first slot is ~link), and per slot the
 * primitive's id (`slot_prim`, MuonTriangleDesc/MuonSphereDesc.prim_id) and
 * whether the slot ends its leaf (`slot_last`). */
int muon_gpu_scene_bvh(const MuonScene *scene, MuonBvhInfo *info, void *nodes, int32_t *slot_prim,
                       uint8_t *slot_last);

/* ---- learned path guiding --------------------------------------------
 * No counterpart in the reference (which has no learned component): a small
 * MLP predicts, per shading point, a mixture of 8 anisotropic lobes over
 * directions (2D Gaussians in the tangent plane of each lobe's mean, projected
 * to the sphere, plus a small uniform part); the path tracer samples it with
 * probability mixture_fraction and its own sampler otherwise, weighting every
 * sample by the combined density, so the estimate stays unbiased whatever the
 * network predicts. The network (one-blob encoded position, normal, outgoing
 * direction and roughness -> 5 layers of 64 -> 64 outputs; BF16 tcgen05
 * tensor-core inference, FP32 training with Adam) learns online from the
 * radiance samples of the guide's own renders. */
typedef struct MuonGuide MuonGuide;

/* What the network learns and which rays it guides (MuonGuideConfig.targets). */
#define MUON_GUIDE_DIRECT 0 /* where direct light arrives; guides the light-hit (MIS) ray,
                               continuations sample the BRDF */
#define MUON_GUIDE_ALL 1    /* all incident light; guides the MIS ray and continuations */

typedef struct MuonGuideConfig {
  int32_t batch;            /* training batch (0: 2^18)                            */
  int32_t wave_paths;       /* paths per wavefront of guided renders (0: 2^24)     */
  int32_t record_bounces;   /* first vertices of a path that are guided and kept as
                               training samples (0: 4); deeper ones sample the BRDF */
  int32_t pool_capacity;    /* training samples kept, newest first (0: 2^22)       */
  float learning_rate;      /* Adam step size (0: 1e-3)                            */
  float mixture_fraction;   /* probability that a guided ray samples the mixture
                               rather than the BRDF (0: 0.95 with MUON_GUIDE_DIRECT,
                               0.5 with MUON_GUIDE_ALL)                            */
  int32_t targets;          /* MUON_GUIDE_DIRECT or MUON_GUIDE_ALL                 */
  int32_t reserved;         /* 0                                                   */
  uint64_t seed;            /* network initialisation and batch selection          */
} MuonGuideConfig;

/* Number of FP32 network parameters (weights [in][out] then biases, per layer). */
#define MUON_GUIDE_PARAMS 33088

int muon_gpu_guide_create(MuonScene *scene, const MuonGuideConfig *config, MuonGuide **out);
void muon_gpu_guide_destroy(MuonGuide *guide);
/* Path-traced render of the guide's scene (device film, as
 * muon_gpu_render_device) sampling with the current network; its path
 * vertices become training samples. params->integrator must be the path
 * tracer; params->wave_paths is the guide's. The tensor-core inference waits
 * for its matrix units with a bound: if a wait gives up, this call (and
 * every later render, forward or sample call of the same guide) returns
 * MUON_ERR_TIMEOUT; destroy the guide. */
int muon_gpu_guide_render_device(MuonGuide *guide, const MuonRenderParams *params, double *d_sum, double *d_sum_sq,
                                 uint32_t *d_count);
/* `steps` Adam steps on batches drawn from the collected samples; the mean
 * loss of the last step goes to *loss when not NULL. */
int muon_gpu_guide_train(MuonGuide *guide, int32_t steps, double *loss);
/* Network outputs (n x 64 raw values) for features (n x 8), on the
 * tensor-core inference path; host arrays. */
int muon_gpu_guide_forward(MuonGuide *guide, const float *features, int64_t n, float *out);
/* Directions drawn from the network's mixture at features (n x 8), one per
 * row, with the given uniforms in [0, 1) (n x 3), and the mixture density of
 * each direction (per steradian): the sampling and density a guided render
 * uses, for inspecting a trained guide and for tests. Host arrays. */
int muon_gpu_guide_sample(MuonGuide *guide, const float *features, const float *u, int64_t n, float *dirs,
                          float *pdf);
/* Gradients (MUON_GUIDE_PARAMS values) of the mean loss over one batch of n
 * samples (features n x 8, unit directions n x 3, weights n) and the loss;
 * host arrays. */
int muon_gpu_guide_gradients(MuonGuide *guide, const float *features, const float *dirs, const float *weights,
                             int32_t n, float *grad, double *loss);
int muon_gpu_guide_get_params(const MuonGuide *guide, float *params);
int muon_gpu_guide_set_params(MuonGuide *guide, const float *params);
/* Training samples collected so far. */
int muon_gpu_guide_samples(const MuonGuide *guide, uint64_t *count);
/* No counterpart in the reference (which has no device waits). Writes the
 * guide's wait-status word from the host: 1 is what an inference kernel
 * leaves when one of its tensor-core waits gives up, 0 clears it. Lets a
 * host (or a test) exercise its MUON_ERR_TIMEOUT handling without making a
 * device wait run out. */
int muon_gpu_guide_set_status(MuonGuide *guide, int32_t status);

/* Thread-local description of the last failure on this thread. */
const char *muon_gpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* MUON_GPU_H_ */
