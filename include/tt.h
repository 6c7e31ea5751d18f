/*
 * tt.h — C ABI of the GB300 path-tracing core (libtt.so).
 *
 * The reference (TrenchantTracer) has no plugin or FFI layer: its hot path sits behind C++
 * classes and device functions. Every entry point below replaces one of those interfaces
 * and names it (file:line in the reference project). Conventions:
 *   - every call returns a tt_status; tt_last_error_string() describes the last failure
 *     on the calling thread;
 *   - device buffers are plain pointers into the current CUDA device's memory; host
 *     buffers are plain host pointers; `stream` is a cudaStream_t (NULL = legacy stream);
 *   - handles are not thread-safe; distinct handles may be used from distinct threads.
 */
#ifndef TT_H
#define TT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tt_status {
    TT_OK = 0,
    TT_ERR_INVALID = 1,  /* bad argument */
    TT_ERR_IO = 2,       /* file missing, short read or write */
    TT_ERR_CUDA = 3,     /* a CUDA runtime call failed */
    TT_ERR_TIMEOUT = 4,  /* a device-side bounded wait ran out */
    TT_ERR_BOUNDS = 5,   /* a device-side bounds check fired (stack / queue overflow) */
    TT_ERR_OOM = 6,      /* host or device allocation failed */
    TT_ERR_FORMAT = 7,   /* malformed JSON / OBJ / .hdr / bvh.cache */
    TT_ERR_NO_DEVICE = 8 /* no CUDA device visible */
} tt_status;

/* A ray, byte-compatible with the reference's Ray (include/geometry/Ray.h:10-13): 32 B. */
typedef struct tt_ray {
    float ox, oy, oz;
    float dx, dy, dz;
    float tmin, tmax;
} tt_ray;

/* The closest/any hit: Hit::index (original triangle id, -1 = miss) and Hit::distance
 * (include/geometry/Hit.h:7-15). On a miss t = ray.tmax, as in the reference. 8 B. */
typedef struct tt_hit {
    int32_t id;
    float t;
} tt_hit;

/* The full hit record of intersect(): id, Hit::matIndex, t and the interpolated,
 * unnormalised Hit::normal (IntersectKernel.cuh:264,288-289). 24 B. */
typedef struct tt_hit_ext {
    int32_t id;
    int32_t mat;
    float t;
    float nx, ny, nz;
} tt_hit_ext;

/* The 7 x u32 header of bvh.cache, in file order (BVHCompact.cpp:319-338). */
typedef struct tt_bvh_header {
    uint32_t nodes;       /* float4 count of the node array (4 per inner node) */
    uint32_t tri_count;   /* triangle references emitted into leaves */
    uint32_t leaf_count;
    uint32_t vertices;    /* float4 count: 3 per triangle + 1 terminator per leaf */
    uint32_t normals;     /* same indexing as vertices */
    uint32_t tri_indices; /* int32 count, same indexing as vertices */
    uint32_t mat_indices; /* uint32 count, same indexing as vertices */
} tt_bvh_header;

/* CameraMeta (include/core/Camera.h:8-16), byte for byte: 60 B. */
typedef struct tt_camera_meta {
    int32_t width, height;
    float position[3];
    float view[3];
    float up[3];
    float fov[2];
    float aperture;
    float focal;
} tt_camera_meta;

/* RenderMeta (include/core/Renderer.h:24-31), byte for byte: 20 B. */
typedef struct tt_render_meta {
    int32_t frame_number;
    uint32_t hashed_frame;
    int32_t samples;
    float pi;
    float two_pi;
} tt_render_meta;

/* A material, flattened (the reference keeps a polymorphic MaterialUnion,
 * include/material/MaterialUnion.h). kind: 0 Diff, 1 Metal, 2 Spec, 3 Refr, 4 Coat (the
 * reference's MaterialType values, include/material/Material.h:11-13), 5 GGX conductor,
 * 6 dielectric. color = diffuseColor (Diff, Coat) / color (Metal, Spec) / F0 (GGX);
 * color2 = specularColor (Coat). 64 B. */
typedef struct tt_material {
    int32_t kind;
    float emission[3];
    float color[3];
    float color2[3];
    float roughness; /* GGX: alpha = roughness^2 */
    float ior;       /* dielectric */
    float pad[4];
} tt_material;

/* An analytic object of the scene JSON (include/geometry/{Plane,Sphere}.h). kind: 0 Sphere,
 * 3 Plane (the reference's GeometryType values). Plane: p0, p1, p2 (a parallelogram); Sphere:
 * radius and position in p0. 64 B. */
typedef struct tt_geometry {
    int32_t kind;
    int32_t material;
    float radius;
    float pad;
    float p0[3];
    float p1[3];
    float p2[3];
    float pad2[3];
} tt_geometry;

typedef struct tt_scene tt_scene; /* host triangle soup + materials (core/Scene.h) */
typedef struct tt_renderer tt_renderer; /* device materials, analytic objects, environment */
typedef struct tt_bvh tt_bvh;     /* host compact SBVH arrays (bvh/BVHCompact.h) */
typedef struct tt_dbvh tt_dbvh;   /* device-resident compact SBVH */

/* ---- errors ---------------------------------------------------------------------- */
const char *tt_last_error_string(void);
const char *tt_version(void);

/* ---- scene ingest (host) ---------------------------------------------------------- */
/* Config(path) + SceneLoader::load (src/util/Config.cpp:3-22, src/loader/SceneLoader.cpp:8-29):
 * the same scene JSON, OBJ, material-JSON and RGBE .hdr formats. */
tt_status tt_scene_load_json(const char *config_path, tt_scene **out);
/* Scene::add(Object*) on arrays already in memory (src/core/Scene.cpp:7-23): vertices and
 * normals are xyz float triples; vidx/nidx are 3 indices per triangle; mat is one material
 * index per triangle (may be NULL = all 0). */
tt_status tt_scene_create(const float *vertices, int32_t num_vertices, const float *normals,
                          int32_t num_normals, const int32_t *vidx, const int32_t *nidx,
                          const uint32_t *mat, int32_t num_triangles, tt_scene **out);
/* counts: [triangles, vertices, normals, materials, analytic geometries] */
tt_status tt_scene_counts(const tt_scene *scene, int32_t counts[5]);
/* copies of the triangle soup: any pointer may be NULL */
tt_status tt_scene_arrays(const tt_scene *scene, float *vertices, float *normals, int32_t *vidx,
                          int32_t *nidx, uint32_t *mat);
/* The environment map HDRLoader::load read for the scene (src/loader/HDRLoader.cpp:5-65):
 * width, height and, when rgb != NULL, w*h*3 linear floats, row 0 first. 0 x 0 = none. */
tt_status tt_scene_env(const tt_scene *scene, int32_t *width, int32_t *height, float *rgb);
/* Replaces the environment map (width*height*3 linear floats, row 0 first; 0 x 0 = none).
 * TT_ERR_INVALID, leaving the scene's map in place, for a negative, infinite or NaN texel. */
tt_status tt_scene_set_env(tt_scene *scene, int32_t width, int32_t height, const float *rgb);
/* Materials and analytic objects: counts via tt_scene_counts; `out` may be NULL. The setters
 * refuse (TT_ERR_INVALID) material kinds outside 0-6 and analytic objects other than spheres (0)
 * and planes (3). */
tt_status tt_scene_materials(const tt_scene *scene, tt_material *out);
tt_status tt_scene_set_materials(tt_scene *scene, const tt_material *materials, int32_t count);
tt_status tt_scene_geometries(const tt_scene *scene, tt_geometry *out);
tt_status tt_scene_set_geometries(tt_scene *scene, const tt_geometry *geometries, int32_t count);
void tt_scene_free(tt_scene *scene);

/* ---- SBVH build and the compact layout (host) ------------------------------------ */
/* BVH::BVH(scene, SAHHelper, splitAlpha) + BVHCompact::createCompact
 * (src/bvh/BVH.cpp:3-63, src/bvh/BVHCompact.cpp:88-250). SAHHelper::setLeafPreferences
 * (src/bvh/SAHHelper.cpp:51-54) gives leaf_min/leaf_max; the reference defaults are
 * split_alpha 1e-5, leaf_min 1, leaf_max 0x7FFFFFF. threads <= 0 uses all host cores; the
 * output does not depend on the thread count. TT_ERR_INVALID for a triangle with a NaN or
 * infinite vertex coordinate (the reference has no check; its sorts are undefined there). */
tt_status tt_bvh_build(const tt_scene *scene, float split_alpha, int32_t leaf_min,
                       int32_t leaf_max, int32_t threads, tt_bvh **out);
/* BVHCompact::save / BVHCompact(FILE*) (src/bvh/BVHCompact.cpp:319-375, :23-79). */
tt_status tt_bvh_save(const tt_bvh *bvh, const char *path);
tt_status tt_bvh_load(const char *path, tt_bvh **out);
tt_status tt_bvh_header_get(const tt_bvh *bvh, tt_bvh_header *out);
/* borrowed pointers to the host arrays (valid until tt_bvh_free) */
tt_status tt_bvh_arrays(const tt_bvh *bvh, const void **nodes, const void **vertices,
                        const void **normals, const int32_t **tri_indices,
                        const uint32_t **mat_indices);
void tt_bvh_free(tt_bvh *bvh);

/* ---- device BVH and traversal ----------------------------------------------------- */
/* The device half of BVHCompact (cudaMalloc + cudaMemcpy + texture objects,
 * src/bvh/BVHCompact.cpp:196-317): uploads the arrays to the current device. */
tt_status tt_bvh_upload(const tt_bvh *bvh, tt_dbvh **out);
void tt_dbvh_free(tt_dbvh *dbvh);

/* Kernel shape used by the traversal calls on `bvh` (a tuning knob; the reference launches one
 * ray per thread, src/core/RenderKernel.cu:221-231):
 *   0 TT_VARIANT_WARP       each warp traces 32 consecutive rays, stack in local memory
 *   1 TT_VARIANT_WARP_SH16  as 0, the lowest 16 stack entries in shared memory
 *   2 TT_VARIANT_WARP_SH32  as 0, the lowest 32 stack entries in shared memory
 *   3 TT_VARIANT_DYNAMIC    every lane claims a new ray as soon as it finishes one
 *   4 TT_VARIANT_WARP_VOTE  as 0, with the reference's warp-vote leaf postponement
 *                           (IntersectKernel.cuh:180-203)
 *   5 TT_VARIANT_SORTED     (default) as 1, over the rays in the order of a counting sort by direction
 *                           octant and origin cell (device scratch of ~17 MB + 8 B per ray)
 *   6 TT_VARIANT_SH16_OCC   as 1, compiled for 12 resident blocks per SM (fewer registers)
 *   7 TT_VARIANT_SORTED_OCC as 5, compiled for 12 resident blocks per SM
 * All variants but 4 return the per-ray result of the reference's algorithm and are identical;
 * variant 4 can differ from them in float corner cases, as the reference's own kernel does. */
#define TT_VARIANT_WARP 0
#define TT_VARIANT_WARP_SH16 1
#define TT_VARIANT_WARP_SH32 2
#define TT_VARIANT_DYNAMIC 3
#define TT_VARIANT_WARP_VOTE 4
#define TT_VARIANT_SORTED 5
#define TT_VARIANT_SH16_OCC 6
#define TT_VARIANT_SORTED_OCC 7
#define TT_NUM_VARIANTS 8
tt_status tt_dbvh_set_variant(tt_dbvh *bvh, int32_t variant);
/* How many bytes of the node array's top levels the trace launches keep persisting in L2 (an
 * access-policy window over the start of the array, where tt_bvh_upload lays the tree's top
 * levels out breadth first; the persisting set-aside is a limit of the calling process's
 * context). 0 = no window. No counterpart in the reference. */
tt_status tt_dbvh_set_l2_window(tt_dbvh *bvh, int64_t bytes);
tt_status tt_dbvh_get_variant(const tt_dbvh *bvh, int32_t *variant);
/* Autotuner: traces the n device rays with every variant (the warp-vote one only when
 * include_vote != 0), three launches each, keeps the fastest for `bvh` and writes each
 * variant's best time in ms to ms_out[variant] (TT_NUM_VARIANTS floats; skipped variants get
 * 0; may be NULL). Synchronises `stream`. */
tt_status tt_dbvh_autotune(tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit *d_hits,
                           int32_t closest, int32_t include_vote, void *stream, float *ms_out);

/* intersect(ray, bvh, needClosestHit) (include/geometry/IntersectKernel.cuh:78-296) over n
 * rays in device memory; hits are written to device memory. closest = 1 is the closest hit,
 * 0 the any hit (first accepted triangle in traversal order). */
tt_status tt_trace(const tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit *d_hits,
                   int32_t closest, void *stream);
/* as tt_trace, writing the full hit record (material index and interpolated normal). */
tt_status tt_trace_ext(const tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit_ext *d_hits,
                       int32_t closest, void *stream);
/* as tt_trace with HOST buffers: copies rays in, traces and copies hits out on `stream`
 * through a device staging area owned by `bvh`, and synchronises the stream before returning
 * (page-locked host buffers get full copy bandwidth). Returns the device error word like
 * tt_dbvh_check. */
tt_status tt_trace_host(const tt_dbvh *bvh, const tt_ray *h_rays, int64_t n, tt_hit *h_hits,
                        int32_t closest, void *stream);
/* Synchronises `stream`, then reads and clears the device error word that tt_trace /
 * tt_trace_ext calls on `bvh` set: TT_ERR_BOUNDS if a traversal stack would have overflowed
 * (the reference's 64-entry stack has no check, IntersectKernel.cuh:8,164-165), TT_ERR_TIMEOUT
 * if a traversal reached its iteration cap (a corrupt BVH), TT_OK otherwise. Rays that fail
 * this way are reported as misses. */
tt_status tt_dbvh_check(const tt_dbvh *bvh, void *stream);
/* The key the ordered variants (TT_VARIANT_SORTED, TT_VARIANT_SORTED_OCC) sort a ray set by,
 * computed on the host; no counterpart in the reference. keys[i] holds ray i's origin cell above
 * its 8-bit direction cell (a 16 x 16 octahedral map); the origin cell indexes a grid over the
 * scene bounds lo..hi whose bits go to the longest remaining cell side first, 13 bits for 2^22
 * rays or more and 2 fewer per quartering of n (6 at least). *key_bits receives the key width.
 * A caller may sort its rays by these keys on the host to trace them coherently. */
tt_status tt_ray_order_keys(const tt_ray *rays, int64_t n, const float lo[3], const float hi[3], uint32_t *keys,
                            int32_t *key_bits);
/* The same keys computed on the device by the ordering kernels' own key function, for n device
 * rays (16-byte aligned) into d_keys; no counterpart in the reference. Launch only. A check that
 * the host keys above are the device's, bit for bit. */
tt_status tt_ray_order_keys_device(const tt_ray *d_rays, int64_t n, const float lo[3], const float hi[3],
                                   uint32_t *d_keys, int32_t *key_bits, void *stream);

/* Allocation-free tracing with HOST ray and hit buffers. No counterpart in the reference: it is
 * an addition for callers that cannot allocate device memory, such as a host application whose
 * device memory belongs to its own arena (it uploads the BVH into that memory itself and passes
 * the arrays here), or a frame loop that must not stall on the device-wide synchronisation a
 * cudaMalloc can cause. tt_trace_host allocates its device staging on first use and whenever a
 * call needs more; this entry point never allocates (no cudaMalloc, cudaFree or allocating
 * library call). Ray and hit staging, the work counter and the error word live in one fixed
 * ~10 MiB array inside libtt.so. The array is reserved on a device when the library's device
 * code is first loaded there (CUDA loads modules lazily by default: at the first libtt call that
 * uses the device) and is held until the process exits, so a caller whose arena will take all
 * device memory makes a warm-up call on each device before its arena grows: with n = 0 this
 * entry point only loads the library's device code on the current device (reserving the array)
 * and looks up the array's address, and returns TT_OK, or the CUDA error if that fails.
 *   d_nodes, d_vertices, d_tri_indices  the caller's device copies of the compact BVH arrays
 *                                       (the layout of tt_bvh_arrays / bvh.cache); 16-, 16- and
 *                                       4-byte aligned
 *   n                                   at most TT_NOALLOC_MAX_RAYS rays per call; larger n is
 *                                       rejected with TT_ERR_INVALID and a message
 * Results are those of tt_trace_host with the default kernel variant. The stream is
 * synchronised before returning. The first call on each device also looks up the device address
 * of the staging array; make that first call (the warm-up) before any stream capture. All calls
 * share the one array: calls that overlap on the GPU (other host threads, other streams) race. */
/* ---- camera and frame metadata (host) ---------------------------------------------------- */
/* Camera(config) + Camera::setFovx(fovx) + Camera::getCameraMeta() for the scene's camera block
 * (src/core/Camera.cpp:12-44, :115-140; the reference's main uses fovx = 45). */
tt_status tt_camera_meta_from_scene(const tt_scene *scene, float fovx, tt_camera_meta *out);
/* RenderMeta of frame `frame_number` (1 for the first frame): hashed_frame =
 * WangHash::encode(frame_number) (src/util/WangHash.cpp:8-15, Renderer.cpp:107) and the
 * reference's PI = 3.14156265f and TWO_PI constants (Renderer.cpp:5-6). */
tt_status tt_render_meta_init(int32_t frame_number, int32_t samples, tt_render_meta *out);
uint32_t tt_wang_hash(uint32_t a);

/* ---- path tracing ------------------------------------------------------------------------- */
/* The renderer's device state: the scene's materials, analytic Plane/Sphere objects and
 * environment map, over an uploaded BVH (which must outlive the renderer); the device half of
 * Renderer::Renderer (src/core/Renderer.cpp:8-57) without the GL parts. */
tt_status tt_renderer_create(const tt_dbvh *bvh, const tt_scene *scene, tt_renderer **out);
void tt_renderer_free(tt_renderer *renderer);
/* One frame of the reference's path tracer, Renderer::render / pathTracingKernel
 * (src/core/RenderKernel.cu:97-233): adds sum_s L / samples of every pixel to d_accum
 * (width*height*3 floats, row 0 = the image's bottom row, as the reference stores it). Uses
 * curand XORWOW streams seeded as the reference does, so a frame equals the reference kernel's
 * for the same inputs. Launch only. */
tt_status tt_render_compat(tt_renderer *renderer, const tt_camera_meta *cam, const tt_render_meta *meta,
                           float *d_accum, void *stream);
/* Synchronises `stream` and reports traversal errors of the renderer's launches. */
tt_status tt_renderer_check(tt_renderer *renderer, void *stream);

/* One material interaction of the reference's path loop (src/core/RenderKernel.cu:64-91): the
 * ray that hit, the Hit record renderKernel built (raw interpolated normal and distance, then
 * n / nl from normalize() and point from hitPoint(), include/geometry/IntersectKernel.cuh:62-76),
 * the throughput mask and the curand XORWOW state (48 bytes) going in; the next ray, mask and
 * state coming out of the material's sampler (include/material/{Diff,Metal,Spec,Refr,Coat}Impl.cuh);
 * u0 is the first uniform the incoming state yields. `kind` is the reference's MaterialType
 * (0 DIFF, 1 METAL, 2 SPEC, 3 REFR, 4 COAT), `material` the index into the scene's materials.
 * 256 bytes. */
typedef struct tt_compat_interaction {
    int32_t kind, thread, material, seq;
    float o[3], d[3], tmin, tmax;
    float normal[3], distance;
    float n[3], nl[3], point[3];
    float mask[3];
    uint32_t rng[12];
    float out_o[3], out_d[3], out_mask[3];
    uint32_t out_rng[12];
    float u0;
    int32_t pad[2];
} tt_compat_interaction;
/* Diagnostic (no counterpart in the reference): re-runs recorded interactions through
 * tt_render_compat's own per-hit arithmetic. For each of the n device records of d_in, d_out gets
 * a copy whose n / nl / point are recomputed by this renderer from (o, d, normal, distance), and
 * whose out_* fields and u0 come from this renderer's sampler of `kind` run on the record's
 * incoming ray, hit (n, nl, point as recorded), mask and curand state. Two more kinds:
 *   5  an environment lookup at a path's miss (hdrSample, include/hdr/HDRKernel.cuh:6-42):
 *      out_mask gets the radiance this renderer looks up for direction d;
 *   6  a sample's primary ray (src/core/RenderKernel.cu:131-197) for the pixel that thread
 *      `thread` of tt_render_compat's launch over `cam` renders: out_o / out_d / tmin / tmax get
 *      the ray, out_rng the curand state after its draws; the state going in is `rng`, or, with
 *      seq < 0, the one the frame seeds for that thread (WangHash(frame) + thread).
 * Lets a caller holding interactions recorded inside the reference's own kernel compare one
 * bounce at a time instead of whole frames. Launch only. */
tt_status tt_compat_replay(const tt_renderer *renderer, const tt_camera_meta *cam, const tt_render_meta *meta,
                           const tt_compat_interaction *d_in, int64_t n, tt_compat_interaction *d_out,
                           void *stream);

/* Parameters of the native path tracer (no counterpart in the reference, which always runs 10
 * bounces with curand streams). */
typedef struct tt_render_params {
    int32_t spp;           /* samples per pixel of this call */
    int32_t sample_offset; /* global index of the first sample (progressive rendering) */
    int32_t max_depth;     /* bounces at most (the reference's fixed value is 10) */
    int32_t rr_depth;      /* Russian roulette from this bounce on (>= max_depth: off) */
    uint32_t seed;         /* PCG32 state seed; the stream of a path is its global index */
    float env_scale;       /* environment radiance factor (the reference uses 2) */
    float ray_eps;         /* new-ray origin offset along the normal, x max(1, |p|_inf) */
    int32_t flags;         /* TT_RENDER_* bits */
} tt_render_params;
#define TT_RENDER_ACCUM_F64 1          /* d_accum holds doubles */
#define TT_RENDER_NO_ENV_SAMPLING 2    /* BSDF sampling only (no environment light sampling / MIS) */
/* Fills `out` with the defaults: spp 1, offset 0, max_depth 8, rr_depth 4, seed 1, env_scale 1,
 * ray_eps 1e-4, flags 0. */
tt_status tt_render_params_default(tt_render_params *out);
/* Native wavefront path tracer (Lambert, GGX conductor, dielectric, environment light sampling
 * by a 2D CDF with MIS, Russian roulette, PCG32 streams; the reference's own material kinds are
 * mapped as the header of tt_render_native.cu lists; a camera with aperture > 1e-5 is a thin
 * lens focused at `focal` along the view direction). Adds the sum of spp samples of every pixel
 * to d_accum (width*height*3 floats, or doubles with TT_RENDER_ACCUM_F64; row 0 = the image's top
 * row). The pixel sums are added in sample order, so the result is the same for every launch
 * shape. Launch only; deterministic for given inputs. */
tt_status tt_render_native(tt_renderer *renderer, const tt_camera_meta *cam, const tt_render_params *params,
                           void *d_accum, void *stream);
/* One query of tt_native_sample_probe (160 bytes): the inputs, then what the native renderer's
 * own device code returned for them. */
typedef struct tt_sample_probe {
    /* in */
    int32_t material;    /* what 0: index into the scene's materials */
    int32_t entering;    /* what 0: 1 when wo is on the side the normal points to (dielectrics) */
    float n[3], wo[3];   /* what 0: unit normal facing wo, unit direction towards the viewer */
    float u[3];          /* uniform numbers in [0, 1) the sampler consumes */
    int32_t pad0;
    uint64_t pcg_state, pcg_seq; /* what 2: pcg32_srandom_r(initstate, initseq) */
    /* out */
    float wi[3];         /* sampled direction (what 0, 1) */
    float weight[3];     /* what 0: f |cos| / pdf; what 1: the environment radiance */
    float pdf;           /* solid-angle pdf of the sample (0: a specular choice or no sample) */
    float eval_pdf;      /* what 0: the pdf bsdf_eval gives for wi; what 1: env_pdf of wi */
    float eval[3];       /* what 0: f |cos| that bsdf_eval gives for wi */
    int32_t specular;
    uint32_t pcg_out[8]; /* what 2: the stream's first eight outputs */
    int32_t texel;       /* what 1: the texel (row * env_w + column) the CDF searches chose */
    int32_t pad1[3];
} tt_sample_probe;
/* Diagnostic (no counterpart in the reference, whose samplers are other ones): runs the native
 * path tracer's own sampling code on n device queries. what 0: the BSDF sampler of the query's
 * material (Lambert, GGX conductor, dielectric, Spec, Coat) and bsdf_eval at the sampled
 * direction; what 1: the environment map's 2D-CDF sampler with u[0], u[1] and env_pdf at the
 * sampled direction (the scene must have an environment); what 2: the PCG32 generator the
 * renderer's paths draw from. Lets tests check the samplers' distributions against their stated
 * densities. Launch only. */
tt_status tt_native_sample_probe(const tt_renderer *renderer, int32_t what, tt_sample_probe *d_queries, int64_t n,
                                 void *stream);
/* The environment's sampling tables built by tt_renderer_create: marginal CDF (env_h + 1 floats)
 * and conditional CDFs (env_h * (env_w + 1) floats), copied to host buffers (either may be
 * NULL). */
tt_status tt_renderer_env_tables(const tt_renderer *renderer, float *marginal, float *conditional);

/* Launch shape of the native path tracer's kernels (no counterpart in the reference). */
typedef struct tt_launch_shape {
    int32_t block;        /* threads per block: 64, 128 or 256 */
    int32_t stack_shared; /* traversal stack entries per thread kept in shared memory: 0, 8 or 16 */
    int32_t wave_paths;   /* paths in flight per wave (queue capacity): 1 .. 2^26 */
    int32_t ordered;      /* 1: order each extension queue by origin and direction cell before
                             tracing it (coherent queues, e.g. camera rays, are left alone) */
    int32_t streamed;     /* 1: a render of more paths than one wave streams them through a pool
                             of wave_paths slots that is refilled with new camera paths as paths
                             end (no refill for cached renders, or when max_depth * wave_paths
                             exceeds 2^29), so every bounce launch traces a full queue; 0: waves
                             of wave_paths paths, each traced bounce by bounce to its end */
    float ms;             /* tt_batch_autotune: the trial's time; otherwise 0 */
} tt_launch_shape;
/* Default: 128 threads, 16 shared entries, 2^22 paths, unordered, streamed. Results do not depend
 * on the shape: every pixel adds its samples in sample order whatever the shape. */
tt_status tt_renderer_set_launch(tt_renderer *renderer, const tt_launch_shape *shape);
tt_status tt_renderer_get_launch(const tt_renderer *renderer, tt_launch_shape *shape);
/* Counters of the native path tracer since the last reset: out[0] extension rays (closest hit),
 * out[1] shadow rays (any hit), out[2] paths. Synchronous. */
tt_status tt_renderer_stats(tt_renderer *renderer, uint64_t *out, int32_t reset);
/* Kernels the native path tracer issued since the last reset (launched, or captured into a batch's
 * graph), counted on the host: its own kernels and the ordering kernels, not a cached render's
 * network kernels. */
tt_status tt_renderer_launches(tt_renderer *renderer, uint64_t *out, int32_t reset);

/* Batched rendering (no counterpart in the reference): many views of any size and sample count
 * rendered by one sequence of persistent wavefront kernels over a shared path index space, which
 * tt_batch_render captures once as a CUDA graph and replays. Every view's image is bit-identical
 * to tt_render_native of that view with the batch's parameters and the view's spp, sample
 * offset and seed. */
typedef struct tt_view {
    tt_camera_meta cam;    /* image size, pinhole and thin lens (aperture > 1e-5: lens radius, focal:
                              distance of the focal plane along the view direction) */
    int32_t spp;
    int32_t sample_offset;
    uint32_t seed;
    int32_t reserved;
} tt_view;
typedef struct tt_batch tt_batch;
/* params: max_depth, rr_depth, env_scale, ray_eps and flags apply to every view; its spp,
 * sample_offset and seed are ignored. The batch keeps a pointer to the renderer. */
tt_status tt_batch_create(tt_renderer *renderer, const tt_view *views, int32_t n, const tt_render_params *params,
                          tt_batch **out);
/* Paths of the whole batch, and the length of its accumulation buffer: view k's width*height*3
 * block follows view k-1's (floats, or doubles with TT_RENDER_ACCUM_F64). */
tt_status tt_batch_info(const tt_batch *batch, int64_t *total_paths, int64_t *accum_elems);
/* Adds every view's samples to d_accum. use_graph = 1: the first call (and any call after the
 * buffer, the launch shape or the renderer's path state changed) captures the kernel sequence as
 * a CUDA graph; later calls replay it. use_graph = 0: plain launches. Launch only. */
tt_status tt_batch_render(tt_batch *batch, void *d_accum, int32_t use_graph, void *stream);
/* Nodes of the captured graph (0 before the first graph render). */
tt_status tt_batch_graph_kernels(const tt_batch *batch, int32_t *kernels);
/* Times the batch's first paths under launch shapes in two stages: block x stack_shared (9
 * trials, written first to results) at 2^22-path waves, ordered and streamed, on a quarter of
 * the sample (at least 2^22 paths); then the fastest block and stack_shared at wave_paths in
 * {2^20, 2^22, 2^24, 2^26}, ordered or not, streamed or not (waves that would hold the whole
 * sample twice over are skipped, and a sample that fits one wave is timed in waves only), on
 * sample_paths paths (0: 2^28; at most the batch). Keeps the fastest stage-2 trial as the
 * renderer's shape and writes up to max_results trials to results (at most 9 + 16).
 * Synchronous; touches no accumulation buffer. */
tt_status tt_batch_autotune(tt_batch *batch, int64_t sample_paths, void *stream, tt_launch_shape *results,
                            int32_t max_results, int32_t *n_results);
tt_status tt_batch_free(tt_batch *batch);

/* Learned radiance cache (no counterpart in the reference): an MLP (160 encoded inputs, five
 * hidden layers of 64 with ReLU, RGB = exp(output)) with BF16 weights and FP32 accumulation on
 * tensor cores, trained online by Adam on a relative L2 loss from radiance the path tracer
 * itself measures. A feature record is 16 floats: position, direction towards the previous
 * vertex, shading normal, roughness, albedo (3), material kind / 8, 2 zeros. */
typedef struct tt_cache tt_cache;
typedef struct tt_cache_params {
    float lr, beta1, beta2, eps; /* Adam (defaults 1e-2, 0.9, 0.99, 1e-10) */
    float ema;                   /* inference weights = exponential average of the weights (0.95) */
    int32_t batch;               /* records per training step (16384) */
    int32_t steps;               /* training steps per rendered wave (4) */
    int32_t train_paths;         /* training paths per wave: traced to full depth, no cache (65536) */
    float spread_c;              /* end a path (from its second vertex on) when its spread exceeds
                                    spread_c x its pixel footprint (0.01); < 0: never */
    uint32_t seed;               /* weight initialisation (1) */
    int32_t use_ema;             /* render with the averaged weights (1) */
    float bbox_lo[3], bbox_hi[3];/* scene bounds of the position encoding */
    int32_t mma_kind;            /* the tensor-core kernels of inference and training: 0 tcgen05 +
                                    TMEM (default), 1 mma.sync */
    int32_t wait_limit;          /* tcgen05 inference: clock cycles one wait for a copy or a product
                                    may take before it counts as run out (0: about a second). A wait
                                    that runs out ends the launch with tt_cache_check reporting
                                    TT_ERR_TIMEOUT; tests set a tiny limit to exercise that path */
} tt_cache_params;
tt_status tt_cache_params_default(tt_cache_params *params);
tt_status tt_cache_create(const tt_cache_params *params, tt_cache **out);
tt_status tt_cache_free(tt_cache *cache);
/* Number of FP32 weights (27136): per layer [out][in], layers 160x64, 4 x 64x64, 64x8 (rows 3..7
 * of the last layer are padding and stay 0). */
tt_status tt_cache_param_count(int32_t *n);
/* which: 0 master weights, 1 averaged weights, 2 the last gradient (tt_cache_gradient). */
tt_status tt_cache_get_weights(const tt_cache *cache, float *h_weights, int32_t which);
/* Sets master and averaged weights (and their BF16 copies); resets the optimiser. */
tt_status tt_cache_set_weights(tt_cache *cache, const float *h_weights);
/* Encoded inputs of n <= batch records as n x 160 BF16 (tests). */
tt_status tt_cache_encode(tt_cache *cache, const float *d_records, int64_t n, void *d_encoded, void *stream);
/* Radiance (n x 3 floats) of n records. Launch only. */
tt_status tt_cache_infer(tt_cache *cache, const float *d_records, int64_t n, float *d_rgb, int32_t use_ema,
                         void *stream);
/* Gradient of the mean loss over n <= batch records w.r.t. the weights (host, tt_cache_param_count
 * floats) and the loss; no update. Synchronous. */
tt_status tt_cache_gradient(tt_cache *cache, const float *d_records, const float *d_targets, int64_t n,
                            float *h_gradient, float *h_loss, void *stream);
/* `steps` Adam steps over consecutive slices of `batch` of n records (targets: n x 3 radiance);
 * h_loss (optional) receives the mean loss. Synchronous only when h_loss is given. */
tt_status tt_cache_train(tt_cache *cache, const float *d_records, const float *d_targets, int64_t n, int32_t steps,
                         float *h_loss, void *stream);
/* Adam steps taken so far. */
tt_status tt_cache_steps(const tt_cache *cache, int32_t *steps);
/* The tensor-core kernels' error word (a bounded wait that ran out); synchronises `stream`. */
tt_status tt_cache_check(tt_cache *cache, void *stream);
/* The native path tracer with the cache: a path that is not a training path ends at the first
 * vertex from its second on where its spread exceeds spread_c x its pixel footprint, adding
 * throughput x (emission + cache radiance); training paths (cache params train_paths per wave,
 * spread evenly) are traced in full and leave a record at that vertex whose target is the
 * radiance they measured from there on; after each wave the cache takes its training steps
 * (train = 1). Otherwise as tt_render_native (with spread_c < 0 and train = 0 it is
 * bit-identical to it). */
tt_status tt_render_cached(tt_renderer *renderer, tt_cache *cache, const tt_camera_meta *cam,
                           const tt_render_params *params, void *d_accum, int32_t train, void *stream);

#define TT_NOALLOC_MAX_RAYS (1 << 18)
tt_status tt_trace_host_noalloc(const void *d_nodes, const void *d_vertices, const int32_t *d_tri_indices,
                                const tt_ray *h_rays, int64_t n, tt_hit *h_hits, int32_t closest,
                                void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TT_H */
