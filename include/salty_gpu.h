/* salty_gpu.h -- C ABI of the GB300-native Salty path-tracing hot path.
 *
 * The reference (ProjectAsura/Salty) is one Windows executable with an in-process C++
 * plugin API; it has no DLL or FFI.  Each entry point below replaces a piece of that
 * API (paths are relative to the reference project's src/ directory):
 *
 *   salty_scene_upload   Scene construction: Mesh::Create(n, Vertex*, IMaterial*)
 *                        (src/s3d_mesh.cpp:539), material factories
 *                        (src/s3d_materialfactory.cpp:28-132), PinholeCamera::Update
 *                        (include/s3d_camera.h:63-90), Scene members
 *                        (include/s3d_scene.h:98-103)
 *   salty_scene_set_instances  Instance (src/s3d_instance.cpp:22-101)
 *   salty_scene_set_spheres    Sphere (src/s3d_sphere.cpp:22-115), Scene::GetLight
 *                        (include/s3d_scene.h:84-90)
 *   salty_bvh_build      BVH8::Create / SplitSAH (src/s3d_bvh8.cpp:254-342,401-479)
 *   salty_trace          Scene::Intersect -> BVH8::IsHit -> Triangle::IsHit
 *                        (include/s3d_scene.h:63-75, src/s3d_bvh8.cpp:191-206,
 *                        src/s3d_triangle.cpp:73-105)
 *   salty_render         PathTracer::TracePath / Radiance / NextEventEstimation
 *                        (src/s3d_pt.cpp:182-353)
 *   salty_tonemap        ToneMapper::Map (src/s3d_tonemapper.cpp:206-353) and the sRGB8
 *                        conversion of PathTracer::Capture (src/s3d_pt.cpp:145-171)
 *   salty_denoise_nlm    FilterNLM (src/s3d_denoiser.cpp:19-95)
 *
 * Conventions.  Every call returns salty_status (0 = OK) and is synchronous on the
 * context's own CUDA stream.  Array arguments marked "host or device" may be either;
 * the library checks with cudaPointerGetAttributes and copies host arrays itself.
 * The caller keeps ownership of every array it passes.  A context is used by one host
 * thread at a time; separate contexts may run on separate threads.  Sizes are 64-bit.
 */
#ifndef SALTY_GPU_H
#define SALTY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SALTY_ABI_VERSION 2

typedef enum salty_status {
    SALTY_OK = 0,
    SALTY_ERR_INVALID_ARG = 1,
    SALTY_ERR_OOM = 2,
    SALTY_ERR_CUDA = 3,
    SALTY_ERR_TIMEOUT = 4,        /* a bounded device-side wait gave up */
    SALTY_ERR_QUEUE_OVERFLOW = 5, /* a device queue or traversal stack ran out of room */
    SALTY_ERR_CANCELLED = 6,      /* salty_ctx_cancel was called during the render */
    SALTY_ERR_NOT_BUILT = 7,      /* salty_trace/salty_render before salty_bvh_build */
    SALTY_ERR_CAPACITY = 8        /* input larger than a documented maximum */
} salty_status;

typedef struct salty_ctx salty_ctx;
typedef struct salty_scene salty_scene;

/* ---------------------------------------------------------------- context */
/* Replaces the process-wide state of PathTracer::Run (src/s3d_pt.cpp:77-132). */
salty_status salty_ctx_create(salty_ctx** out, int device);
void salty_ctx_destroy(salty_ctx* ctx);
/* Last error text of this context ("" if none).  Valid until the next call. */
const char* salty_last_error(const salty_ctx* ctx);
int salty_abi_version(void);
/* Requests that a running salty_render stop (any thread): the render returns
 * SALTY_ERR_CANCELLED after its current graph launch, at most 256 iterations of the path
 * loop. */
void salty_ctx_cancel(salty_ctx* ctx);

/* Page-locked host memory for fast copies (cudaHostAlloc). */
salty_status salty_host_alloc(salty_ctx* ctx, size_t bytes, void** out);
void salty_host_free(salty_ctx* ctx, void* p);

/* ---------------------------------------------------------------- scene */
enum { SALTY_LAMBERT = 0, SALTY_MIRROR = 1, SALTY_GLASS = 2, SALTY_GGX = 3, SALTY_PHONG = 4, SALTY_PLASTIC = 5 };

/* IMaterial (include/s3d_material.h:35-42): Lambert (src/s3d_lambert.cpp), Mirror
 * (src/s3d_mirror.cpp), Glass (src/s3d_glass.cpp), Phong (src/s3d_phong.cpp: color is the
 * specular colour), Plastic (src/s3d_plastic.cpp: color diffuse, specular, power) and a GGX
 * conductor (the reference only has SampleGGX, include/s3d_math.h:2985-2993). */
typedef struct salty_material {
    int32_t type;
    float color[3];     /* Lambert albedo / mirror, glass, GGX specular colour */
    float emission[3];
    float ior;          /* glass */
    float roughness;    /* GGX: alpha = roughness^2 */
    float specular[3];  /* Plastic: specular colour (color is its diffuse colour) */
    float power;        /* Phong, Plastic: lobe exponent (> 0) */
    int32_t color_map;  /* 1 + index of a texture that multiplies the base colour, 0 = none
                         * (TexturedMaterial, src/s3d_texturedmaterial.cpp:63-87) */
} salty_material;

/* PinholeCamera (include/s3d_camera.h:63-100) and ThinLensCamera (:150-267).  fov is the
 * reference's linear screen half-extent factor (a 40 degree field of view is
 * fov = 2 tan 20 deg).  lens_radius > 0 makes a thin lens focused at focal_distance
 * (0: |target - pos|, as ThinLensCamera::Update).  The compat profile reproduces the
 * reference's lens (offset in the world xy plane, focal plane z = const, a z-aligned
 * view); the physical profile puts the lens in the camera's screen axes and the focal
 * plane perpendicular to the view direction. */
typedef struct salty_camera {
    float pos[3], target[3], up[3];
    float fov;
    float near_clip;
    float lens_radius;
    float focal_distance;
} salty_camera;

/* An RGB float image; texel (x, y) is rgb[3 * (y * width + x)].  Sampled bilinearly with
 * the reference's wrap (Texture::SampleColor, src/s3d_texture.cpp:925-952). */
typedef struct salty_texture {
    int32_t width, height;
    const float* rgb;          /* host or device */
} salty_texture;

typedef struct salty_scene_desc {
    const float* tri_pos;      /* n_tris * 9: v0, v1, v2 (host or device) */
    const float* tri_nrm;      /* n_tris * 9 shading normals, or NULL (geometric) */
    const int32_t* tri_mat;    /* n_tris material indices, or NULL (all 0) */
    int64_t n_tris;
    const salty_material* mats;  /* host */
    int32_t n_mats;
    /* One-sided parallelogram area light, emitting along cross(edge_a, edge_b).  The
     * library adds its two triangles to the scene (indices n_tris, n_tris + 1). */
    int32_t has_light;
    float light_corner[3], light_edge_a[3], light_edge_b[3], light_emission[3];
    /* Directional sun: unit direction towards the sun, irradiance on a surface facing it,
     * and the angular radius of its disk in radians (0: a delta light, reachable only by
     * next-event estimation; > 0: a uniform disk of that radius, sampled by NEE and hit by
     * BSDF-sampled rays, the two combined by multiple importance sampling). */
    int32_t has_sun;
    float sun_dir[3], sun_radiance[3];
    float sun_half_angle;
    float sky[3];              /* constant sky radiance (Scene::SampleIBL) */
    salty_camera camera;
    /* Textures (Texture, src/s3d_texture.cpp): colour maps and an environment map. */
    const float* tri_uv;       /* n_tris * 6 texture coordinates (host or device), or NULL */
    const struct salty_texture* textures;  /* host table */
    int32_t n_textures;
    int32_t ibl_map;           /* 1 + index of a sphere-mapped environment texture that replaces
                                * the constant sky (Texture::SampleColor(dir)), 0 = none */
    float ibl_scale;           /* environment radiance = texel * ibl_scale (Scene::SampleIBL: 10) */
} salty_scene_desc;

salty_status salty_scene_upload(salty_ctx* ctx, const salty_scene_desc* desc, salty_scene** out);
void salty_scene_destroy(salty_ctx* ctx, salty_scene* scene);
/* Replaces the scene's camera (Scene::m_pCamera / PinholeCamera::Update,
 * include/s3d_camera.h:63-90) without touching geometry or BVH.  Render the next frame
 * with accumulate = 0: the film's samples belong to the old view. */
salty_status salty_scene_set_camera(salty_ctx* ctx, salty_scene* scene, const salty_camera* camera);

/* ---------------------------------------------------------------- meshes */
/* A mesh in host memory, owned by the library (salty_mesh_free). */
typedef struct salty_mesh {
    int64_t n_tris;
    float* tri_pos;             /* n_tris * 9 */
    float* tri_nrm;             /* n_tris * 9 vertex normals */
    float* tri_uv;              /* n_tris * 6 texture coordinates */
    int32_t* tri_mat;           /* n_tris material indices */
    int32_t n_mats;
    salty_material* mats;
    int32_t* mat_texture;       /* per material: its colour map's texture index, or -1 */
    int32_t n_textures;
    const char* texture_names;  /* n_textures x 256 bytes, names relative to the file */
} salty_mesh;

/* Reads an SMD file (Mesh::LoadFromFile, src/s3d_mesh.cpp:250-465; version 2): matte ->
 * Lambert, mirror, dielectric -> Glass, glossy -> Phong, plastic.  Texture maps are listed
 * but not applied.  Triangles with a negative material index take material 0.  ctx may
 * be NULL (no GPU is needed; errors then come without a message). */
salty_status salty_mesh_load_smd(salty_ctx* ctx, const char* path, salty_mesh** out);
void salty_mesh_free(salty_mesh* mesh);

/* Places n_tris triangles by a row-major 3x4 affine matrix (x' = M[0..2].x + M[3], ...):
 * positions by the matrix, normals by the inverse transpose of its linear part,
 * renormalised.  Instance (src/s3d_instance.cpp:22-101) keeps one copy of a mesh under
 * several transforms in a two-level BVH; here each placement is a transformed copy in the
 * scene's single BVH (same images, memory per copy).  nrm_in/nrm_out may be NULL. */
salty_status salty_mesh_transform(const float* matrix, int64_t n_tris, const float* pos_in, const float* nrm_in,
                                  float* pos_out, float* nrm_out);

/* ---------------------------------------------------------------- instances */
/* One placed copy of a mesh: the scene's triangles [first_tri, first_tri + n_tris) under a
 * row-major 3x4 object-to-world matrix (x' = M[0..2].x + M[3], ...; invertible). */
typedef struct salty_instance {
    int64_t first_tri;
    int64_t n_tris;
    float object_to_world[12];
} salty_instance;

/* Instance (src/s3d_instance.cpp:22-101): makes the scene's world n placed copies of its
 * meshes, each stored once, in a two-level BVH -- a top-level BVH over the instances' world
 * boxes whose leaves lead into one BVH per distinct mesh, which rays enter transformed to
 * object space (directions not renormalised, so hit distances stay world distances; the
 * reference renormalises, which makes distances of scaled instances incomparable).  Call
 * after salty_scene_upload and before salty_bvh_build; n = 0 returns to the flat scene.
 * The area light stays in world space.  Triangle ids (salty_trace, hit records) are then
 * virtual: instance i's triangle j is id base_i + j, base_i the triangle count of the
 * instances before it, the light's two triangles last.  Instanced scenes render through
 * salty_render (not salty_render_batch).  instances: host array. */
salty_status salty_scene_set_instances(salty_ctx* ctx, salty_scene* scene, const salty_instance* instances,
                                       int32_t n);

/* An analytic sphere (Sphere, src/s3d_sphere.cpp:22-115). */
typedef struct salty_sphere {
    float center[3];
    float radius;       /* > 0 */
    int32_t material;   /* index into the scene's material table */
    int32_t light;      /* nonzero: also a light of the scene, sampled by next-event estimation
                         * with its material's emission */
} salty_sphere;

/* Sphere shapes of the scene, in the same BVH as its triangles: hits report id n_tris + k
 * for sphere k (n_tris counting the area light's two triangles), t as for triangles and
 * u = v = 0.  Spheres marked as lights join the light list after the area light, in input
 * order; next-event estimation picks one light uniformly (Scene::GetLight,
 * include/s3d_scene.h:84-90), in the compat profile with Sphere::Sample's point on the
 * radius + 0.1 sphere and pdf 1/(4 pi r^2) (src/s3d_sphere.cpp:106-115), in the physical
 * profile with a direction uniform in the cone the sphere subtends, combined with BSDF
 * sampling by MIS.  Call after salty_scene_upload and before salty_bvh_build; n = 0 removes
 * them.  Not combined with instances; sphere scenes render through salty_render (not
 * salty_render_batch).  spheres: host array. */
salty_status salty_scene_set_spheres(salty_ctx* ctx, salty_scene* scene, const salty_sphere* spheres, int32_t n);

/* ---------------------------------------------------------------- BVH */
typedef struct salty_build_opts {
    int32_t bins;          /* SAH bins per axis, 8..32 (default 32) */
    int32_t max_leaf;      /* triangles per leaf, 1..3 (default 3) */
    float   trav_cost;     /* binary-build SAH: node cost relative to one triangle test (default
                            * 0.3, i.e. small leaves, which trace fastest here; 0 = default) */
} salty_build_opts;

typedef struct salty_bvh_info {
    int64_t n_nodes;       /* BVH8 nodes (80 bytes each) */
    int64_t n_binary;      /* binary nodes built before the collapse */
    int32_t depth;         /* BVH8 depth (root = 1) */
    int32_t binary_depth;
    double  sah_cost;      /* SAH cost of the BVH8 (node cost 1, triangle cost 1) */
    float   build_ms;      /* device time of the whole build (CUDA events) */
} salty_bvh_info;

/* Device binned-SAH build collapsed to 8-wide nodes with 8-bit quantised child boxes.
 * opts may be NULL (defaults).  info may be NULL. */
salty_status salty_bvh_build(salty_ctx* ctx, salty_scene* scene, const salty_build_opts* opts,
                             salty_bvh_info* info);

/* ---------------------------------------------------------------- trace */
typedef struct salty_ray { float org[3]; float tmin; float dir[3]; float tmax; } salty_ray; /* 32 B */
typedef struct salty_hit { float t; int32_t id; float u, v; } salty_hit;                    /* 16 B */

enum {
    SALTY_TRACE_ANY_HIT = 1 << 0,     /* stop at the first hit (occlusion); default closest */
    SALTY_TRACE_WATERTIGHT = 1 << 1,  /* watertight test; default: the reference's test */
    SALTY_TRACE_COUNTERS = 1 << 2     /* count node/triangle fetches (slower) */
};

/* Closest or any hit for n rays.  Closest hit: the smallest t the triangle test accepts
 * in [tmin, tmax]; equal t goes to the lowest triangle index.  Misses: id = -1, t = +inf.
 * u, v: barycentric weights of v1, v2.  rays/hits: host or device.  Triangle ids are
 * scene input indices. */
salty_status salty_trace(salty_ctx* ctx, salty_scene* scene, const salty_ray* rays, int64_t n,
                         uint32_t flags, salty_hit* hits);

typedef struct salty_trace_stats {
    double  kernel_ms;       /* device time of the traversal kernel(s), CUDA events */
    double  total_ms;        /* device time of the call including copies */
    int64_t rays;
    int64_t node_fetches;    /* SALTY_TRACE_COUNTERS only */
    int64_t tri_fetches;     /* SALTY_TRACE_COUNTERS only */
    int64_t h2d_bytes, d2h_bytes;
    int64_t launches;        /* traversal kernel launches of the call */
} salty_trace_stats;
/* Statistics of the last salty_trace on this context. */
salty_status salty_last_trace_stats(const salty_ctx* ctx, salty_trace_stats* out);

/* ---------------------------------------------------------------- render */
enum { SALTY_PROFILE_COMPAT = 0, SALTY_PROFILE_PHYSICAL = 1 };
enum { SALTY_TM_NONE = -1, SALTY_TM_REINHARD = 0, SALTY_TM_UNCHARTED2 = 1, SALTY_TM_ACES = 2 };

typedef struct salty_render_opts {
    int32_t width, height;
    int32_t spp;            /* samples per pixel added by this call */
    int32_t max_depth;      /* path segments (PathTracer::Config::MaxBounceCount) */
    int32_t rr_depth;       /* physical profile: Russian roulette from this depth */
    int32_t profile;        /* SALTY_PROFILE_* */
    uint64_t seed;
    int32_t accumulate;     /* 0: clear the film first; 1: add to it (progressive) */
    int32_t fp64;           /* accumulate in double (converged oracle images) */
    int32_t tonemap;        /* SALTY_TM_* for srgb8 output */
    int32_t ref_oetf;       /* 1: the reference's pow(1.055x, 1/2.4) - 0.055 OETF */
    /* Optional window of the width x height frame (all 0: the whole frame).  Pixels keep
     * their full-frame rays and random streams, so a window renders exactly the same
     * samples as the matching pixels of a full render; the film and the outputs are
     * crop_w x crop_h. */
    int32_t crop_x, crop_y, crop_w, crop_h;
} salty_render_opts;

typedef struct salty_render_stats {
    double  ms;               /* device time of the render call */
    int64_t samples;          /* camera samples in the film after the call */
    int64_t rays;             /* primary + extension + shadow rays traced by the call */
    int64_t paths;            /* camera paths traced by the call */
} salty_render_stats;

/* Renders opts->spp samples per pixel into the scene's film (wavefront path tracer), then
 * writes the film's per-pixel mean (mean_rgb, W*H*3 float), the variance of that mean
 * (var_rgb) and the tonemapped sRGB8 image (srgb8, W*H*3).  Any output may be NULL;
 * outputs are host or device. */
salty_status salty_render(salty_ctx* ctx, salty_scene* scene, const salty_render_opts* opts,
                          float* mean_rgb, float* var_rgb, uint8_t* srgb8, salty_render_stats* stats);

/* Renders several scenes in one pass: their samples share the wavefront queues of one
 * CUDA graph per wave, their BVHs are walked from one concatenated arena (built on the
 * first call for a set of scenes and kept while none of them is rebuilt), and each scene's
 * own film receives its samples exactly as salty_render with the same options would add
 * them (identical values).  PathTracer::Run (src/s3d_pt.cpp:77-132) renders one scene per
 * process; this is the batched form of it.  opts[i] belongs to scenes[i]; all scenes share
 * one profile; a scene may appear once.  total (may be NULL): device time, samples, rays
 * and paths of the whole batch.  Read each film with salty_render (spp = 0, accumulate = 1)
 * or salty_film_read. */
salty_status salty_render_batch(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts,
                                int32_t n, salty_render_stats* total);

/* Launch shapes of the renderer and the traversal kernel (per context). */
typedef struct salty_tuning {
    int32_t trace_block;     /* traversal threads per block: 64, 128 or 256 */
    int32_t trace_pool;      /* rays a warp takes from the queue per refill, 32..4096 */
    int32_t trace_postpone;  /* fewest lanes that test a triangle group together, 1..32 */
    int32_t shade_block;     /* shading threads per block, a multiple of 32 in 64..1024 */
    int32_t trace_regs;      /* traversal registers per thread: 64, or 56 (more resident warps) */
    int64_t wave_paths;      /* paths in flight (queue capacity), 2^16..2^27; default 2^24
                              * (352 bytes of path state per path plus per-sample buffers of
                              * up to 7x as many samples at 48 bytes: about 11 GB for a
                              * depth-12 render of that many samples or more; smaller renders
                              * allocate what they use) */
} salty_tuning;
salty_status salty_get_tuning(salty_ctx* ctx, salty_tuning* out);
salty_status salty_set_tuning(salty_ctx* ctx, const salty_tuning* t);
/* Picks the tuning for a render: trial renders of the batch with at most trial_spp samples
 * per pixel, timed with CUDA events, one pass of coordinate descent over wave_paths,
 * shade_block, trace_block, trace_regs, trace_pool and trace_postpone.  Leaves the best tuning set on
 * the context (also copied to out and its trial time to best_ms; either may be NULL) and
 * each film holding its last trial render: render with accumulate = 0 afterwards.  BVH node
 * width (8) and traversal stack depth (from the BVH depth) are fixed by the build. */
salty_status salty_autotune(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts, int32_t n,
                            int32_t trial_spp, salty_tuning* out, float* best_ms);
/* Picks the traversal launch shape (trace_block with trace_regs as pairs, then trace_pool,
 * then trace_postpone) for salty_trace of these rays on this scene, timing launches with
 * CUDA events; sets it on the context.  rays host or device; hits are discarded. */
salty_status salty_autotune_trace(salty_ctx* ctx, salty_scene* scene, const salty_ray* rays, int64_t n,
                                  uint32_t flags, salty_tuning* out, float* best_ms);

/* Film sums as stored (W*H*3 each): FP32 sum + Kahan compensation, or FP64 sums when the
 * film was rendered with fp64.  Arrays host or device; NULL skips. */
salty_status salty_film_read(salty_ctx* ctx, salty_scene* scene, double* sum, double* sumsq,
                             int64_t* samples);

/* Checkpoint / resume of a progressive render (the reference's dead app saved a BMP every
 * 29.9 s, src/s3d_app.cpp:491-501; this keeps the estimator's state instead).  Checkpoint:
 * per-pixel sums and sums of squares (W*H*3 doubles each), the FP32 film's Kahan
 * compensation (W*H*3 floats; pass NULL for an FP64 film), the first-hit feature sums (W*H*7
 * floats) and the sample count; any output may be NULL.  Restore: the film takes that state
 * for the frame/window/precision `opts` describe, and a salty_render with accumulate = 1 and
 * the same options then continues it exactly as if it had never stopped (comp and aov may be
 * NULL: zeros). */
salty_status salty_film_checkpoint(salty_ctx* ctx, salty_scene* scene, double* sum, double* sumsq, float* comp,
                                   float* aov, int64_t* samples);
salty_status salty_film_restore(salty_ctx* ctx, salty_scene* scene, const salty_render_opts* opts,
                                const double* sum, const double* sumsq, const float* comp, const float* aov,
                                int64_t samples);

/* Mean first-hit features of the film (the learned denoiser's auxiliary inputs): albedo
 * (W*H*3), shading normal facing the camera (W*H*3) and 1/(1 + hit distance) (W*H; 0 where
 * the camera ray escapes).  Arrays host or device; NULL skips. */
salty_status salty_film_aov(salty_ctx* ctx, salty_scene* scene, float* albedo, float* normal, float* depth);

/* ---------------------------------------------------------------- post */
/* ToneMapper::Map on a W*H*3 linear image, optionally followed by the sRGB8 conversion.
 * out_rgb / out_srgb8 may be NULL.  Arrays host or device. */
salty_status salty_tonemap(salty_ctx* ctx, int32_t type, int32_t width, int32_t height,
                           const float* rgb, float* out_rgb, uint8_t* out_srgb8, int32_t ref_oetf,
                           float* ave_lw, float* max_lw);

/* salty_tonemap, for callers that must not allocate device memory when they tonemap.
 * No counterpart in the reference: it exists for hosts that cannot call cudaMalloc at the
 * point where they tonemap -- a real-time viewer that tonemaps every frame inside its
 * render loop (cudaMalloc synchronises the whole device, which such a loop cannot afford),
 * or an engine that owns all GPU memory and forbids allocation after start-up.
 *   - Arrays are device memory of the context's GPU only: d_rgb (W*H*3 float), d_out_rgb
 *     and/or d_out_srgb8 (either may be NULL, not both).  The call allocates nothing and
 *     does not wait: it enqueues three kernels on `stream` (a cudaStream_t; NULL = the
 *     context's own stream) and returns; synchronise that stream before reading the outputs.
 *   - The context's own stream does not wait for work on other streams (the legacy default
 *     stream included, where most callers produce d_rgb): order the work that writes d_rgb
 *     before the call (an event or a synchronisation), or pass the producer's own stream.
 *   - Its scratch is a fixed 64 KiB device array inside the library, present on every GPU
 *     that loads the library until the process exits; images are limited to 16,777,216
 *     pixels (4096 x 4096).  Larger images return SALTY_ERR_CAPACITY before any launch.
 *   - The first call on each device looks up that array's device address once (with the
 *     device current); make that first call before any stream capture.
 *   - Every call reuses the same array and overwrites all of it that it reads, so nothing
 *     carries over between calls -- but calls that overlap on the GPU (other streams,
 *     other host threads) race on it: serialise them.
 * Results equal salty_tonemap's to within rounding: the log-luminance sum is added in a
 * different order (16-byte aligned inputs add four pixels' logarithms in FP32 before the
 * FP64 sum), and the log-average's exponential and the curve parameters are evaluated on
 * the GPU rather than on the host, so the scale factor can differ in the last bits. */
salty_status salty_tonemap_noalloc(salty_ctx* ctx, void* stream, int32_t type, int32_t width, int32_t height,
                                   const float* d_rgb, float* d_out_rgb, uint8_t* d_out_srgb8, int32_t ref_oetf);

/* FilterNLM as the reference defines it: RGBA, 5x5 patch, 13x13 search, h = sigma = coeff. */
salty_status salty_denoise_nlm_ref(salty_ctx* ctx, int32_t width, int32_t height, float coeff,
                                   const float* rgba, float* out);

/* Variance-scaled NLM on RGB with per-pixel variance of the mean (W*H*3 each):
 * search window (2 search_r + 1)^2, patch (2 patch_r + 1)^2, strength k. */
salty_status salty_denoise_nlm(salty_ctx* ctx, int32_t width, int32_t height, int32_t search_r,
                               int32_t patch_r, float k, const float* rgb, const float* var,
                               float* out);

/* ---------------------------------------------------------------- learned denoiser
 * No reference counterpart: the reference's only denoiser is FilterNLM
 * (src/s3d_denoiser.cpp:19-95).  A 5-level U-Net (3x3 convolutions, 16->32->48->64->80->96
 * channels, skip connections, about 566k parameters) whose convolutions run as implicit
 * GEMMs on the tensor cores in BF16 with FP32 accumulation, trained with Adam on an L1
 * loss in log(1 + colour) space.
 *
 * Features: n images of h x w pixels, 11 floats per pixel in this order: colour (the noisy
 * mean, linear), first-hit albedo (3), first-hit normal (3), 1/(1 + first-hit distance)
 * -- salty_film_read's mean followed by salty_film_aov's three planes -- and the colour's
 * noise level in log space, mean over channels of sqrt(var_c) / (1 + colour_c) with var the
 * variance of the mean.  h and w must be multiples of 16 and n*h*w at most 2^26.  Arrays
 * are host or device. */
typedef struct salty_unet salty_unet;

/* He-uniform initial weights from `seed`, zero biases. */
salty_status salty_unet_create(salty_ctx* ctx, uint64_t seed, salty_unet** out);
void salty_unet_destroy(salty_ctx* ctx, salty_unet* net);
/* Number of FP32 parameters: per layer, weights [9][cout][cin] then biases [cout]. */
int64_t salty_unet_param_count(const salty_unet* net);
/* Copies the FP32 parameters and/or the gradients of the last train step (either may be NULL). */
salty_status salty_unet_get_params(salty_ctx* ctx, salty_unet* net, float* params, float* grads);
salty_status salty_unet_set_params(salty_ctx* ctx, salty_unet* net, const float* params);
/* The optimiser's state (Adam first and second moments, one float per parameter each, and
 * the step count), for checkpointing a training run; any output of get may be NULL. */
salty_status salty_unet_get_adam(salty_ctx* ctx, salty_unet* net, float* m, float* v, int64_t* step);
salty_status salty_unet_set_adam(salty_ctx* ctx, salty_unet* net, const float* m, const float* v, int64_t step);
/* Denoised linear RGB, n*h*w*3 floats. */
salty_status salty_unet_forward(salty_ctx* ctx, salty_unet* net, const float* features, int32_t n, int32_t h,
                                int32_t w, float* out_rgb);
/* One step on a batch: forward, loss against target_rgb (n*h*w*3 linear), gradients, and,
 * when lr > 0, an Adam update (beta 0.9, 0.999, eps 1e-8).  With lr == 0 only the loss and
 * the gradients are computed.  *loss (may be NULL) = mean |y - log(1 + target)| over pixels
 * and colour channels, y = log(1 + input colour) + the network's correction. */
salty_status salty_unet_train_step(salty_ctx* ctx, salty_unet* net, const float* features, const float* target_rgb,
                                   int32_t n, int32_t h, int32_t w, float lr, float* loss);
/* Denoises the scene's film (the frame or window of the last salty_render) in one device
 * pass: film mean, variance and first-hit features -> features (borders reflected up to
 * multiples of 16) -> network.  out_rgb: film width * height * 3 floats, host or device.
 * NLM (salty_denoise_nlm) is the fallback where no trained weights exist. */
salty_status salty_denoise_unet(salty_ctx* ctx, salty_unet* net, salty_scene* scene, float* out_rgb);
/* The same, averaged over `mirrors` mirror images of the frame (1: as salty_denoise_unet;
 * 2: also left-right; 4: also top-bottom and both; 8: also the transposes of those four,
 * i.e. every symmetry of the pixel grid) -- a self-ensemble that lowers the network's own
 * error at the cost of `mirrors` forward passes. */
salty_status salty_denoise_unet_ensemble(salty_ctx* ctx, salty_unet* net, salty_scene* scene, int32_t mirrors,
                                        float* out_rgb);
/* The kernel of the network's convolutions: SALTY_CONV_TCGEN05 (default; fifth-generation
 * tensor cores, accumulators in tensor memory, inputs staged by the TMA copy engine where
 * they sit in one tensor), SALTY_CONV_TCGEN05_CP_ASYNC (the same MMAs with every input
 * staged by cp.async) or SALTY_CONV_MMA_SYNC (warp-level mma.sync).  All give the same
 * result up to the order of the FP32 sums.  The weight gradients follow: with the tcgen05
 * kinds they are tensor-core GEMMs summed in a fixed order (a training step is
 * deterministic); with SALTY_CONV_MMA_SYNC, mma.sync tiles added by FP32 atomics. */
enum { SALTY_CONV_TCGEN05 = 0, SALTY_CONV_MMA_SYNC = 1, SALTY_CONV_TCGEN05_CP_ASYNC = 2 };
salty_status salty_unet_set_conv_kernel(salty_ctx* ctx, salty_unet* net, int32_t kind);

/* ---------------------------------------------------------------- inputs */
/* The traversal microbenchmark's seeded inputs (host arrays): a triangle soup with
 * centroids uniform in [0,1]^3 and vertices within +-0.005, and rays from a radius-2
 * sphere about (0.5,0.5,0.5) towards uniform points of the cube. */
salty_status salty_microbench_soup(uint64_t seed, int64_t n, float* tri_pos);
salty_status salty_microbench_rays(uint64_t seed, int64_t n, float tmin, salty_ray* rays);

#ifdef __cplusplus
}
#endif
#endif /* SALTY_GPU_H */
