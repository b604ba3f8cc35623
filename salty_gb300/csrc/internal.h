// internal.h -- shared host/device definitions of libsalty_gpu (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/salty_gpu.h"

namespace salty {

// ------------------------------------------------------------------ BVH8 node
// 80 bytes, read as five 16-byte loads:
//   w0: origin p (3 x f32), packed exponents ex|ey<<8|ez<<16 | imask<<24
//   w1: child_base, tri_base, meta[0..3], meta[4..7]
//   w2: qlo_x[8], qlo_y[8]      w3: qlo_z[8], qhi_x[8]      w4: qhi_y[8], qhi_z[8]
// Child slot s covers [p + qlo*2^e, p + qhi*2^e] per axis (e = byte - 127); the
// quantised box contains the child's exact box.  Slot bit a is 1 when the child lies on
// the high side of the node centre along axis a, so visiting slots in increasing order
// of (slot XOR ray-octant) is roughly front to back.  imask bit s: slot s is an inner
// node, numbered child_base + popc(imask & ((1<<s)-1)); its meta byte is
// (1 << 5) | (24 + s).  A leaf slot's meta byte is (((1 << count) - 1) << 5) | offset:
// triangles tri_base + offset .. + count - 1.  So (meta >> 5) << (meta & 31) is the
// slot's bit pattern in a 32-bit hit mask (triangles 0..23, inner children 24..31,
// after XOR-ing inner slots with the ray octant).  Empty slots have meta 0 and
// qlo = 255 > qhi = 0, an empty box.
struct alignas(16) Bvh8Node {
    uint4 w[5];
};
static_assert(sizeof(Bvh8Node) == 80, "node layout");

constexpr int kMaxLeafTris = 3;
constexpr int kMaxNodeTris = 24;

// Leaf-ordered triangle: three float4, v0.xyz + input id (int bits), v1.xyz, v2.xyz.
constexpr int kTriFloat4 = 3;

// Binary build node (32 bytes).  count > 0: leaf over prim positions [a, a + count);
// count == 0: inner node with children a and a + 1.
struct alignas(16) BNode {
    float lo[3];
    int a;
    float hi[3];
    int count;
};

// ------------------------------------------------------------------ errors
struct ErrorSink {
    std::string msg;
    salty_status fail(salty_status s, const char* fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        msg = buf;
        return s;
    }
};

#define SALTY_TRY_CUDA(sink, expr)                                                              \
    do {                                                                                        \
        cudaError_t e__ = (expr);                                                               \
        if (e__ != cudaSuccess)                                                                 \
            return (sink).fail(e__ == cudaErrorMemoryAllocation ? SALTY_ERR_OOM : SALTY_ERR_CUDA, \
                               "%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e__)); \
    } while (0)

#define SALTY_TRY(expr)                       \
    do {                                      \
        salty_status s__ = (expr);            \
        if (s__ != SALTY_OK) return s__;      \
    } while (0)

// ------------------------------------------------------------------ device buffers
// Grow-only device allocation (cudaMalloc); contents are not preserved on growth.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        release();
        size_t want = n ? n : 1;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        else p = nullptr;
        return e;
    }
};

// ------------------------------------------------------------------ scene
struct GpuMaterial {
    int type;
    float color[3];
    float emission[3];
    float ior;
    float roughness;
    float rr_threshold;  // compat dice threshold max(colour, 0.01)
    float specular[3];   // Plastic
    float power;         // Phong, Plastic lobe exponent
    int color_map;       // texture multiplying the base colour, -1 none
};

// A texture in the scene's texel array: float4 texels (rgb, unused) from `offset`.
struct GpuTexture {
    long long offset;
    int width, height;
};

struct SceneConsts {
    int has_light;
    float lc[3], la[3], lb[3], ln[3], le[3];
    float larea;
    int light_tri0;      // first light triangle id (n_tris of the input), -1 if none
    int has_sun;
    float sun_dir[3], sun_rad[3];
    int sun_disk;            // 1: finite disk (sun_cos_max < 1), 0: delta light
    float sun_cos_max;       // cos of the disk's angular radius
    float sun_L[3];          // disk radiance = irradiance / solid angle
    float sun_pdf;           // 1 / solid angle
    float sun_t[3], sun_b[3];  // tangent frame around sun_dir
    float sky[3];
    float cam_pos[3], cam_cx[3], cam_cy[3], cam_cz[3];
    float cam_fov, cam_near;
    float cam_target[3], cam_up[3];
    float cam_lens, cam_focal;  // thin lens radius (0: pinhole), focal distance
    int ibl_map;                // environment texture, -1: constant sky
    float ibl_scale;
    int n_lights;               // has_light + sphere lights (Scene::GetLight's list)
    int sph_base;               // id of the first sphere (kNoSpheres: none)
};

struct Film {
    int width = 0, height = 0;           // film (window) size
    int frame_w = 0, frame_h = 0;        // frame the window belongs to
    int crop_x = 0, crop_y = 0;
    int fp64 = 0;
    int64_t samples = 0;
    DevBuf<float> sum, comp, sumsq;      // FP32 sum with Kahan compensation
    DevBuf<double> sum64, sumsq64;       // FP64 film
    DevBuf<float> aov;                   // first-hit feature sums, 7 per pixel
};

struct Bvh {
    DevBuf<Bvh8Node> nodes;
    DevBuf<float4> tris;        // leaf order, kTriFloat4 per triangle
    int64_t n_nodes = 0;
    int64_t n_tris = 0;         // leaf-order triangles
    int32_t depth = 0;
    bool built = false;
    uint64_t generation = 0;    // bumped by every build (batch arenas key on it)
    salty_bvh_info info{};
};

// One placed copy of a mesh in a two-level BVH, as the traversal reads it: the world-to-
// object transform for rays, the mesh's BVH root in the scene's node arena and the virtual
// triangle id of the instance's first triangle.
struct alignas(16) InstRec {
    float w2o[12];      // row-major 3x4
    unsigned root;      // the mesh's BVH8 root node
    int vbase;          // instance triangle j has id vbase + j
    int first;          // scene index of the mesh's first triangle
    int pad;
};
// The same instance as shading reads it: object-to-world transform of positions and the
// normal matrix (inverse transpose of its linear part).
struct alignas(16) InstShade {
    float o2w[12];
    float nrm[9];
    float pad[3];
};

// What one traversal launch walks: a BVH (or a batch arena of concatenated BVHs) and, per
// ray, the node it starts at.  With `inst`, node 0 starts a top-level BVH whose leaf
// entries are instances (two levels).
constexpr int kNoSpheres = 0x7fffffff;
constexpr int kSphLight = 1 << 30;  // flag in a sphere's material word: the sphere is a light

struct TraceTarget {
    const Bvh8Node* nodes = nullptr;
    const float4* tris = nullptr;
    int depth = 0;
    const int* roots = nullptr;  // per-ray root node, or null (node 0)
    const InstRec* inst = nullptr;
    int sph_base = kNoSpheres;   // first sphere id (leaf entries from it on are spheres)
};

// Launch shape of the traversal kernel, chosen by salty_autotune.
struct TraceTuning {
    int block = 128;     // threads per block: 64, 128 or 256
    int pool = 64;       // rays a warp takes from the global cursor per refill
    int postpone = 1;    // fewest lanes that test a triangle group together (1: never postpone)
    int regs = 56;       // register budget per thread: 64, or 56 (more resident warps: 9 blocks of 128)
};

}  // namespace salty

struct salty_scene {
    int64_t n_tris = 0;          // including the two light triangles
    int64_t n_input = 0;         // triangles given by the caller
    salty::DevBuf<float> pos;    // n_tris * 9
    salty::DevBuf<float> nrm;    // n_tris * 9
    salty::DevBuf<int> mat;      // n_tris
    salty::DevBuf<salty::GpuMaterial> mats;
    int n_mats = 0;
    salty::DevBuf<float> uv;     // n_tris * 6 (zeros when none were given)
    salty::DevBuf<salty::GpuTexture> textures;
    salty::DevBuf<float4> texels;
    int n_textures = 0;
    int64_t n_texels = 0;
    salty::SceneConsts consts{};
    salty::Bvh bvh;
    salty::Film film;
    // Instance (src/s3d_instance.cpp:22-101): when n_inst > 0 the world is these placed
    // copies of the scene's meshes (the light's triangles are one more, untransformed)
    std::vector<salty_instance> inst_host;
    salty::DevBuf<salty::InstRec> inst_rec;
    salty::DevBuf<salty::InstShade> inst_shade;
    salty::DevBuf<int> inst_vbase;  // n_inst + 1 prefix sums of triangle counts
    int n_inst = 0;
    int64_t n_virtual = 0;          // triangles of all instances
    // Sphere shapes (src/s3d_sphere.cpp:22-115): ids n_tris + k, in the same BVH
    std::vector<salty_sphere> sph_host;
    salty::DevBuf<float4> sph;      // centre, radius
    salty::DevBuf<int> sph_mat;     // material index
    salty::DevBuf<int> sph_lights;  // the spheres that are lights, in input order
    int n_sph = 0;
    int n_sph_lights = 0;
};

namespace salty {
// Launch shapes of the renderer, chosen by salty_autotune (include/salty_gpu.h).
struct Tuning {
    TraceTuning trace;
    // Paths in flight (queue capacity).  Every traversal launch ends with a tail of a few
    // long walks; freed queue slots are refilled with new samples each iteration, so the
    // launches stay full and a moderate queue already amortises the tails (1080p
    // heightfield, 64 spp: 1,360 Mrays/s at 2^22, 1,567 at 2^24, 1,633 at 2^26).  352 bytes
    // of path state per path plus 48 bytes per sample of the per-sample buffers: about 11 GB
    // at 2^24 for a depth-12 render.
    long long wave_paths = 1ll << 24;
    int shade_block = 256;             // threads per block of the shading kernels
};

// Device queues of the wavefront renderer, kept by the context between renders.
struct WaveStore {
    DevBuf<float4> rays[2], W[2], L[2], hits, nee, srays, shits, lbuf, abuf;
    DevBuf<uint4> meta[2];
    DevBuf<int> roots[2], sroots;
    DevBuf<int> counts, done;
    DevBuf<long long> ctl;
    DevBuf<unsigned long long> stats, tc0, tc1, tc2, tc3;  // tc*: traversal cursors of the two halves
};

// Scenes of a batch render concatenated: nodes and leaf triangles of every BVH back to
// back (child, triangle and id fields rebased), triangle attributes and materials likewise.
struct BatchArena {
    std::vector<std::pair<const void*, uint64_t>> key;  // (scene, BVH generation) per slot
    DevBuf<Bvh8Node> nodes;
    DevBuf<float4> tris;
    DevBuf<float> pos, nrm, uv;
    DevBuf<int> mat;
    DevBuf<GpuMaterial> mats;
    DevBuf<GpuTexture> textures;
    DevBuf<float4> texels;
    std::vector<long long> node_off, id_off, tex_off;
    int depth = 0;
};
}  // namespace salty

struct salty_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaStream_t aux_stream = nullptr;            // the render's second queue half
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaEvent_t ev[8] = {};
    salty::ErrorSink err;
    salty_trace_stats last_trace{};
    volatile int cancel = 0;
    // scratch shared by calls on this context
    salty::DevBuf<unsigned char> scratch;
    salty::DevBuf<float4> ray_buf;
    salty::DevBuf<float4> hit_buf;
    salty::DevBuf<unsigned long long> counters;
    salty::DevBuf<int> status;   // device status word(s)
    void* pinned = nullptr;      // small pinned readback area
    salty::Tuning tune;
    salty::WaveStore waves;
    salty::BatchArena arena;
    salty::DevBuf<unsigned char> slots;  // SceneSlot table of the current render
};

namespace salty {
// bvh_build.cu
salty_status build_bvh(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts);
// a BVH over n triangles (9 floats each, device) into `out`; root box lo, hi (host)
salty_status build_bvh_tris(salty_ctx* ctx, const float* d_pos, int n, const salty_build_opts& opts, Bvh& out,
                            float root_box[6]);
// instance.cu
salty_status build_instanced(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts);
salty_status build_with_spheres(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts);
// trace.cu
salty_status trace_launch(salty_ctx* ctx, salty_scene* sc, const float4* d_rays, long long n,
                          const int* n_dev, uint32_t flags, float4* d_hits,
                          unsigned long long* d_counters, cudaStream_t st, int* d_status);
salty_status trace_launch(salty_ctx* ctx, const TraceTarget& tgt, const TraceTuning& tune, const float4* d_rays,
                          long long n, const int* n_dev, uint32_t flags, float4* d_hits,
                          unsigned long long* d_counters, cudaStream_t st, int* d_status);
// render.cu
salty_status render(salty_ctx* ctx, salty_scene* sc, const salty_render_opts& o,
                    salty_render_stats* stats);
salty_status render_batch(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts, int n,
                          salty_render_stats* total);
salty_status check_render_opts(salty_ctx* ctx, const salty_scene* sc, const salty_render_opts* o);
salty_status film_outputs(salty_ctx* ctx, salty_scene* sc, const salty_render_opts& o,
                          float* d_mean, float* d_var, uint8_t* d_srgb);
salty_status film_features(salty_ctx* ctx, salty_scene* sc, float* d_mean, float* d_var, float* d_albedo,
                           float* d_normal, float* d_depth);
// post.cu
salty_status tonemap_device(salty_ctx* ctx, int type, int w, int h, const float* d_rgb,
                            float* d_out, uint8_t* d_srgb, int ref_oetf, float* ave, float* mx);
salty_status nlm_ref_device(salty_ctx* ctx, int w, int h, float coeff, const float* d_in,
                            float* d_out);
salty_status nlm_var_device(salty_ctx* ctx, int w, int h, int search_r, int patch_r, float k,
                            const float* d_rgb, const float* d_var, float* d_out);

inline bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
}  // namespace salty
