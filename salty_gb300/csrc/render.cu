// render.cu -- wavefront path tracer.
//
// Replaces PathTracer::TracePath / Radiance / NextEventEstimation (src/s3d_pt.cpp:182-353),
// which walk one path at a time per OpenMP thread.  Here the paths in flight live in queues
// on the device, split into two halves that run concurrently, and each iteration is, per half,
//   generate new camera paths into the queue's free slots
//   extend   closest-hit traversal of every live path         (trace.cu kernel)
//   shade1   next-event estimation: builds the shadow-ray queue
//   shadow   traversal of the shadow queue                     (trace.cu kernel)
//   shade2   adds unoccluded light, samples the BSDF, Russian roulette, and compacts the
//            surviving paths into the next queue (warp ballot + one atomic per warp)
// then, for both halves together, accumulate the samples whose paths have all ended to the
// film in sample order (Kahan-compensated FP32, or FP64) and plan the next iteration's new
// samples.  Queue lengths stay in device memory, so the whole frame is one CUDA graph whose
// conditional while-node repeats the iterations; each half's launches fill the SMs the
// other half's traversal tail leaves idle.
//
// Two estimators:
//   SALTY_PROFILE_COMPAT reproduces the reference's estimator: pixel-centre rays, uniform
//     hemisphere Lambert sampling weighted by albedo, dice-based termination without
//     reweighting (src/s3d_lambert.cpp:64-86), Mirror (src/s3d_mirror.cpp:59-71), the
//     Schlick Glass with its 1/0.5 branch weights (src/s3d_glass.cpp:60-128), NEE through
//     a closest-hit shadow ray with the reference's MIS weight (src/s3d_pt.cpp:251-292),
//     and the reference's triangle test with t in [1e-3, 1e12].
//   SALTY_PROFILE_PHYSICAL is an unbiased estimator for the same scenes: jittered pixels,
//     cosine-weighted Lambert, exact-Fresnel dielectric, GGX, balance-heuristic MIS
//     between BSDF sampling and the one-sided area light, a directional sun (delta, or a
//     disk sampled by NEE and hit by BSDF rays, combined by MIS), constant sky, Russian
//     roulette from rr_depth (survival min(1, max W), rolled only below 1), watertight
//     triangle test; camera rays start at t = 1e-4, rays leaving a surface at t = 0 from an
//     origin pushed off it (spawn).
// The first bounce of every sample also records the denoiser's features (albedo, shading
// normal, 1/(1 + distance)), averaged in the film next to the radiance.
// Random numbers: one PCG stream (include/s3d_math.h:2769-2817 step) per (pixel, sample).
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "internal.h"

namespace salty {
namespace {

constexpr float kPi = 3.1415926535897932384626433832795f;
constexpr float k2Pi = 6.283185307179586476925286766559f;
constexpr float kFHitMin = 1e-3f, kFHitMax = 1e12f;  // include/s3d_math.h:44-45
constexpr float kEps = 1e-4f;

// ---------------------------------------------------------------- RNG
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
struct Rng {
    unsigned long long s;
    __device__ __forceinline__ unsigned u32() {
        unsigned long long old = s;
        s = old * 6364136223846793005ull + 1442695040888963407ull;
        unsigned xs = (unsigned)(((old >> 18) ^ old) >> 27);
        unsigned rot = (unsigned)(old >> 59);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
    }
    __device__ __forceinline__ float f32() { return __fdiv_rn((float)u32(), 4294967296.0f); }
};
__device__ __forceinline__ Rng rng_for(unsigned long long seed, unsigned long long pixel, unsigned long long sample) {
    Rng r;
    r.s = mix64(seed ^ mix64((pixel << 32) | (sample & 0xffffffffull))) + 1442695040888963407ull;
    (void)r.u32();
    return r;
}

// ---------------------------------------------------------------- vectors
struct V {
    float x, y, z;
};
__device__ __forceinline__ V mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator*(V a, V b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V operator*(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V operator-(V a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V cross(V a, V b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float maxc(V a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ V safe_unit(V v) {
    float m = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return m > 0.0f ? mk(v.x / m, v.y / m, v.z / m) : v;
}
__device__ __forceinline__ V reflect(V i, V n) {
    float d2 = 2.0f * dot(n, i);
    return mk(i.x - d2 * n.x, i.y - d2 * n.y, i.z - d2 * n.z);
}
// Duff et al. 2017 (include/s3d_math.h:2875-2886)
__device__ __forceinline__ void tangent_space(V n, V& t, V& b) {
    float s = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (s + n.z);
    float bb = n.x * n.y * a;
    t = mk(1.0f + s * n.x * n.x * a, s * bb, -s * n.x);
    b = mk(bb, s + n.y * n.y * a, -n.y);
}
__device__ __forceinline__ V ld3(const float* p) { return mk(p[0], p[1], p[2]); }

// Origin of a ray leaving the surface point p in direction w: p pushed off the surface along
// the geometric normal ng (either orientation) to the side w points to, by 256 units in the
// last place of each coordinate, or by 2^-16 near the world origin where ulps are tiny
// (Waechter and Binder, "A Fast and Robust Method for Avoiding Self-Intersection", Ray
// Tracing Gems, 2019).  Rays spawned this way start at t = 0.
__device__ __forceinline__ float nudge(float p, float n) {
    const int o = (int)(256.0f * n);
    const float q = __int_as_float(__float_as_int(p) + (p < 0.0f ? -o : o));
    return fabsf(p) < 1.0f / 32.0f ? p + n * (1.0f / 65536.0f) : q;
}
__device__ __forceinline__ V spawn(V p, V ng, V w) {
    const V n = (ng.x * w.x + ng.y * w.y + ng.z * w.z) >= 0.0f ? ng : mk(-ng.x, -ng.y, -ng.z);
    return mk(nudge(p.x, n.x), nudge(p.y, n.y), nudge(p.z, n.z));
}
__device__ __forceinline__ V xyz(float4 v) { return mk(v.x, v.y, v.z); }

// ---------------------------------------------------------------- state
struct PathSoA {
    float4* W;      // throughput xyz, w = prev bsdf pdf
    float4* L;      // radiance xyz, w = unused
    uint4* meta;    // x,y = rng state, z = wave-local sample slot, w = depth | prev_delta<<16
};

struct Camera {
    float pos[3], cx[3], cy[3], cz[3];
    float dir[3], u[3], v[3];  // unit view direction and screen axes
    float lens, focal;         // thin lens radius (0: pinhole) and focal distance
};

// One scene of a batch (one slot for a plain render).  Its samples are the global sample
// indices [sample_off, sample_off + npx * spp), sample g -> (s, p) = divmod(g - sample_off,
// npx); its film pixels are [pixel_off, pixel_off + npx) of the batch's pixel space.
struct SceneSlot {
    SceneConsts k;              // light_tri0 in the ids of the batch's triangle arrays
    Camera cam;
    int width, height;          // the frame
    int crop_x, crop_y, film_w, film_h;
    int spp, max_depth, rr_depth, profile;
    int root;                   // BVH root node (batch arena index)
    int pad;
    long long npx;
    unsigned long long seed;
    float *sum, *comp, *sumsq, *aov;  // the scene's film (FP32 + Kahan, or FP64 below)
    double *sum64, *sumsq64;
};

struct WaveParams {
    const float* pos;
    const float* nrm;
    const float* uv;
    const int* mat;
    const GpuMaterial* mats;
    const GpuTexture* textures;
    const float4* texels;
    const SceneSlot* slots;
    const long long* sample_off;  // per slot, then the total (n_slots + 1 entries)
    const long long* pixel_off;   // per slot, then the total
    const InstRec* irec;          // instances (two-level scenes, one slot), or null
    const InstShade* ishade;
    const int* ivbase;            // n_inst + 1 first virtual ids
    const float4* sph;            // spheres (one scene): centre, radius
    const int* sph_mat;           // material | kSphLight when the sphere is a light
    const int* sph_lights;        // the light spheres, in light-list order
    int n_inst;
    int n_slots;
    int capacity;                 // paths in flight (queue length), cap_a + cap_b
    int cap_a, cap_b;             // the two halves' queue lengths
    int chunk;                    // samples per accumulation chunk
    long long ring;               // per-sample buffer entries: ring_chunks * chunk
    int ring_chunks;
    int launch_iters;             // iterations per graph launch
    long long iter_limit;         // iterations after which the render is declared stuck
    long long total_samples;
};

// Path state word meta.w: depth (bits 0..15), previous vertex delta (bit 16), slot (17..31).
constexpr int kSlotShift = 17;
constexpr int kMaxSlots = 1 << (32 - kSlotShift);
__device__ __forceinline__ unsigned pack_w(int depth, bool delta, int slot) {
    return (unsigned)depth | ((delta ? 1u : 0u) << 16) | ((unsigned)slot << kSlotShift);
}

struct WaveBuffers {
    float4* rays[2];
    PathSoA path[2];
    int* roots[2];     // per queued ray: BVH root of its scene (null for one scene)
    int* sroots;
    float4* hits;
    float4* nee;       // 2 per path: contribution xyz, w = shadow-queue index (int bits, -1 none)
    float4* srays;     // shadow queue rays (2 per path)
    float4* shits;
    float4* lbuf;      // per wave-local sample: radiance xyz
    float4* abuf;      // per wave-local sample, first hit: 2 x float4 (albedo, 1/(1+t)) (normal, 0)
    int* counts;       // [0] queue A len, [1] queue B len, [2] shadow len
    long long* ctl;    // the sample stream, see enum Ctl (shared by the halves)
    long long* gen;    // this half's pending generation: first sample, count, first queue slot
    int* done;         // per ring chunk: its samples whose paths have ended
    unsigned long long* stats;  // [0] rays traced, [1] paths
};

constexpr long long kMaxRingChunks = 16;  // per-sample buffers: at most 16 chunks of half a queue
constexpr long long kMinSplit = 1 << 16;  // queues of at least this many paths run as two halves
constexpr int kLaunchIters = 256;          // iterations per graph launch (cancellation granularity)

// Control words of the regenerating wavefront (ctl[]).
enum Ctl : int {
    kNext = 0,      // next global sample to start
    kAccBase = 1,   // samples below this are in the films
    kAccN = 2,      // samples [kAccBase, kAccBase + kAccN) are ready to accumulate
    kIters = 3,     // iterations run
    kLaunchEnd = 4, // this graph launch stops after iteration kLaunchEnd
    kGenA = 5,      // half A's pending generation (3 words, WaveBuffers::gen)
    kStuck = 8,     // set when kIters passed the iteration limit
    kGenB = 9,      // half B's pending generation (3 words)
    kCtlWords = 12
};

// the last slot whose offset is <= g (slots with no samples or pixels are skipped)
__device__ __forceinline__ int find_slot(const long long* off, int lo, int hi, long long g) {
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------- kernels
// Camera rays for the pending samples [g0, g0 + n) of the batch, appended to queue q at
// slots [slot0, slot0 + n); sample g of slot S -> (sample s, film pixel fp) = divmod(g -
// S.sample_off, S.npx).  PinholeCamera::GetRay (include/s3d_camera.h:95-100) with
// separately rounded operations.
__global__ void k_generate(WaveParams P, WaveBuffers B, int q) {
    const long long g0 = B.gen[0];
    const int n = (int)B.gen[1], slot0 = (int)B.gen[2];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const long long g = g0 + j;
        const int i = slot0 + j;                          // queue slot
        const unsigned r = (unsigned)(g % P.ring);        // per-sample buffer entry
        const int sid = P.n_slots == 1 ? 0 : find_slot(P.sample_off, 0, P.n_slots - 1, g);
        const SceneSlot& S = P.slots[sid];
        const long long gl = g - P.sample_off[sid];
        const long long s = gl / S.npx, fp = gl % S.npx;
        const int px = S.crop_x + (int)(fp % S.film_w), py = S.crop_y + (int)(fp / S.film_w);
        const long long p = (long long)py * S.width + px;  // full-frame pixel: its random stream
        Rng rng = rng_for(S.seed, (unsigned long long)p, (unsigned long long)s);
        float fx, fy;
        if (S.profile == SALTY_PROFILE_COMPAT) {
            fx = __fsub_rn(__fdiv_rn(__fadd_rn(0.5f, (float)px), (float)S.width), 0.5f);
            fy = __fsub_rn(__fdiv_rn(__fadd_rn(0.5f, (float)py), (float)S.height), 0.5f);
        } else {
            float jx = rng.f32(), jy = rng.f32();
            fx = __fsub_rn(__fdiv_rn(__fadd_rn(jx, (float)px), (float)S.width), 0.5f);
            fy = __fsub_rn(__fdiv_rn(__fadd_rn(jy, (float)py), (float)S.height), 0.5f);
        }
        float sp[3], d[3];  // screen point, direction
        for (int a = 0; a < 3; ++a) {
            sp[a] = __fadd_rn(__fadd_rn(__fmul_rn(S.cam.cx[a], fx), __fmul_rn(S.cam.cy[a], fy)), S.cam.cz[a]);
            d[a] = __fsub_rn(sp[a], S.cam.pos[a]);
        }
        const float mag = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
        const float tmin = S.profile == SALTY_PROFILE_COMPAT ? kFHitMin : kEps;
        const float tmax = S.profile == SALTY_PROFILE_COMPAT ? kFHitMax : INFINITY;
        V org = mk(S.cam.pos[0], S.cam.pos[1], S.cam.pos[2]);
        V dir = mk(__fdiv_rn(d[0], mag), __fdiv_rn(d[1], mag), __fdiv_rn(d[2], mag));
        if (S.cam.lens > 0.0f) {
            // ThinLensCamera::GetRay (include/s3d_camera.h:206-222): compat keeps the
            // reference's world-xy lens and z = const focal plane, physical uses the
            // screen axes and a focal plane perpendicular to the view
            const float th = k2Pi * rng.f32();
            const float rad = S.cam.lens * sqrtf(fmaxf(rng.f32(), 0.0f));
            float sn, cs;
            sincosf(th, &sn, &cs);
            const float lx = rad * cs, ly = rad * sn;
            V focus;
            if (S.profile == SALTY_PROFILE_COMPAT) {
                focus = org + dir * (S.cam.focal / fabsf(dir.z));
                org = org + mk(lx, ly, 0.0f);
            } else {
                focus = org + dir * (S.cam.focal / dot(dir, ld3(S.cam.dir)));
                org = org + ld3(S.cam.u) * lx + ld3(S.cam.v) * ly;
            }
            dir = safe_unit(focus - org);
        }
        B.rays[q][2 * i] = make_float4(org.x, org.y, org.z, tmin);
        B.rays[q][2 * i + 1] = make_float4(dir.x, dir.y, dir.z, tmax);
        if (B.roots[q]) B.roots[q][i] = S.root;
        B.path[q].W[i] = make_float4(1.f, 1.f, 1.f, 0.f);
        B.path[q].L[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        B.path[q].meta[i] = make_uint4((unsigned)rng.s, (unsigned)(rng.s >> 32), r, pack_w(0, true, sid));
        B.abuf[2 * r] = make_float4(0.f, 0.f, 0.f, 0.f);
        B.abuf[2 * r + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

struct Surf {
    V p, ng, ngf, ns, nsf;
    bool into;
};

// The scene triangle behind a hit id: the id itself, or, in a scene of instances, the mesh
// triangle of the (virtual) id and its instance (inst = -1 when there are none).
__device__ __forceinline__ int mesh_tri(const WaveParams& P, int id, int& inst) {
    inst = -1;
    if (P.n_inst == 0) return id;
    int lo = 0, hi = P.n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.ivbase[mid] <= id) lo = mid;
        else hi = mid - 1;
    }
    inst = lo;
    return P.irec[lo].first + (id - P.ivbase[lo]);
}
__device__ __forceinline__ V inst_point(const InstShade& S, V p) {
    return mk(S.o2w[0] * p.x + S.o2w[1] * p.y + S.o2w[2] * p.z + S.o2w[3],
              S.o2w[4] * p.x + S.o2w[5] * p.y + S.o2w[6] * p.z + S.o2w[7],
              S.o2w[8] * p.x + S.o2w[9] * p.y + S.o2w[10] * p.z + S.o2w[11]);
}
// Triangle::CalcParam's normal (src/s3d_triangle.cpp:107-121), not normalised, in world
// space: Instance::CalcParam (src/s3d_instance.cpp:80-84) applies the inverse transpose
__device__ __forceinline__ V interp_normal(const WaveParams& P, int mt, int inst, float u, float v) {
    const float* np = P.nrm + (size_t)mt * 9;
    const float al = 1.0f - u - v;
    const V n = mk(np[0] * al + np[3] * u + np[6] * v, np[1] * al + np[4] * u + np[7] * v,
                   np[2] * al + np[5] * u + np[8] * v);
    if (inst < 0) return n;
    const float* m = P.ishade[inst].nrm;
    return mk(m[0] * n.x + m[1] * n.y + m[2] * n.z, m[3] * n.x + m[4] * n.y + m[5] * n.z,
              m[6] * n.x + m[7] * n.y + m[8] * n.z);
}

__device__ __forceinline__ Surf surface(const WaveParams& P, int mt, int inst, float t, float u, float v, V o, V d) {
    Surf s;
    s.p = o + d * t;
    const float* tp = P.pos + (size_t)mt * 9;
    V v0 = ld3(tp), v1 = ld3(tp + 3), v2 = ld3(tp + 6);
    if (inst >= 0) {
        const InstShade& S = P.ishade[inst];
        v0 = inst_point(S, v0);
        v1 = inst_point(S, v1);
        v2 = inst_point(S, v2);
    }
    s.ng = safe_unit(cross(v1 - v0, v2 - v0));
    s.into = dot(s.ng, d) < 0.0f;
    s.ngf = s.into ? s.ng : -s.ng;
    s.ns = safe_unit(interp_normal(P, mt, inst, u, v));
    s.nsf = dot(s.ns, d) < 0.0f ? s.ns : -s.ns;
    return s;
}

// Texture::SampleColor (src/s3d_texture.cpp:925-952): bilinear, weights taken before the
// wrap, indices wrapped as |i % size| (which mirrors negative ones, as the reference does).
__device__ V tex_sample(const WaveParams& P, int map, float u, float v) {
    const GpuTexture t = P.textures[map];
    float fx = u * (float)(t.width - 1), fy = v * (float)(t.height - 1);
    if (!(fabsf(fx) < 1e9f)) fx = 0.0f;  // NaN / huge coordinates: keep the index arithmetic defined
    if (!(fabsf(fy) < 1e9f)) fy = 0.0f;
    int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    int x1 = x0 + 1, y1 = y0 + 1;
    const float xw0 = (float)x1 - fx, xw1 = fx - (float)x0, yw0 = (float)y1 - fy, yw1 = fy - (float)y0;
    x0 = abs(x0 % t.width);
    x1 = abs(x1 % t.width);
    y0 = abs(y0 % t.height);
    y1 = abs(y1 % t.height);
    const float4* T = P.texels + t.offset;
    const float4 c00 = T[(long long)y0 * t.width + x0], c01 = T[(long long)y1 * t.width + x0];
    const float4 c10 = T[(long long)y0 * t.width + x1], c11 = T[(long long)y1 * t.width + x1];
    return (xyz(c00) * yw0 + xyz(c01) * yw1) * xw0 + (xyz(c10) * yw0 + xyz(c11) * yw1) * xw1;
}

// Texture::SampleColor(dir) (src/s3d_texture.cpp:957-972): latitude-longitude lookup
__device__ V tex_sphere(const WaveParams& P, int map, V d) {
    const float theta = acosf(fminf(1.0f, fmaxf(-1.0f, d.y)));
    float u = 0.0f;
    const float v = theta * (1.0f / kPi);
    if (!(fabsf(d.x) <= FLT_EPSILON) && !(fabsf(d.z) <= FLT_EPSILON)) {
        const float phi = atan2f(d.z, d.x);
        u = (d.z < 0.0f ? phi + k2Pi : phi) * (1.0f / k2Pi);
    }
    return tex_sample(P, map, u, v);
}

// radiance arriving from the environment along d (Scene::SampleIBL, include/s3d_scene.h:81-82)
__device__ __forceinline__ V environment(const WaveParams& P, const SceneConsts& k, V d) {
    return k.ibl_map >= 0 ? tex_sphere(P, k.ibl_map, d) * k.ibl_scale : ld3(k.sky);
}

// the material's colour map at the hit (Triangle::CalcParam's texture coordinate), or 1
__device__ __forceinline__ V color_map(const WaveParams& P, const GpuMaterial& m, int id, float b1, float b2) {
    if (m.color_map < 0) return mk(1.0f, 1.0f, 1.0f);
    const float* t = P.uv + (size_t)id * 6;
    const float a = 1.0f - b1 - b2;
    return tex_sample(P, m.color_map, t[0] * a + t[2] * b1 + t[4] * b2, t[1] * a + t[3] * b1 + t[5] * b2);
}

__device__ __forceinline__ bool is_light(const SceneConsts& k, int id) {
    return k.light_tri0 >= 0 && id >= k.light_tri0 && id < k.light_tri0 + 2;
}

// ---------------------------------------------------------------- hits on spheres
// What shading needs to find behind a hit id: the material and either the mesh triangle
// (with its instance) or the sphere.
struct HitRef {
    int mat;
    int mtri;  // mesh triangle, -1 on a sphere
    int inst;  // instance of the triangle, -1 when none
    int sph;   // sphere index, -1 on a triangle
};
__device__ __forceinline__ HitRef hit_ref(const WaveParams& P, const SceneConsts& K, int id) {
    HitRef r;
    if (id >= K.sph_base) {
        r.sph = id - K.sph_base;
        r.mtri = -1;
        r.inst = -1;
        r.mat = P.sph_mat[r.sph] & (kSphLight - 1);
    } else {
        r.sph = -1;
        r.mtri = mesh_tri(P, id, r.inst);
        r.mat = P.mat[r.mtri];
    }
    return r;
}
__device__ __forceinline__ V sph_center(const WaveParams& P, int k) { return xyz(P.sph[k]); }
// Sphere::CalcParam (src/s3d_sphere.cpp:94-104): the outward normal at p ...
__device__ __forceinline__ V sph_normal(const WaveParams& P, int k, V p) { return safe_unit(p - sph_center(P, k)); }
// ... and the texture coordinate (phi / 2 pi, (pi - theta) / pi), phi = atan2(n.x, n.z)
// in [0, 2 pi), theta = acos(n.y)
__device__ __forceinline__ V sph_color_map(const WaveParams& P, const GpuMaterial& m, V n) {
    const float theta = acosf(fminf(1.0f, fmaxf(-1.0f, n.y)));
    float phi = atan2f(n.x, n.z);
    if (phi < 0.0f) phi += k2Pi;
    return tex_sample(P, m.color_map, phi * (1.0f / k2Pi), (kPi - theta) * (1.0f / kPi));
}
// the material's colour map at the hit point p (barycentrics b1, b2 on a triangle), or 1
__device__ __forceinline__ V hit_color_map(const WaveParams& P, const GpuMaterial& m, const HitRef& r, float b1,
                                           float b2, V p) {
    if (m.color_map < 0) return mk(1.0f, 1.0f, 1.0f);
    if (r.sph >= 0) return sph_color_map(P, m, sph_normal(P, r.sph, p));
    return color_map(P, m, r.mtri, b1, b2);
}
// unit shading normal, not oriented
__device__ __forceinline__ V hit_normal(const WaveParams& P, const HitRef& r, float b1, float b2, V p) {
    if (r.sph >= 0) return sph_normal(P, r.sph, p);
    return safe_unit(interp_normal(P, r.mtri, r.inst, b1, b2));
}
__device__ __forceinline__ Surf hit_surface(const WaveParams& P, const HitRef& r, float t, float b1, float b2, V o,
                                            V d) {
    if (r.sph < 0) return surface(P, r.mtri, r.inst, t, b1, b2, o, d);
    Surf s;
    s.p = o + d * t;
    s.ng = sph_normal(P, r.sph, s.p);
    s.into = dot(s.ng, d) < 0.0f;
    s.ngf = s.into ? s.ng : -s.ng;
    s.ns = s.ng;
    s.nsf = s.ngf;
    return s;
}

// Solid angle pdf of sampling sphere light k uniformly in the cone it subtends from x (0
// when x is inside): 1 / (2 pi (1 - cos theta_max)), 1 - cos = sin^2 / (1 + cos).
__device__ __forceinline__ float sph_cone_pdf(const WaveParams& P, int k, V x, float& cos_max) {
    const float4 sp = P.sph[k];
    const V w = xyz(sp) - x;
    const float d2 = dot(w, w), r2 = sp.w * sp.w;
    if (!(d2 > r2)) { cos_max = 1.0f; return 0.0f; }
    const float s2 = r2 / d2;
    cos_max = sqrtf(fmaxf(0.0f, 1.0f - s2));
    return 1.0f / (k2Pi * (s2 / (1.0f + cos_max)));
}

__device__ __forceinline__ float ggx_d(float nh, float a2) {
    float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * k * k);
}
__device__ __forceinline__ float ggx_g1(float nv, float a2) { return 2.0f * nv / (nv + sqrtf(a2 + (1.0f - a2) * nv * nv)); }
__device__ __forceinline__ V schlick(V f0, float c) {
    float m = 1.0f - c, m2 = m * m, m5 = m2 * m2 * m;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}
// SamplePhong (include/s3d_math.h:2976-2982): cos(theta) = (1 - v)^(1 / (n + 1))
__device__ __forceinline__ V sample_phong(float u, float v, float n) {
    float p = k2Pi * u;
    float ct = powf(1.0f - v, 1.0f / (n + 1.0f));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float sp, cp;
    sincosf(p, &sp, &cp);
    return mk(st * cp, st * sp, ct);
}
// Normalised Phong lobe around the mirror direction of wo (physical profile):
// f = (n + 2) / (2 pi) cos^n, sampled with pdf (n + 1) / (2 pi) cos^n.
__device__ __forceinline__ float phong_lobe(V n, V wo, V wi, float power, float& pdf) {
    V r = reflect(-wo, n);
    float c = dot(r, wi);
    if (c <= 0.0f) { pdf = 0.0f; return 0.0f; }
    float cn = powf(c, power);
    pdf = (power + 1.0f) / k2Pi * cn;
    return (power + 2.0f) / k2Pi * cn;
}
// Plastic (physical profile): Schlick F (R0 = 0.04) at the outgoing angle weighs a Phong
// lobe (specular) against a Lambert base (1 - F); the lobe is sampled with probability
// clamp(F, 0.1, 0.9) and the mixture pdf is used.
__device__ __forceinline__ float plastic_fresnel(float cos_o) {
    float m = 1.0f - fmaxf(cos_o, 0.0f), m2 = m * m;
    return 0.04f + 0.96f * m2 * m2 * m;
}
__device__ __forceinline__ float plastic_ps(float F) { return fminf(0.9f, fmaxf(0.1f, F)); }

// f(wo, wi) without the cosine, and the BSDF-sampling pdf (physical profile)
__device__ __forceinline__ V phys_eval(const GpuMaterial& m, V n, V wo, V wi, float& pdf) {
    V col = ld3(m.color);
    float ni = dot(n, wi);
    if (m.type == SALTY_PHONG) {
        float lp;
        float f = phong_lobe(n, wo, wi, m.power, lp);
        pdf = lp;
        return col * f;
    }
    if (m.type == SALTY_PLASTIC) {
        float lp;
        float fl = phong_lobe(n, wo, wi, m.power, lp);
        float F = plastic_fresnel(dot(n, wo)), ps = plastic_ps(F);
        pdf = ps * lp + (1.0f - ps) * fmaxf(ni, 0.0f) / kPi;
        return ld3(m.specular) * (F * fl) + col * ((1.0f - F) / kPi);
    }
    if (m.type == SALTY_GGX) {
        float a = m.roughness * m.roughness, a2 = a * a;
        float no = dot(n, wo);
        V h = safe_unit(wo + wi);
        float nh = dot(n, h), oh = dot(wo, h);
        if (no <= 0.0f || ni <= 0.0f || nh <= 0.0f || oh <= 0.0f) { pdf = 0.0f; return mk(0, 0, 0); }
        float D = ggx_d(nh, a2), G = ggx_g1(no, a2) * ggx_g1(ni, a2);
        pdf = D * nh / (4.0f * oh);
        return schlick(col, oh) * (D * G / (4.0f * no * ni));
    }
    pdf = ni / kPi;
    return col * (1.0f / kPi);
}

// warp-aggregated append: returns this lane's slot in a queue of counter `ctr`
__device__ __forceinline__ int warp_append(bool want, int* ctr) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return -1;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(ctr, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// NEE for the live paths of queue `q`: appends shadow rays, stores contributions.
// The shading kernels gather path state, hits and triangle attributes from HBM: capped at 64
// registers (from 85 and 92, a few spilled values) they keep four 256-thread blocks per SM
// in flight instead of two, and the 1080p heightfield frame runs 2.8 % faster.
__global__ void __maxnreg__(64) k_shade1(WaveParams P, WaveBuffers B, int q) {
    const int n = B.counts[q];
    const int stride = gridDim.x * blockDim.x;
    const int lim = (n + 31) & ~31;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lim; i += stride) {
        bool live = i < n;
        float4 h = live ? B.hits[i] : make_float4(0, 0, 0, 0);
        int id = __float_as_int(h.y);
        bool want_l = false, want_s = false;
        float4 ray_l0, ray_l1, ray_s0, ray_s1;
        V cl = mk(0, 0, 0), cs = mk(0, 0, 0);
        float4 e1x = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // compat sphere light: dist^2, pdf, index + 1
        const uint4 mt = live ? B.path[q].meta[i] : make_uint4(0, 0, 0, 0);
        const int slot = (int)(mt.w >> kSlotShift);
        const SceneSlot& S = P.slots[slot];
        const SceneConsts& K = S.k;
        if (live && id >= 0 && !is_light(K, id)) {
            const HitRef hr = hit_ref(P, K, id);
            GpuMaterial m = P.mats[hr.mat];
            const float4 r0 = B.rays[q][2 * i], r1 = B.rays[q][2 * i + 1];
            V o = xyz(r0), d = xyz(r1);
            const V hp = mk(__fadd_rn(o.x, __fmul_rn(d.x, h.x)), __fadd_rn(o.y, __fmul_rn(d.y, h.x)),
                            __fadd_rn(o.z, __fmul_rn(d.z, h.x)));
            // TexturedMaterial::GetBaseColor: the colour map multiplies the base colour
            const V tx = hit_color_map(P, m, hr, h.z, h.w, hp);
            m.color[0] *= tx.x; m.color[1] *= tx.y; m.color[2] *= tx.z;
            const bool delta = (m.type == SALTY_MIRROR || m.type == SALTY_GLASS);
            Rng rng;
            rng.s = (unsigned long long)mt.x | ((unsigned long long)mt.y << 32);
            if (S.profile == SALTY_PROFILE_COMPAT) {
                if (!delta && K.n_lights > 0) {
                    const V p = hp;
                    const V nrm = hit_normal(P, hr, h.z, h.w, p);
                    // Scene::GetLight (include/s3d_scene.h:84-90): one light, uniformly
                    const int li = (int)(rng.u32() % (unsigned)K.n_lights);
                    const V fs = ld3(m.color) * (1.0f / kPi);
                    if (li < K.has_light) {
                        float u = rng.f32(), w = rng.f32();
                        V lp = ld3(K.lc) + ld3(K.la) * u + ld3(K.lb) * w;
                        float pdf = 1.0f / K.larea;
                        V ld = lp - p;
                        float dist2 = dot(ld, ld);
                        ld = safe_unit(ld);
                        float cos_s = fabsf(dot(nrm, ld));
                        float cos_l = fabsf(dot(ld3(K.ln), -ld));
                        float G = cos_s * cos_l / dist2;
                        float brdf_pdf = fabsf(ld.z / kPi) * cos_l / dist2;
                        float mis = pdf / (brdf_pdf + pdf);
                        cl = ld3(K.le) * fs * mis * (G / pdf);
                        want_l = true;
                        ray_l0 = make_float4(p.x, p.y, p.z, kFHitMin);
                        ray_l1 = make_float4(ld.x, ld.y, ld.z, kFHitMax);
                    } else {
                        // Sphere::Sample (src/s3d_sphere.cpp:106-115): a point on the sphere
                        // of radius r + 0.1, pdf 1 / (4 pi r^2); the light's normal and the
                        // rest of the estimate wait for the shadow ray's hit (k_shade2)
                        const int k = P.sph_lights[li - K.has_light];
                        const float4 sp = P.sph[k];
                        const float a1 = k2Pi * rng.f32();
                        const float z = 1.0f - 2.0f * rng.f32();
                        const float rr = sqrtf(1.0f - z * z);
                        const V lp = xyz(sp) + safe_unit(mk(rr * cosf(a1), rr * sinf(a1), z)) * (sp.w + 1e-1f);
                        const float pdf = 1.0f / (4.0f * kPi * sp.w * sp.w);
                        V ld = lp - p;
                        const float dist2 = dot(ld, ld);
                        ld = safe_unit(ld);
                        cl = fs * fabsf(dot(nrm, ld));
                        e1x = make_float4(dist2, pdf, __int_as_float(k + 1), 0.0f);
                        want_l = true;
                        ray_l0 = make_float4(p.x, p.y, p.z, kFHitMin);
                        ray_l1 = make_float4(ld.x, ld.y, ld.z, kFHitMax);
                    }
                }
            } else {
                if (!delta) {
                    Surf s = hit_surface(P, hr, h.x, h.z, h.w, o, d);
                    V wo = -d;
                    if (K.n_lights > 0) {
                        // one light of the list, uniformly (the draw only with two or more)
                        int li = 0;
                        if (K.n_lights > 1) li = min((int)(rng.f32() * (float)K.n_lights), K.n_lights - 1);
                        const float psel = 1.0f / (float)K.n_lights;
                        if (li < K.has_light) {
                            float u1 = rng.f32(), u2 = rng.f32();
                            V lp = ld3(K.lc) + ld3(K.la) * u1 + ld3(K.lb) * u2;
                            V wi = lp - s.p;
                            float dist2 = dot(wi, wi), dist = sqrtf(dist2);
                            wi = wi * (1.0f / dist);
                            float cos_l = dot(ld3(K.ln), -wi);
                            float cos_s = dot(s.nsf, wi), cos_g = dot(s.ngf, wi);
                            if (cos_l > 0.0f && cos_s > 0.0f && cos_g > 0.0f) {
                                float pdf_b;
                                V f = phys_eval(m, s.nsf, wo, wi, pdf_b);
                                float pdf_l = psel * dist2 / (cos_l * K.larea);
                                float mis = pdf_l / (pdf_l + pdf_b);
                                cl = f * ld3(K.le) * (cos_s * mis / pdf_l);
                                want_l = true;
                                const V so = spawn(s.p, s.ng, wi);
                                ray_l0 = make_float4(so.x, so.y, so.z, 0.0f);
                                ray_l1 = make_float4(wi.x, wi.y, wi.z, dist * (1.0f - 1e-4f));
                            }
                        } else {
                            // a direction uniform in the cone the sphere subtends
                            const int k = P.sph_lights[li - K.has_light];
                            const float u1 = rng.f32(), u2 = rng.f32();
                            float cos_max;
                            const float pdf_c = sph_cone_pdf(P, k, s.p, cos_max);
                            if (pdf_c > 0.0f) {
                                const float4 sp = P.sph[k];
                                const V w = xyz(sp) - s.p;
                                const float dc = sqrtf(dot(w, w));
                                const V wz = w * (1.0f / dc);
                                const float one_m = (1.0f - cos_max) * u1;  // 1 - cos theta
                                const float ct = 1.0f - one_m;
                                const float st = sqrtf(fmaxf(0.0f, one_m * (2.0f - one_m)));
                                float sp_, cp_;
                                sincosf(k2Pi * u2, &sp_, &cp_);
                                V tx_, ty_;
                                tangent_space(wz, tx_, ty_);
                                const V wi = safe_unit(tx_ * (st * cp_) + ty_ * (st * sp_) + wz * ct);
                                // distance to the near side, (dc^2 - r^2) / (dc cos + sqrt(r^2 -
                                // dc^2 sin^2)): no cancellation at the cone's edge
                                const float hs = sp.w * sp.w - dc * dc * st * st;
                                const float dist = (dc * dc - sp.w * sp.w) / (dc * ct + sqrtf(fmaxf(0.0f, hs)));
                                const float cos_s = dot(s.nsf, wi), cos_g = dot(s.ngf, wi);
                                if (cos_s > 0.0f && cos_g > 0.0f && dist > 0.0f) {
                                    float pdf_b;
                                    V f = phys_eval(m, s.nsf, wo, wi, pdf_b);
                                    const float pdf_l = psel * pdf_c;
                                    const float mis = pdf_l / (pdf_l + pdf_b);
                                    const V le = ld3(P.mats[P.sph_mat[k] & (kSphLight - 1)].emission);
                                    cl = f * le * (cos_s * mis / pdf_l);
                                    want_l = true;
                                    // the shadow ray runs from the light point back to the
                                    // surface: from just outside the sphere it cannot meet
                                    // the sphere itself, which a ray towards a grazing point
                                    // on its silhouette could, by rounding
                                    const V lq = s.p + wi * dist;
                                    const V qs = spawn(lq, safe_unit(lq - xyz(sp)), -wi);
                                    const V ps = spawn(s.p, s.ng, wi);
                                    V back = ps - qs;
                                    const float blen = sqrtf(dot(back, back));
                                    back = back * (1.0f / blen);
                                    ray_l0 = make_float4(qs.x, qs.y, qs.z, 0.0f);
                                    ray_l1 = make_float4(back.x, back.y, back.z, blen * (1.0f - 1e-4f));
                                }
                            }
                        }
                    }
                    if (K.has_sun) {
                        V wi = ld3(K.sun_dir);
                        if (K.sun_disk) {
                            // uniform direction in the sun's cone
                            float u1 = rng.f32(), u2 = rng.f32();
                            float ct = 1.0f - u1 * (1.0f - K.sun_cos_max);
                            float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                            float sp, cp;
                            sincosf(k2Pi * u2, &sp, &cp);
                            wi = safe_unit(ld3(K.sun_t) * (st * cp) + ld3(K.sun_b) * (st * sp) + wi * ct);
                        }
                        float cos_s = dot(s.nsf, wi), cos_g = dot(s.ngf, wi);
                        if (cos_s > 0.0f && cos_g > 0.0f) {
                            float pdf_b;
                            V f = phys_eval(m, s.nsf, wo, wi, pdf_b);
                            if (K.sun_disk) {
                                float mis = K.sun_pdf / (K.sun_pdf + pdf_b);
                                cs = f * ld3(K.sun_L) * (cos_s * mis / K.sun_pdf);
                            } else {
                                cs = f * ld3(K.sun_rad) * cos_s;
                            }
                            want_s = true;
                            const V so = spawn(s.p, s.ng, wi);
                            ray_s0 = make_float4(so.x, so.y, so.z, 0.0f);
                            ray_s1 = make_float4(wi.x, wi.y, wi.z, INFINITY);
                        }
                    }
                }
            }
            B.path[q].meta[i] = make_uint4((unsigned)rng.s, (unsigned)(rng.s >> 32), mt.z, mt.w);
        }
        const int ql = warp_append(want_l, &B.counts[2]);
        const int qs = warp_append(want_s, &B.counts[2]);
        if (want_l) {
            B.srays[2 * ql] = ray_l0;
            B.srays[2 * ql + 1] = ray_l1;
            if (B.sroots) B.sroots[ql] = S.root;
        }
        if (want_s) {
            B.srays[2 * qs] = ray_s0;
            B.srays[2 * qs + 1] = ray_s1;
            if (B.sroots) B.sroots[qs] = S.root;
        }
        if (live) {
            B.nee[2 * i] = make_float4(cl.x, cl.y, cl.z, __int_as_float(want_l ? ql : -1));
            B.nee[2 * i + 1] = make_float4(want_s ? cs.x : e1x.x, want_s ? cs.y : e1x.y, want_s ? cs.z : e1x.z,
                                           __int_as_float(want_s ? qs : -1));
        }
    }
}

// BSDF sampling, Russian roulette, compaction of queue q into queue q^1.
__global__ void __maxnreg__(64) k_shade2(WaveParams P, WaveBuffers B, int q) {
    const int n = B.counts[q];
    const int stride = gridDim.x * blockDim.x;
    const int lim = (n + 31) & ~31;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lim; i += stride) {
        const bool live = i < n;
        bool cont = false;
        float4 nr0, nr1, nW, nL;
        uint4 nmeta;
        int root = 0, ended = -1;
        if (live) {
            const float4 h = B.hits[i];
            const int id = __float_as_int(h.y);
            float4 W4 = B.path[q].W[i], L4 = B.path[q].L[i];
            uint4 mt = B.path[q].meta[i];
            const int slot = (int)(mt.w >> kSlotShift);
            const int depth = (int)(mt.w & 0xffffu);
            const SceneSlot& S = P.slots[slot];
            const SceneConsts& K = S.k;
            const bool compat = S.profile == SALTY_PROFILE_COMPAT;
            root = S.root;
            V W = xyz(W4), L = xyz(L4);
            float prev_pdf = W4.w;
            const bool prev_delta = (mt.w >> 16) & 1u;
            Rng rng;
            rng.s = (unsigned long long)mt.x | ((unsigned long long)mt.y << 32);
            const float4 r0 = B.rays[q][2 * i], r1 = B.rays[q][2 * i + 1];
            V o = xyz(r0), d = xyz(r1);
            // unoccluded light
            const float4 e0 = B.nee[2 * i], e1 = B.nee[2 * i + 1];
            const int q0 = __float_as_int(e0.w), q1 = __float_as_int(e1.w);
            const int sk = compat ? __float_as_int(e1.z) - 1 : -1;  // compat: sampled light sphere
            if (q0 >= 0 && sk >= 0) {
                // NextEventEstimation with a sphere light (src/s3d_pt.cpp:274-288): accepted
                // when the shadow ray's first hit is that sphere; the light's normal is taken
                // where the ray hit it, the distance is the sampled point's
                const float4 sh = B.shits[q0];
                if (__float_as_int(sh.y) == K.sph_base + sk) {
                    const V sd = xyz(B.srays[2 * q0 + 1]);
                    const V hp = xyz(B.srays[2 * q0]) + sd * sh.x;
                    const float cos_l = fabsf(dot(sph_normal(P, sk, hp), -sd));
                    const float dist2 = e1.x, pdf = e1.y;
                    const float brdf_pdf = fabsf(sd.z / kPi) * cos_l / dist2;
                    const float mis = pdf / (brdf_pdf + pdf);
                    const V le = ld3(P.mats[P.sph_mat[sk] & (kSphLight - 1)].emission);
                    L = L + W * le * xyz(e0) * (mis * (cos_l / dist2) / pdf);
                }
            } else if (q0 >= 0) {
                const int sid = __float_as_int(B.shits[q0].y);
                bool vis = compat ? (sid >= 0 && is_light(K, sid)) : (sid < 0);
                if (vis) L = L + W * xyz(e0);
            }
            if (q1 >= 0) {
                const int sid = __float_as_int(B.shits[q1].y);
                if (sid < 0) L = L + W * xyz(e1);
            }
            if (depth == 0 && id >= 0) {
                // first-hit features of the sample (denoiser inputs): albedo, 1/(1+t),
                // shading normal facing the camera
                const HitRef ar = hit_ref(P, K, id);
                const GpuMaterial am = P.mats[ar.mat];
                const V ap = o + d * h.x;
                V n = hit_normal(P, ar, h.z, h.w, ap);
                if (dot(n, d) > 0.0f) n = -n;
                const bool emitter = is_light(K, id);
                const V atx = hit_color_map(P, am, ar, h.z, h.w, ap);
                B.abuf[2 * mt.z] = make_float4(emitter ? 1.0f : am.color[0] * atx.x, emitter ? 1.0f : am.color[1] * atx.y,
                                               emitter ? 1.0f : am.color[2] * atx.z, 1.0f / (1.0f + h.x));
                B.abuf[2 * mt.z + 1] = make_float4(n.x, n.y, n.z, 0.0f);
            }
            if (id < 0) {
                L = L + W * environment(P, K, d);
                // an escaping ray inside the sun's disk (physical profile, finite sun)
                if (!compat && K.has_sun && K.sun_disk && dot(d, ld3(K.sun_dir)) >= K.sun_cos_max) {
                    const float w = prev_delta ? 1.0f : prev_pdf / (prev_pdf + K.sun_pdf);
                    L = L + W * ld3(K.sun_L) * w;
                }
            } else if (compat) {
                const HitRef hr = hit_ref(P, K, id);
                const GpuMaterial m = P.mats[hr.mat];
                V pos = mk(__fadd_rn(o.x, __fmul_rn(d.x, h.x)), __fadd_rn(o.y, __fmul_rn(d.y, h.x)),
                           __fadd_rn(o.z, __fmul_rn(d.z, h.x)));
                const V tx = hit_color_map(P, m, hr, h.z, h.w, pos);  // TexturedMaterial::Shade scales the weight
                L = L + W * ld3(m.emission);
                V normal = hit_normal(P, hr, h.z, h.w, pos);
                V nm = dot(normal, d) < 0.0f ? normal : -normal;
                V col = ld3(m.color), out, wgt;
                bool dice = false;
                if (m.type == SALTY_MIRROR) {
                    out = safe_unit(reflect(d, nm));
                    wgt = col;
                } else if (m.type == SALTY_GLASS) {
                    V refl = safe_unit(reflect(d, nm));
                    bool into = dot(normal, nm) > 0.0f;
                    float nc = 1.0f, nt = m.ior;
                    float nnt = into ? nc / nt : nt / nc;
                    float ddn = dot(d, nm);
                    float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
                    if (cos2t < 0.0f) {
                        out = refl;
                        wgt = col;
                    } else {
                        V refr = safe_unit(d * nnt - normal * (into ? 1.0f : -1.0f) * (ddn * nnt + sqrtf(cos2t)));
                        float a = nt - nc, b = nt + nc, R0 = a * a / (b * b);
                        float c = 1.0f - (into ? -ddn : dot(refr, normal));
                        float c2 = c * c;
                        float Re = R0 + (1.0f - R0) * (c2 * c2 * c), Tr = 1.0f - Re;
                        float Pp = 0.25f + 0.5f * Re;
                        if (rng.f32() < Pp) { out = refl; wgt = col * (Re / (Pp * 0.5f)); }
                        else { out = refr; wgt = col * (Tr / ((1.0f - Pp) * 0.5f)); }
                    }
                } else if (m.type == SALTY_PHONG) {
                    // Phong::Shade (src/s3d_phong.cpp:65-88)
                    float uu = rng.f32(), vv = rng.f32();
                    V sd = sample_phong(uu, vv, m.power);
                    V w = safe_unit(reflect(d, nm)), t, b;
                    tangent_space(w, t, b);
                    out = safe_unit(t * sd.x + b * sd.y + w * sd.z);
                    dice = rng.f32() >= m.rr_threshold;
                    wgt = col * fabsf(dot(out, nm));
                } else if (m.type == SALTY_PLASTIC) {
                    // Plastic::Shade (src/s3d_plastic.cpp:71-142): R0 = 0.5, diffuse branch
                    // with P = (R + 0.5) / 2 weighted R / P, Phong branch (1 - R) / (1 - P)
                    float t1 = 1.0f - fabsf(dot(normal, d));
                    float R = 0.5f + 0.5f * t1 * t1 * t1 * t1 * t1;
                    float Pd = (R + 0.5f) * 0.5f;
                    if (rng.f32() <= Pd) {
                        V t, b;
                        tangent_space(nm, t, b);
                        float uu = rng.f32(), vv = rng.f32();
                        float rr = sqrtf(1.0f - uu * uu), ph = k2Pi * vv;
                        float sp, cp;
                        sincosf(ph, &sp, &cp);
                        out = safe_unit(t * (rr * cp) + b * (rr * sp) + nm * uu);
                        dice = rng.f32() >= m.rr_threshold;
                        wgt = col * (R / Pd);
                    } else {
                        float uu = rng.f32(), vv = rng.f32();
                        V sd = sample_phong(uu, vv, m.power);
                        V w = safe_unit(reflect(d, nm)), t, b;
                        tangent_space(w, t, b);
                        out = safe_unit(t * sd.x + b * sd.y + w * sd.z);
                        dice = rng.f32() >= m.rr_threshold;  // derived from the diffuse threshold
                        wgt = ld3(m.specular) * (dot(out, nm) * (1.0f - R) / (1.0f - Pd));
                    }
                } else {
                    V t, b;
                    tangent_space(nm, t, b);
                    float uu = rng.f32(), vv = rng.f32();
                    float rr = sqrtf(1.0f - uu * uu), ph = k2Pi * vv;
                    float sp, cp;
                    sincosf(ph, &sp, &cp);
                    out = safe_unit(t * (rr * cp) + b * (rr * sp) + nm * uu);
                    dice = rng.f32() >= m.rr_threshold;
                    wgt = col;
                }
                W = W * (wgt * tx);
                bool stop = dice || (W.x < FLT_EPSILON && W.y < FLT_EPSILON && W.z < FLT_EPSILON) ||
                            depth + 1 >= S.max_depth;
                if (!stop) {
                    cont = true;
                    nr0 = make_float4(pos.x, pos.y, pos.z, kFHitMin);
                    nr1 = make_float4(out.x, out.y, out.z, kFHitMax);
                    nW = make_float4(W.x, W.y, W.z, 0.0f);
                }
            } else if (is_light(K, id)) {
                float cos_l = dot(ld3(K.ln), -d);
                if (cos_l > 0.0f) {
                    if (prev_delta) L = L + W * ld3(K.le);
                    else {
                        float pdf_l = h.x * h.x / (cos_l * K.larea * (float)K.n_lights);
                        float mis = prev_pdf / (prev_pdf + pdf_l);
                        L = L + W * ld3(K.le) * mis;
                    }
                }
            } else {
                const HitRef hr = hit_ref(P, K, id);
                GpuMaterial m = P.mats[hr.mat];
                Surf s = hit_surface(P, hr, h.x, h.z, h.w, o, d);
                const V tx = hit_color_map(P, m, hr, h.z, h.w, s.p);
                m.color[0] *= tx.x; m.color[1] *= tx.y; m.color[2] *= tx.z;
                if (hr.sph >= 0 && (P.sph_mat[hr.sph] & kSphLight) && !prev_delta) {
                    // a light sphere reached by BSDF sampling: MIS against the cone sampling
                    // of next-event estimation from the previous vertex (the ray's origin)
                    float cos_max;
                    const float pdf_l = sph_cone_pdf(P, hr.sph, o, cos_max) / (float)K.n_lights;
                    L = L + W * ld3(m.emission) * (prev_pdf / (prev_pdf + pdf_l));
                } else {
                    L = L + W * ld3(m.emission);
                }
                V col = ld3(m.color), wi, wgt;
                float pdf = 0.0f;
                bool is_delta = false, dead = false;
                if (m.type == SALTY_MIRROR) {
                    wi = reflect(d, s.nsf);
                    wgt = col;
                    is_delta = true;
                } else if (m.type == SALTY_GLASS) {
                    float eta = s.into ? 1.0f / m.ior : m.ior;
                    float cosi = -dot(d, s.nsf);
                    float sin2t = eta * eta * (1.0f - cosi * cosi);
                    float F = 1.0f, cost = 0.0f;
                    if (sin2t < 1.0f) {
                        cost = sqrtf(1.0f - sin2t);
                        float rs = (eta * cosi - cost) / (eta * cosi + cost);
                        float rp = (cosi - eta * cost) / (cosi + eta * cost);
                        F = 0.5f * (rs * rs + rp * rp);
                    }
                    float xi = rng.f32();
                    if (xi < F) wi = reflect(d, s.nsf);
                    else wi = safe_unit(d * eta + s.nsf * (eta * cosi - cost));
                    wgt = col;
                    is_delta = true;
                } else if (m.type == SALTY_GGX) {
                    float a = m.roughness * m.roughness, a2 = a * a;
                    float r1 = rng.f32(), r2 = rng.f32();
                    float ph = k2Pi * r1;
                    float ct = sqrtf((1.0f - r2) / fmaxf(r2 * (a2 - 1.0f) + 1.0f, 1e-8f));
                    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                    V t, b;
                    tangent_space(s.nsf, t, b);
                    float sp, cp;
                    sincosf(ph, &sp, &cp);
                    V hh = safe_unit(t * (st * cp) + b * (st * sp) + s.nsf * ct);
                    wi = reflect(d, hh);
                    V wo = -d;
                    float no = dot(s.nsf, wo), ni = dot(s.nsf, wi), nh = dot(s.nsf, hh), oh = dot(wo, hh);
                    if (ni <= 0.0f || no <= 0.0f || oh <= 0.0f || dot(s.ngf, wi) <= 0.0f) {
                        dead = true;
                    } else {
                        float G = ggx_g1(no, a2) * ggx_g1(ni, a2);
                        wgt = schlick(col, oh) * (G * oh / (no * nh));
                        pdf = ggx_d(nh, a2) * nh / (4.0f * oh);
                    }
                } else if (m.type == SALTY_PHONG || m.type == SALTY_PLASTIC) {
                    bool lobe = true;
                    V wo = -d;
                    if (m.type == SALTY_PLASTIC) lobe = rng.f32() < plastic_ps(plastic_fresnel(dot(s.nsf, wo)));
                    float r1 = rng.f32(), r2 = rng.f32();
                    V t, b;
                    if (lobe) {
                        V sd = sample_phong(r1, r2, m.power);
                        V rd = reflect(d, s.nsf);
                        tangent_space(rd, t, b);
                        wi = safe_unit(t * sd.x + b * sd.y + rd * sd.z);
                    } else {
                        float rr = sqrtf(r1), ph = k2Pi * r2;
                        float z = sqrtf(fmaxf(0.0f, 1.0f - r1));
                        tangent_space(s.nsf, t, b);
                        float sp, cp;
                        sincosf(ph, &sp, &cp);
                        wi = safe_unit(t * (rr * cp) + b * (rr * sp) + s.nsf * z);
                    }
                    const float ni = dot(s.nsf, wi);
                    if (ni <= 0.0f || dot(s.ngf, wi) <= 0.0f) {
                        dead = true;
                    } else {
                        V f = phys_eval(m, s.nsf, wo, wi, pdf);
                        if (!(pdf > 0.0f)) dead = true;
                        else wgt = f * (ni / pdf);
                    }
                } else {
                    float r1 = rng.f32(), r2 = rng.f32();
                    float rr = sqrtf(r1), ph = k2Pi * r2;
                    float z = sqrtf(fmaxf(0.0f, 1.0f - r1));
                    V t, b;
                    tangent_space(s.nsf, t, b);
                    float sp, cp;
                    sincosf(ph, &sp, &cp);
                    wi = safe_unit(t * (rr * cp) + b * (rr * sp) + s.nsf * z);
                    if (dot(s.ngf, wi) <= 0.0f) dead = true;
                    wgt = col;
                    pdf = dot(s.nsf, wi) / kPi;
                }
                if (!dead) {
                    W = W * wgt;
                    bool stop = (W.x <= 0.0f && W.y <= 0.0f && W.z <= 0.0f);
                    if (!stop && depth >= S.rr_depth) {
                        // survival min(1, max W): lossless chains of mirror or glass bounces
                        // (W still 1) are never cut, so their weights never grow
                        const float qv = fminf(1.0f, maxc(W));
                        if (qv < 1.0f) {
                            if (rng.f32() >= qv) stop = true;
                            else W = W * (1.0f / qv);
                        }
                    }
                    if (depth + 1 >= S.max_depth) stop = true;
                    if (!stop) {
                        cont = true;
                        const V so = spawn(s.p, s.ng, wi);
                        nr0 = make_float4(so.x, so.y, so.z, 0.0f);
                        nr1 = make_float4(wi.x, wi.y, wi.z, INFINITY);
                        nW = make_float4(W.x, W.y, W.z, pdf);
                        mt.w = pack_w(depth + 1, is_delta, slot);
                    }
                }
            }
            nL = make_float4(L.x, L.y, L.z, 0.0f);
            nmeta = make_uint4((unsigned)rng.s, (unsigned)(rng.s >> 32), mt.z,
                               compat ? pack_w(depth + 1, false, slot) : mt.w);
            if (!cont) {
                B.lbuf[mt.z] = nL;
                ended = (int)(mt.z / (unsigned)P.chunk);
            }
        }
        // the ended sample's chunk: one atomic per distinct chunk of the warp
        const unsigned peers = __match_any_sync(0xffffffffu, ended);
        if (ended >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&B.done[ended], __popc(peers));
        const int qi = warp_append(cont, &B.counts[q ^ 1]);
        if (cont) {
            B.rays[q ^ 1][2 * qi] = nr0;
            B.rays[q ^ 1][2 * qi + 1] = nr1;
            B.path[q ^ 1].W[qi] = nW;
            B.path[q ^ 1].L[qi] = nL;
            B.path[q ^ 1].meta[qi] = nmeta;
            if (B.roots[q ^ 1]) B.roots[q ^ 1][qi] = root;
        }
    }
}

// After the shading of queue q in both halves: counts their rays, empties those queues and
// the shadow queues, and finds the samples ready for the films -- the longest run of whole
// chunks, from the first sample not yet accumulated, whose paths have all ended.
__global__ void k_iter_end(WaveParams P, WaveBuffers A, WaveBuffers B, int q) {
    A.stats[0] += (unsigned long long)(A.counts[q] + A.counts[2] + B.counts[q] + B.counts[2]);
    A.counts[q] = 0;
    A.counts[2] = 0;
    B.counts[q] = 0;
    B.counts[2] = 0;
    const long long base = A.ctl[kAccBase];
    long long n = 0;
    for (int k = 0; k < P.ring_chunks; ++k) {
        const long long c0 = base + n;
        if (c0 >= P.total_samples) break;
        const long long size = min((long long)P.chunk, P.total_samples - c0);
        if (A.done[(c0 / P.chunk) % P.ring_chunks] != (int)size) break;
        n += size;
    }
    A.ctl[kAccN] = n;
}

// New samples for the halves' queues q: up to the free slots of half A, then of half B, as
// far as free per-sample entries allow (samples below kAccBase + ring).
__device__ void plan_generation(const WaveParams& P, WaveBuffers& A, WaveBuffers& B, int q) {
    long long* c = A.ctl;
    const int have_a = A.counts[q], have_b = B.counts[q];
    const long long limit = min(P.total_samples, c[kAccBase] + P.ring);
    const long long avail = max(0LL, limit - c[kNext]);
    const long long add_a = min((long long)(P.cap_a - have_a), avail);
    const long long add_b = min((long long)(P.cap_b - have_b), avail - add_a);
    A.gen[0] = c[kNext];
    A.gen[1] = add_a;
    A.gen[2] = have_a;
    B.gen[0] = c[kNext] + add_a;
    B.gen[1] = add_b;
    B.gen[2] = have_b;
    c[kNext] += add_a + add_b;
    A.counts[q] = have_a + (int)add_a;
    B.counts[q] = have_b + (int)add_b;
    A.stats[1] += (unsigned long long)(add_a + add_b);
}

// After the accumulation: frees the accumulated chunks, plans the next generation (queues
// q ^ 1) and decides whether the graph launch runs another iteration.
__global__ void k_iter_next(WaveParams P, WaveBuffers A, WaveBuffers B, int q, cudaGraphConditionalHandle more,
                            int last) {
    long long* c = A.ctl;
    const long long n = c[kAccN];
    for (long long g = c[kAccBase]; g < c[kAccBase] + n; g += P.chunk) A.done[(g / P.chunk) % P.ring_chunks] = 0;
    c[kAccBase] += n;
    c[kAccN] = 0;
    plan_generation(P, A, B, q ^ 1);
    c[kIters] += 1;
    if (c[kIters] > P.iter_limit) c[kStuck] = 1;
    if (last) {
        const bool go = c[kAccBase] < P.total_samples && c[kIters] < c[kLaunchEnd] && !c[kStuck];
        cudaGraphSetConditional(more, go ? 1u : 0u);
    }
}

// Start of a render: nothing accumulated, the first samples pending for queues 0.
__global__ void k_render_init(WaveParams P, WaveBuffers A, WaveBuffers B) {
    for (int k = 0; k < kCtlWords; ++k) A.ctl[k] = 0;
    for (int k = 0; k < P.ring_chunks; ++k) A.done[k] = 0;
    for (int k = 0; k < 3; ++k) {
        A.counts[k] = 0;
        B.counts[k] = 0;
    }
    A.stats[0] = 0;
    A.stats[1] = 0;
    plan_generation(P, A, B, 0);
}

// Start of a graph launch: run at most launch_iters iterations.
__global__ void k_launch_begin(WaveParams P, WaveBuffers B) { B.ctl[kLaunchEnd] = B.ctl[kIters] + P.launch_iters; }

// Adds the wave's samples to the films: one thread per film pixel of the slots the wave
// touches, that pixel's samples in index order.
__global__ void k_accumulate(WaveParams P, WaveBuffers B) {
    const long long g0 = B.ctl[kAccBase];
    const long long n = B.ctl[kAccN];
    if (n <= 0) return;
    const int s0 = P.n_slots == 1 ? 0 : find_slot(P.sample_off, 0, P.n_slots - 1, g0);
    const int s1 = P.n_slots == 1 ? 0 : find_slot(P.sample_off, s0, P.n_slots - 1, g0 + n - 1);
    const long long p_begin = P.pixel_off[s0], p_end = P.pixel_off[s1 + 1];
    for (long long gp = p_begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; gp < p_end;
         gp += (long long)gridDim.x * blockDim.x) {
        const int sid = s0 == s1 ? s0 : find_slot(P.pixel_off, s0, s1, gp);
        const SceneSlot& S = P.slots[sid];
        const long long npx = S.npx, p = gp - P.pixel_off[sid];
        // the wave in slot-local sample indices [a, b), within the slot's npx * spp
        const long long base = P.sample_off[sid];
        const long long a = g0 - base;
        long long b = g0 + n - base;
        if (b > npx * S.spp) b = npx * S.spp;
        // samples s of this pixel with a <= s * npx + p < b
        const long long lo = a - p, hi = b - 1 - p;
        if (hi < 0) continue;
        const long long s_lo = lo <= 0 ? 0 : (lo + npx - 1) / npx;
        const long long s_hi = hi / npx;
        if (s_lo > s_hi) continue;
        // per-sample entry of slot-local sample index j: (base + j) % ring
        if (S.sum64) {
            double a0 = S.sum64[3 * p], a1 = S.sum64[3 * p + 1], a2 = S.sum64[3 * p + 2];
            double b0 = S.sumsq64[3 * p], b1 = S.sumsq64[3 * p + 1], b2 = S.sumsq64[3 * p + 2];
            for (long long sm = s_lo; sm <= s_hi; ++sm) {
                float4 l = B.lbuf[(base + sm * npx + p) % P.ring];
                a0 += l.x; a1 += l.y; a2 += l.z;
                b0 += (double)l.x * l.x; b1 += (double)l.y * l.y; b2 += (double)l.z * l.z;
            }
            S.sum64[3 * p] = a0; S.sum64[3 * p + 1] = a1; S.sum64[3 * p + 2] = a2;
            S.sumsq64[3 * p] = b0; S.sumsq64[3 * p + 1] = b1; S.sumsq64[3 * p + 2] = b2;
        } else {
            float sm3[3], c[3], q2[3];
            for (int k = 0; k < 3; ++k) { sm3[k] = S.sum[3 * p + k]; c[k] = S.comp[3 * p + k]; q2[k] = S.sumsq[3 * p + k]; }
            for (long long sm = s_lo; sm <= s_hi; ++sm) {
                float4 l = B.lbuf[(base + sm * npx + p) % P.ring];
                float v[3] = {l.x, l.y, l.z};
                for (int k = 0; k < 3; ++k) {
                    // Kahan-compensated sum
                    float y = __fsub_rn(v[k], c[k]);
                    float t = __fadd_rn(sm3[k], y);
                    c[k] = __fsub_rn(__fsub_rn(t, sm3[k]), y);
                    sm3[k] = t;
                    q2[k] = __fadd_rn(q2[k], __fmul_rn(v[k], v[k]));
                }
            }
            for (int k = 0; k < 3; ++k) { S.sum[3 * p + k] = sm3[k]; S.comp[3 * p + k] = c[k]; S.sumsq[3 * p + k] = q2[k]; }
        }
        // first-hit features: albedo (3), normal (3), 1/(1+t) (1)
        float f[7];
        for (int k = 0; k < 7; ++k) f[k] = S.aov[7 * p + k];
        for (long long sm = s_lo; sm <= s_hi; ++sm) {
            const long long wi = (base + sm * npx + p) % P.ring;
            const float4 f0 = B.abuf[2 * wi], f1 = B.abuf[2 * wi + 1];
            f[0] += f0.x; f[1] += f0.y; f[2] += f0.z; f[6] += f0.w;
            f[3] += f1.x; f[4] += f1.y; f[5] += f1.z;
        }
        for (int k = 0; k < 7; ++k) S.aov[7 * p + k] = f[k];
    }
}


// Mean first-hit features of the film: albedo W*H*3, normal W*H*3, 1/(1+t) W*H.
__global__ void k_aov_out(const float* __restrict__ aov, long long npx, double count, float* albedo, float* normal,
                          float* depth) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        const float inv = count > 0 ? (float)(1.0 / count) : 0.0f;
        for (int k = 0; k < 3; ++k) {
            if (albedo) albedo[3 * p + k] = aov[7 * p + k] * inv;
            if (normal) normal[3 * p + k] = aov[7 * p + 3 + k] * inv;
        }
        if (depth) depth[p] = aov[7 * p + 6] * inv;
    }
}

__global__ void k_film_out(const float* sum, const float* sumsq, const double* sum64, const double* sumsq64,
                           long long n, double count, float* mean, float* var) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double s = sum64 ? sum64[i] : (double)sum[i];
        double q = sum64 ? sumsq64[i] : (double)sumsq[i];
        double m = count > 0 ? s / count : 0.0;
        if (mean) mean[i] = (float)m;
        if (var) {
            double v = count > 1 ? (q / count - m * m) * count / (count - 1.0) / count : 0.0;
            var[i] = (float)(v > 0 ? v : 0.0);
        }
    }
}

// Batch arena: copies of a scene's BVH and triangles with their indices moved by the
// scene's offsets in the arena.
__global__ void k_arena_nodes(const Bvh8Node* __restrict__ src, long long n, unsigned node_off, unsigned leaf_off,
                              Bvh8Node* __restrict__ dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        Bvh8Node v = src[i];
        v.w[1].x += node_off;  // child_base
        v.w[1].y += leaf_off;  // tri_base
        dst[i] = v;
    }
}

__global__ void k_arena_tris(const float4* __restrict__ src, long long n, int id_off, float4* __restrict__ dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 a = src[3 * i];
        a.w = __int_as_float(__float_as_int(a.w) + id_off);  // input id
        dst[3 * i] = a;
        dst[3 * i + 1] = src[3 * i + 1];
        dst[3 * i + 2] = src[3 * i + 2];
    }
}

__global__ void k_arena_mats(const GpuMaterial* __restrict__ src, int n, int tex_off, GpuMaterial* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        GpuMaterial m = src[i];
        if (m.color_map >= 0) m.color_map += tex_off;
        dst[i] = m;
    }
}

__global__ void k_arena_textures(const GpuTexture* __restrict__ src, int n, long long texel_off,
                                 GpuTexture* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        GpuTexture t = src[i];
        t.offset += texel_off;
        dst[i] = t;
    }
}

__global__ void k_arena_mat(const int* __restrict__ src, long long n, int mat_off, int* __restrict__ dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i] + mat_off;
}

int grid_of(long long n, int per_sm_blocks, int num_sms, int block = 256) {
    long long g = (n + block - 1) / block, cap = (long long)num_sms * per_sm_blocks;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

namespace {

// Resets the film when the call does not continue it (PathTracer::TracePath clears RT at
// the start of a run, src/s3d_pt.cpp:297-353).
salty_status prepare_film(salty_ctx* ctx, salty_scene* sc, const salty_render_opts& o) {
    auto& E = ctx->err;
    cudaStream_t st = ctx->stream;
    Film& F = sc->film;
    const bool cropped = o.crop_w > 0 && o.crop_h > 0;
    const int fw = cropped ? o.crop_w : o.width, fh = cropped ? o.crop_h : o.height;
    const int cx = cropped ? o.crop_x : 0, cy = cropped ? o.crop_y : 0;
    const long long npx = (long long)fw * fh;
    const bool fresh = !o.accumulate || F.width != fw || F.height != fh || F.fp64 != o.fp64 || F.frame_w != o.width ||
                       F.frame_h != o.height || F.crop_x != cx || F.crop_y != cy;
    if (!fresh) return SALTY_OK;
    F.width = fw;
    F.height = fh;
    F.frame_w = o.width;
    F.frame_h = o.height;
    F.crop_x = cx;
    F.crop_y = cy;
    F.fp64 = o.fp64;
    F.samples = 0;
    SALTY_TRY_CUDA(E, F.aov.ensure(npx * 7));
    SALTY_TRY_CUDA(E, cudaMemsetAsync(F.aov.p, 0, npx * 7 * sizeof(float), st));
    if (o.fp64) {
        SALTY_TRY_CUDA(E, F.sum64.ensure(npx * 3));
        SALTY_TRY_CUDA(E, F.sumsq64.ensure(npx * 3));
        SALTY_TRY_CUDA(E, cudaMemsetAsync(F.sum64.p, 0, npx * 3 * sizeof(double), st));
        SALTY_TRY_CUDA(E, cudaMemsetAsync(F.sumsq64.p, 0, npx * 3 * sizeof(double), st));
    } else {
        SALTY_TRY_CUDA(E, F.sum.ensure(npx * 3));
        SALTY_TRY_CUDA(E, F.comp.ensure(npx * 3));
        SALTY_TRY_CUDA(E, F.sumsq.ensure(npx * 3));
        SALTY_TRY_CUDA(E, cudaMemsetAsync(F.sum.p, 0, npx * 3 * sizeof(float), st));
        SALTY_TRY_CUDA(E, cudaMemsetAsync(F.comp.p, 0, npx * 3 * sizeof(float), st));
        SALTY_TRY_CUDA(E, cudaMemsetAsync(F.sumsq.p, 0, npx * 3 * sizeof(float), st));
    }
    return SALTY_OK;
}

// PinholeCamera::Update (include/s3d_camera.h:63-90), host floats, aspect of the frame
Camera camera_of(const SceneConsts& k, int width, int height) {
    Camera c;
    float aspect = (float)width / (float)height;
    float dir[3] = {k.cam_target[0] - k.cam_pos[0], k.cam_target[1] - k.cam_pos[1], k.cam_target[2] - k.cam_pos[2]};
    auto unitv = [](float* v) {
        float m = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] /= m; v[1] /= m; v[2] /= m;
    };
    auto crossv = [](const float* a, const float* b, float* r) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    unitv(dir);
    float cx[3], cy[3];
    crossv(dir, k.cam_up, cx);
    unitv(cx);
    for (int a = 0; a < 3; ++a) cx[a] = cx[a] * k.cam_fov * aspect;
    crossv(dir, cx, cy);
    unitv(cy);
    for (int a = 0; a < 3; ++a) {
        cy[a] = cy[a] * k.cam_fov;
        c.pos[a] = k.cam_pos[a];
        c.cx[a] = cx[a];
        c.cy[a] = cy[a];
        c.cz[a] = k.cam_pos[a] + dir[a] * k.cam_near;
        c.dir[a] = dir[a];
    }
    float u[3] = {cx[0], cx[1], cx[2]}, v[3] = {cy[0], cy[1], cy[2]};
    unitv(u);
    unitv(v);
    float foc[3] = {k.cam_target[0] - k.cam_pos[0], k.cam_target[1] - k.cam_pos[1], k.cam_target[2] - k.cam_pos[2]};
    for (int a = 0; a < 3; ++a) { c.u[a] = u[a]; c.v[a] = v[a]; }
    c.lens = k.cam_lens;
    c.focal = k.cam_focal > 0.0f ? k.cam_focal : std::sqrt(foc[0] * foc[0] + foc[1] * foc[1] + foc[2] * foc[2]);
    return c;
}

// Builds (or reuses) the arena of a batch; offsets per slot in ctx->arena.
salty_status ensure_arena(salty_ctx* ctx, salty_scene* const* scenes, int n) {
    auto& E = ctx->err;
    BatchArena& A = ctx->arena;
    std::vector<std::pair<const void*, uint64_t>> key(n);
    for (int i = 0; i < n; ++i) key[i] = {scenes[i], scenes[i]->bvh.generation};
    if (key == A.key && A.nodes.p) return SALTY_OK;
    A.key.clear();
    long long nn = 0, nl = 0, nt = 0, nm = 0, ntex = 0, ntx = 0;
    A.node_off.assign(n, 0);
    A.id_off.assign(n, 0);
    A.tex_off.assign(n, 0);
    std::vector<long long> leaf_off(n), mat_off(n), texel_off(n);
    int depth = 0;
    for (int i = 0; i < n; ++i) {
        const salty_scene* sc = scenes[i];
        A.node_off[i] = nn;
        leaf_off[i] = nl;
        A.id_off[i] = nt;
        mat_off[i] = nm;
        A.tex_off[i] = ntex;
        texel_off[i] = ntx;
        nn += sc->bvh.n_nodes;
        nl += sc->bvh.n_tris;
        nt += sc->n_tris;
        nm += sc->n_mats;
        ntex += sc->n_textures;
        ntx += sc->n_texels;
        depth = std::max(depth, (int)sc->bvh.depth);
    }
    if (nn >= (1ll << 31) || nl >= (1ll << 31) || nt >= (1ll << 31))
        return E.fail(SALTY_ERR_CAPACITY, "a batch holds at most 2^31 - 1 nodes and triangles");
    SALTY_TRY_CUDA(E, A.nodes.ensure(nn));
    SALTY_TRY_CUDA(E, A.tris.ensure(nl * kTriFloat4));
    SALTY_TRY_CUDA(E, A.pos.ensure(nt * 9));
    SALTY_TRY_CUDA(E, A.nrm.ensure(nt * 9));
    SALTY_TRY_CUDA(E, A.uv.ensure(nt * 6));
    SALTY_TRY_CUDA(E, A.textures.ensure(std::max(ntex, 1ll)));
    SALTY_TRY_CUDA(E, A.texels.ensure(std::max(ntx, 1ll)));
    SALTY_TRY_CUDA(E, A.mat.ensure(nt));
    SALTY_TRY_CUDA(E, A.mats.ensure(nm));
    cudaStream_t st = ctx->stream;
    for (int i = 0; i < n; ++i) {
        const salty_scene* sc = scenes[i];
        const int g = ctx->num_sms * 4;
        k_arena_nodes<<<g, 256, 0, st>>>(sc->bvh.nodes.p, sc->bvh.n_nodes, (unsigned)A.node_off[i],
                                         (unsigned)leaf_off[i], A.nodes.p + A.node_off[i]);
        k_arena_tris<<<g, 256, 0, st>>>(sc->bvh.tris.p, sc->bvh.n_tris, (int)A.id_off[i],
                                        A.tris.p + leaf_off[i] * kTriFloat4);
        k_arena_mat<<<g, 256, 0, st>>>(sc->mat.p, sc->n_tris, (int)mat_off[i], A.mat.p + A.id_off[i]);
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(A.pos.p + A.id_off[i] * 9, sc->pos.p, sc->n_tris * 9 * sizeof(float),
                                          cudaMemcpyDeviceToDevice, st));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(A.nrm.p + A.id_off[i] * 9, sc->nrm.p, sc->n_tris * 9 * sizeof(float),
                                          cudaMemcpyDeviceToDevice, st));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(A.uv.p + A.id_off[i] * 6, sc->uv.p, sc->n_tris * 6 * sizeof(float),
                                          cudaMemcpyDeviceToDevice, st));
        k_arena_mats<<<1, 256, 0, st>>>(sc->mats.p, sc->n_mats, (int)A.tex_off[i], A.mats.p + mat_off[i]);
        if (sc->n_textures > 0) {
            k_arena_textures<<<1, 256, 0, st>>>(sc->textures.p, sc->n_textures, texel_off[i],
                                                A.textures.p + A.tex_off[i]);
            SALTY_TRY_CUDA(E, cudaMemcpyAsync(A.texels.p + texel_off[i], sc->texels.p, sc->n_texels * sizeof(float4),
                                              cudaMemcpyDeviceToDevice, st));
        }
    }
    SALTY_TRY_CUDA(E, cudaGetLastError());
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
    A.depth = depth;
    A.key = key;
    return SALTY_OK;
}

}  // namespace

salty_status render_batch(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts, int n,
                          salty_render_stats* total) {
    auto& E = ctx->err;
    cudaStream_t st = ctx->stream;
    if (n < 1 || n > kMaxSlots) return E.fail(SALTY_ERR_INVALID_ARG, "a batch holds 1..%d scenes", kMaxSlots);
    for (int i = 0; i < n; ++i) SALTY_TRY(prepare_film(ctx, scenes[i], opts[i]));
    // what the traversal walks: the scene itself, or the batch arena
    TraceTarget tgt;
    const float *pos, *nrm, *uv;
    const int* mat;
    const GpuMaterial* mats;
    const GpuTexture* textures;
    const float4* texels;
    if (n > 1)
        for (int i = 0; i < n; ++i)
            if (scenes[i]->n_inst > 0 || scenes[i]->n_sph > 0)
                return E.fail(SALTY_ERR_INVALID_ARG,
                              "scene %d of the batch holds instances or spheres: render it with salty_render", i);
    if (n == 1) {
        tgt.nodes = scenes[0]->bvh.nodes.p;
        tgt.tris = scenes[0]->bvh.tris.p;
        tgt.depth = scenes[0]->bvh.depth;
        tgt.inst = scenes[0]->n_inst > 0 ? scenes[0]->inst_rec.p : nullptr;
        tgt.sph_base = scenes[0]->n_sph > 0 ? (int)scenes[0]->n_tris : kNoSpheres;
        pos = scenes[0]->pos.p;
        nrm = scenes[0]->nrm.p;
        uv = scenes[0]->uv.p;
        mat = scenes[0]->mat.p;
        mats = scenes[0]->mats.p;
        textures = scenes[0]->textures.p;
        texels = scenes[0]->texels.p;
    } else {
        SALTY_TRY(ensure_arena(ctx, scenes, n));
        const BatchArena& A = ctx->arena;
        tgt.nodes = A.nodes.p;
        tgt.tris = A.tris.p;
        tgt.depth = A.depth;
        pos = A.pos.p;
        nrm = A.nrm.p;
        uv = A.uv.p;
        mat = A.mat.p;
        mats = A.mats.p;
        textures = A.textures.p;
        texels = A.texels.p;
    }
    // slot table
    std::vector<SceneSlot> slots(n);
    std::vector<long long> offs(2 * (n + 1));
    long long* sample_off = offs.data();
    long long* pixel_off = offs.data() + n + 1;
    long long samples = 0, pixels = 0;
    int max_depth = 0;
    for (int i = 0; i < n; ++i) {
        const salty_render_opts& o = opts[i];
        salty_scene* sc = scenes[i];
        Film& F = sc->film;
        SceneSlot& S = slots[i];
        std::memset(&S, 0, sizeof S);
        S.k = sc->consts;
        if (n > 1 && S.k.light_tri0 >= 0) S.k.light_tri0 += (int)ctx->arena.id_off[i];
        if (n > 1 && S.k.ibl_map >= 0) S.k.ibl_map += (int)ctx->arena.tex_off[i];
        S.cam = camera_of(sc->consts, o.width, o.height);
        S.width = o.width;
        S.height = o.height;
        S.crop_x = F.crop_x;
        S.crop_y = F.crop_y;
        S.film_w = F.width;
        S.film_h = F.height;
        S.spp = o.spp;
        S.max_depth = o.max_depth;
        S.rr_depth = o.rr_depth;
        S.profile = o.profile;
        S.root = n > 1 ? (int)ctx->arena.node_off[i] : 0;
        S.npx = (long long)F.width * F.height;
        S.seed = o.seed + 0x9e3779b97f4a7c15ull * (unsigned long long)F.samples;  // new streams per progressive call
        if (o.fp64) {
            S.sum64 = F.sum64.p;
            S.sumsq64 = F.sumsq64.p;
        } else {
            S.sum = F.sum.p;
            S.comp = F.comp.p;
            S.sumsq = F.sumsq.p;
        }
        S.aov = F.aov.p;
        sample_off[i] = samples;
        pixel_off[i] = pixels;
        samples += S.npx * o.spp;
        pixels += S.npx;
        if (o.spp > 0) max_depth = std::max(max_depth, o.max_depth);
        if (o.profile != opts[0].profile)
            return E.fail(SALTY_ERR_INVALID_ARG, "the scenes of a batch share one profile");
    }
    sample_off[n] = samples;
    pixel_off[n] = pixels;
    if (samples == 0) {
        if (total) *total = salty_render_stats{};
        return SALTY_OK;
    }
    const size_t slot_bytes = (size_t)n * sizeof(SceneSlot), off_bytes = offs.size() * sizeof(long long);
    const size_t slot_region = (slot_bytes + 255) / 256 * 256;
    SALTY_TRY_CUDA(E, ctx->slots.ensure(slot_region + off_bytes));
    unsigned char* dslots = ctx->slots.p;
    long long* doffs = reinterpret_cast<long long*>(dslots + slot_region);
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(dslots, slots.data(), slot_bytes, cudaMemcpyHostToDevice, st));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(doffs, offs.data(), off_bytes, cudaMemcpyHostToDevice, st));

    // queues: `cap` paths in flight; per-sample buffers (radiance, first-hit features) for
    // `ring` samples, in chunks of `chunk` that enter the films in sample order
    const Tuning& T = ctx->tune;
    const long long cap = std::min<long long>(samples, T.wave_paths);
    const long long chunk = std::max<long long>(1, cap / 2);
    const long long chunks_total = (samples + chunk - 1) / chunk;
    // enough chunks for the samples started during a path's lifetime (max_depth iterations,
    // about half a queue each), at most kMaxRingChunks and 2^27 samples (6.4 GB)
    const int ring_chunks = (int)std::max<long long>(
        1, std::min<long long>({chunks_total, kMaxRingChunks, (long long)max_depth + 2,
                                std::max<long long>(2, (1ll << 27) / chunk)}));
    const long long ring = chunk * ring_chunks;
    WaveStore& S = ctx->waves;
    const bool batch = n > 1;
    for (int i = 0; i < 2; ++i) {
        SALTY_TRY_CUDA(E, S.rays[i].ensure(cap * 2));
        SALTY_TRY_CUDA(E, S.W[i].ensure(cap));
        SALTY_TRY_CUDA(E, S.L[i].ensure(cap));
        SALTY_TRY_CUDA(E, S.meta[i].ensure(cap));
        if (batch) SALTY_TRY_CUDA(E, S.roots[i].ensure(cap));
    }
    if (batch) SALTY_TRY_CUDA(E, S.sroots.ensure(cap * 2));
    SALTY_TRY_CUDA(E, S.hits.ensure(cap));
    SALTY_TRY_CUDA(E, S.nee.ensure(cap * 2));
    SALTY_TRY_CUDA(E, S.srays.ensure(cap * 4));
    SALTY_TRY_CUDA(E, S.shits.ensure(cap * 2));
    SALTY_TRY_CUDA(E, S.lbuf.ensure(ring));
    SALTY_TRY_CUDA(E, S.abuf.ensure(ring * 2));
    SALTY_TRY_CUDA(E, S.counts.ensure(16));
    SALTY_TRY_CUDA(E, S.ctl.ensure(kCtlWords));
    SALTY_TRY_CUDA(E, S.done.ensure(kMaxRingChunks));
    SALTY_TRY_CUDA(E, S.stats.ensure(4));
    for (auto* tc : {&S.tc0, &S.tc1, &S.tc2, &S.tc3}) SALTY_TRY_CUDA(E, tc->ensure(4));
    SALTY_TRY_CUDA(E, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));

    WaveParams P;
    P.pos = pos;
    P.nrm = nrm;
    P.uv = uv;
    P.mat = mat;
    P.mats = mats;
    P.textures = textures;
    P.texels = texels;
    P.slots = reinterpret_cast<const SceneSlot*>(dslots);
    P.sample_off = doffs;
    P.pixel_off = doffs + n + 1;
    P.n_inst = (n == 1) ? scenes[0]->n_inst : 0;
    P.irec = P.n_inst ? scenes[0]->inst_rec.p : nullptr;
    P.ishade = P.n_inst ? scenes[0]->inst_shade.p : nullptr;
    P.ivbase = P.n_inst ? scenes[0]->inst_vbase.p : nullptr;
    const bool sph = n == 1 && scenes[0]->n_sph > 0;
    P.sph = sph ? scenes[0]->sph.p : nullptr;
    P.sph_mat = sph ? scenes[0]->sph_mat.p : nullptr;
    P.sph_lights = sph ? scenes[0]->sph_lights.p : nullptr;
    P.n_slots = n;
    P.capacity = (int)cap;
    // two halves of the queue run concurrently (a render of fewer paths uses half A alone)
    P.cap_a = (int)(cap >= kMinSplit ? cap / 2 : cap);
    P.cap_b = (int)cap - P.cap_a;
    P.chunk = (int)chunk;
    P.ring = ring;
    P.ring_chunks = ring_chunks;
    P.launch_iters = kLaunchIters;
    // every path ends within max_depth iterations of its start, and an iteration that finds
    // the queue empty starts at least one chunk's samples: a bound with a margin of 2
    P.iter_limit = 2 * (chunks_total + 2) * (long long)(max_depth + 2);
    P.total_samples = samples;

    // the halves' views of the queues: half B starts cap_a paths in (2 rays and 2 shadow
    // rays per path), with its own queue lengths and generation plan
    auto half = [&](long long off, int counts_off, int gen_word) {
        WaveBuffers h;
        for (int i = 0; i < 2; ++i) {
            h.rays[i] = S.rays[i].p + 2 * off;
            h.path[i] = PathSoA{S.W[i].p + off, S.L[i].p + off, S.meta[i].p + off};
            h.roots[i] = batch ? S.roots[i].p + off : nullptr;
        }
        h.sroots = batch ? S.sroots.p + 2 * off : nullptr;
        h.hits = S.hits.p + off;
        h.nee = S.nee.p + 2 * off;
        h.srays = S.srays.p + 4 * off;
        h.shits = S.shits.p + 2 * off;
        h.lbuf = S.lbuf.p;
        h.abuf = S.abuf.p;
        h.counts = S.counts.p + counts_off;
        h.ctl = S.ctl.p;
        h.gen = S.ctl.p + gen_word;
        h.done = S.done.p;
        h.stats = S.stats.p;
        return h;
    };
    WaveBuffers BA = half(0, 0, kGenA), BB = half(P.cap_a, 8, kGenB);

    const bool compat = opts[0].profile == SALTY_PROFILE_COMPAT;
    const uint32_t ext_flags = compat ? 0u : (uint32_t)SALTY_TRACE_WATERTIGHT;
    const uint32_t sh_flags = compat ? 0u : (uint32_t)(SALTY_TRACE_WATERTIGHT | SALTY_TRACE_ANY_HIT);
    const int sb = T.shade_block;
    const int agrid = grid_of(std::min<long long>(pixels, ring), 2048 / 256, ctx->num_sms);

    // The render is one CUDA graph: a conditional while-node whose body runs two
    // iterations (queue 0, then queue 1) of
    //   for each half, on its own stream: generate new samples into the free queue slots ->
    //   extension rays -> NEE -> shadow rays -> BSDF sampling and compaction into the
    //   other queue;
    //   joined: accumulate the chunks whose samples have all ended -> plan the next
    //   generation,
    // and repeats while samples remain (at most kLaunchIters iterations per launch, so a
    // cancellation is seen between launches).  Every path lives in the queue until it
    // ends, so each launch of the traversal sees a full queue instead of the shrinking
    // depth levels of a fixed wave, and while one half's traversal finishes its longest
    // walks the other half's launches take the idle SMs.
    // SALTY_RENDER_HOST_LOOP=1 launches the same iterations from a host loop instead (16 per
    // step): the kernels inside a conditional graph body are invisible to some profilers.
    const char* hl = std::getenv("SALTY_RENDER_HOST_LOOP");
    const bool host_loop = hl && std::atoi(hl) != 0;
    cudaGraphConditionalHandle more = 0;
    // one half's shading and traversal for queue q, on stream hs
    auto run_half = [&](const WaveBuffers& H, long long hcap, unsigned long long* tc_ext, unsigned long long* tc_sh,
                        cudaStream_t hs, int q) -> salty_status {
        const int hgrid = grid_of(hcap, 2048 / sb, ctx->num_sms, sb);
        TraceTarget ext = tgt, shd = tgt;
        ext.roots = H.roots[q];
        shd.roots = H.sroots;
        k_generate<<<hgrid, sb, 0, hs>>>(P, H, q);
        SALTY_TRY(trace_launch(ctx, ext, T.trace, H.rays[q], hcap, &H.counts[q], ext_flags, H.hits, tc_ext, hs,
                               ctx->status.p));
        k_shade1<<<hgrid, sb, 0, hs>>>(P, H, q);
        SALTY_TRY(trace_launch(ctx, shd, T.trace, H.srays, 2 * hcap, &H.counts[2], sh_flags, H.shits, tc_sh, hs,
                               ctx->status.p));
        k_shade2<<<hgrid, sb, 0, hs>>>(P, H, q);
        return SALTY_OK;
    };
    const bool split = P.cap_b > 0;
    auto iteration_pair = [&](bool in_graph) -> salty_status {
        for (int q = 0; q < 2; ++q) {
            // half B on the auxiliary stream, forked from and joined back into st (in the
            // host loop both halves run on st, one after the other)
            const cudaStream_t sb_stream = in_graph && split ? ctx->aux_stream : st;
            if (in_graph && split) {
                SALTY_TRY_CUDA(E, cudaEventRecord(ctx->fork_ev, st));
                SALTY_TRY_CUDA(E, cudaStreamWaitEvent(sb_stream, ctx->fork_ev, 0));
            }
            SALTY_TRY(run_half(BA, P.cap_a, S.tc0.p, S.tc1.p, st, q));
            if (split) SALTY_TRY(run_half(BB, P.cap_b, S.tc2.p, S.tc3.p, sb_stream, q));
            if (in_graph && split) {
                SALTY_TRY_CUDA(E, cudaEventRecord(ctx->join_ev, sb_stream));
                SALTY_TRY_CUDA(E, cudaStreamWaitEvent(st, ctx->join_ev, 0));
            }
            k_iter_end<<<1, 1, 0, st>>>(P, BA, BB, q);
            k_accumulate<<<agrid, 256, 0, st>>>(P, BA);
            k_iter_next<<<1, 1, 0, st>>>(P, BA, BB, q, more, in_graph && q == 1 ? 1 : 0);
        }
        return SALTY_OK;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    struct GraphGuard {
        cudaGraph_t& g;
        cudaGraphExec_t& x;
        ~GraphGuard() {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
        }
    } guard{graph, exec};
    if (!host_loop) {
        SALTY_TRY_CUDA(E, cudaGraphCreate(&graph, 0));
        SALTY_TRY_CUDA(E, cudaGraphConditionalHandleCreate(&more, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNode_t begin_node, loop_node;
        {
            cudaKernelNodeParams kp{};
            void* args[] = {&P, &BA};
            kp.func = reinterpret_cast<void*>(k_launch_begin);
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(1);
            kp.kernelParams = args;
            SALTY_TRY_CUDA(E, cudaGraphAddKernelNode(&begin_node, graph, nullptr, 0, &kp));
        }
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = more;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        SALTY_TRY_CUDA(E, cudaGraphAddNode(&loop_node, graph, &begin_node, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        SALTY_TRY_CUDA(E, cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                                        cudaStreamCaptureModeThreadLocal));
        const salty_status cap_status = iteration_pair(true);
        cudaGraph_t captured = body;
        cudaError_t ce = cudaStreamEndCapture(st, &captured);
        if (cap_status != SALTY_OK) return cap_status;
        SALTY_TRY_CUDA(E, ce);
        SALTY_TRY_CUDA(E, cudaGraphInstantiate(&exec, graph, 0));
    }

    cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1];
    SALTY_TRY_CUDA(E, cudaEventRecord(e0, st));
    k_render_init<<<1, 1, 0, st>>>(P, BA, BB);
    salty_status rs = SALTY_OK;
    long long hc[kCtlWords];
    const int pairs_per_step = 8;
    const long long max_launches = P.iter_limit / (host_loop ? 2 * pairs_per_step : kLaunchIters) + 2;
    for (long long launch = 0;; ++launch) {
        if (launch > max_launches) { rs = E.fail(SALTY_ERR_TIMEOUT, "render made no progress"); break; }
        if (host_loop) {
            k_launch_begin<<<1, 1, 0, st>>>(P, BA);
            for (int k = 0; k < pairs_per_step && rs == SALTY_OK; ++k) rs = iteration_pair(false);
            if (rs != SALTY_OK) break;
        } else {
            cudaError_t le = cudaGraphLaunch(exec, st);
            if (le != cudaSuccess) { rs = E.fail(SALTY_ERR_CUDA, "graph launch: %s", cudaGetErrorString(le)); break; }
        }
        cudaError_t re = cudaMemcpyAsync(hc, S.ctl.p, sizeof hc, cudaMemcpyDeviceToHost, st);
        if (re == cudaSuccess) re = cudaStreamSynchronize(st);
        if (re != cudaSuccess) { rs = E.fail(SALTY_ERR_CUDA, "render: %s", cudaGetErrorString(re)); break; }
        if (hc[kStuck]) { rs = E.fail(SALTY_ERR_TIMEOUT, "render made no progress in %lld iterations", hc[kIters]); break; }
        if (hc[kAccBase] >= samples) break;
        if (ctx->cancel) { rs = E.fail(SALTY_ERR_CANCELLED, "render cancelled"); break; }
    }
    SALTY_TRY_CUDA(E, cudaEventRecord(e1, st));
    SALTY_TRY_CUDA(E, cudaEventSynchronize(e1));
    SALTY_TRY_CUDA(E, cudaGetLastError());
    if (rs != SALTY_OK) return rs;
    int status = 0;
    SALTY_TRY_CUDA(E, cudaMemcpy(&status, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) return E.fail(SALTY_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
    unsigned long long hs[2];
    SALTY_TRY_CUDA(E, cudaMemcpy(hs, S.stats.p, sizeof hs, cudaMemcpyDeviceToHost));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    for (int i = 0; i < n; ++i) scenes[i]->film.samples += opts[i].spp;
    if (total) {
        total->ms = ms;
        total->samples = n == 1 ? scenes[0]->film.samples : samples;
        total->rays = (int64_t)hs[0];
        total->paths = (int64_t)hs[1];
    }
    return SALTY_OK;
}

salty_status render(salty_ctx* ctx, salty_scene* sc, const salty_render_opts& o, salty_render_stats* stats) {
    salty_scene* one[1] = {sc};
    SALTY_TRY(render_batch(ctx, one, &o, 1, stats));
    if (stats) stats->samples = sc->film.samples;
    return SALTY_OK;
}

salty_status film_outputs(salty_ctx* ctx, salty_scene* sc, const salty_render_opts& o, float* d_mean, float* d_var,
                          uint8_t* d_srgb) {
    auto& E = ctx->err;
    Film& F = sc->film;
    const long long n = (long long)F.width * F.height * 3;
    DevBuf<float> tmp;
    float* mean = d_mean;
    if (!mean && d_srgb) {
        SALTY_TRY_CUDA(E, tmp.ensure(n));
        mean = tmp.p;
    }
    k_film_out<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(F.fp64 ? nullptr : F.sum.p, F.fp64 ? nullptr : F.sumsq.p,
                                                         F.fp64 ? F.sum64.p : nullptr, F.fp64 ? F.sumsq64.p : nullptr,
                                                         n, (double)F.samples, mean, d_var);
    SALTY_TRY_CUDA(E, cudaGetLastError());
    if (d_srgb) {
        int tm = o.tonemap < 0 ? SALTY_TM_REINHARD : o.tonemap;
        SALTY_TRY(tonemap_device(ctx, tm, F.width, F.height, mean, nullptr, d_srgb, o.ref_oetf, nullptr, nullptr));
    }
    return SALTY_OK;
}

// Mean, variance of the mean and mean first-hit features of the film, all on the device
// (any output may be null).  The film must hold samples.
salty_status film_features(salty_ctx* ctx, salty_scene* sc, float* d_mean, float* d_var, float* d_albedo,
                           float* d_normal, float* d_depth) {
    Film& F = sc->film;
    const long long npx = (long long)F.width * F.height;
    if (npx == 0 || F.samples == 0 || !F.aov.p) return ctx->err.fail(SALTY_ERR_NOT_BUILT, "the film is empty");
    if (d_mean || d_var)
        k_film_out<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(
            F.fp64 ? nullptr : F.sum.p, F.fp64 ? nullptr : F.sumsq.p, F.fp64 ? F.sum64.p : nullptr,
            F.fp64 ? F.sumsq64.p : nullptr, npx * 3, (double)F.samples, d_mean, d_var);
    if (d_albedo || d_normal || d_depth)
        k_aov_out<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(F.aov.p, npx, (double)F.samples, d_albedo, d_normal,
                                                            d_depth);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

}  // namespace salty

// Checkpoint and resume of a progressive film: its raw state out and back in.
extern "C" salty_status salty_film_checkpoint(salty_ctx* ctx, salty_scene* sc, double* sum, double* sumsq, float* comp,
                                              float* aov, int64_t* samples) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    if (!sc) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "null scene");
    SALTY_TRY(salty_film_read(ctx, sc, sum, sumsq, samples));
    const Film& F = sc->film;
    const long long npx = (long long)F.width * F.height;
    if (npx == 0) return SALTY_OK;
    cudaSetDevice(ctx->device);
    if (comp) {
        if (F.fp64) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "an FP64 film has no compensation terms");
        SALTY_TRY_CUDA(ctx->err, cudaMemcpy(comp, F.comp.p, npx * 3 * sizeof(float), cudaMemcpyDefault));
    }
    if (aov) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(aov, F.aov.p, npx * 7 * sizeof(float), cudaMemcpyDefault));
    return SALTY_OK;
}

extern "C" salty_status salty_film_restore(salty_ctx* ctx, salty_scene* sc, const salty_render_opts* o,
                                           const double* sum, const double* sumsq, const float* comp, const float* aov,
                                           int64_t samples) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    SALTY_TRY(check_render_opts(ctx, sc, o));
    if (!sum || !sumsq || samples < 0) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad film state");
    if (comp && o->fp64) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "an FP64 film has no compensation terms");
    cudaSetDevice(ctx->device);
    salty_render_opts fresh = *o;
    fresh.accumulate = 0;
    SALTY_TRY(prepare_film(ctx, sc, fresh));  // sizes and zeroes the film as the options say
    Film& F = sc->film;
    const long long n = (long long)F.width * F.height * 3;
    auto put = [&](float* dst32, double* dst64, const double* src) -> salty_status {
        if (dst64) {
            SALTY_TRY_CUDA(ctx->err, cudaMemcpy(dst64, src, n * sizeof(double), cudaMemcpyDefault));
            return SALTY_OK;
        }
        std::vector<double> h(n);
        SALTY_TRY_CUDA(ctx->err, cudaMemcpy(h.data(), src, n * sizeof(double), cudaMemcpyDefault));
        std::vector<float> hf(h.begin(), h.end());
        SALTY_TRY_CUDA(ctx->err, cudaMemcpy(dst32, hf.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        return SALTY_OK;
    };
    SALTY_TRY(put(F.fp64 ? nullptr : F.sum.p, F.fp64 ? F.sum64.p : nullptr, sum));
    SALTY_TRY(put(F.fp64 ? nullptr : F.sumsq.p, F.fp64 ? F.sumsq64.p : nullptr, sumsq));
    if (comp) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(F.comp.p, comp, n * sizeof(float), cudaMemcpyDefault));
    if (aov) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(F.aov.p, aov, n / 3 * 7 * sizeof(float), cudaMemcpyDefault));
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(ctx->stream));
    F.samples = samples;
    return SALTY_OK;
}

extern "C" salty_status salty_film_read(salty_ctx* ctx, salty_scene* sc, double* sum, double* sumsq,
                                        int64_t* samples) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    if (!sc) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "null scene");
    Film& F = sc->film;
    if (samples) *samples = F.samples;
    const long long n = (long long)F.width * F.height * 3;
    if (n == 0) return SALTY_OK;
    cudaSetDevice(ctx->device);
    auto fetch = [&](double* dst, const double* s64, const float* s32) -> salty_status {
        if (!dst) return SALTY_OK;
        DevBuf<double> tmp;
        const double* src = s64;
        if (!s64) {
            SALTY_TRY_CUDA(ctx->err, tmp.ensure(n));
            // widen on the host side of the copy: copy floats then convert
            std::vector<float> h(n);
            SALTY_TRY_CUDA(ctx->err, cudaMemcpy(h.data(), s32, n * sizeof(float), cudaMemcpyDeviceToHost));
            std::vector<double> hd(h.begin(), h.end());
            SALTY_TRY_CUDA(ctx->err, cudaMemcpy(dst, hd.data(), n * sizeof(double), cudaMemcpyDefault));
            return SALTY_OK;
        }
        SALTY_TRY_CUDA(ctx->err, cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDefault));
        return SALTY_OK;
    };
    SALTY_TRY(fetch(sum, F.fp64 ? F.sum64.p : nullptr, F.sum.p));
    SALTY_TRY(fetch(sumsq, F.fp64 ? F.sumsq64.p : nullptr, F.sumsq.p));
    return SALTY_OK;
}

extern "C" salty_status salty_film_aov(salty_ctx* ctx, salty_scene* sc, float* albedo, float* normal, float* depth) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    if (!sc) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "null scene");
    Film& F = sc->film;
    const long long npx = (long long)F.width * F.height;
    if (npx == 0 || !F.aov.p) return ctx->err.fail(SALTY_ERR_NOT_BUILT, "the film is empty");
    cudaSetDevice(ctx->device);
    auto& E = ctx->err;
    float* outs[3] = {albedo, normal, depth};
    const long long sizes[3] = {npx * 3, npx * 3, npx};
    DevBuf<float> tmp[3];
    float* dev[3];
    for (int i = 0; i < 3; ++i) {
        dev[i] = outs[i];
        if (outs[i] && !is_device_ptr(outs[i])) {
            SALTY_TRY_CUDA(E, tmp[i].ensure(sizes[i]));
            dev[i] = tmp[i].p;
        }
    }
    k_aov_out<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(F.aov.p, npx, (double)F.samples, dev[0], dev[1], dev[2]);
    SALTY_TRY_CUDA(E, cudaGetLastError());
    for (int i = 0; i < 3; ++i)
        if (outs[i] && dev[i] != outs[i])
            SALTY_TRY_CUDA(E, cudaMemcpyAsync(outs[i], dev[i], sizes[i] * sizeof(float), cudaMemcpyDeviceToHost,
                                              ctx->stream));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}
