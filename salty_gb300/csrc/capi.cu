// capi.cu -- the extern "C" entry points of libsalty_gpu (include/salty_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "internal.h"

using namespace salty;

namespace {

// ---------------------------------------------------------------- host helpers
struct V3 {
    float x, y, z;
};
inline V3 v3(const float* p) { return {p[0], p[1], p[2]}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Vector3::UnitVector (include/s3d_math.h:830-842)
inline V3 unit(V3 v) {
    float m = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return {v.x / m, v.y / m, v.z / m};
}
inline void put(float* d, V3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

__global__ void k_geometric_normals(const float* __restrict__ pos, float* __restrict__ nrm, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pos + i * 9;
    float e1x = p[3] - p[0], e1y = p[4] - p[1], e1z = p[5] - p[2];
    float e2x = p[6] - p[0], e2y = p[7] - p[1], e2z = p[8] - p[2];
    float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    float m = sqrtf(nx * nx + ny * ny + nz * nz);
    if (m > 0.0f) { nx /= m; ny /= m; nz /= m; }
    for (int k = 0; k < 3; ++k) {
        nrm[i * 9 + k * 3] = nx;
        nrm[i * 9 + k * 3 + 1] = ny;
        nrm[i * 9 + k * 3 + 2] = nz;
    }
}

// bad[0]: triangles with a non-finite coordinate; bad[1]: material index out of range.
__global__ void k_validate(const float* __restrict__ pos, const int* __restrict__ mat, long long n, int n_mats,
                           int* bad) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool finite = true;
    for (int k = 0; k < 9; ++k) finite &= isfinite(pos[i * 9 + k]);
    if (!finite) atomicAdd(&bad[0], 1);
    if (mat[i] < 0 || mat[i] >= n_mats) atomicAdd(&bad[1], 1);
}

__global__ void k_rgb_to_texels(const float* __restrict__ rgb, long long n, float4* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
}

__global__ void k_fill_int(int* p, long long n, int v) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

salty_status copy_in(salty_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!bytes) return SALTY_OK;
    SALTY_TRY_CUDA(ctx->err, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
    return SALTY_OK;
}

// ---------------------------------------------------------------- PCG (generators)
// PCG-XSH-RR 64/32 as the reference's PCG class (include/s3d_math.h:2769-2817).
struct Pcg {
    uint64_t s;
    explicit Pcg(uint64_t seed) : s(seed + 1442695040888963407ull) { next(); }
    uint32_t next() {
        uint64_t old = s;
        s = old * 6364136223846793005ull + 1442695040888963407ull;
        uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
    }
    float f32() { return (float)next() / (float)0xffffffffu; }
};

}  // namespace

namespace salty {
salty_status check_render_opts(salty_ctx* ctx, const salty_scene* sc, const salty_render_opts* o) {
    auto& E = ctx->err;
    if (!sc || !o) return E.fail(SALTY_ERR_INVALID_ARG, "null scene or options");
    if (o->width <= 0 || o->height <= 0 || o->spp < 0 || o->max_depth < 1 || o->max_depth > 0xffff)
        return E.fail(SALTY_ERR_INVALID_ARG, "bad render size/spp/depth");
    if ((int64_t)o->width * o->height > (1ll << 28)) return E.fail(SALTY_ERR_CAPACITY, "image too large");
    const bool cropped = o->crop_w > 0 || o->crop_h > 0 || o->crop_x != 0 || o->crop_y != 0;
    if (cropped && (o->crop_w <= 0 || o->crop_h <= 0 || o->crop_x < 0 || o->crop_y < 0 ||
                    (int64_t)o->crop_x + o->crop_w > o->width || (int64_t)o->crop_y + o->crop_h > o->height))
        return E.fail(SALTY_ERR_INVALID_ARG, "crop window outside the frame");
    if (o->profile != SALTY_PROFILE_COMPAT && o->profile != SALTY_PROFILE_PHYSICAL)
        return E.fail(SALTY_ERR_INVALID_ARG, "bad profile");
    if (!sc->bvh.built) return E.fail(SALTY_ERR_NOT_BUILT, "salty_bvh_build has not been called");
    return SALTY_OK;
}
}  // namespace salty

extern "C" {

int salty_abi_version(void) { return SALTY_ABI_VERSION; }

salty_status salty_ctx_create(salty_ctx** out, int device) {
    if (!out) return SALTY_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return SALTY_ERR_CUDA;
    }
    if (device < 0 || device >= count) return SALTY_ERR_INVALID_ARG;
    auto* c = new (std::nothrow) salty_ctx();
    if (!c) return SALTY_ERR_OOM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaHostAlloc(&c->pinned, 1 << 16, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return SALTY_ERR_CUDA;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    if (c->counters.ensure(64) != cudaSuccess || c->status.ensure(16) != cudaSuccess) {
        salty_ctx_destroy(c);
        return SALTY_ERR_OOM;
    }
    *out = c;
    return SALTY_OK;
}

void salty_ctx_destroy(salty_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    delete ctx;
}

const char* salty_last_error(const salty_ctx* ctx) { return ctx ? ctx->err.msg.c_str() : "null context"; }

void salty_ctx_cancel(salty_ctx* ctx) {
    if (ctx) ctx->cancel = 1;
}

salty_status salty_host_alloc(salty_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    SALTY_TRY_CUDA(ctx->err, cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
    return SALTY_OK;
}

void salty_host_free(salty_ctx* ctx, void* p) {
    (void)ctx;
    if (p) cudaFreeHost(p);
}

// ---------------------------------------------------------------- scene
salty_status salty_scene_upload(salty_ctx* ctx, const salty_scene_desc* d, salty_scene** out) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!d || !out) return E.fail(SALTY_ERR_INVALID_ARG, "null scene description");
    *out = nullptr;
    if (d->n_tris < 0 || (d->n_tris > 0 && !d->tri_pos)) return E.fail(SALTY_ERR_INVALID_ARG, "bad triangle array");
    if (d->n_mats < 0 || (d->n_mats > 0 && !d->mats)) return E.fail(SALTY_ERR_INVALID_ARG, "bad material table");
    if (d->n_tris + (d->has_light ? 2 : 0) <= 0) return E.fail(SALTY_ERR_INVALID_ARG, "scene has no triangles");
    if (d->n_tris > (int64_t)0x3fffffff - 2) return E.fail(SALTY_ERR_CAPACITY, "too many triangles");
    cudaSetDevice(ctx->device);
    auto* sc = new (std::nothrow) salty_scene();
    if (!sc) return E.fail(SALTY_ERR_OOM, "host allocation failed");
    const int64_t n_in = d->n_tris;
    const int64_t n = n_in + (d->has_light ? 2 : 0);
    sc->n_input = n_in;
    sc->n_tris = n;
    auto fail = [&](salty_status s) { delete sc; return s; };
#define UP_TRY(expr)                          \
    do {                                      \
        salty_status s_ = (expr);             \
        if (s_ != SALTY_OK) return fail(s_);  \
    } while (0)
#define UP_CUDA(expr)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess) return fail(E.fail(SALTY_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_))); \
    } while (0)
    UP_CUDA(sc->pos.ensure((size_t)n * 9));
    UP_CUDA(sc->nrm.ensure((size_t)n * 9));
    UP_CUDA(sc->mat.ensure((size_t)n));
    UP_TRY(copy_in(ctx, sc->pos.p, d->tri_pos, (size_t)n_in * 9 * sizeof(float)));
    if (d->tri_nrm) UP_TRY(copy_in(ctx, sc->nrm.p, d->tri_nrm, (size_t)n_in * 9 * sizeof(float)));
    else if (n_in > 0)
        k_geometric_normals<<<(unsigned)((n_in + 255) / 256), 256, 0, ctx->stream>>>(sc->pos.p, sc->nrm.p, n_in);
    if (d->tri_mat) UP_TRY(copy_in(ctx, sc->mat.p, d->tri_mat, (size_t)n_in * sizeof(int)));
    else if (n_in > 0) k_fill_int<<<(unsigned)((n_in + 255) / 256), 256, 0, ctx->stream>>>(sc->mat.p, n_in, 0);

    std::vector<GpuMaterial> mats(d->n_mats + 1);
    for (int i = 0; i < d->n_mats; ++i) {
        const salty_material& m = d->mats[i];
        if (m.type < SALTY_LAMBERT || m.type > SALTY_PLASTIC)
            return fail(E.fail(SALTY_ERR_INVALID_ARG, "material %d: bad type", i));
        if ((m.type == SALTY_PHONG || m.type == SALTY_PLASTIC) && !(m.power > 0.0f && m.power < 1e6f))
            return fail(E.fail(SALTY_ERR_INVALID_ARG, "material %d: power must be in (0, 1e6)", i));
        GpuMaterial g{};
        g.type = m.type;
        for (int c = 0; c < 3; ++c) { g.color[c] = m.color[c]; g.emission[c] = m.emission[c]; }
        g.ior = m.ior > 0 ? m.ior : 1.5f;
        g.roughness = m.roughness;
        for (int c = 0; c < 3; ++c) g.specular[c] = m.specular[c];
        g.power = m.power;
        g.color_map = m.color_map - 1;
        if (g.color_map < -1 || g.color_map >= d->n_textures)
            return fail(E.fail(SALTY_ERR_INVALID_ARG, "material %d: color_map outside the texture table", i));
        // Lambert::Lambert (src/s3d_lambert.cpp:22-31), Phong::Phong (src/s3d_phong.cpp:22-31),
        // Plastic::Plastic (src/s3d_plastic.cpp:22-37): max(colour, 0.01)
        g.rr_threshold = std::max(std::max(std::max(m.color[0], m.color[1]), m.color[2]), 0.01f);
        mats[i] = g;
    }
    SceneConsts& k = sc->consts;
    std::memset(&k, 0, sizeof(k));
    k.light_tri0 = -1;
    k.sph_base = kNoSpheres;
    k.n_lights = d->has_light ? 1 : 0;
    if (d->has_light) {
        // the light: a black Lambert emitter (two-sided in the compat profile)
        GpuMaterial lm{};
        lm.type = SALTY_LAMBERT;
        lm.color_map = -1;
        for (int c = 0; c < 3; ++c) lm.emission[c] = d->light_emission[c];
        lm.rr_threshold = 0.01f;
        mats[d->n_mats] = lm;
        k.has_light = 1;
        V3 c = v3(d->light_corner), a = v3(d->light_edge_a), b = v3(d->light_edge_b);
        V3 cr = cross(a, b);
        k.larea = std::sqrt(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
        if (!(k.larea > 0)) return fail(E.fail(SALTY_ERR_INVALID_ARG, "degenerate light"));
        put(k.lc, c); put(k.la, a); put(k.lb, b); put(k.ln, unit(cr));
        for (int i = 0; i < 3; ++i) k.le[i] = d->light_emission[i];
        k.light_tri0 = (int)n_in;
        V3 p0 = c, p1 = add(c, a), p2 = add(add(c, a), b), p3 = add(c, b);
        float lt[18], ln[18];
        V3 q[6] = {p0, p1, p2, p0, p2, p3};
        V3 nn = unit(cr);
        for (int i = 0; i < 6; ++i) { put(lt + i * 3, q[i]); put(ln + i * 3, nn); }
        int lmi[2] = {d->n_mats, d->n_mats};
        UP_CUDA(cudaMemcpyAsync(sc->pos.p + n_in * 9, lt, sizeof lt, cudaMemcpyHostToDevice, ctx->stream));
        UP_CUDA(cudaMemcpyAsync(sc->nrm.p + n_in * 9, ln, sizeof ln, cudaMemcpyHostToDevice, ctx->stream));
        UP_CUDA(cudaMemcpyAsync(sc->mat.p + n_in, lmi, sizeof lmi, cudaMemcpyHostToDevice, ctx->stream));
        UP_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    sc->n_mats = d->n_mats + (d->has_light ? 1 : 0);
    if (sc->n_mats == 0) {  // no table: one grey Lambert
        GpuMaterial g{};
        g.type = SALTY_LAMBERT;
        g.color_map = -1;
        g.color[0] = g.color[1] = g.color[2] = 0.75f;
        g.rr_threshold = 0.75f;
        mats[0] = g;
        sc->n_mats = 1;
    }
    if (n_in > 0) {
        const int n_user_mats = std::max(d->n_mats, 1);
        int* bad = ctx->status.p + 4;
        UP_CUDA(cudaMemsetAsync(bad, 0, 2 * sizeof(int), ctx->stream));
        k_validate<<<(unsigned)((n_in + 255) / 256), 256, 0, ctx->stream>>>(sc->pos.p, sc->mat.p, n_in, n_user_mats, bad);
        int hb[2] = {0, 0};
        UP_CUDA(cudaMemcpyAsync(hb, bad, sizeof hb, cudaMemcpyDeviceToHost, ctx->stream));
        UP_CUDA(cudaStreamSynchronize(ctx->stream));
        if (hb[0]) return fail(E.fail(SALTY_ERR_INVALID_ARG, "%d triangles have non-finite vertices", hb[0]));
        if (hb[1]) return fail(E.fail(SALTY_ERR_INVALID_ARG, "%d triangles reference a material outside 0..%d", hb[1], n_user_mats - 1));
    }
    // texture coordinates and textures
    UP_CUDA(sc->uv.ensure((size_t)n * 6));
    UP_CUDA(cudaMemsetAsync(sc->uv.p, 0, (size_t)n * 6 * sizeof(float), ctx->stream));
    if (d->tri_uv && n_in > 0) UP_TRY(copy_in(ctx, sc->uv.p, d->tri_uv, (size_t)n_in * 6 * sizeof(float)));
    if (d->n_textures < 0 || (d->n_textures > 0 && !d->textures))
        return fail(E.fail(SALTY_ERR_INVALID_ARG, "bad texture table"));
    {
        std::vector<GpuTexture> tt(std::max(d->n_textures, 1));
        long long texels = 0;
        for (int t = 0; t < d->n_textures; ++t) {
            const salty_texture& x = d->textures[t];
            if (x.width <= 0 || x.height <= 0 || !x.rgb || (long long)x.width * x.height > (1ll << 28))
                return fail(E.fail(SALTY_ERR_INVALID_ARG, "texture %d: bad size or data", t));
            tt[t] = GpuTexture{texels, x.width, x.height};
            texels += (long long)x.width * x.height;
        }
        UP_CUDA(sc->textures.ensure(tt.size()));
        UP_CUDA(sc->texels.ensure((size_t)std::max(texels, 1ll)));
        DevBuf<float> stage;
        for (int t = 0; t < d->n_textures; ++t) {
            const salty_texture& x = d->textures[t];
            const long long np = (long long)x.width * x.height;
            UP_CUDA(stage.ensure((size_t)np * 3));
            UP_TRY(copy_in(ctx, stage.p, x.rgb, (size_t)np * 3 * sizeof(float)));
            k_rgb_to_texels<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(stage.p, np,
                                                                                    sc->texels.p + tt[t].offset);
            UP_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        UP_CUDA(cudaMemcpyAsync(sc->textures.p, tt.data(), sizeof(GpuTexture) * tt.size(), cudaMemcpyHostToDevice,
                                ctx->stream));
        UP_CUDA(cudaStreamSynchronize(ctx->stream));
        sc->n_textures = d->n_textures;
        sc->n_texels = texels;
    }
    if (d->ibl_map < 0 || d->ibl_map > d->n_textures)
        return fail(E.fail(SALTY_ERR_INVALID_ARG, "ibl_map outside the texture table"));
    k.ibl_map = d->ibl_map - 1;
    k.ibl_scale = d->ibl_scale > 0.0f ? d->ibl_scale : 10.0f;
    UP_CUDA(sc->mats.ensure(sc->n_mats));
    UP_CUDA(cudaMemcpyAsync(sc->mats.p, mats.data(), sizeof(GpuMaterial) * sc->n_mats, cudaMemcpyHostToDevice,
                            ctx->stream));
    k.has_sun = d->has_sun;
    for (int i = 0; i < 3; ++i) {
        k.sun_dir[i] = d->sun_dir[i];
        k.sun_rad[i] = d->sun_radiance[i];
        k.sky[i] = d->sky[i];
    }
    if (d->has_sun) {
        if (!(d->sun_half_angle >= 0.0f) || d->sun_half_angle > 0.5f)
            return fail(E.fail(SALTY_ERR_INVALID_ARG, "sun_half_angle must be in [0, 0.5] radians"));
        V3 sd = unit(v3(d->sun_dir));
        put(k.sun_dir, sd);
        k.sun_disk = d->sun_half_angle > 0.0f;
        k.sun_cos_max = std::cos((double)d->sun_half_angle);
        // solid angle of the cone (the pdf of a uniform direction in it), in double since
        // 1 - cos is tiny for small disks; the disk's radiance L makes the irradiance on a
        // surface facing the sun, L pi sin^2(half angle), equal to sun_radiance
        const double ca = std::cos((double)d->sun_half_angle);
        const double omega = 2.0 * 3.14159265358979323846 * (1.0 - ca);
        const double facing = 3.14159265358979323846 * (1.0 - ca) * (1.0 + ca);
        k.sun_pdf = k.sun_disk ? (float)(1.0 / omega) : 0.0f;
        for (int i = 0; i < 3; ++i) k.sun_L[i] = k.sun_disk ? (float)(d->sun_radiance[i] / facing) : 0.0f;
        // Duff et al. 2017 frame around the sun direction
        float s = sd.z >= 0.0f ? 1.0f : -1.0f, a = -1.0f / (s + sd.z), b = sd.x * sd.y * a;
        V3 t{1.0f + s * sd.x * sd.x * a, s * b, -s * sd.x}, bb{b, s + sd.y * sd.y * a, -sd.y};
        put(k.sun_t, t);
        put(k.sun_b, bb);
    }
    // PinholeCamera::Update (include/s3d_camera.h:63-90) minus the aspect, applied per render
    const salty_camera& cam = d->camera;
    for (int i = 0; i < 3; ++i) {
        k.cam_pos[i] = cam.pos[i];
        k.cam_target[i] = cam.target[i];
        k.cam_up[i] = cam.up[i];
    }
    k.cam_fov = cam.fov;
    k.cam_near = cam.near_clip > 0 ? cam.near_clip : 1.0f;
    if (!(cam.lens_radius >= 0.0f) || !(cam.focal_distance >= 0.0f))
        return fail(E.fail(SALTY_ERR_INVALID_ARG, "camera lens radius and focal distance must be >= 0"));
    k.cam_lens = cam.lens_radius;
    k.cam_focal = cam.focal_distance;
    UP_CUDA(cudaStreamSynchronize(ctx->stream));
    UP_CUDA(cudaGetLastError());
#undef UP_TRY
#undef UP_CUDA
    *out = sc;
    return SALTY_OK;
}

salty_status salty_scene_set_camera(salty_ctx* ctx, salty_scene* scene, const salty_camera* cam) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    if (!scene || !cam) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "null scene or camera");
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(cam->pos[i]) || !std::isfinite(cam->target[i]) || !std::isfinite(cam->up[i]))
            return ctx->err.fail(SALTY_ERR_INVALID_ARG, "camera has a non-finite component");
    if (!(cam->fov > 0.0f) || !std::isfinite(cam->fov))
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "camera fov must be positive");
    salty::SceneConsts& k = scene->consts;
    for (int i = 0; i < 3; ++i) {
        k.cam_pos[i] = cam->pos[i];
        k.cam_target[i] = cam->target[i];
        k.cam_up[i] = cam->up[i];
    }
    k.cam_fov = cam->fov;
    k.cam_near = cam->near_clip > 0 ? cam->near_clip : 1.0f;
    if (!(cam->lens_radius >= 0.0f) || !(cam->focal_distance >= 0.0f))
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "camera lens radius and focal distance must be >= 0");
    k.cam_lens = cam->lens_radius;
    k.cam_focal = cam->focal_distance;
    return SALTY_OK;
}

void salty_scene_destroy(salty_ctx* ctx, salty_scene* scene) {
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    delete scene;
}

salty_status salty_bvh_build(salty_ctx* ctx, salty_scene* scene, const salty_build_opts* opts,
                             salty_bvh_info* info) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    if (!scene) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "null scene");
    salty_build_opts o{32, 3, 0.3f};
    if (opts) {
        if (opts->bins) o.bins = opts->bins;
        if (opts->max_leaf) o.max_leaf = opts->max_leaf;
        if (opts->trav_cost > 0) o.trav_cost = opts->trav_cost;
    }
    if (o.bins < 2 || o.bins > 32) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bins must be 2..32");
    if (o.max_leaf < 1 || o.max_leaf > kMaxLeafTris) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "max_leaf must be 1..3");
    cudaSetDevice(ctx->device);
    scene->bvh.built = false;
    SALTY_TRY(build_bvh(ctx, scene, o));
    if (info) *info = scene->bvh.info;
    return SALTY_OK;
}

// ---------------------------------------------------------------- trace
salty_status salty_trace(salty_ctx* ctx, salty_scene* sc, const salty_ray* rays, int64_t n, uint32_t flags,
                         salty_hit* hits) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!sc) return E.fail(SALTY_ERR_INVALID_ARG, "null scene");
    if (n < 0 || (n > 0 && (!rays || !hits))) return E.fail(SALTY_ERR_INVALID_ARG, "bad ray/hit arrays");
    if (flags & ~(uint32_t)(SALTY_TRACE_ANY_HIT | SALTY_TRACE_WATERTIGHT | SALTY_TRACE_COUNTERS))
        return E.fail(SALTY_ERR_INVALID_ARG, "unknown trace flags 0x%x", flags);
    if (!sc->bvh.built) return E.fail(SALTY_ERR_NOT_BUILT, "salty_bvh_build has not been called");
    cudaSetDevice(ctx->device);
    salty_trace_stats stats{};
    stats.rays = n;
    if (n == 0) {
        ctx->last_trace = stats;
        return SALTY_OK;
    }
    const bool din = is_device_ptr(rays) && ((uintptr_t)rays % 16 == 0);
    const bool dout = is_device_ptr(hits) && ((uintptr_t)hits % 16 == 0);
    cudaStream_t st = ctx->stream;
    SALTY_TRY_CUDA(E, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    cudaEvent_t t0 = ctx->ev[2], k0 = ctx->ev[3], k1 = ctx->ev[4], t1 = ctx->ev[5];
    SALTY_TRY_CUDA(E, cudaEventRecord(t0, st));
    unsigned long long counts[3] = {0, 0, 0};
    double kernel_ms = 0.0;
    if (din && dout) {
        SALTY_TRY_CUDA(E, cudaEventRecord(k0, st));
        SALTY_TRY(trace_launch(ctx, sc, (const float4*)rays, n, nullptr, flags, (float4*)hits, ctx->counters.p, st,
                               ctx->status.p));
        stats.launches = 1;
        SALTY_TRY_CUDA(E, cudaEventRecord(k1, st));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(counts, ctx->counters.p, sizeof counts, cudaMemcpyDeviceToHost, st));
        SALTY_TRY_CUDA(E, cudaEventRecord(t1, st));
        SALTY_TRY_CUDA(E, cudaEventSynchronize(t1));
        float ms = 0;
        cudaEventElapsedTime(&ms, k0, k1);
        kernel_ms = ms;
    } else {
        // Host arrays: chunks alternate between two device slots so the copies of one
        // chunk overlap the traversal of the other.
        const long long chunk = 1ll << 21;
        const long long nch = (n + chunk - 1) / chunk;
        const long long slot_rays = std::min<long long>(chunk, n);
        SALTY_TRY_CUDA(E, ctx->ray_buf.ensure((size_t)2 * 2 * slot_rays));
        SALTY_TRY_CUDA(E, ctx->hit_buf.ensure((size_t)2 * slot_rays));
        cudaStream_t ss[2] = {ctx->stream, ctx->copy_stream};
        cudaEvent_t slot_free[2] = {ctx->ev[6], ctx->ev[7]};
        SALTY_TRY_CUDA(E, cudaEventRecord(k0, st));
        SALTY_TRY_CUDA(E, cudaStreamWaitEvent(ss[1], k0, 0));
        for (long long c = 0; c < nch; ++c) {
            const int s = (int)(c & 1);
            const long long b = c * chunk, m = std::min(chunk, n - b);
            float4* rb = ctx->ray_buf.p + (size_t)s * 2 * slot_rays;
            float4* hb = ctx->hit_buf.p + (size_t)s * slot_rays;
            const float4* rin = din ? (const float4*)(rays + b) : rb;
            float4* hout = dout ? (float4*)(hits + b) : hb;
            if (!din) {
                SALTY_TRY_CUDA(E, cudaMemcpyAsync(rb, rays + b, (size_t)m * sizeof(salty_ray), cudaMemcpyDefault, ss[s]));
                stats.h2d_bytes += m * (int64_t)sizeof(salty_ray);
            }
            SALTY_TRY(trace_launch(ctx, sc, rin, m, nullptr, flags, hout, ctx->counters.p + 4 * s, ss[s], ctx->status.p));
            ++stats.launches;
            if (!dout) {
                SALTY_TRY_CUDA(E, cudaMemcpyAsync(hits + b, hb, (size_t)m * sizeof(salty_hit), cudaMemcpyDefault, ss[s]));
                stats.d2h_bytes += m * (int64_t)sizeof(salty_hit);
            }
            SALTY_TRY_CUDA(E, cudaEventRecord(slot_free[s], ss[s]));
            (void)slot_free;
            if (flags & SALTY_TRACE_COUNTERS) {
                SALTY_TRY_CUDA(E, cudaStreamSynchronize(ss[s]));
                unsigned long long cc[3];
                SALTY_TRY_CUDA(E, cudaMemcpy(cc, ctx->counters.p + 4 * s, sizeof cc, cudaMemcpyDeviceToHost));
                counts[1] += cc[1];
                counts[2] += cc[2];
            }
        }
        SALTY_TRY_CUDA(E, cudaEventRecord(ctx->ev[6], ss[1]));
        SALTY_TRY_CUDA(E, cudaStreamWaitEvent(st, ctx->ev[6], 0));
        SALTY_TRY_CUDA(E, cudaEventRecord(k1, st));
        SALTY_TRY_CUDA(E, cudaEventRecord(t1, st));
        SALTY_TRY_CUDA(E, cudaEventSynchronize(t1));
        float ms = 0;
        cudaEventElapsedTime(&ms, k0, k1);
        kernel_ms = ms;
    }
    SALTY_TRY_CUDA(E, cudaGetLastError());
    int status = 0;
    SALTY_TRY_CUDA(E, cudaMemcpy(&status, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost));
    float total = 0;
    cudaEventElapsedTime(&total, t0, t1);
    stats.kernel_ms = kernel_ms;
    stats.total_ms = total;
    stats.node_fetches = (int64_t)counts[1];
    stats.tri_fetches = (int64_t)counts[2];
    ctx->last_trace = stats;
    if (status) return E.fail(SALTY_ERR_QUEUE_OVERFLOW, "traversal stack overflow (BVH depth %d)", sc->bvh.depth);
    return SALTY_OK;
}

salty_status salty_last_trace_stats(const salty_ctx* ctx, salty_trace_stats* out) {
    if (!ctx || !out) return SALTY_ERR_INVALID_ARG;
    *out = ctx->last_trace;
    return SALTY_OK;
}

// ---------------------------------------------------------------- render / post

salty_status salty_render(salty_ctx* ctx, salty_scene* sc, const salty_render_opts* o, float* mean_rgb,
                          float* var_rgb, uint8_t* srgb8, salty_render_stats* stats) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    SALTY_TRY(check_render_opts(ctx, sc, o));
    const bool cropped = o->crop_w > 0 || o->crop_h > 0 || o->crop_x != 0 || o->crop_y != 0;
    cudaSetDevice(ctx->device);
    ctx->cancel = 0;
    salty_render_stats st{};
    SALTY_TRY(render(ctx, sc, *o, &st));
    if (stats) *stats = st;
    if (!mean_rgb && !var_rgb && !srgb8) return SALTY_OK;
    const size_t npx = cropped ? (size_t)o->crop_w * o->crop_h : (size_t)o->width * o->height;
    const bool dm = !mean_rgb || is_device_ptr(mean_rgb), dv = !var_rgb || is_device_ptr(var_rgb),
               ds = !srgb8 || is_device_ptr(srgb8);
    float *tm = nullptr, *tv = nullptr;
    uint8_t* ts = nullptr;
    DevBuf<float> bm, bv;
    DevBuf<uint8_t> bs;
    if (mean_rgb && !dm) { SALTY_TRY_CUDA(E, bm.ensure(npx * 3)); tm = bm.p; } else tm = mean_rgb;
    if (var_rgb && !dv) { SALTY_TRY_CUDA(E, bv.ensure(npx * 3)); tv = bv.p; } else tv = var_rgb;
    if (srgb8 && !ds) { SALTY_TRY_CUDA(E, bs.ensure(npx * 3)); ts = bs.p; } else ts = srgb8;
    SALTY_TRY(film_outputs(ctx, sc, *o, tm, tv, ts));
    if (mean_rgb && !dm) SALTY_TRY_CUDA(E, cudaMemcpyAsync(mean_rgb, tm, npx * 12, cudaMemcpyDeviceToHost, ctx->stream));
    if (var_rgb && !dv) SALTY_TRY_CUDA(E, cudaMemcpyAsync(var_rgb, tv, npx * 12, cudaMemcpyDeviceToHost, ctx->stream));
    if (srgb8 && !ds) SALTY_TRY_CUDA(E, cudaMemcpyAsync(srgb8, ts, npx * 3, cudaMemcpyDeviceToHost, ctx->stream));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}

salty_status salty_film_read(salty_ctx* ctx, salty_scene* sc, double* sum, double* sumsq, int64_t* samples);

salty_status salty_render_batch(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts,
                                int32_t n, salty_render_stats* total) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!scenes || !opts || n < 1) return E.fail(SALTY_ERR_INVALID_ARG, "empty batch");
    for (int i = 0; i < n; ++i) {
        SALTY_TRY(check_render_opts(ctx, scenes[i], &opts[i]));
        for (int j = 0; j < i; ++j)
            if (scenes[j] == scenes[i]) return E.fail(SALTY_ERR_INVALID_ARG, "scene %d appears twice in the batch", i);
    }
    cudaSetDevice(ctx->device);
    ctx->cancel = 0;
    return render_batch(ctx, scenes, opts, n, total);
}

salty_status salty_get_tuning(salty_ctx* ctx, salty_tuning* out) {
    if (!ctx || !out) return SALTY_ERR_INVALID_ARG;
    out->trace_block = ctx->tune.trace.block;
    out->trace_pool = ctx->tune.trace.pool;
    out->trace_postpone = ctx->tune.trace.postpone;
    out->shade_block = ctx->tune.shade_block;
    out->trace_regs = ctx->tune.trace.regs;
    out->wave_paths = ctx->tune.wave_paths;
    return SALTY_OK;
}

salty_status salty_set_tuning(salty_ctx* ctx, const salty_tuning* t) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!t) return E.fail(SALTY_ERR_INVALID_ARG, "null tuning");
    if (t->trace_block != 64 && t->trace_block != 128 && t->trace_block != 256)
        return E.fail(SALTY_ERR_INVALID_ARG, "trace_block must be 64, 128 or 256");
    if (t->trace_pool < 32 || t->trace_pool > 4096) return E.fail(SALTY_ERR_INVALID_ARG, "trace_pool must be 32..4096");
    if (t->trace_postpone < 1 || t->trace_postpone > 32)
        return E.fail(SALTY_ERR_INVALID_ARG, "trace_postpone must be 1..32");
    if (t->shade_block < 64 || t->shade_block > 1024 || t->shade_block % 32)
        return E.fail(SALTY_ERR_INVALID_ARG, "shade_block must be a multiple of 32 in 64..1024");
    if (t->trace_regs != 64 && t->trace_regs != 56) return E.fail(SALTY_ERR_INVALID_ARG, "trace_regs must be 64 or 56");
    if (t->wave_paths < (1 << 16) || t->wave_paths > (1 << 27))
        return E.fail(SALTY_ERR_INVALID_ARG, "wave_paths must be 2^16..2^27");
    ctx->tune.trace.block = t->trace_block;
    ctx->tune.trace.pool = t->trace_pool;
    ctx->tune.trace.postpone = t->trace_postpone;
    ctx->tune.shade_block = t->shade_block;
    ctx->tune.trace.regs = t->trace_regs;
    ctx->tune.wave_paths = t->wave_paths;
    return SALTY_OK;
}

salty_status salty_autotune_trace(salty_ctx* ctx, salty_scene* sc, const salty_ray* rays, int64_t n, uint32_t flags,
                                  salty_tuning* out, float* best_ms) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!sc || !rays || n <= 0) return E.fail(SALTY_ERR_INVALID_ARG, "null scene or no rays");
    if (flags & ~(uint32_t)(SALTY_TRACE_ANY_HIT | SALTY_TRACE_WATERTIGHT))
        return E.fail(SALTY_ERR_INVALID_ARG, "unknown trace flags 0x%x", flags);
    if (!sc->bvh.built) return E.fail(SALTY_ERR_NOT_BUILT, "salty_bvh_build has not been called");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    SALTY_TRY_CUDA(E, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    const float4* d_rays = reinterpret_cast<const float4*>(rays);
    DevBuf<float4> copy;
    if (!is_device_ptr(rays) || (uintptr_t)rays % 16) {
        SALTY_TRY_CUDA(E, copy.ensure((size_t)n * 2));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(copy.p, rays, (size_t)n * sizeof(salty_ray), cudaMemcpyDefault, st));
        d_rays = copy.p;
    }
    DevBuf<float4> hits;
    SALTY_TRY_CUDA(E, hits.ensure((size_t)n));
    // time of one launch under the context's current tuning: the better of two, after one untimed
    auto time_of = [&](float* ms) -> salty_status {
        float best = 1e30f;
        for (int r = 0; r < 3; ++r) {
            SALTY_TRY_CUDA(E, cudaEventRecord(ctx->ev[3], st));
            SALTY_TRY(trace_launch(ctx, sc, d_rays, n, nullptr, flags, hits.p, ctx->counters.p, st, ctx->status.p));
            SALTY_TRY_CUDA(E, cudaEventRecord(ctx->ev[4], st));
            SALTY_TRY_CUDA(E, cudaEventSynchronize(ctx->ev[4]));
            float m = 0;
            cudaEventElapsedTime(&m, ctx->ev[3], ctx->ev[4]);
            if (r > 0) best = std::min(best, m);
        }
        *ms = best;
        return SALTY_OK;
    };
    const TraceTuning start = ctx->tune.trace;
    TraceTuning best = start;
    float best_t = 0;
    salty_status s = time_of(&best_t);
    const int block_regs[][2] = {{64, 64}, {128, 64}, {256, 64}, {64, 56}, {128, 56}};
    const int pool[] = {64, 128, 256};
    const int postpone[] = {1, 4, 7, 10};
    auto consider = [&](TraceTuning t) -> salty_status {
        ctx->tune.trace = t;
        float ms = 0;
        SALTY_TRY(time_of(&ms));
        if (ms < best_t * 0.995f) { best_t = ms; best = t; }
        return SALTY_OK;
    };
    for (auto& br : block_regs) {
        if (s != SALTY_OK) break;
        TraceTuning t = best;
        t.block = br[0];
        t.regs = br[1];
        if (t.block != best.block || t.regs != best.regs) s = consider(t);
    }
    for (int v : pool) {
        if (s != SALTY_OK) break;
        TraceTuning t = best;
        t.pool = v;
        if (v != best.pool) s = consider(t);
    }
    for (int v : postpone) {
        if (s != SALTY_OK) break;
        TraceTuning t = best;
        t.postpone = v;
        if (v != best.postpone) s = consider(t);
    }
    ctx->tune.trace = s == SALTY_OK ? best : start;
    if (s != SALTY_OK) return s;
    int status = 0;
    SALTY_TRY_CUDA(E, cudaMemcpy(&status, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) return E.fail(SALTY_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
    if (best_ms) *best_ms = best_t;
    return out ? salty_get_tuning(ctx, out) : SALTY_OK;
}

salty_status salty_autotune(salty_ctx* ctx, salty_scene* const* scenes, const salty_render_opts* opts, int32_t n,
                            int32_t trial_spp, salty_tuning* out, float* best_ms) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!scenes || !opts || n < 1) return E.fail(SALTY_ERR_INVALID_ARG, "empty batch");
    if (trial_spp < 1) return E.fail(SALTY_ERR_INVALID_ARG, "trial_spp must be >= 1");
    std::vector<salty_render_opts> trial(opts, opts + n);
    for (auto& o : trial) {
        o.spp = std::min(o.spp, trial_spp);
        o.accumulate = 0;
    }
    for (int i = 0; i < n; ++i) SALTY_TRY(check_render_opts(ctx, scenes[i], &trial[i]));
    cudaSetDevice(ctx->device);
    long long samples = 0;
    for (int i = 0; i < n; ++i) {
        const bool cr = trial[i].crop_w > 0 && trial[i].crop_h > 0;
        samples += (long long)(cr ? trial[i].crop_w : trial[i].width) * (cr ? trial[i].crop_h : trial[i].height) *
                   trial[i].spp;
    }
    // time of one trial render under a tuning: the better of two runs (device time)
    auto time_of = [&](const Tuning& t, float* ms) -> salty_status {
        ctx->tune = t;
        float best = 1e30f;
        for (int r = 0; r < 2; ++r) {
            salty_render_stats st{};
            SALTY_TRY(render_batch(ctx, scenes, trial.data(), n, &st));
            best = std::min(best, (float)st.ms);
        }
        *ms = best;
        return SALTY_OK;
    };
    const Tuning start = ctx->tune;
    Tuning best = start;
    float best_t = 0;
    salty_status s = time_of(best, &best_t);
    // coordinate descent, one pass over the knobs
    const long long waves[] = {1ll << 22, 1ll << 24, 1ll << 26, 1ll << 27};
    const int shade[] = {128, 256, 512};
    // traversal block size and register budget interact (registers x threads x blocks per
    // SM against the shared stack), so they are searched as pairs
    const int block_regs[][2] = {{64, 64}, {128, 64}, {256, 64}, {64, 56}, {128, 56}};
    const int pool[] = {64, 128, 256};
    const int postpone[] = {1, 4, 7, 10};
    auto try_knob = [&](auto set, const auto& values) -> salty_status {
        for (auto v : values) {
            Tuning t = best;
            if (!set(t, v)) continue;
            float ms = 0;
            SALTY_TRY(time_of(t, &ms));
            if (ms < best_t * 0.995f) { best_t = ms; best = t; }
        }
        return SALTY_OK;
    };
    if (s == SALTY_OK)
        s = try_knob([&](Tuning& t, long long v) {
                // capacities at or above the sample count all run one wave
                if (std::min(v, samples) == std::min(best.wave_paths, samples)) return false;
                t.wave_paths = v;
                return true;
            }, waves);
    if (s == SALTY_OK)
        s = try_knob([&](Tuning& t, int v) { if (v == best.shade_block) return false; t.shade_block = v; return true; },
                     shade);
    if (s == SALTY_OK)
        s = try_knob([&](Tuning& t, const int* v) {
                if (v[0] == best.trace.block && v[1] == best.trace.regs) return false;
                t.trace.block = v[0];
                t.trace.regs = v[1];
                return true;
            }, block_regs);
    if (s == SALTY_OK)
        s = try_knob([&](Tuning& t, int v) { if (v == best.trace.pool) return false; t.trace.pool = v; return true; },
                     pool);
    if (s == SALTY_OK)
        s = try_knob([&](Tuning& t, int v) {
                if (v == best.trace.postpone) return false;
                t.trace.postpone = v;
                return true;
            }, postpone);
    ctx->tune = s == SALTY_OK ? best : start;
    if (s != SALTY_OK) return s;
    if (best_ms) *best_ms = best_t;
    return out ? salty_get_tuning(ctx, out) : SALTY_OK;
}

salty_status salty_tonemap(salty_ctx* ctx, int32_t type, int32_t w, int32_t h, const float* rgb, float* out_rgb,
                           uint8_t* out_srgb8, int32_t ref_oetf, float* ave_lw, float* max_lw) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (w <= 0 || h <= 0 || !rgb) return E.fail(SALTY_ERR_INVALID_ARG, "bad image");
    if (type < SALTY_TM_REINHARD || type > SALTY_TM_ACES) return E.fail(SALTY_ERR_INVALID_ARG, "bad tonemap type");
    cudaSetDevice(ctx->device);
    const size_t npx = (size_t)w * h;
    DevBuf<float> bi, bo;
    DevBuf<uint8_t> bs;
    const float* di = rgb;
    if (!is_device_ptr(rgb)) {
        SALTY_TRY_CUDA(E, bi.ensure(npx * 3));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(bi.p, rgb, npx * 12, cudaMemcpyHostToDevice, ctx->stream));
        di = bi.p;
    }
    float* dout = out_rgb;
    bool hout = out_rgb && !is_device_ptr(out_rgb);
    if (hout) { SALTY_TRY_CUDA(E, bo.ensure(npx * 3)); dout = bo.p; }
    uint8_t* ds = out_srgb8;
    bool hs = out_srgb8 && !is_device_ptr(out_srgb8);
    if (hs) { SALTY_TRY_CUDA(E, bs.ensure(npx * 3)); ds = bs.p; }
    SALTY_TRY(tonemap_device(ctx, type, w, h, di, dout, ds, ref_oetf, ave_lw, max_lw));
    if (hout) SALTY_TRY_CUDA(E, cudaMemcpyAsync(out_rgb, dout, npx * 12, cudaMemcpyDeviceToHost, ctx->stream));
    if (hs) SALTY_TRY_CUDA(E, cudaMemcpyAsync(out_srgb8, ds, npx * 3, cudaMemcpyDeviceToHost, ctx->stream));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}

salty_status salty_denoise_nlm_ref(salty_ctx* ctx, int32_t w, int32_t h, float coeff, const float* rgba, float* out) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (w <= 0 || h <= 0 || !rgba || !out) return E.fail(SALTY_ERR_INVALID_ARG, "bad image");
    cudaSetDevice(ctx->device);
    const size_t npx = (size_t)w * h;
    DevBuf<float> bi, bo;
    const float* di = rgba;
    if (!is_device_ptr(rgba)) {
        SALTY_TRY_CUDA(E, bi.ensure(npx * 4));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(bi.p, rgba, npx * 16, cudaMemcpyHostToDevice, ctx->stream));
        di = bi.p;
    }
    float* dout = out;
    bool hout = !is_device_ptr(out);
    if (hout) { SALTY_TRY_CUDA(E, bo.ensure(npx * 4)); dout = bo.p; }
    SALTY_TRY(nlm_ref_device(ctx, w, h, coeff, di, dout));
    if (hout) SALTY_TRY_CUDA(E, cudaMemcpyAsync(out, dout, npx * 16, cudaMemcpyDeviceToHost, ctx->stream));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}

salty_status salty_denoise_nlm(salty_ctx* ctx, int32_t w, int32_t h, int32_t search_r, int32_t patch_r, float k,
                               const float* rgb, const float* var, float* out) {
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (w <= 0 || h <= 0 || !rgb || !var || !out) return E.fail(SALTY_ERR_INVALID_ARG, "bad image");
    if (search_r < 0 || search_r > 32 || patch_r < 0 || patch_r > 8)
        return E.fail(SALTY_ERR_INVALID_ARG, "search_r must be 0..32 and patch_r 0..8");
    cudaSetDevice(ctx->device);
    const size_t npx = (size_t)w * h;
    DevBuf<float> bi, bv, bo;
    const float* di = rgb;
    const float* dv = var;
    if (!is_device_ptr(rgb)) {
        SALTY_TRY_CUDA(E, bi.ensure(npx * 3));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(bi.p, rgb, npx * 12, cudaMemcpyHostToDevice, ctx->stream));
        di = bi.p;
    }
    if (!is_device_ptr(var)) {
        SALTY_TRY_CUDA(E, bv.ensure(npx * 3));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(bv.p, var, npx * 12, cudaMemcpyHostToDevice, ctx->stream));
        dv = bv.p;
    }
    float* dout = out;
    bool hout = !is_device_ptr(out);
    if (hout) { SALTY_TRY_CUDA(E, bo.ensure(npx * 3)); dout = bo.p; }
    SALTY_TRY(nlm_var_device(ctx, w, h, search_r, patch_r, k, di, dv, dout));
    if (hout) SALTY_TRY_CUDA(E, cudaMemcpyAsync(out, dout, npx * 12, cudaMemcpyDeviceToHost, ctx->stream));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}

// ---------------------------------------------------------------- inputs
// Triangle soup: centroid c ~ U[0,1]^3 (three draws), then for each vertex k and axis a
// in order, v[k][a] = c[a] + (draw - 0.5f) * 0.01f.
salty_status salty_microbench_soup(uint64_t seed, int64_t n, float* tri_pos) {
    if (n < 0 || (n > 0 && !tri_pos)) return SALTY_ERR_INVALID_ARG;
    Pcg r(seed);
    for (int64_t i = 0; i < n; ++i) {
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = r.f32();
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                float j = (r.f32() - 0.5f) * 0.01f;
                tri_pos[i * 9 + k * 3 + a] = c[a] + j;
            }
    }
    return SALTY_OK;
}

// Rays: origin uniform on the radius-2 sphere about (0.5, 0.5, 0.5) (Marsaglia 1972, in
// double), target ~ U[0,1]^3, direction = Vector3::UnitVector(target - origin)
// (include/s3d_math.h:830-842), tmin given, tmax = +inf.
salty_status salty_microbench_rays(uint64_t seed, int64_t n, float tmin, salty_ray* rays) {
    if (n < 0 || (n > 0 && !rays)) return SALTY_ERR_INVALID_ARG;
    Pcg r(seed);
    for (int64_t i = 0; i < n; ++i) {
        double a, b, s;
        do {
            a = 2.0 * (double)r.f32() - 1.0;
            b = 2.0 * (double)r.f32() - 1.0;
            s = a * a + b * b;
        } while (s >= 1.0);
        double q = 2.0 * std::sqrt(1.0 - s);
        float o[3];
        o[0] = (float)(0.5 + 2.0 * (a * q));
        o[1] = (float)(0.5 + 2.0 * (b * q));
        o[2] = (float)(0.5 + 2.0 * (1.0 - 2.0 * s));
        float t[3];
        for (int k = 0; k < 3; ++k) t[k] = r.f32();
        float d0 = t[0] - o[0], d1 = t[1] - o[1], d2 = t[2] - o[2];
        float mag = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        salty_ray& out = rays[i];
        out.org[0] = o[0]; out.org[1] = o[1]; out.org[2] = o[2];
        out.tmin = tmin;
        out.dir[0] = d0 / mag; out.dir[1] = d1 / mag; out.dir[2] = d2 / mag;
        out.tmax = INFINITY;
    }
    return SALTY_OK;
}

}  // extern "C"
