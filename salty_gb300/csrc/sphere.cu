// sphere.cu -- analytic spheres (Sphere, src/s3d_sphere.cpp:22-115) as shapes of a scene.
//
// A sphere is one more primitive of the scene's BVH8: the build sees it as a degenerate
// triangle (box min, box max, box min) whose bounds are the sphere's box, and afterwards
// its leaf entry is rewritten to (centre, id) (radius, 0, 0, 0) -- the layout the
// traversal's sphere test reads (traverse.cuh, leaf ids from n_tris on).  Shading finds the
// sphere's material and light status in small per-scene tables (render.cu).
#include <cmath>

#include "internal.h"

namespace salty {
namespace {

// positions of the build's stand-in triangles: (lo, hi, lo) per sphere
__global__ void k_sph_boxes(const float4* __restrict__ sph, int n, float* __restrict__ pos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s = sph[i];
    float* p = pos + (size_t)i * 9;
    p[0] = s.x - s.w; p[1] = s.y - s.w; p[2] = s.z - s.w;
    p[3] = s.x + s.w; p[4] = s.y + s.w; p[5] = s.z + s.w;
    p[6] = p[0]; p[7] = p[1]; p[8] = p[2];
}

// leaf entries of spheres: (centre, id) (radius, 0, 0, 0) (0, 0, 0, 0)
__global__ void k_sph_leaves(float4* __restrict__ tris, long long n, int base, const float4* __restrict__ sph) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4* e = tris + i * kTriFloat4;
        const int id = __float_as_int(e[0].w);
        if (id < base) continue;
        const float4 s = sph[id - base];
        e[0] = make_float4(s.x, s.y, s.z, __int_as_float(id));
        e[1] = make_float4(s.w, 0.0f, 0.0f, 0.0f);
        e[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

}  // namespace

salty_status build_with_spheres(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts) {
    auto& E = ctx->err;
    cudaStream_t st = ctx->stream;
    const long long nt = sc->n_tris, n = nt + sc->n_sph;
    if (n > (long long)0x3fffffff) return E.fail(SALTY_ERR_CAPACITY, "too many primitives (%lld)", n);
    DevBuf<float> pos;
    SALTY_TRY_CUDA(E, pos.ensure((size_t)n * 9));
    if (nt > 0)
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(pos.p, sc->pos.p, (size_t)nt * 9 * sizeof(float), cudaMemcpyDeviceToDevice, st));
    k_sph_boxes<<<(sc->n_sph + 255) / 256, 256, 0, st>>>(sc->sph.p, sc->n_sph, pos.p + (size_t)nt * 9);
    SALTY_TRY_CUDA(E, cudaGetLastError());
    float box[6];
    SALTY_TRY(build_bvh_tris(ctx, pos.p, (int)n, opts, sc->bvh, box));
    k_sph_leaves<<<(unsigned)std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8), 256, 0, st>>>(
        sc->bvh.tris.p, n, (int)nt, sc->sph.p);
    SALTY_TRY_CUDA(E, cudaGetLastError());
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
    return SALTY_OK;
}

}  // namespace salty

extern "C" salty_status salty_scene_set_spheres(salty_ctx* ctx, salty_scene* scene, const salty_sphere* spheres,
                                                int32_t n) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!scene) return E.fail(SALTY_ERR_INVALID_ARG, "null scene");
    if (n < 0 || (n > 0 && !spheres)) return E.fail(SALTY_ERR_INVALID_ARG, "bad sphere list");
    if (n > 0 && scene->n_inst > 0) return E.fail(SALTY_ERR_INVALID_ARG, "spheres are not combined with instances");
    // the caller's materials: the table without the area light's own
    const int user_mats = std::max(1, scene->n_mats - (scene->consts.has_light ? 1 : 0));
    std::vector<float4> cr(n);
    std::vector<int> mat(n), lights;
    for (int i = 0; i < n; ++i) {
        const salty_sphere& s = spheres[i];
        if (!std::isfinite(s.center[0]) || !std::isfinite(s.center[1]) || !std::isfinite(s.center[2]) ||
            !std::isfinite(s.radius) || !(s.radius > 0.0f))
            return E.fail(SALTY_ERR_INVALID_ARG, "sphere %d: centre or radius invalid", i);
        if (s.material < 0 || s.material >= user_mats)
            return E.fail(SALTY_ERR_INVALID_ARG, "sphere %d: material %d outside the table", i, s.material);
        cr[i] = make_float4(s.center[0], s.center[1], s.center[2], s.radius);
        mat[i] = s.material | (s.light ? kSphLight : 0);
        if (s.light) lights.push_back(i);
    }
    cudaSetDevice(ctx->device);
    if (n > 0) {
        SALTY_TRY_CUDA(E, scene->sph.ensure(n));
        SALTY_TRY_CUDA(E, scene->sph_mat.ensure(n));
        SALTY_TRY_CUDA(E, scene->sph_lights.ensure(std::max<size_t>(1, lights.size())));
        cudaStream_t st = ctx->stream;
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(scene->sph.p, cr.data(), n * sizeof(float4), cudaMemcpyHostToDevice, st));
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(scene->sph_mat.p, mat.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
        if (!lights.empty())
            SALTY_TRY_CUDA(E, cudaMemcpyAsync(scene->sph_lights.p, lights.data(), lights.size() * sizeof(int),
                                              cudaMemcpyHostToDevice, st));
        SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
    }
    scene->sph_host.assign(spheres, spheres + n);
    scene->n_sph = n;
    scene->n_sph_lights = (int)lights.size();
    scene->consts.sph_base = n > 0 ? (int)scene->n_tris : kNoSpheres;
    scene->consts.n_lights = (scene->consts.has_light ? 1 : 0) + scene->n_sph_lights;
    scene->bvh.built = false;
    return SALTY_OK;
}
