// instance.cu -- two-level BVHs: placed copies of meshes, each mesh stored once.
//
// Replaces Instance (src/s3d_instance.cpp:22-101), which wraps a shape with a world matrix,
// transforms the ray into object space in IsHit and the normal back in CalcParam.  Here a
// scene's instances share the scene's triangle arrays: salty_scene_set_instances names, per
// instance, a triangle range (its mesh) and a 3x4 object-to-world matrix.  The build then
//   1. builds one BVH8 per distinct mesh over its triangles in object space,
//   2. builds a top-level BVH8 over the instances' world boxes (the mesh box's eight corners
//      transformed -- the reference transforms only two corners, include/s3d_math.h:
//      2267-2272, which loses parts of rotated meshes), each instance one leaf entry,
//   3. writes all of them into the scene's node and triangle arrays, top level first, with
//      child and triangle bases rebased, and an instance table for traversal (world-to-
//      object matrix, mesh root node, first virtual id) and shading (object-to-world and
//      normal matrices).
// The traversal kernel enters an instance when the walk reaches its leaf entry and returns
// to the top level when the mesh's walk is over (trace.cu).  Ray directions are not
// renormalised in object space, so hit distances compare across instances.
#include <algorithm>
#include <cmath>
#include <map>

#include "internal.h"

namespace salty {
namespace {

__global__ void k_inst_nodes(const Bvh8Node* __restrict__ src, long long n, unsigned node_off, unsigned tri_off,
                             Bvh8Node* __restrict__ dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        Bvh8Node v = src[i];
        v.w[1].x += node_off;  // child base
        v.w[1].y += tri_off;   // triangle base
        dst[i] = v;
    }
}

// 3x4 affine inverse in double; false when singular
bool invert34(const float* m, float* inv) {
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], k = m[10];
    const double A = e * k - f * h, B = -(d * k - f * g), Cc = d * h - e * g;
    const double det = a * A + b * B + c * Cc;
    if (!(std::fabs(det) > 1e-30) || !std::isfinite(det)) return false;
    const double id = 1.0 / det;
    const double r[9] = {A * id, -(b * k - c * h) * id, (b * f - c * e) * id,
                         B * id, (a * k - c * g) * id, -(a * f - c * d) * id,
                         Cc * id, -(a * h - b * g) * id, (a * e - b * d) * id};
    const double t[3] = {m[3], m[7], m[11]};
    for (int i = 0; i < 3; ++i) {
        inv[4 * i + 0] = (float)r[3 * i + 0];
        inv[4 * i + 1] = (float)r[3 * i + 1];
        inv[4 * i + 2] = (float)r[3 * i + 2];
        inv[4 * i + 3] = (float)(-(r[3 * i] * t[0] + r[3 * i + 1] * t[1] + r[3 * i + 2] * t[2]));
    }
    return true;
}

}  // namespace

salty_status build_instanced(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts) {
    auto& E = ctx->err;
    cudaStream_t st = ctx->stream;
    const int ni = sc->n_inst;
    const std::vector<salty_instance>& I = sc->inst_host;
    // 1. one BVH per distinct mesh
    std::map<std::pair<int64_t, int64_t>, int> mesh_of;
    std::vector<std::pair<int64_t, int64_t>> meshes;
    std::vector<int> inst_mesh(ni);
    for (int i = 0; i < ni; ++i) {
        auto key = std::make_pair(I[i].first_tri, I[i].n_tris);
        auto it = mesh_of.find(key);
        if (it == mesh_of.end()) {
            it = mesh_of.emplace(key, (int)meshes.size()).first;
            meshes.push_back(key);
        }
        inst_mesh[i] = it->second;
    }
    const int nm = (int)meshes.size();
    std::vector<Bvh> blas(nm);
    std::vector<float> mbox(6 * (size_t)nm);
    int blas_depth = 0;
    double build_ms = 0.0;
    for (int m = 0; m < nm; ++m) {
        SALTY_TRY(build_bvh_tris(ctx, sc->pos.p + meshes[m].first * 9, (int)meshes[m].second, opts, blas[m],
                                 &mbox[6 * (size_t)m]));
        blas_depth = std::max(blas_depth, (int)blas[m].depth);
        build_ms += blas[m].info.build_ms;
    }
    // 2. the top level over the instances' world boxes, each given as a degenerate triangle
    // (lo, hi, lo) whose box is the instance's
    std::vector<float> boxes(9 * (size_t)ni);
    for (int i = 0; i < ni; ++i) {
        const float* M = I[i].object_to_world;
        const float* b = &mbox[6 * (size_t)inst_mesh[i]];
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 8; ++c) {
            const double p[3] = {b[(c & 1) ? 3 : 0], b[(c & 2) ? 4 : 1], b[(c & 4) ? 5 : 2]};
            for (int r = 0; r < 3; ++r) {
                const double w = M[4 * r] * p[0] + M[4 * r + 1] * p[1] + M[4 * r + 2] * p[2] + M[4 * r + 3];
                lo[r] = std::min(lo[r], w);
                hi[r] = std::max(hi[r], w);
            }
        }
        for (int r = 0; r < 3; ++r) {
            // rounded outwards to float, with a relative margin for the transforms' rounding
            const double pad = 1e-6 * std::max(std::fabs(lo[r]), std::fabs(hi[r])) + 1e-30;
            boxes[9 * (size_t)i + r] = boxes[9 * (size_t)i + 6 + r] = std::nextafter((float)(lo[r] - pad), -INFINITY);
            boxes[9 * (size_t)i + 3 + r] = std::nextafter((float)(hi[r] + pad), INFINITY);
        }
    }
    DevBuf<float> dboxes;
    SALTY_TRY_CUDA(E, dboxes.ensure(boxes.size()));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(dboxes.p, boxes.data(), boxes.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    Bvh tlas;
    float tbox[6];
    SALTY_TRY(build_bvh_tris(ctx, dboxes.p, ni, opts, tlas, tbox));
    build_ms += tlas.info.build_ms;
    // 3. one node array and one triangle array: the top level, then every mesh
    long long nn = tlas.n_nodes, nt = tlas.n_tris;
    std::vector<long long> node_off(nm), tri_off(nm);
    for (int m = 0; m < nm; ++m) {
        node_off[m] = nn;
        tri_off[m] = nt;
        nn += blas[m].n_nodes;
        nt += blas[m].n_tris;
    }
    if (nn >= (1ll << 31) || nt >= (1ll << 31)) return E.fail(SALTY_ERR_CAPACITY, "instanced BVH too large");
    Bvh& B = sc->bvh;
    SALTY_TRY_CUDA(E, B.nodes.ensure((size_t)nn));
    SALTY_TRY_CUDA(E, B.tris.ensure((size_t)nt * kTriFloat4));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(B.nodes.p, tlas.nodes.p, tlas.n_nodes * sizeof(Bvh8Node),
                                      cudaMemcpyDeviceToDevice, st));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(B.tris.p, tlas.tris.p, tlas.n_tris * kTriFloat4 * sizeof(float4),
                                      cudaMemcpyDeviceToDevice, st));
    for (int m = 0; m < nm; ++m) {
        k_inst_nodes<<<ctx->num_sms * 4, 256, 0, st>>>(blas[m].nodes.p, blas[m].n_nodes, (unsigned)node_off[m],
                                                       (unsigned)tri_off[m], B.nodes.p + node_off[m]);
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(B.tris.p + tri_off[m] * kTriFloat4, blas[m].tris.p,
                                          blas[m].n_tris * kTriFloat4 * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    }
    // instance tables
    std::vector<InstRec> rec(ni);
    std::vector<InstShade> shade(ni);
    std::vector<int> vbase(ni + 1);
    long long vb = 0;
    for (int i = 0; i < ni; ++i) {
        InstRec& R = rec[i];
        if (!invert34(I[i].object_to_world, R.w2o))
            return E.fail(SALTY_ERR_INVALID_ARG, "instance %d: the matrix is not invertible", i);
        R.root = (unsigned)node_off[inst_mesh[i]];
        R.vbase = (int)vb;
        R.first = (int)I[i].first_tri;
        R.pad = 0;
        InstShade& S = shade[i];
        std::copy(I[i].object_to_world, I[i].object_to_world + 12, S.o2w);
        // normal matrix = transpose of the inverse's linear part
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S.nrm[3 * r + c] = R.w2o[4 * c + r];
        S.pad[0] = S.pad[1] = S.pad[2] = 0.0f;
        vbase[i] = (int)vb;
        vb += I[i].n_tris;
    }
    vbase[ni] = (int)vb;
    SALTY_TRY_CUDA(E, sc->inst_rec.ensure(ni));
    SALTY_TRY_CUDA(E, sc->inst_shade.ensure(ni));
    SALTY_TRY_CUDA(E, sc->inst_vbase.ensure(ni + 1));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(sc->inst_rec.p, rec.data(), ni * sizeof(InstRec), cudaMemcpyHostToDevice, st));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(sc->inst_shade.p, shade.data(), ni * sizeof(InstShade), cudaMemcpyHostToDevice,
                                      st));
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(sc->inst_vbase.p, vbase.data(), (ni + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                      st));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));  // the host tables above go out of scope
    sc->n_virtual = vb;
    B.n_nodes = nn;
    B.n_tris = nt;
    // stack: the top level's groups, three entries to enter an instance, the mesh's groups
    B.depth = (int)tlas.depth + blas_depth + 2;
    B.built = true;
    B.generation = tlas.generation;
    B.info.n_nodes = nn;
    B.info.n_binary = tlas.info.n_binary;
    for (const Bvh& b : blas) B.info.n_binary += b.info.n_binary;
    B.info.depth = (int)tlas.depth + blas_depth;
    B.info.binary_depth = tlas.info.binary_depth;
    B.info.sah_cost = tlas.info.sah_cost;
    B.info.build_ms = (float)build_ms;
    // the light's ids are virtual too: its instance is the last
    sc->consts.light_tri0 = sc->consts.has_light ? vbase[ni - 1] : -1;
    return SALTY_OK;
}

}  // namespace salty

extern "C" salty_status salty_scene_set_instances(salty_ctx* ctx, salty_scene* scene, const salty_instance* inst,
                                                  int32_t n) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (!scene) return E.fail(SALTY_ERR_INVALID_ARG, "null scene");
    if (n < 0 || (n > 0 && !inst)) return E.fail(SALTY_ERR_INVALID_ARG, "bad instance list");
    if (n > 0 && scene->n_sph > 0) return E.fail(SALTY_ERR_INVALID_ARG, "instances are not combined with spheres");
    const int64_t n_mesh_tris = scene->n_input;
    std::vector<salty_instance> v;
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        const salty_instance& x = inst[i];
        if (x.first_tri < 0 || x.n_tris <= 0 || x.first_tri + x.n_tris > n_mesh_tris)
            return E.fail(SALTY_ERR_INVALID_ARG, "instance %d: triangles [%lld, %lld) outside the scene's %lld", i,
                          (long long)x.first_tri, (long long)(x.first_tri + x.n_tris), (long long)n_mesh_tris);
        float tmp[12];
        for (float f : x.object_to_world)
            if (!std::isfinite(f)) return E.fail(SALTY_ERR_INVALID_ARG, "instance %d: matrix is not finite", i);
        if (!invert34(x.object_to_world, tmp))
            return E.fail(SALTY_ERR_INVALID_ARG, "instance %d: the matrix is not invertible", i);
        total += x.n_tris;
        v.push_back(x);
    }
    if (n > 0 && scene->consts.has_light) {
        // the light's two triangles, appended after the caller's, stay in world space
        salty_instance L{};
        L.first_tri = scene->n_input;
        L.n_tris = 2;
        L.object_to_world[0] = L.object_to_world[5] = L.object_to_world[10] = 1.0f;
        v.push_back(L);
        total += 2;
    }
    if (total >= (1ll << 31) - 1) return E.fail(SALTY_ERR_CAPACITY, "instances hold more than 2^31 - 1 triangles");
    scene->inst_host = v;
    scene->n_inst = (int)v.size();
    scene->n_virtual = total;
    if (n == 0) scene->consts.light_tri0 = scene->consts.has_light ? (int)scene->n_input : -1;
    scene->bvh.built = false;
    return SALTY_OK;
}
