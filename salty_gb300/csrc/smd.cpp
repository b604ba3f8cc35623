// smd.cpp -- the SMD mesh format (Mesh::LoadFromFile, src/s3d_mesh.cpp:250-465) and mesh
// instancing by transform, on the host.
//
// File layout (little endian, version 2):
//   header   magic "SMD\0", u32 version = 2, u32 data header size = 24,
//            u32 triangles, materials, textures, triangle / material / texture struct sizes
//   textures textures x char[256] file names (relative to the file's directory)
//   materials materials x (s32 type, then by type)
//            0 matte      color[3] emissive[3] s32 map                      28 bytes
//            1 mirror     color[3] emissive[3] s32 map                      28
//            2 dielectric color[3] f32 ior emissive[3] s32 map              32
//            3 glossy     color[3] f32 power emissive[3] s32 map            32
//            4 plastic    diffuse[3] specular[3] f32 power emissive[3] s32 map s32 map  48
//   triangles triangles x (3 x (position[3] normal[3] texcoord[2]), s32 material)   100
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

namespace {

constexpr uint32_t kSmdVersion = 2;
constexpr uint32_t kDataHeaderSize = 24;
constexpr size_t kTriangleBytes = 100;

struct Reader {
    FILE* f;
    bool ok = true;
    template <typename T>
    T get() {
        T v{};
        if (ok && std::fread(&v, sizeof v, 1, f) != 1) ok = false;
        return v;
    }
    void floats(float* dst, int n) {
        for (int i = 0; i < n; ++i) dst[i] = get<float>();
    }
};

// The mesh handed out is the public base of its store.
struct MeshStore : salty_mesh {
    std::vector<float> pos, nrm, uv;
    std::vector<int32_t> mat, tex;
    std::vector<salty_material> mats;
    std::vector<char> names;
    void publish() {
        n_tris = (int64_t)mat.size();
        tri_pos = pos.data();
        tri_nrm = nrm.data();
        tri_uv = uv.data();
        tri_mat = mat.data();
        n_mats = (int32_t)mats.size();
        salty_mesh::mats = mats.data();
        mat_texture = tex.data();
        n_textures = (int32_t)(names.size() / 256);
        texture_names = names.data();
    }
};

}  // namespace

extern "C" {

salty_status salty_mesh_load_smd(salty_ctx* ctx, const char* path, salty_mesh** out) {
    salty::ErrorSink local;  // no context (no GPU needed to read a file): status only
    auto& E = ctx ? ctx->err : local;
    if (!path || !out) return E.fail(SALTY_ERR_INVALID_ARG, "null path or output");
    FILE* f = std::fopen(path, "rb");
    if (!f) return E.fail(SALTY_ERR_INVALID_ARG, "cannot open %s", path);
    Reader r{f};
    auto* st = new (std::nothrow) MeshStore{};
    if (!st) {
        std::fclose(f);
        return E.fail(SALTY_ERR_OOM, "host allocation failed");
    }
    auto fail = [&](const char* why) {
        std::fclose(f);
        delete st;
        return E.fail(SALTY_ERR_INVALID_ARG, "%s: %s", path, why);
    };
    char magic[4];
    for (char& c : magic) c = r.get<char>();
    const uint32_t version = r.get<uint32_t>(), dh = r.get<uint32_t>();
    const uint32_t n_tris = r.get<uint32_t>(), n_mats = r.get<uint32_t>(), n_tex = r.get<uint32_t>();
    const uint32_t tri_size = r.get<uint32_t>();
    (void)r.get<uint32_t>();
    (void)r.get<uint32_t>();
    if (!r.ok) return fail("truncated header");
    if (std::memcmp(magic, "SMD", 4) != 0) return fail("not an SMD file");
    if (version != kSmdVersion) return fail("unsupported version");
    if (dh != kDataHeaderSize) return fail("bad data header size");
    if (n_tris == 0 || n_mats == 0) return fail("no triangles or no materials");
    if (tri_size != kTriangleBytes && tri_size != 0) return fail("bad triangle size");
    if (n_tris > (1u << 30) || n_mats > (1u << 20) || n_tex > (1u << 20)) return fail("counts too large");
    st->names.resize((size_t)n_tex * 256);
    if (n_tex && std::fread(st->names.data(), 256, n_tex, f) != n_tex) return fail("truncated texture table");
    for (uint32_t t = 0; t < n_tex; ++t) st->names[(size_t)t * 256 + 255] = '\0';
    st->mats.resize(n_mats);
    st->tex.assign(n_mats, -1);
    for (uint32_t i = 0; i < n_mats; ++i) {
        salty_material& m = st->mats[i];
        std::memset(&m, 0, sizeof m);
        m.ior = 1.5f;
        const int32_t type = r.get<int32_t>();
        int32_t map = -1;
        switch (type) {
            case 0:  // matte -> Lambert (MaterialFactory::CreateLambert)
            case 1:  // mirror
                m.type = type == 0 ? SALTY_LAMBERT : SALTY_MIRROR;
                r.floats(m.color, 3);
                r.floats(m.emission, 3);
                map = r.get<int32_t>();
                break;
            case 2:  // dielectric -> Glass
                m.type = SALTY_GLASS;
                r.floats(m.color, 3);
                m.ior = r.get<float>();
                r.floats(m.emission, 3);
                map = r.get<int32_t>();
                break;
            case 3:  // glossy -> Phong
                m.type = SALTY_PHONG;
                r.floats(m.color, 3);
                m.power = r.get<float>();
                r.floats(m.emission, 3);
                map = r.get<int32_t>();
                break;
            case 4:  // plastic
                m.type = SALTY_PLASTIC;
                r.floats(m.color, 3);
                r.floats(m.specular, 3);
                m.power = r.get<float>();
                r.floats(m.emission, 3);
                map = r.get<int32_t>();
                (void)r.get<int32_t>();  // specular map: unused by the reference's Plastic
                break;
            default:
                return fail("unknown material type");
        }
        if (!r.ok) return fail("truncated material table");
        st->tex[i] = (map >= 0 && (uint32_t)map < n_tex) ? map : -1;
    }
    st->pos.resize((size_t)n_tris * 9);
    st->nrm.resize((size_t)n_tris * 9);
    st->uv.resize((size_t)n_tris * 6);
    st->mat.resize(n_tris);
    for (uint32_t t = 0; t < n_tris; ++t) {
        for (int k = 0; k < 3; ++k) {
            r.floats(&st->pos[(size_t)t * 9 + 3 * k], 3);
            r.floats(&st->nrm[(size_t)t * 9 + 3 * k], 3);
            r.floats(&st->uv[(size_t)t * 6 + 2 * k], 2);
        }
        const int32_t id = r.get<int32_t>();
        if (!r.ok) return fail("truncated triangle table");
        if (id >= (int32_t)n_mats) return fail("material index out of range");
        // the reference passes a null material for id < 0 (src/s3d_mesh.cpp:445); a flat
        // scene needs one, so such triangles take material 0
        st->mat[t] = id >= 0 ? id : 0;
    }
    std::fclose(f);
    st->publish();
    *out = st;
    return SALTY_OK;
}

void salty_mesh_free(salty_mesh* mesh) {
    delete static_cast<MeshStore*>(mesh);
}

salty_status salty_mesh_transform(const float* matrix, int64_t n_tris, const float* pos_in, const float* nrm_in,
                                  float* pos_out, float* nrm_out) {
    if (!matrix || n_tris < 0 || (n_tris > 0 && (!pos_in || !pos_out))) return SALTY_ERR_INVALID_ARG;
    const float* M = matrix;  // row-major 3x4: x' = M[0..2] . x + M[3], ...
    // normals by the inverse transpose of the linear part (cofactor matrix; the scale of
    // the result does not matter, normals are renormalised)
    const double a = M[0], b = M[1], c = M[2], d = M[4], e = M[5], f = M[6], g = M[8], h = M[9], i = M[10];
    const double C[9] = {e * i - f * h, f * g - d * i, d * h - e * g,
                         c * h - b * i, a * i - c * g, b * g - a * h,
                         b * f - c * e, c * d - a * f, a * e - b * d};
    const double det = a * C[0] + b * C[1] + c * C[2];
    if (!(std::fabs(det) > 0.0)) return SALTY_ERR_INVALID_ARG;
    const double sgn = det < 0 ? -1.0 : 1.0;
    for (int64_t t = 0; t < n_tris; ++t) {
        for (int k = 0; k < 3; ++k) {
            const float* p = pos_in + t * 9 + 3 * k;
            float* q = pos_out + t * 9 + 3 * k;
            const float x = p[0], y = p[1], z = p[2];
            for (int r = 0; r < 3; ++r) q[r] = M[4 * r] * x + M[4 * r + 1] * y + M[4 * r + 2] * z + M[4 * r + 3];
            if (nrm_in && nrm_out) {
                const float* n = nrm_in + t * 9 + 3 * k;
                double v[3];
                for (int r = 0; r < 3; ++r) v[r] = sgn * (C[3 * r] * n[0] + C[3 * r + 1] * n[1] + C[3 * r + 2] * n[2]);
                const double len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                float* o = nrm_out + t * 9 + 3 * k;
                for (int r = 0; r < 3; ++r) o[r] = len > 0 ? (float)(v[r] / len) : 0.0f;
            }
        }
    }
    return SALTY_OK;
}

}  // extern "C"
