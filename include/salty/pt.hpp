// salty/pt.hpp -- C++ host API over libsalty_gpu, shaped like the reference's own.
//
// A Salty host builds a Scene from meshes, materials, a light and a pinhole camera and
// calls PathTracer::Run(Config); this header keeps those names and their meaning so such a
// host switches to the GPU by swapping headers.  Reference counterparts (paths relative to
// the reference project's src/):
//   Config                   PathTracer::Config            include/s3d_pt.h:33-40
//   PathTracer::Run          PathTracer::Run / TracePath   src/s3d_pt.cpp:77-132, 297-353
//   PathTracer::Capture      PathTracer::Capture           src/s3d_pt.cpp:137-176
//   Material::Lambert/...    Lambert/Mirror/Glass::Create  src/s3d_materialfactory.cpp:28-132
//   Scene::AddMesh           Mesh::Create(n, Vertex*, IMaterial*)  src/s3d_mesh.cpp:539
//   PinholeCamera            PinholeCamera::Update         include/s3d_camera.h:63-90
//   Vertex                   Vertex                        include/s3d_shape.h:27-32
// Differences: Run takes the Scene instead of hard-coding TestScene (src/s3d_pt.cpp:113);
// errors are C++ exceptions carrying the library's status and message instead of bool /
// nullptr; the area light is a parallelogram (the reference can only sample spheres).
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../salty_gpu.h"

namespace salty {

struct Vector3 {
    float x = 0, y = 0, z = 0;
};
using Color3 = Vector3;
struct Vector2 {
    float x = 0, y = 0;
};

struct Vertex {
    Vector3 Position;
    Vector3 Normal;
    Vector2 TexCoord;
};

class Error : public std::runtime_error {
public:
    Error(salty_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    salty_status status;
};

inline void check(salty_status s, salty_ctx* ctx, const char* what) {
    if (s != SALTY_OK)
        throw Error(s, std::string(what) + ": " + (ctx ? salty_last_error(ctx) : "no context"));
}

struct Config {
    int Width = 960;
    int Height = 540;
    int MaxBounceCount = 32;
    float MaxRenderingSec = 59.8f;
    int CpuCoreCount = 1;            // accepted for source compatibility; unused on the GPU
    // GPU additions
    int SamplesPerPass = 4;          // samples per pixel per progressive pass
    int RussianRouletteDepth = 3;    // physical estimator only
    int Profile = SALTY_PROFILE_PHYSICAL;
    int ToneMapping = SALTY_TM_ACES; // the reference captures with ACES (src/s3d_pt.cpp:43)
    uint64_t Seed = 3141592;         // the reference seeds its PCG with 3141592 (src/s3d_pt.cpp:304)
    int MaxPasses = 0;               // > 0: stop after this many passes even before the time budget
    // Time-budgeted runs (MaxPasses == 0): each pass doubles the samples of the last while two
    // such passes still fit the remaining budget.  Large passes fill the wavefront's queues,
    // so more samples fit the budget; the image is the same as with fixed passes of the same
    // total (sample k of a pixel is the same in any pass split).
    bool GrowPasses = true;
};

struct Material {
    salty_material m{};
    static Material Lambert(Color3 diffuse, Color3 emissive = {}) { return make(SALTY_LAMBERT, diffuse, emissive, 1.5f, 0.f); }
    static Material Mirror(Color3 specular, Color3 emissive = {}) { return make(SALTY_MIRROR, specular, emissive, 1.5f, 0.f); }
    static Material Glass(Color3 specular, float ior, Color3 emissive = {}) {
        return make(SALTY_GLASS, specular, emissive, ior, 0.f);
    }
    static Material GGX(Color3 specular, float roughness) { return make(SALTY_GGX, specular, {}, 1.5f, roughness); }
    // MaterialFactory::CreatePhong / CreatePlastic (src/s3d_materialfactory.cpp:28-132)
    static Material Phong(Color3 specular, float power, Color3 emissive = {}) {
        Material r = make(SALTY_PHONG, specular, emissive, 1.5f, 0.f);
        r.m.power = power;
        return r;
    }
    // TexturedMaterial (src/s3d_texturedmaterial.cpp): a texture of Scene::AddTexture scales
    // the base colour
    Material& SetColorMap(int texture) {
        m.color_map = texture + 1;
        return *this;
    }
    static Material Plastic(Color3 diffuse, Color3 specular, float power, Color3 emissive = {}) {
        Material r = make(SALTY_PLASTIC, diffuse, emissive, 1.5f, 0.f);
        r.m.specular[0] = specular.x; r.m.specular[1] = specular.y; r.m.specular[2] = specular.z;
        r.m.power = power;
        return r;
    }

private:
    static Material make(int type, Color3 c, Color3 e, float ior, float rough) {
        Material r;
        r.m.type = type;
        r.m.color[0] = c.x; r.m.color[1] = c.y; r.m.color[2] = c.z;
        r.m.emission[0] = e.x; r.m.emission[1] = e.y; r.m.emission[2] = e.z;
        r.m.ior = ior;
        r.m.roughness = rough;
        return r;
    }
};

struct PinholeCamera {
    Vector3 Position, Target, Upward{0, 1, 0};
    float Fov = 1.0f;        // the reference's linear screen extent (2 tan(half angle))
    float NearClip = 1.0f;
    float LensRadius = 0.0f;     // > 0: a thin lens (ThinLensCamera)
    float FocalDistance = 0.0f;  // 0: |Target - Position|
    void Update(Vector3 position, Vector3 target, Vector3 upward, float fov, float /*aspect: from Config*/,
                float nearClip) {
        Position = position; Target = target; Upward = upward; Fov = fov; NearClip = nearClip;
    }
};

// ThinLensCamera::Update (include/s3d_camera.h:167-196): a pinhole plus a lens radius,
// focused at the target distance.
struct ThinLensCamera : PinholeCamera {
    void Update(Vector3 position, Vector3 target, Vector3 upward, float fov, float aspect, float nearClip,
                float lensRadius) {
        PinholeCamera::Update(position, target, upward, fov, aspect, nearClip);
        LensRadius = lensRadius;
        FocalDistance = 0.0f;
    }
};

class Scene {
public:
    // Mesh::Create(vertexCount, pVertices, pMaterial): three vertices per triangle.
    void AddMesh(const std::vector<Vertex>& vertices, const Material& material) {
        if (vertices.size() % 3 != 0) throw Error(SALTY_ERR_INVALID_ARG, "AddMesh: vertex count is not a multiple of 3");
        const int id = (int)mats_.size();
        mats_.push_back(material.m);
        for (const Vertex& v : vertices) {
            pos_.insert(pos_.end(), {v.Position.x, v.Position.y, v.Position.z});
            nrm_.insert(nrm_.end(), {v.Normal.x, v.Normal.y, v.Normal.z});
            uv_.insert(uv_.end(), {v.TexCoord.x, v.TexCoord.y});
        }
        for (size_t i = 0; i < vertices.size() / 3; ++i) mat_.push_back(id);
    }
    // Mesh::Create(filename) (src/s3d_mesh.cpp:250-465), optionally placed as an Instance by
    // a row-major 3x4 matrix (normals by its inverse transpose); returns the triangle count.
    int64_t AddSmd(const char* path, const float* matrix3x4 = nullptr) {
        salty_mesh* m = nullptr;
        const salty_status st = salty_mesh_load_smd(nullptr, path, &m);
        if (st != SALTY_OK) throw Error(st, std::string("cannot load ") + path);
        const size_t n = (size_t)m->n_tris, p0 = pos_.size();
        pos_.resize(p0 + n * 9);
        nrm_.resize(p0 + n * 9);
        if (matrix3x4) {
            salty_mesh_transform(matrix3x4, m->n_tris, m->tri_pos, m->tri_nrm, pos_.data() + p0, nrm_.data() + p0);
        } else {
            std::copy(m->tri_pos, m->tri_pos + n * 9, pos_.begin() + p0);
            std::copy(m->tri_nrm, m->tri_nrm + n * 9, nrm_.begin() + p0);
        }
        uv_.insert(uv_.end(), m->tri_uv, m->tri_uv + n * 6);
        const int base = (int)mats_.size();
        mats_.insert(mats_.end(), m->mats, m->mats + m->n_mats);
        for (size_t t = 0; t < n; ++t) mat_.push_back(base + m->tri_mat[t]);
        salty_mesh_free(m);
        return (int64_t)n;
    }
    // Texture (src/s3d_texture.cpp): float RGB, texel (x, y) at rgb[3 * (y * width + x)];
    // returns its index for Material::SetColorMap and SetEnvironment.
    int AddTexture(int width, int height, std::vector<float> rgb) {
        if (width <= 0 || height <= 0 || rgb.size() != (size_t)width * height * 3)
            throw Error(SALTY_ERR_INVALID_ARG, "AddTexture: size does not match the texels");
        tex_data_.push_back(std::move(rgb));
        tex_.push_back(salty_texture{width, height, nullptr});
        return (int)tex_.size() - 1;
    }
    // Scene::SampleIBL with a latitude-longitude texture (radiance = texel * scale)
    void SetEnvironment(int texture, float scale = 10.0f) { ibl_ = texture + 1; ibl_scale_ = scale; }
    void SetQuadLight(Vector3 corner, Vector3 edgeA, Vector3 edgeB, Color3 emission) {
        has_light_ = true;
        light_ = {corner, edgeA, edgeB, emission};
    }
    void SetSun(Vector3 dirTowardsSun, Color3 irradiance) {
        has_sun_ = true;
        sun_ = {dirTowardsSun, irradiance};
    }
    void SetSky(Color3 radiance) { sky_ = radiance; }
    void SetCamera(const PinholeCamera& c) { camera_ = c; }

    salty_scene_desc Describe() const {
        salty_scene_desc d{};
        d.tri_pos = pos_.data();
        d.tri_nrm = nrm_.data();
        d.tri_mat = mat_.data();
        d.n_tris = (int64_t)mat_.size();
        d.mats = mats_.data();
        d.n_mats = (int32_t)mats_.size();
        d.has_light = has_light_;
        put(d.light_corner, light_.corner); put(d.light_edge_a, light_.a); put(d.light_edge_b, light_.b);
        put(d.light_emission, light_.e);
        d.has_sun = has_sun_;
        put(d.sun_dir, sun_.dir); put(d.sun_radiance, sun_.e);
        put(d.sky, sky_);
        put(d.camera.pos, camera_.Position); put(d.camera.target, camera_.Target); put(d.camera.up, camera_.Upward);
        d.camera.fov = camera_.Fov;
        d.camera.near_clip = camera_.NearClip;
        d.camera.lens_radius = camera_.LensRadius;
        d.camera.focal_distance = camera_.FocalDistance;
        d.tri_uv = uv_.data();
        for (size_t t = 0; t < tex_.size(); ++t) tex_[t].rgb = tex_data_[t].data();
        d.textures = tex_.data();
        d.n_textures = (int32_t)tex_.size();
        d.ibl_map = ibl_;
        d.ibl_scale = ibl_scale_;
        return d;
    }

private:
    static void put(float* d, Vector3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }
    struct Light { Vector3 corner, a, b; Color3 e; } light_{};
    struct Sun { Vector3 dir; Color3 e; } sun_{};
    std::vector<float> pos_, nrm_, uv_;
    std::vector<int32_t> mat_;
    std::vector<salty_material> mats_;
    std::vector<std::vector<float>> tex_data_;
    mutable std::vector<salty_texture> tex_;
    int32_t ibl_ = 0;
    float ibl_scale_ = 10.0f;
    bool has_light_ = false, has_sun_ = false;
    Color3 sky_{};
    PinholeCamera camera_{};
};

class PathTracer {
public:
    explicit PathTracer(int device = 0) { check(salty_ctx_create(&ctx_, device), nullptr, "salty_ctx_create"); }
    ~PathTracer() {
        if (scene_) salty_scene_destroy(ctx_, scene_);
        salty_ctx_destroy(ctx_);
    }
    PathTracer(const PathTracer&) = delete;
    PathTracer& operator=(const PathTracer&) = delete;

    // TracePath: progressive passes of SamplesPerPass samples until MaxRenderingSec (or
    // MaxPasses), then Capture("final.png") unless capturePath is empty.
    bool Run(const Config& config, const Scene& scene, const char* capturePath = "final.png") {
        config_ = config;
        if (scene_) salty_scene_destroy(ctx_, scene_);
        scene_ = nullptr;
        const salty_scene_desc d = scene.Describe();
        check(salty_scene_upload(ctx_, &d, &scene_), ctx_, "salty_scene_upload");
        check(salty_bvh_build(ctx_, scene_, nullptr, nullptr), ctx_, "salty_bvh_build");
        const auto t0 = std::chrono::steady_clock::now();
        passes_ = 0;
        samples_ = 0;
        int spp = config_.SamplesPerPass;
        for (;;) {
            salty_render_opts o = opts(passes_ > 0);
            o.spp = spp;
            salty_render_stats st{};
            check(salty_render(ctx_, scene_, &o, nullptr, nullptr, nullptr, &st), ctx_, "salty_render");
            ++passes_;
            samples_ += spp;
            const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (secs >= config_.MaxRenderingSec || (config_.MaxPasses > 0 && passes_ >= config_.MaxPasses)) break;
            if (config_.GrowPasses && config_.MaxPasses <= 0) {
                const double per_spp = secs / samples_, left = config_.MaxRenderingSec - secs;
                if (2.0 * spp * per_spp * 2.0 <= left && spp < (1 << 20)) spp *= 2;
            }
        }
        if (capturePath && *capturePath) Capture(capturePath);
        return true;
    }

    int Passes() const { return passes_; }
    // Samples per pixel rendered by the last Run.
    long long SamplesPerPixel() const { return samples_; }

    // Per-pixel mean radiance of the film (W*H*3).
    std::vector<float> Image() {
        std::vector<float> img((size_t)config_.Width * config_.Height * 3);
        salty_render_opts o = opts(true);
        o.spp = 0;
        check(salty_render(ctx_, scene_, &o, img.data(), nullptr, nullptr, nullptr), ctx_, "salty_render(read)");
        return img;
    }

    // Capture: tonemap + the reference's sRGB8 conversion, then a PNG file.
    std::vector<uint8_t> Capture(const char* filename) {
        std::vector<uint8_t> rgb((size_t)config_.Width * config_.Height * 3);
        salty_render_opts o = opts(true);
        o.spp = 0;
        check(salty_render(ctx_, scene_, &o, nullptr, nullptr, rgb.data(), nullptr), ctx_, "salty_render(capture)");
        if (filename && *filename) write_png(filename, config_.Width, config_.Height, rgb);
        return rgb;
    }

    salty_ctx* Context() { return ctx_; }

    // Minimal PNG writer (stored deflate blocks): 8-bit RGB.
    static void write_png(const char* path, int w, int h, const std::vector<uint8_t>& rgb) {
        std::vector<uint8_t> raw;
        raw.reserve((size_t)h * (w * 3 + 1));
        for (int y = 0; y < h; ++y) {
            raw.push_back(0);
            raw.insert(raw.end(), rgb.begin() + (size_t)y * w * 3, rgb.begin() + (size_t)(y + 1) * w * 3);
        }
        std::vector<uint8_t> z = {0x78, 0x01};
        uint32_t a = 1, b = 0;
        for (uint8_t c : raw) { a = (a + c) % 65521; b = (b + a) % 65521; }
        for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
            const size_t n = std::min<size_t>(65535, raw.size() - off);
            const bool last = off + n >= raw.size();
            z.push_back(last ? 1 : 0);
            z.push_back(n & 0xff); z.push_back(n >> 8);
            z.push_back(~n & 0xff); z.push_back((~n >> 8) & 0xff);
            z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
            if (last) break;
        }
        const uint32_t adler = (b << 16) | a;
        for (int s = 24; s >= 0; s -= 8) z.push_back((adler >> s) & 0xff);
        FILE* f = std::fopen(path, "wb");
        if (!f) throw Error(SALTY_ERR_INVALID_ARG, std::string("cannot open ") + path);
        const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
        std::fwrite(sig, 1, 8, f);
        uint8_t ihdr[13] = {0};
        be32(ihdr, (uint32_t)w); be32(ihdr + 4, (uint32_t)h);
        ihdr[8] = 8; ihdr[9] = 2;
        chunk(f, "IHDR", ihdr, 13);
        chunk(f, "IDAT", z.data(), z.size());
        chunk(f, "IEND", nullptr, 0);
        std::fclose(f);
    }

private:
    salty_render_opts opts(bool accumulate) const {
        salty_render_opts o{};
        o.width = config_.Width;
        o.height = config_.Height;
        o.spp = config_.SamplesPerPass;
        o.max_depth = config_.MaxBounceCount;
        o.rr_depth = config_.RussianRouletteDepth;
        o.profile = config_.Profile;
        o.seed = config_.Seed;
        o.accumulate = accumulate ? 1 : 0;
        o.tonemap = config_.ToneMapping;
        o.ref_oetf = 1;
        return o;
    }
    static void be32(uint8_t* p, uint32_t v) { p[0] = v >> 24; p[1] = v >> 16; p[2] = v >> 8; p[3] = v; }
    static uint32_t crc32(const uint8_t* d, size_t n, uint32_t c) {
        for (size_t i = 0; i < n; ++i) {
            c ^= d[i];
            for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
        }
        return c;
    }
    static void chunk(FILE* f, const char* type, const uint8_t* data, size_t n) {
        uint8_t len[4];
        be32(len, (uint32_t)n);
        std::fwrite(len, 1, 4, f);
        std::fwrite(type, 1, 4, f);
        if (n) std::fwrite(data, 1, n, f);
        uint32_t c = crc32((const uint8_t*)type, 4, 0xffffffffu);
        c = crc32(data, n, c) ^ 0xffffffffu;
        uint8_t cb[4];
        be32(cb, c);
        std::fwrite(cb, 1, 4, f);
    }

    salty_ctx* ctx_ = nullptr;
    salty_scene* scene_ = nullptr;
    Config config_{};
    int passes_ = 0;
    long long samples_ = 0;
};

}  // namespace salty
