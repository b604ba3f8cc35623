// sref_harness.cpp -- C entry points into the UNMODIFIED Salty reference,
// compiled from the reference's own sources (see oracle/Makefile).
//
// TEST INFRASTRUCTURE ONLY.  The tests, the smoke check and the CPU-baseline
// leg of the benchmark load the resulting oracle/_ref/libsalty_ref.so to pin
// the oracle restatement and the GPU path; no shipped code links it.
//
// What it drives, all through the reference's own public API:
//   * Triangle::Create + BVH8::Create + BVH8::IsHit      (src/s3d_triangle.cpp:22-105,
//     src/s3d_bvh8.cpp:191-206,401-479): closest-hit traversal over a triangle soup,
//     exactly what Mesh::Init/Mesh::IsHit do (src/s3d_mesh.cpp:470-504).
//   * PathTracer::Radiance / NextEventEstimation        (src/s3d_pt.cpp:182-292) with
//     a Scene subclass (include/s3d_scene.h:22-109), Mesh::Create(n, Vertex*, IMaterial*)
//     (src/s3d_mesh.cpp:539), Lambert/Mirror/Glass materials and PinholeCamera
//     (include/s3d_camera.h:63-100).  Radiance is private, so this file widens access
//     before including s3d_pt.h.  The reference has no area-light sampling for meshes
//     (IShape::Sample is a no-op, include/s3d_shape.h:67), so a QuadLight IShape is
//     supplied here through the reference's own plugin interface.
//   * ToneMapper::Map (src/s3d_tonemapper.cpp:206-353) and FilterNLM
//     (src/s3d_denoiser.cpp:19-95).
//   * PathTracer::Capture (src/s3d_pt.cpp:137-176): ACES + sRGB8 + PNG file.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

// private members of the reference's classes (Texture texels, PathTracer state, camera
// generator) are set directly by this harness
#define private public
#define protected public
#include <s3d_math.h>
#include <s3d_shape.h>
#include <s3d_material.h>
#include <s3d_triangle.h>
#include <s3d_sphere.h>
#include <s3d_bvh8.h>
#include <s3d_mesh.h>
#include <s3d_lambert.h>
#include <s3d_phong.h>
#include <s3d_plastic.h>
#include <s3d_mirror.h>
#include <s3d_glass.h>
#include <s3d_texture.h>
#include <s3d_tonemapper.h>
#include <s3d_denoiser.h>
#include <s3d_texturedmaterial.h>
#include <s3d_camera.h>
#include <s3d_scene.h>
#include <s3d_pt.h>
#undef private
#undef protected

using namespace s3d;

namespace {

double now_sec() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int resolve_threads(int n) {
    if (n > 0) return n;
    unsigned hw = std::thread::hardware_concurrency();
    return hw ? (int)hw : 1;
}

template <typename F>
void run_parallel(long count, int nthreads, long chunk, const F& fn) {
    std::atomic<long> next{0};
    auto worker = [&]() {
        for (;;) {
            long b = next.fetch_add(chunk);
            if (b >= count) break;
            long e = std::min(count, b + chunk);
            for (long i = b; i < e; ++i) fn(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

Vector3 v3(const float* p) { return Vector3(p[0], p[1], p[2]); }

struct Soup {
    std::vector<IShape*> tris;
    IShape* root = nullptr;
    IMaterial* mat = nullptr;
    std::unordered_map<const IShape*, int> index;
};

// Area light: a parallelogram made of two reference Triangles.  Hits report
// this object as the shape, so the reference's shadow test
// (light == shadowRecord.pShape, src/s3d_pt.cpp:274) recognises it.
class QuadLight : public IShape {
public:
    QuadLight(const Vector3& c, const Vector3& a, const Vector3& b, IMaterial* mat)
        : m_C(c), m_A(a), m_B(b), m_Mat(mat) {
        Vector3 n = Vector3::Cross(a, b);
        m_Area = n.Length();
        m_N = Vector3::UnitVector(n);
        Vertex v[6];
        Vector3 p0 = c, p1 = c + a, p2 = c + a + b, p3 = c + b;
        Vector3 ps[6] = {p0, p1, p2, p0, p2, p3};
        for (int i = 0; i < 6; ++i) { v[i].Position = ps[i]; v[i].Normal = m_N; v[i].TexCoord = Vector2(0, 0); }
        m_T[0] = Triangle::Create(&v[0], mat);
        m_T[1] = Triangle::Create(&v[3], mat);
        Vector3 mn = Vector3::Min(Vector3::Min(p0, p1), Vector3::Min(p2, p3));
        Vector3 mx = Vector3::Max(Vector3::Max(p0, p1), Vector3::Max(p2, p3));
        m_Box = BoundingBox(mn, mx);
    }
    ~QuadLight() override { SafeRelease(m_T[0]); SafeRelease(m_T[1]); }
    void AddRef() override { ++m_Count; }
    void Release() override { if (--m_Count == 0) delete this; }
    u32 GetCount() const override { return m_Count; }
    bool IsHit(const RaySet& rs, HitRecord& rec) const override {
        bool hit = m_T[0]->IsHit(rs, rec);
        hit |= m_T[1]->IsHit(rs, rec);
        if (hit) rec.pShape = this;
        return hit;
    }
    BoundingBox GetBox() const override { return m_Box; }
    Vector3 GetCenter() const override { return m_Box.center; }
    void CalcParam(const Vector3&, const Vector2&, Vector3* n, Vector2* uv) const override {
        *n = m_N; *uv = Vector2(0, 0);
    }
    void Sample(PCG& rnd, Vector3* pos, float* pdf) override {
        float u = rnd.GetAsF32();
        float w = rnd.GetAsF32();
        *pos = m_C + m_A * u + m_B * w;
        *pdf = 1.0f / m_Area;
    }
private:
    u32 m_Count = 1;
    Vector3 m_C, m_A, m_B, m_N;
    float m_Area = 0;
    IMaterial* m_Mat;
    IShape* m_T[2] = {nullptr, nullptr};
    BoundingBox m_Box;
};

}  // namespace

extern "C" {

struct sref_material {
    int type;            // 0 Lambert, 1 Mirror, 2 Glass, 4 Phong, 5 Plastic
    float color[3];      // Plastic: diffuse
    float emission[3];
    float ior;
    float specular[3];   // Plastic
    float power;         // Phong, Plastic
    int color_map;       // 1 + texture index (TexturedMaterial), 0 = none
};

struct sref_texture {
    int width, height;
    const float* rgb;    // texel (x, y) at rgb[3 * (y * width + x)]
};

struct sref_scene_desc {
    const float* tri_pos;    // n_tris * 9
    const float* tri_nrm;    // n_tris * 9 (shading normals)
    const int* tri_mat;      // n_tris
    long n_tris;
    const sref_material* mats;
    int n_mats;
    int has_light;
    float light_corner[3], light_edge_a[3], light_edge_b[3], light_emission[3];
    float cam_pos[3], cam_target[3], cam_up[3];
    float cam_fov, cam_near;
    float sky_over_10;       // constant sky radiance / 10 (Scene::SampleIBL scales by 10)
    const char* tmp_dir;     // where the 2x2 sky .hdr file is written
    float cam_lens;          // > 0: ThinLensCamera with this lens radius
    const float* tri_uv;     // n_tris * 6, or NULL
    const sref_texture* textures;
    int n_textures;
    int ibl_map;             // 1 + texture index of the environment (replaces the constant sky), 0 = none
    const float* spheres;    // n_spheres * 6: centre xyz, radius, material, light (0/1)
    int n_spheres;
};

// ---------------------------------------------------------------- traversal
void* sref_soup_create(const float* pos9, long n, double* build_seconds) {
    auto* s = new Soup();
    s->mat = Lambert::Create(Color3(0.5f, 0.5f, 0.5f));
    s->tris.resize(n);
    for (long i = 0; i < n; ++i) {
        Vertex v[3];
        for (int k = 0; k < 3; ++k) {
            v[k].Position = v3(pos9 + i * 9 + k * 3);
            v[k].Normal = Vector3(0, 1, 0);
            v[k].TexCoord = Vector2(0, 0);
        }
        s->tris[i] = Triangle::Create(v, s->mat);
        s->index[s->tris[i]] = (int)i;
    }
    std::vector<IShape*> work(s->tris);
    double t0 = now_sec();
    s->root = BVH8::Create(work.size(), work.data());
    if (build_seconds) *build_seconds = now_sec() - t0;
    return s;
}

void sref_soup_destroy(void* h) {
    auto* s = (Soup*)h;
    if (!s) return;
    SafeRelease(s->root);
    for (auto* t : s->tris) SafeRelease(t);
    SafeRelease(s->mat);
    delete s;
}

// rays: n x 8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax).  The reference has
// fixed limits (F_HIT_MIN = 1e-3, F_HIT_MAX = 1e12, include/s3d_math.h:44-45),
// so tmin/tmax are ignored.  Outputs: triangle index or -1, t, barycentrics.
double sref_soup_trace(void* h, const float* rays, long n, int nthreads,
                       int32_t* ids, float* t, float* bu, float* bv) {
    auto* s = (Soup*)h;
    nthreads = resolve_threads(nthreads);
    double t0 = now_sec();
    run_parallel(n, nthreads, 256, [&](long i) {
        const float* r = rays + i * 8;
        RaySet rs = MakeRaySet(Vector3(r[0], r[1], r[2]), Vector3(r[4], r[5], r[6]));
        HitRecord rec;
        bool hit = s->root->IsHit(rs, rec);
        if (hit) {
            ids[i] = s->index.at(rec.pShape);
            t[i] = rec.distance;
            if (bu) bu[i] = rec.barycentric.x;
            if (bv) bv[i] = rec.barycentric.y;
        } else {
            ids[i] = -1;
            t[i] = rec.distance;
            if (bu) bu[i] = 0;
            if (bv) bv[i] = 0;
        }
    });
    return now_sec() - t0;
}

// ---------------------------------------------------------------- rendering
struct SrefScene;
}  // extern "C"

namespace {
class HarnessScene : public Scene {
public:
    std::vector<Texture> textures;
    PinholeCamera camera;
    ThinLensCamera lens;
    float lens_radius = 0.0f;
    std::vector<IMaterial*> mats;
};
}  // namespace

struct SrefScene {
    HarnessScene scene;
};

extern "C" {

// A Texture (src/s3d_texture.cpp) holding the given float texels, as its loaders leave it.
static void fill_texture(Texture& t, const sref_texture& x) {
    t.Term();
    t.m_Width = x.width;
    t.m_Height = x.height;
    t.m_Size = (u32)(x.width * x.height);
    t.m_pColors = new Color3[t.m_Size];
    for (u32 i = 0; i < t.m_Size; ++i) t.m_pColors[i] = Color3(x.rgb[3 * i], x.rgb[3 * i + 1], x.rgb[3 * i + 2]);
}

void* sref_scene_create(const sref_scene_desc* d, int width, int height) {
    auto* h = new SrefScene();
    HarnessScene& sc = h->scene;
    sc.textures.resize(d->n_textures > 0 ? d->n_textures : 0);
    for (int t = 0; t < d->n_textures; ++t) fill_texture(sc.textures[t], d->textures[t]);
    for (int m = 0; m < d->n_mats; ++m) {
        const sref_material& sm = d->mats[m];
        Color3 c(sm.color[0], sm.color[1], sm.color[2]);
        Color3 e(sm.emission[0], sm.emission[1], sm.emission[2]);
        IMaterial* mat = nullptr;
        if (sm.type == 1) mat = Mirror::Create(c, e);
        else if (sm.type == 2) mat = Glass::Create(c, sm.ior, e);
        else if (sm.type == 4) mat = Phong::Create(c, sm.power, e);
        else if (sm.type == 5)
            mat = Plastic::Create(c, Color3(sm.specular[0], sm.specular[1], sm.specular[2]), sm.power, e);
        else mat = Lambert::Create(c, e);
        if (sm.color_map > 0 && sm.color_map <= (int)sc.textures.size()) {
            IMaterial* tm = TexturedMaterial::Create(&sc.textures[sm.color_map - 1], mat);
            SafeRelease(mat);
            mat = tm;
        }
        sc.mats.push_back(mat);
    }
    // one Mesh per material, vertices in input order
    for (int m = 0; m < d->n_mats; ++m) {
        std::vector<Vertex> verts;
        for (long i = 0; i < d->n_tris; ++i) {
            if (d->tri_mat[i] != m) continue;
            for (int k = 0; k < 3; ++k) {
                Vertex v;
                v.Position = v3(d->tri_pos + i * 9 + k * 3);
                v.Normal = v3(d->tri_nrm + i * 9 + k * 3);
                v.TexCoord = d->tri_uv ? Vector2(d->tri_uv[i * 6 + 2 * k], d->tri_uv[i * 6 + 2 * k + 1]) : Vector2(0, 0);
                verts.push_back(v);
            }
        }
        if (verts.empty()) continue;
        IShape* mesh = Mesh::Create((u32)verts.size(), verts.data(), sc.mats[m]);
        sc.m_Shapes.push_back(mesh);
    }
    if (d->has_light) {
        Color3 e(d->light_emission[0], d->light_emission[1], d->light_emission[2]);
        IMaterial* lm = Lambert::Create(Color3(0, 0, 0), e);
        sc.mats.push_back(lm);
        auto* q = new QuadLight(v3(d->light_corner), v3(d->light_edge_a), v3(d->light_edge_b), lm);
        sc.m_Shapes.push_back(q);
        sc.m_pLightList.push_back(q);
    }
    // the reference's own Sphere shape (src/s3d_sphere.cpp); light spheres join the light
    // list after the quad light, in input order
    for (int k = 0; k < d->n_spheres; ++k) {
        const float* p = d->spheres + 6 * k;
        IShape* sp = Sphere::Create(p[3], Vector3(p[0], p[1], p[2]), sc.mats[(int)p[4]]);
        sc.m_Shapes.push_back(sp);
        if (p[5] != 0.0f) sc.m_pLightList.push_back(sp);
    }
    sc.camera.Update(v3(d->cam_pos), v3(d->cam_target), v3(d->cam_up), d->cam_fov,
                     float(width) / float(height), d->cam_near);
    sc.m_pCamera = &sc.camera;
    sc.lens_radius = d->cam_lens;
    if (d->cam_lens > 0.0f)
        sc.lens.Update(v3(d->cam_pos), v3(d->cam_target), v3(d->cam_up), d->cam_fov, float(width) / float(height),
                       d->cam_near, d->cam_lens);

    if (d->ibl_map > 0 && d->ibl_map <= d->n_textures) {
        // an environment texture as the IBL (Scene::SampleIBL scales it by 10)
        fill_texture(sc.m_IBL, d->textures[d->ibl_map - 1]);
        return h;
    }
    // Constant sky through the reference's own HDR loader: a 2x2 flat RGBE file.
    std::string path = std::string(d->tmp_dir ? d->tmp_dir : "/tmp") + "/sref_sky_" +
                       std::to_string((long)(uintptr_t)h) + ".hdr";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (f) {
        std::fputs("#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2 +X 2\n", f);
        unsigned char px[4] = {0, 0, 0, 0};
        float v = d->sky_over_10;
        if (v > 1e-32f) {
            int ex;
            float m = std::frexp(v, &ex) * 256.0f / v;
            unsigned char c = (unsigned char)(v * m);
            px[0] = px[1] = px[2] = c;
            px[3] = (unsigned char)(ex + 128);
        }
        for (int i = 0; i < 4; ++i) std::fwrite(px, 1, 4, f);
        std::fclose(f);
        sc.m_IBL.Init(path.c_str(), TFF_HDR);
        std::remove(path.c_str());
    }
    return h;
}

void sref_scene_destroy(void* p) {
    auto* h = (SrefScene*)p;
    if (!h) return;
    for (auto* s : h->scene.m_Shapes) SafeRelease(s);
    h->scene.m_Shapes.clear();
    h->scene.m_pLightList.clear();
    for (auto* m : h->scene.mats) SafeRelease(m);
    delete h;
}

// Renders spp samples per pixel with PathTracer::Radiance, pixel-centre rays as
// in PathTracer::TracePath (src/s3d_pt.cpp:318-331).  Each image row restarts
// the PCG at SetSeed(seed * 1000003 + row), so results do not depend on the
// thread count.  Outputs per-pixel sums of L and of L^2 (double).
double sref_render(void* p, int width, int height, int spp, int max_bounce, uint64_t seed,
                   int nthreads, double* sum, double* sumsq) {
    auto* h = (SrefScene*)p;
    nthreads = resolve_threads(nthreads);
    double t0 = now_sec();
    run_parallel(height, nthreads, 1, [&](long y) {
        PathTracer pt;
        pt.m_pScene = &h->scene;
        pt.m_Config.Width = width;
        pt.m_Config.Height = height;
        pt.m_Config.MaxBounceCount = max_bounce;
        pt.m_Config.MaxRenderingSec = 1e9f;
        pt.m_Config.CpuCoreCount = 1;
        pt.m_Updatable = true;
        pt.m_Random.SetSeed(seed * 1000003ull + (uint64_t)y);
        // a thin lens samples its aperture with its own generator on every GetRay
        // (include/s3d_camera.h:206-222): one camera copy per row, seeded per row
        ThinLensCamera lens = h->scene.lens;
        lens.m_Random.SetSeed((unsigned)(seed * 7919ull + (uint64_t)y + 1));
        for (int x = 0; x < width; ++x) {
            const float fx = (0.5f + x) / width - 0.5f, fy = (0.5f + y) / height - 0.5f;
            Ray ray = h->scene.GetRay(fx, fy);
            double s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
            for (int k = 0; k < spp; ++k) {
                if (h->scene.lens_radius > 0.0f) ray = lens.GetRay(fx, fy);
                Color3 L = pt.Radiance(ray);
                s[0] += L.x; s[1] += L.y; s[2] += L.z;
                q[0] += (double)L.x * L.x; q[1] += (double)L.y * L.y; q[2] += (double)L.z * L.z;
            }
            long idx = (long)y * width + x;
            for (int c = 0; c < 3; ++c) { sum[idx * 3 + c] = s[c]; if (sumsq) sumsq[idx * 3 + c] = q[c]; }
        }
        pt.m_pScene = nullptr;
    });
    return now_sec() - t0;
}

// ---------------------------------------------------------------- post
void sref_tonemap(int type, int width, int height, const float* rgb, float* out) {
    std::vector<Color3> in((size_t)width * height), res((size_t)width * height);
    for (size_t i = 0; i < in.size(); ++i) in[i] = Color3(rgb[i * 3], rgb[i * 3 + 1], rgb[i * 3 + 2]);
    ToneMapper::Map((TONE_MAPPING_TYPE)type, width, height, in.data(), res.data());
    for (size_t i = 0; i < res.size(); ++i) { out[i * 3] = res[i].x; out[i * 3 + 1] = res[i].y; out[i * 3 + 2] = res[i].z; }
}

void sref_nlm(int width, int height, float coeff, const float* rgba, float* out) {
    std::vector<Color4> in((size_t)width * height), res((size_t)width * height);
    for (size_t i = 0; i < in.size(); ++i) in[i] = Color4(rgba[i * 4], rgba[i * 4 + 1], rgba[i * 4 + 2], rgba[i * 4 + 3]);
    FilterNLM(width, height, coeff, in.data(), res.data());
    for (size_t i = 0; i < res.size(); ++i) {
        out[i * 4] = res[i].x; out[i * 4 + 1] = res[i].y; out[i * 4 + 2] = res[i].z; out[i * 4 + 3] = res[i].w;
    }
}

// PathTracer::Capture on an accumulated image: ACES tonemap, clamp, the
// reference's sRGB OETF and 8-bit rounding, written as PNG by stb.
void sref_capture_png(int width, int height, const float* rgb, const char* path) {
    PathTracer pt;
    pt.m_Config.Width = width;
    pt.m_Config.Height = height;
    pt.m_RenderTarget = new Color3[(size_t)width * height];
    pt.m_Intermediate = new Color3[(size_t)width * height];
    for (size_t i = 0; i < (size_t)width * height; ++i)
        pt.m_RenderTarget[i] = Color3(rgb[i * 3], rgb[i * 3 + 1], rgb[i * 3 + 2]);
    pt.Capture(path);
}

}  // extern "C"
