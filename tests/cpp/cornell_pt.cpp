// Renders the Cornell box through the C++ host API (include/salty/pt.hpp) the way a
// Salty host drives PathTracer::Run, and prints the pass count and image mean.
// Usage: cornell_pt <out.png> [passes] [budget seconds]
// passes 0: a time-budgeted run (MaxRenderingSec = budget, passes growing).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "salty/pt.hpp"

using salty::Vector3;
using salty::Vertex;

static void quad(std::vector<Vertex>& v, Vector3 p0, Vector3 p1, Vector3 p2, Vector3 p3) {
    Vector3 e1{p1.x - p0.x, p1.y - p0.y, p1.z - p0.z}, e2{p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
    Vector3 n{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    float m = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
    n = {n.x / m, n.y / m, n.z / m};
    for (Vector3 p : {p0, p1, p2, p0, p2, p3}) v.push_back(Vertex{p, n, {}});
}

int main(int argc, char** argv) {
    const char* out = argc > 1 ? argv[1] : "final.png";
    int passes = argc > 2 ? std::atoi(argv[2]) : 8;
    const float budget = argc > 3 ? (float)std::atof(argv[3]) : 1.0f;
    salty::Scene scene;
    std::vector<Vertex> white, red, green;
    quad(white, {0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 0, 0});
    quad(white, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1});
    quad(white, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1});
    quad(red, {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0});
    quad(green, {0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1});
    scene.AddMesh(white, salty::Material::Lambert({0.75f, 0.75f, 0.75f}));
    scene.AddMesh(red, salty::Material::Lambert({0.75f, 0.25f, 0.25f}));
    scene.AddMesh(green, salty::Material::Lambert({0.25f, 0.75f, 0.25f}));
    scene.SetQuadLight({0.375f, 0.999f, 0.375f}, {0.25f, 0, 0}, {0, 0, 0.25f}, {17, 12, 4});
    salty::PinholeCamera cam;
    cam.Update({0.5f, 0.5f, -1.4f}, {0.5f, 0.5f, 0.0f}, {0, 1, 0}, 2.0f * std::tan(20.0f * 3.14159265f / 180.0f), 1.0f,
               1.0f);
    scene.SetCamera(cam);
    salty::Config cfg;
    cfg.Width = 128;
    cfg.Height = 128;
    cfg.MaxBounceCount = 8;
    cfg.MaxRenderingSec = passes > 0 ? 1e9f : budget;
    cfg.MaxPasses = passes;
    cfg.SamplesPerPass = 4;
    try {
        salty::PathTracer pt(0);
        pt.Run(cfg, scene, out);
        std::vector<float> img = pt.Image();
        double s[3] = {0, 0, 0};
        for (size_t i = 0; i < img.size(); ++i) s[i % 3] += img[i];
        const double n = (double)cfg.Width * cfg.Height;
        std::printf("passes %d spp %lld mean %.6f %.6f %.6f\n", pt.Passes(), pt.SamplesPerPixel(), s[0] / n, s[1] / n,
                    s[2] / n);
    } catch (const salty::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", (int)e.status, e.what());
        return 2;
    }
    return 0;
}
