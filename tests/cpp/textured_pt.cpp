// Renders a textured, environment-lit scene with an SMD mesh placed twice, through the C++
// host API (include/salty/pt.hpp), and prints the pass count and image mean.
// Usage: textured_pt <mesh.smd> <out.png> [passes]
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "salty/pt.hpp"

using salty::Vector3;
using salty::Vertex;

int main(int argc, char** argv) {
    if (argc < 3) return 1;
    const int passes = argc > 3 ? std::atoi(argv[3]) : 4;
    salty::Scene scene;
    // a 64 x 64 checkerboard on a floor quad, texture coordinates from (x, z)
    std::vector<float> checker(64 * 64 * 3);
    for (int y = 0; y < 64; ++y)
        for (int x = 0; x < 64; ++x)
            for (int c = 0; c < 3; ++c) checker[3 * (y * 64 + x) + c] = ((x / 8 + y / 8) % 2) ? 0.8f : 0.2f;
    const int tex = scene.AddTexture(64, 64, checker);
    std::vector<float> sky(16 * 8 * 3, 0.1f);  // a dim environment map (x 10)
    scene.SetEnvironment(scene.AddTexture(16, 8, sky));
    std::vector<Vertex> floor;
    const Vector3 n{0, 1, 0};
    const Vector3 p[4] = {{-2, 0, -2}, {-2, 0, 2}, {2, 0, 2}, {2, 0, -2}};
    for (int i : {0, 1, 2, 0, 2, 3}) floor.push_back(Vertex{p[i], n, {(p[i].x + 2) / 4, (p[i].z + 2) / 4}});
    scene.AddMesh(floor, salty::Material::Lambert({0.9f, 0.9f, 0.9f}).SetColorMap(tex));
    // the SMD mesh twice: as it is, and moved and scaled (an Instance)
    const int64_t n0 = scene.AddSmd(argv[1]);
    const float m[12] = {0.5f, 0, 0, 1.0f, 0, 0.5f, 0, 0, 0, 0, 0.5f, 0.5f};
    const int64_t n1 = scene.AddSmd(argv[1], m);
    if (n0 <= 0 || n1 != n0) return 3;
    scene.SetSun({0.3f, 0.8f, 0.5f}, {2, 2, 2});
    salty::PinholeCamera cam;
    cam.Update({0, 1.5f, -4}, {0, 0.3f, 0}, {0, 1, 0}, 0.8f, 1.0f, 1.0f);
    scene.SetCamera(cam);
    salty::Config cfg;
    cfg.Width = 96;
    cfg.Height = 64;
    cfg.MaxBounceCount = 6;
    cfg.MaxRenderingSec = 1e9f;
    cfg.MaxPasses = passes;
    cfg.SamplesPerPass = 4;
    try {
        salty::PathTracer pt(0);
        pt.Run(cfg, scene, argv[2]);
        std::vector<float> img = pt.Image();
        double s[3] = {0, 0, 0};
        for (size_t i = 0; i < img.size(); ++i) s[i % 3] += img[i];
        const double np = (double)cfg.Width * cfg.Height;
        std::printf("passes %d mean %.6f %.6f %.6f\n", pt.Passes(), s[0] / np, s[1] / np, s[2] / np);
    } catch (const salty::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", (int)e.status, e.what());
        return 2;
    }
    return 0;
}
