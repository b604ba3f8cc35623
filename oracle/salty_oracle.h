/* salty_oracle.h -- CPU restatement of Salty's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py use it, always as the checker.  The shipped
 * library (libsalty_gpu.so) never links, loads or calls it.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the reference project's src/ directory).  The restatement is pinned against
 * the unmodified reference compiled from its own sources (oracle/Makefile,
 * oracle/_ref/libsalty_ref.so) by tests/test_oracle_pins.py and the committed
 * fixtures in tests/golden/.
 */
#ifndef SALTY_ORACLE_H
#define SALTY_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- PCG-XSH-RR 64/32 (include/s3d_math.h:2769-2817) ---- */
typedef struct { uint64_t state; } opcg;
void     opcg_seed(opcg* r, uint64_t seed);
uint32_t opcg_u32(opcg* r);
float    opcg_f32(opcg* r);

/* ---- traversal microbenchmark inputs ---- */
void oracle_gen_soup(uint64_t seed, long n, float* pos9);
void oracle_gen_rays(uint64_t seed, long n, float tmin, float* rays8);

/* ---- ray/triangle tests ---- */
/* Reference test, same operation order (src/s3d_triangle.cpp:73-105).  Returns 1 on
 * hit with t in [tmin, tmax]; t/u/v written. */
int oracle_tri_ref(const float o[3], const float d[3], const float v0[3], const float v1[3],
                   const float v2[3], float tmin, float tmax, float* t, float* u, float* v);
/* Watertight test (Woop, Benthin, Wald, JCGT 2013). */
int oracle_tri_watertight(const float o[3], const float d[3], const float v0[3], const float v1[3],
                          const float v2[3], float tmin, float tmax, float* t, float* u, float* v);

/* ---- closest / any hit over a triangle soup ----
 * Closest hit = smallest computed t among triangles the chosen test accepts; equal t
 * goes to the lowest triangle index.  The acceleration structure never culls by t, so
 * the answer does not depend on it.  mode: 0 reference test, 1 watertight. */
void* oracle_bvh_create(const float* pos9, long n);
void  oracle_bvh_destroy(void* bvh);
void  oracle_trace(void* bvh, const float* rays8, long n, int mode, int any_hit, int nthreads,
                   int32_t* ids, float* t, float* u, float* v);

/* ---- the reference's own BVH8 (BVH8::Create / BVH8::IsHit, src/s3d_bvh8.cpp), restated
 * for the CPU baseline: same tree, same walk order, same triangle test and ties (the
 * first triangle walked keeps an equal t). ---- */
void*  oracle_refbvh_create(const float* pos9, long n, double* build_seconds);
void   oracle_refbvh_destroy(void* bvh);
void   oracle_refbvh_stats(void* bvh, long* n8, long* n4, long* n_leaf, int* depth);
double oracle_refbvh_trace(void* bvh, const float* rays8, long n, int nthreads, int32_t* ids, float* t, float* u,
                           float* v);

/* ---- rendering ---- */
enum { ORACLE_LAMBERT = 0, ORACLE_MIRROR = 1, ORACLE_GLASS = 2, ORACLE_GGX = 3, ORACLE_PHONG = 4,
       ORACLE_PLASTIC = 5 };
enum { ORACLE_PROFILE_COMPAT = 0, ORACLE_PROFILE_PHYSICAL = 1 };

typedef struct {
    int   type;
    float color[3];
    float emission[3];
    float ior;
    float roughness;
    float specular[3];  /* Plastic: specular colour (color is the diffuse one) */
    float power;        /* Phong / Plastic: lobe exponent */
    int   color_map;    /* 1 + texture index multiplying the base colour, 0 = none */
} oracle_material;

typedef struct {
    int          width, height;
    const float* rgb;   /* texel (x, y) at rgb[3 * (y * width + x)] */
} oracle_texture;

typedef struct {
    const float* tri_pos;   /* n*9 */
    const float* tri_nrm;   /* n*9 shading normals, or NULL (geometric) */
    const int*   tri_mat;   /* n */
    long         n_tris;
    const oracle_material* mats;
    int          n_mats;
    int          has_light;
    float        light_corner[3], light_edge_a[3], light_edge_b[3], light_emission[3];
    int          has_sun;
    float        sun_dir[3];        /* unit, towards the sun */
    float        sun_radiance[3];   /* irradiance on a surface facing the sun */
    float        sun_half_angle;    /* radians; 0 = delta light, > 0 = uniform disk with MIS */
    float        sky[3];            /* constant sky radiance */
    float        cam_pos[3], cam_target[3], cam_up[3];
    float        cam_fov, cam_near; /* fov used linearly as in include/s3d_camera.h:85-86 */
    float        cam_lens;          /* thin-lens radius (0: pinhole) */
    float        cam_focal;         /* focal distance (0: |target - pos|, as ThinLensCamera) */
    const float* tri_uv;            /* n*6 texture coordinates, or NULL */
    const oracle_texture* textures;
    int          n_textures;
    int          ibl_map;           /* 1 + texture index of the environment, 0 = constant sky */
    float        ibl_scale;
    const float* spheres;           /* n_spheres * 6: centre xyz, radius, material, light (0/1) */
    long         n_spheres;
} oracle_scene;

typedef struct {
    int      width, height, spp;
    int      max_depth;     /* path segments, as PathTracer::Config::MaxBounceCount */
    int      rr_depth;      /* physical profile: Russian roulette from this depth */
    int      profile;       /* ORACLE_PROFILE_* */
    uint64_t seed;
    int      nthreads;
    int      row_begin, row_end;   /* render rows [row_begin,row_end); 0,0 = all */
} oracle_render_opts;

/* sum/sumsq: width*height*3 doubles (per-pixel sum of L and of L^2 over spp). */
void oracle_render(const oracle_scene* sc, const oracle_render_opts* o, double* sum, double* sumsq);

/* ---- tonemapping (src/s3d_tonemapper.cpp:38-353) and sRGB8 (src/s3d_pt.cpp:145-171) ---- */
enum { ORACLE_TM_REINHARD = 0, ORACLE_TM_UNCHARTED2 = 1, ORACLE_TM_ACES = 2 };
void oracle_tonemap(int type, int width, int height, const float* rgb, float* out,
                    float* ave_lw, float* max_lw);
/* ref_oetf=1: the reference's pow(1.055x, 1/2.4) - 0.055; 0: standard sRGB. */
void oracle_srgb8(const float* rgb, long n_px, int ref_oetf, uint8_t* out);

/* ---- denoisers ---- */
/* Reference NLM: RGBA, 5x5 patch, 13x13 search, h = sigma = coeff (src/s3d_denoiser.cpp:19-95). */
void oracle_nlm_ref(int width, int height, float coeff, const float* rgba, float* out);
/* Variance-scaled NLM (21x21 search, 7x7 patch by default), RGB + per-pixel variance
 * of the mean (3 channels).  d^2 = mean over patch and channels of
 *   ((a-b)^2 - (va + min(va, vb))) / (eps + k^2 (va + vb)),  w = exp(-max(0, d^2)). */
void oracle_nlm_var(int width, int height, int search_r, int patch_r, float k,
                    const float* rgb, const float* var, float* out);

#ifdef __cplusplus
}
#endif
#endif
