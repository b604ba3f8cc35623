/* salty_oracle.c -- CPU restatement of Salty's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see salty_oracle.h).  Built with -ffp-contract=off
 * so every product and sum is rounded separately, as the reference's MSVC
 * /arch:AVX build does.  Reference citations are relative to the reference
 * project's src/ directory.
 */
#define _GNU_SOURCE
#include "salty_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

/* ------------------------------------------------------------------ PCG */
/* include/s3d_math.h:2769-2817: state = seed + inc, then one step. */
static const uint64_t kPcgMul = 6364136223846793005ull;
static const uint64_t kPcgInc = 1442695040888963407ull;

uint32_t opcg_u32(opcg* r) {
    uint64_t old = r->state;
    r->state = old * kPcgMul + kPcgInc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}
void opcg_seed(opcg* r, uint64_t seed) {
    r->state = seed + kPcgInc;
    (void)opcg_u32(r);
}
/* static_cast<float>(u32) / 0xffffffffui32: the divisor converts to 4294967296.0f */
float opcg_f32(opcg* r) { return (float)opcg_u32(r) / (float)0xffffffffu; }

/* splitmix64 finaliser (Steele, Lea, Flood 2014): per-(pixel, sample) stream seeds. */
static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static uint64_t stream_seed(uint64_t seed, uint64_t pixel, uint64_t sample) {
    return mix64(seed ^ mix64((pixel << 32) | (sample & 0xffffffffull)));
}

/* ------------------------------------------------------- microbenchmark */
/* Triangle soup: centroid c ~ U[0,1]^3 (three draws), then for each vertex k and axis a
 * in order, v[k][a] = c[a] + (draw - 0.5f) * 0.01f. */
void oracle_gen_soup(uint64_t seed, long n, float* pos9) {
    opcg r; opcg_seed(&r, seed);
    for (long i = 0; i < n; ++i) {
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = opcg_f32(&r);
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                float j = (opcg_f32(&r) - 0.5f) * 0.01f;
                pos9[i * 9 + k * 3 + a] = c[a] + j;
            }
    }
}

/* Rays: origin uniform on the sphere of radius 2 about (0.5,0.5,0.5) by Marsaglia's
 * method (1972) in double precision (only +,-,*,sqrt: identical on every IEEE host);
 * target ~ U[0,1]^3; direction = the reference's Vector3::UnitVector(target - origin)
 * (include/s3d_math.h:830-842). */
void oracle_gen_rays(uint64_t seed, long n, float tmin, float* rays8) {
    opcg r; opcg_seed(&r, seed);
    for (long i = 0; i < n; ++i) {
        double a, b, s;
        do {
            a = 2.0 * (double)opcg_f32(&r) - 1.0;
            b = 2.0 * (double)opcg_f32(&r) - 1.0;
            s = a * a + b * b;
        } while (s >= 1.0);
        double q = 2.0 * sqrt(1.0 - s);
        float o[3];
        o[0] = (float)(0.5 + 2.0 * (a * q));
        o[1] = (float)(0.5 + 2.0 * (b * q));
        o[2] = (float)(0.5 + 2.0 * (1.0 - 2.0 * s));
        float t[3];
        for (int k = 0; k < 3; ++k) t[k] = opcg_f32(&r);
        float d[3] = {t[0] - o[0], t[1] - o[1], t[2] - o[2]};
        float mag = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        float* out = rays8 + i * 8;
        out[0] = o[0]; out[1] = o[1]; out[2] = o[2]; out[3] = tmin;
        out[4] = d[0] / mag; out[5] = d[1] / mag; out[6] = d[2] / mag; out[7] = INFINITY;
    }
}

/* ------------------------------------------------------- vector helpers */
typedef struct { float x, y, z; } v3;
static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float maxc(v3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
static inline float length(v3 a) { return sqrtf(dot(a, a)); }
/* Vector3::SafeUnitVector (include/s3d_math.h:847-859) */
static inline v3 safe_unit(v3 v) {
    float mag = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (mag > 0.0f) return mk(v.x / mag, v.y / mag, v.z / mag);
    return v;
}
/* Vector3::UnitVector (include/s3d_math.h:830-842) */
static inline v3 unit(v3 v) {
    float mag = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return mk(v.x / mag, v.y / mag, v.z / mag);
}
/* Vector3::Reflect (include/s3d_math.h:893-903): i - 2 (n.i) n */
static inline v3 reflect(v3 i, v3 n) {
    float d = n.x * i.x + n.y * i.y + n.z * i.z;
    float d2 = 2.0f * d;
    return mk(i.x - d2 * n.x, i.y - d2 * n.y, i.z - d2 * n.z);
}
/* TangentSpace, Duff et al. 2017 (include/s3d_math.h:2875-2886) */
static inline void tangent_space(v3 n, v3* t, v3* b) {
    float s = (n.z >= 0.0f) ? 1.0f : -1.0f;
    float a = -1.0f / (s + n.z);
    float bb = n.x * n.y * a;
    *t = mk(1.0f + s * n.x * n.x * a, s * bb, -s * n.x);
    *b = mk(bb, s + n.y * n.y * a, -n.y);
}

/* ------------------------------------------------------- triangle tests */
/* src/s3d_triangle.cpp:73-105 with Triangle::m_Edge from the constructor (:38-39). */
int oracle_tri_ref(const float o_[3], const float d_[3], const float v0_[3], const float v1_[3],
                   const float v2_[3], float tmin, float tmax, float* t, float* u, float* v) {
    v3 o = ld3(o_), d = ld3(d_), v0 = ld3(v0_), v1 = ld3(v1_), v2 = ld3(v2_);
    v3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    v3 s1 = cross(d, e2);
    float div = dot(s1, e1);
    if (fabsf(div) <= FLT_EPSILON) return 0;
    v3 dv = sub(o, v0);
    float beta = dot(dv, s1) / div;
    if (beta <= 0.0f || beta >= 1.0f) return 0;
    v3 s2 = cross(dv, e1);
    float gamma = dot(d, s2) / div;
    if (gamma <= 0.0f || (beta + gamma) >= 1.0f) return 0;
    float dist = dot(e2, s2) / div;
    if (dist < tmin || dist > tmax) return 0;
    *t = dist; *u = beta; *v = gamma;
    return 1;
}

/* Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013.
 * Edge functions fall back to double when a single-precision one is exactly 0. */
int oracle_tri_watertight(const float o_[3], const float d_[3], const float v0_[3], const float v1_[3],
                          const float v2_[3], float tmin, float tmax, float* t, float* u, float* v) {
    float d[3] = {d_[0], d_[1], d_[2]};
    /* dominant axis, ties to the lower index */
    float ad[3] = {fabsf(d[0]), fabsf(d[1]), fabsf(d[2])};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (d[kz] < 0.0f) { int tmp = kx; kx = ky; ky = tmp; }
    float Sx = d[kx] / d[kz], Sy = d[ky] / d[kz], Sz = 1.0f / d[kz];
    float A[3], B[3], C[3];
    for (int i = 0; i < 3; ++i) { A[i] = v0_[i] - o_[i]; B[i] = v1_[i] - o_[i]; C[i] = v2_[i] - o_[i]; }
    float Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    float Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    float Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    float det = U + V + W;
    if (det == 0.0f) return 0;
    float Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
    float T = U * Az + V * Bz + W * Cz;
    if (det > 0.0f) { if (T < tmin * det || T > tmax * det) return 0; }
    else { if (T > tmin * det || T < tmax * det) return 0; }
    float rcp = 1.0f / det;
    *t = T * rcp; *u = V * rcp; *v = W * rcp;
    return 1;
}

/* ------------------------------------------------------- oracle BVH */
/* A plain median-split binary BVH.  Boxes are tested in double against the ray's line
 * restricted to t >= tmin (minus slack); nothing is culled by the best hit so far, so
 * the closest-hit answer depends only on the triangle test. */
typedef struct { float lo[3], hi[3]; int left, right, first, count; } onode;
typedef struct {
    const float* pos;  /* copy owned */
    long n;
    int* prim;         /* leaf order */
    onode* nodes;
    long n_nodes;
} obvh;

typedef struct { float c[3]; } ocent;

static void tri_bounds(const float* p, float lo[3], float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(p[a], fminf(p[3 + a], p[6 + a]));
        hi[a] = fmaxf(p[a], fmaxf(p[3 + a], p[6 + a]));
    }
}

static const float* g_sort_cent; static int g_sort_axis;
static int cmp_prim(const void* a, const void* b) {
    float ca = g_sort_cent[*(const int*)a * 3 + g_sort_axis];
    float cb = g_sort_cent[*(const int*)b * 3 + g_sort_axis];
    if (ca < cb) return -1;
    if (ca > cb) return 1;
    return (*(const int*)a < *(const int*)b) ? -1 : (*(const int*)a > *(const int*)b);
}

static int obvh_build_rec(obvh* b, const float* cent, int first, int count) {
    long id = b->n_nodes++;
    onode* nd = &b->nodes[id];
    for (int a = 0; a < 3; ++a) { nd->lo[a] = INFINITY; nd->hi[a] = -INFINITY; }
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = first; i < first + count; ++i) {
        float lo[3], hi[3];
        tri_bounds(b->pos + (long)b->prim[i] * 9, lo, hi);
        for (int a = 0; a < 3; ++a) {
            nd->lo[a] = fminf(nd->lo[a], lo[a]); nd->hi[a] = fmaxf(nd->hi[a], hi[a]);
            float c = cent[b->prim[i] * 3 + a];
            clo[a] = fminf(clo[a], c); chi[a] = fmaxf(chi[a], c);
        }
    }
    if (count <= 4) { nd->left = nd->right = -1; nd->first = first; nd->count = count; return (int)id; }
    int axis = 0;
    for (int a = 1; a < 3; ++a) if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    g_sort_cent = cent; g_sort_axis = axis;
    qsort(b->prim + first, count, sizeof(int), cmp_prim);
    int half = count / 2;
    int l = obvh_build_rec(b, cent, first, half);
    int r = obvh_build_rec(b, cent, first + half, count - half);
    nd = &b->nodes[id];
    nd->left = l; nd->right = r; nd->first = 0; nd->count = 0;
    return (int)id;
}

void* oracle_bvh_create(const float* pos9, long n) {
    obvh* b = (obvh*)calloc(1, sizeof(obvh));
    float* p = (float*)malloc(sizeof(float) * 9 * (n > 0 ? n : 1));
    memcpy(p, pos9, sizeof(float) * 9 * n);
    b->pos = p; b->n = n;
    b->prim = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (long i = 0; i < n; ++i) b->prim[i] = (int)i;
    b->nodes = (onode*)malloc(sizeof(onode) * (2 * (n > 0 ? n : 1)));
    float* cent = (float*)malloc(sizeof(float) * 3 * (n > 0 ? n : 1));
    for (long i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a)
            cent[i * 3 + a] = (p[i * 9 + a] + p[i * 9 + 3 + a] + p[i * 9 + 6 + a]) * (1.0f / 3.0f);
    if (n > 0) obvh_build_rec(b, cent, 0, (int)n);
    free(cent);
    return b;
}

void oracle_bvh_destroy(void* h) {
    obvh* b = (obvh*)h;
    if (!b) return;
    free((void*)b->pos); free(b->prim); free(b->nodes); free(b);
}

/* Slab test in double; returns 1 if the line meets the box for some t >= tmin_lo and
 * t <= tmax_hi. */
static int box_hit_d(const onode* nd, const double o[3], const double inv[3], double tmin_lo, double tmax_hi) {
    double t0 = tmin_lo, t1 = tmax_hi;
    for (int a = 0; a < 3; ++a) {
        double lo = ((double)nd->lo[a] - o[a]) * inv[a];
        double hi = ((double)nd->hi[a] - o[a]) * inv[a];
        if (isnan(lo) || isnan(hi)) { /* origin on the slab plane of a parallel ray */
            if (o[a] < nd->lo[a] || o[a] > nd->hi[a]) return 0;
            continue;
        }
        if (lo > hi) { double tmp = lo; lo = hi; hi = tmp; }
        lo -= 1e-9 * fabs(lo) + 1e-12; hi += 1e-9 * fabs(hi) + 1e-12;
        if (lo > t0) t0 = lo;
        if (hi < t1) t1 = hi;
        if (t0 > t1) return 0;
    }
    return 1;
}

typedef struct { int id; float t, u, v; } ohit;

/* cull_slack < 0: never cull by the best hit (parity traversal); otherwise a node is
 * skipped when its entry exceeds best_t * (1 + cull_slack) (render traversal). */
static int obvh_trace_one(const obvh* b, const float* o, const float* d, float tmin, float tmax,
                          int mode, int any_hit, double cull_slack, ohit* out) {
    double od[3] = {o[0], o[1], o[2]}, inv[3];
    for (int a = 0; a < 3; ++a) inv[a] = 1.0 / (double)d[a];
    int stack[128]; int sp = 0;
    out->id = -1; out->t = INFINITY; out->u = out->v = 0.0f;
    if (b->n == 0) return 0;
    stack[sp++] = 0;
    while (sp) {
        const onode* nd = &b->nodes[stack[--sp]];
        double hi = (double)tmax;
        if (cull_slack >= 0.0 && out->id >= 0) hi = (double)out->t * (1.0 + cull_slack) + 1e-12;
        if (!box_hit_d(nd, od, inv, (double)tmin - 1e-6 * fabs((double)tmin) - 1e-12, hi)) continue;
        if (nd->left < 0) {
            for (int i = nd->first; i < nd->first + nd->count; ++i) {
                int p = b->prim[i];
                const float* tp = b->pos + (long)p * 9;
                float t, u, v;
                int h = mode == 0 ? oracle_tri_ref(o, d, tp, tp + 3, tp + 6, tmin, tmax, &t, &u, &v)
                                  : oracle_tri_watertight(o, d, tp, tp + 3, tp + 6, tmin, tmax, &t, &u, &v);
                if (!h) continue;
                if (out->id < 0 || t < out->t || (t == out->t && p < out->id)) {
                    out->id = p; out->t = t; out->u = u; out->v = v;
                    if (any_hit) return 1;
                }
            }
        } else {
            stack[sp++] = nd->right;
            stack[sp++] = nd->left;
        }
    }
    return out->id >= 0;
}

typedef struct {
    const obvh* b; const float* rays; long n; int mode, any_hit;
    int32_t* ids; float *t, *u, *v;
    long next; pthread_mutex_t mu;
} trace_job;

static void* trace_worker(void* arg) {
    trace_job* j = (trace_job*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        long b = j->next; j->next += 1024;
        pthread_mutex_unlock(&j->mu);
        if (b >= j->n) break;
        long e = b + 1024 < j->n ? b + 1024 : j->n;
        for (long i = b; i < e; ++i) {
            const float* r = j->rays + i * 8;
            ohit h;
            obvh_trace_one(j->b, r, r + 4, r[3], r[7], j->mode, j->any_hit, -1.0, &h);
            j->ids[i] = h.id;
            if (j->t) j->t[i] = h.t;
            if (j->u) j->u[i] = h.u;
            if (j->v) j->v[i] = h.v;
        }
    }
    return NULL;
}

static int resolve_threads(int n) {
    if (n > 0) return n;
    long hw = sysconf(_SC_NPROCESSORS_ONLN);
    return hw > 0 ? (int)hw : 1;
}

void oracle_trace(void* bvh, const float* rays8, long n, int mode, int any_hit, int nthreads,
                  int32_t* ids, float* t, float* u, float* v) {
    trace_job j = {(const obvh*)bvh, rays8, n, mode, any_hit, ids, t, u, v, 0, PTHREAD_MUTEX_INITIALIZER};
    nthreads = resolve_threads(nthreads);
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (int i = 1; i < nthreads; ++i) pthread_create(&th[i], NULL, trace_worker, &j);
    trace_worker(&j);
    for (int i = 1; i < nthreads; ++i) pthread_join(th[i], NULL);
}

/* ------------------------------------------------------- the reference's BVH8 */
/* A restatement of the reference's own acceleration structure and walk, for the CPU
 * baseline: the same tree as BVH8::Create builds (src/s3d_bvh8.cpp:254-342,401-479, with
 * BVH4::Create src/s3d_bvh4.cpp:237-325,384-423 and Leaf src/s3d_leaf.cpp:22-35 where a
 * split is refused), walked as BVH8::IsHit / BVH4::IsHit / Leaf::IsHit do
 * (src/s3d_bvh8.cpp:191-206, src/s3d_bvh4.cpp:174-189, src/s3d_leaf.cpp:74-87): a
 * depth-first walk in child order 0..7, every child whose box the line of the ray pierces
 * (BoundingBox8::IsHit, include/s3d_math.h:2549-2586: slabs from -1e12 to 1e12, no clip to
 * the best hit), and Triangle::IsHit (src/s3d_triangle.cpp:73-105) with its shared record
 * (a later triangle must be strictly closer).  Floating-point operations follow the
 * reference's order; min/max follow the SSE/AVX semantics (a < b ? a : b, a > b ? a : b). */
#define RB_BUCKETS 16
#define RB_FMAX FLT_MAX
#define RB_HITMAX 1e12f
#define RB_HITMIN 1e-3f

typedef struct { float mn[3], mx[3], c[3]; int empty; } rbox;

static rbox rbox_empty(void) {
    rbox b;
    for (int a = 0; a < 3; ++a) { b.mn[a] = RB_FMAX; b.mx[a] = -RB_FMAX; b.c[a] = 0.0f; }
    b.empty = 1;
    return b;
}
static rbox rbox_of(const float mn[3], const float mx[3]) {   /* BoundingBox(mini, maxi) */
    rbox b;
    for (int a = 0; a < 3; ++a) { b.mn[a] = mn[a]; b.mx[a] = mx[a]; b.c[a] = (mn[a] + mx[a]) * 0.5f; }
    b.empty = 0;
    return b;
}
static float rmin(float a, float b) { return a < b ? a : b; }
static float rmax(float a, float b) { return a > b ? a : b; }
static rbox rbox_merge(const rbox* a, const rbox* b) {       /* BoundingBox::Merge(box, box) */
    if (!a->empty && !b->empty) {
        float mn[3], mx[3];
        for (int k = 0; k < 3; ++k) { mn[k] = rmin(a->mn[k], b->mn[k]); mx[k] = rmax(a->mx[k], b->mx[k]); }
        return rbox_of(mn, mx);
    }
    if (a->empty && !b->empty) return *b;
    return *a;
}
static rbox rbox_merge_pt(const rbox* a, const float p[3]) { /* BoundingBox::Merge(box, point) */
    if (!a->empty) {
        float mn[3], mx[3];
        for (int k = 0; k < 3; ++k) { mn[k] = rmin(a->mn[k], p[k]); mx[k] = rmax(a->mx[k], p[k]); }
        return rbox_of(mn, mx);
    }
    rbox b;
    for (int k = 0; k < 3; ++k) b.mn[k] = b.mx[k] = b.c[k] = p[k];
    b.empty = 0;
    return b;
}
static float rbox_area(const rbox* b) {                      /* SurfaceArea, include/s3d_math.h:2904-2910 */
    float X = fabsf(b->mx[0] - b->mn[0]), Y = fabsf(b->mx[1] - b->mn[1]), Z = fabsf(b->mx[2] - b->mn[2]);
    return 2.0f * ((X * Y) + (X * Z) + (Y * Z));
}

typedef struct { float v0[3], e1[3], e2[3]; rbox box; } rtri;
/* kind 8 / 4: inner node with that many children and their boxes (SoA); kind 0: a leaf
 * of `count` triangles at tri_index[first ..] */
typedef struct { int kind, first, count; int child[8]; float lo[3][8], hi[3][8]; } rnode;
typedef struct {
    rtri* tris; long n;
    int* idx;                 /* the work array BVH8::Create partitions */
    rnode* nodes; long n_nodes, cap;
    rbox* node_box;           /* GetBox() of every node */
    long n8, n4, n_leaf; int depth;
} rbvh;

static long rb_new_node(rbvh* b) {
    if (b->n_nodes == b->cap) {
        b->cap = b->cap ? b->cap * 2 : 1024;
        b->nodes = (rnode*)realloc(b->nodes, sizeof(rnode) * (size_t)b->cap);
        b->node_box = (rbox*)realloc(b->node_box, sizeof(rbox) * (size_t)b->cap);
    }
    return b->n_nodes++;
}

/* CalcOffset(box, p).a[axis] (src/s3d_bvh8.cpp:75-89) */
static float rb_offset(const rbox* cb, const float p[3], int axis) {
    float o = p[axis] - cb->mn[axis];
    if (cb->mx[axis] > cb->mn[axis]) o /= cb->mx[axis] - cb->mn[axis];
    return o;
}

/* SplitSAH (src/s3d_bvh8.cpp:254-342; BVH4's differs only in its leaf threshold) */
static int rb_split(rbvh* b, int* sh, long count, int min_leaf, long* mid) {
    if (count <= min_leaf) return 0;
    rbox bound = b->tris[sh[0]].box, cen = rbox_empty();
    for (long i = 1; i < count; ++i) bound = rbox_merge(&bound, &b->tris[sh[i]].box);
    cen = rbox_merge_pt(&cen, b->tris[sh[0]].box.c);
    for (long i = 1; i < count; ++i) cen = rbox_merge_pt(&cen, b->tris[sh[i]].box.c);
    float ext[3] = {cen.mx[0] - cen.mn[0], cen.mx[1] - cen.mn[1], cen.mx[2] - cen.mn[2]};
    int axis = (ext[0] > ext[1] && ext[0] > ext[2]) ? 0 : (ext[1] > ext[2] ? 1 : 2);
    if (cen.mx[axis] == cen.mn[axis]) return 0;
    unsigned cnt[RB_BUCKETS];
    rbox bb[RB_BUCKETS];
    for (int k = 0; k < RB_BUCKETS; ++k) { cnt[k] = 0; bb[k] = rbox_empty(); }
    for (long i = 0; i < count; ++i) {
        int k = (int)((float)RB_BUCKETS * rb_offset(&cen, b->tris[sh[i]].box.c, axis));
        if (k == RB_BUCKETS) k = RB_BUCKETS - 1;
        cnt[k]++;
        bb[k] = rbox_merge(&bb[k], &b->tris[sh[i]].box);
    }
    float cost[RB_BUCKETS - 1];
    const float area = rbox_area(&bound);
    for (int i = 0; i < RB_BUCKETS - 1; ++i) {
        rbox b0 = rbox_empty(), b1 = rbox_empty();
        int c0 = 0, c1 = 0;
        for (int j = 0; j <= i; ++j) { b0 = rbox_merge(&b0, &bb[j]); c0 += (int)cnt[j]; }
        for (int j = i + 1; j < RB_BUCKETS; ++j) { b1 = rbox_merge(&b1, &bb[j]); c1 += (int)cnt[j]; }
        cost[i] = 1.0f + ((float)c0 * rbox_area(&b0) + (float)c1 * rbox_area(&b1)) / area;
    }
    float best = cost[0];
    int split = 0;
    for (int i = 1; i < RB_BUCKETS - 1; ++i)
        if (cost[i] < best) { best = cost[i]; split = i; }
    if (!(best < (float)count)) return 0;
    /* std::partition (bidirectional form) with the reference's predicate: the bucket
     * position is compared as a float, `16 * offset <= split` */
    int* first = sh;
    int* last = sh + count;
    for (;;) {
        for (;;) {
            if (first == last) goto done;
            float k = (float)RB_BUCKETS * rb_offset(&cen, b->tris[*first].box.c, axis);
            if (k == (float)RB_BUCKETS) k = (float)(RB_BUCKETS - 1);
            if (k <= (float)split) ++first; else break;
        }
        --last;
        for (;;) {
            if (first == last) goto done;
            float k = (float)RB_BUCKETS * rb_offset(&cen, b->tris[*last].box.c, axis);
            if (k == (float)RB_BUCKETS) k = (float)(RB_BUCKETS - 1);
            if (!(k <= (float)split)) --last; else break;
        }
        int tmp = *first; *first = *last; *last = tmp;
        ++first;
    }
done:
    *mid = first - sh;
    return 1;
}

/* Leaf::Create (src/s3d_leaf.cpp:22-35): its box merges the triangles' boxes */
static long rb_leaf(rbvh* b, int* sh, long count, int depth) {
    long id = rb_new_node(b);
    rnode* nd = &b->nodes[id];
    nd->kind = 0;
    nd->first = (int)(sh - b->idx);
    nd->count = (int)count;
    rbox bx = b->tris[sh[0]].box;
    for (long i = 1; i < count; ++i) bx = rbox_merge(&bx, &b->tris[sh[i]].box);
    b->node_box[id] = bx;
    b->n_leaf++;
    if (depth > b->depth) b->depth = depth;
    return id;
}

/* BVH8 / BVH4 node from its children: BoundingBox8/4 of their GetBox(), and its own
 * GetBox() (the lanes merged) */
static long rb_inner(rbvh* b, int kind, const long* ch) {
    long id = rb_new_node(b);
    rnode* nd = &b->nodes[id];
    nd->kind = kind;
    float mn[3] = {RB_FMAX, RB_FMAX, RB_FMAX}, mx[3] = {-RB_FMAX, -RB_FMAX, -RB_FMAX};
    for (int i = 0; i < kind; ++i) {
        const rbox* cb = &b->node_box[ch[i]];
        nd->child[i] = (int)ch[i];
        for (int a = 0; a < 3; ++a) {
            nd->lo[a][i] = cb->mn[a];
            nd->hi[a][i] = cb->mx[a];
            mn[a] = rmin(mn[a], cb->mn[a]);
            mx[a] = rmax(mx[a], cb->mx[a]);
        }
    }
    b->node_box[id] = rbox_of(mn, mx);
    if (kind == 8) b->n8++; else b->n4++;
    return id;
}

/* BVH4::Create (src/s3d_bvh4.cpp:384-423); its CreateNode is always a Leaf (:94-104) */
static long rb_create4(rbvh* b, int* sh, long count, int depth) {
    if (count <= 4) return rb_leaf(b, sh, count, depth);
    long mid = 0, midL = 0, midR = 0;
    if (!rb_split(b, sh, count, 4, &mid)) return rb_leaf(b, sh, count, depth);
    if (!rb_split(b, sh, mid, 4, &midL)) return rb_leaf(b, sh, count, depth);
    if (!rb_split(b, sh + mid, count - mid, 4, &midR)) return rb_leaf(b, sh, count, depth);
    long i1 = midL, i2 = mid, i3 = mid + midR;
    long ch[4];
    ch[0] = rb_create4(b, sh, i1, depth + 1);
    ch[1] = rb_create4(b, sh + i1, i2 - i1, depth + 1);
    ch[2] = rb_create4(b, sh + i2, i3 - i2, depth + 1);
    ch[3] = rb_create4(b, sh + i3, count - i3, depth + 1);
    return rb_inner(b, 4, ch);
}

/* CreateNode of the BVH8 file (src/s3d_bvh8.cpp:94-110): a Leaf up to 8, else BVH4 */
static long rb_node8(rbvh* b, int* sh, long count, int depth) {
    return count <= 8 ? rb_leaf(b, sh, count, depth) : rb_create4(b, sh, count, depth);
}

/* BVH8::Create (src/s3d_bvh8.cpp:401-479): three levels of binary splits, 8 children */
static long rb_create8(rbvh* b, int* sh, long count, int depth) {
    if (count <= 8) return rb_node8(b, sh, count, depth);
    long mid = 0, midL = 0, midR = 0, m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    if (!rb_split(b, sh, count, 8, &mid)) return rb_node8(b, sh, count, depth);
    if (!rb_split(b, sh, mid, 8, &midL)) return rb_node8(b, sh, count, depth);
    if (!rb_split(b, sh + mid, count - mid, 8, &midR)) return rb_node8(b, sh, count, depth);
    long iB = midL, iC = mid, iD = mid + midR;
    if (!rb_split(b, sh, iB, 8, &m0)) return rb_node8(b, sh, count, depth);
    if (!rb_split(b, sh + iB, iC - iB, 8, &m1)) return rb_node8(b, sh, count, depth);
    if (!rb_split(b, sh + iC, iD - iC, 8, &m2)) return rb_node8(b, sh, count, depth);
    if (!rb_split(b, sh + iD, count - iD, 8, &m3)) return rb_node8(b, sh, count, depth);
    long idx[9] = {0, m0, midL, midL + m1, mid, mid + m2, mid + midR, mid + midR + m3, count};
    long ch[8];
    for (int i = 0; i < 8; ++i) ch[i] = rb_create8(b, sh + idx[i], idx[i + 1] - idx[i], depth + 1);
    return rb_inner(b, 8, ch);
}

void* oracle_refbvh_create(const float* pos9, long n, double* build_seconds) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    rbvh* b = (rbvh*)calloc(1, sizeof(rbvh));
    b->n = n;
    b->tris = (rtri*)malloc(sizeof(rtri) * (size_t)(n ? n : 1));
    b->idx = (int*)malloc(sizeof(int) * (size_t)(n ? n : 1));
    for (long i = 0; i < n; ++i) {   /* Triangle::Triangle (src/s3d_triangle.cpp:22-40) */
        const float* p = pos9 + i * 9;
        rtri* t = &b->tris[i];
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a) {
            t->v0[a] = p[a];
            mn[a] = rmin(rmin(p[a], p[3 + a]), p[6 + a]);
            mx[a] = rmax(rmax(p[a], p[3 + a]), p[6 + a]);
            t->e1[a] = p[3 + a] - p[a];
            t->e2[a] = p[6 + a] - p[a];
        }
        t->box = rbox_of(mn, mx);
        b->idx[i] = (int)i;
    }
    if (n > 0) rb_create8(b, b->idx, n, 1);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (build_seconds) *build_seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    return b;
}

void oracle_refbvh_destroy(void* h) {
    rbvh* b = (rbvh*)h;
    if (!b) return;
    free(b->tris); free(b->idx); free(b->nodes); free(b->node_box); free(b);
}

void oracle_refbvh_stats(void* h, long* n8, long* n4, long* n_leaf, int* depth) {
    const rbvh* b = (const rbvh*)h;
    *n8 = b->n8; *n4 = b->n4; *n_leaf = b->n_leaf; *depth = b->depth;
}

typedef struct { float t, u, v; int id; } rrec;

/* Triangle::IsHit against the shared record (src/s3d_triangle.cpp:73-105) */
static void rb_tri(const rtri* T, int id, const float o[3], const float d[3], rrec* rec) {
    v3 D = ld3(d), e1 = ld3(T->e1), e2 = ld3(T->e2);
    v3 s1 = cross(D, e2);
    float div = dot(s1, e1);
    if (fabsf(div) <= FLT_EPSILON) return;
    v3 dv = sub(ld3(o), ld3(T->v0));
    float beta = dot(dv, s1) / div;
    if (beta <= 0.0f || beta >= 1.0f) return;
    v3 s2 = cross(dv, e1);
    float gamma = dot(D, s2) / div;
    if (gamma <= 0.0f || (beta + gamma) >= 1.0f) return;
    float dist = dot(e2, s2) / div;
    if (dist < RB_HITMIN || dist > RB_HITMAX) return;
    if (dist >= rec->t) return;
    rec->t = dist; rec->u = beta; rec->v = gamma; rec->id = id;
}

/* BoundingBox8/4::IsHit (include/s3d_math.h:2549-2586, 2364-2401): one bit per child */
static unsigned rb_box_mask(const rnode* nd, const float o[3], const float d[3]) {
    unsigned m = 0;
    for (int i = 0; i < nd->kind; ++i) {
        float tmin = -RB_HITMAX, tmax = RB_HITMAX;
        for (int a = 0; a < 3; ++a) {
            float t0 = (nd->lo[a][i] - o[a]) / d[a];
            float t1 = (nd->hi[a][i] - o[a]) / d[a];
            float n = t0 < t1 ? t0 : t1, f = t0 > t1 ? t0 : t1;
            tmin = tmin > n ? tmin : n;
            tmax = tmax < f ? tmax : f;
        }
        if (tmax >= tmin) m |= 1u << i;
    }
    return m;
}

static void rb_trace_one(const rbvh* b, const float o[3], const float d[3], rrec* rec) {
    rec->t = RB_FMAX; rec->u = rec->v = 0.0f; rec->id = -1;
    if (b->n_nodes == 0) return;
    int stack[1024];
    int sp = 0;
    stack[sp++] = (int)(b->n_nodes - 1);   /* the root is built last */
    while (sp) {
        const rnode* nd = &b->nodes[stack[--sp]];
        if (nd->kind == 0) {
            for (int i = 0; i < nd->count; ++i) {
                int id = b->idx[nd->first + i];
                rb_tri(&b->tris[id], id, o, d, rec);
            }
            continue;
        }
        unsigned m = rb_box_mask(nd, o, d);
        for (int i = nd->kind - 1; i >= 0; --i)   /* child 0 is walked first */
            if (m & (1u << i)) stack[sp++] = nd->child[i];
    }
}

typedef struct {
    const rbvh* b; const float* rays; long n; int32_t* ids; float *t, *u, *v;
    long next; pthread_mutex_t mu;
} rtrace_job;

static void* rtrace_worker(void* arg) {
    rtrace_job* j = (rtrace_job*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        long s = j->next; j->next += 256;
        pthread_mutex_unlock(&j->mu);
        if (s >= j->n) break;
        long e = s + 256 < j->n ? s + 256 : j->n;
        for (long i = s; i < e; ++i) {
            const float* r = j->rays + i * 8;
            rrec rec;
            rb_trace_one(j->b, r, r + 4, &rec);
            j->ids[i] = rec.id;
            if (j->t) j->t[i] = rec.t;
            if (j->u) j->u[i] = rec.u;
            if (j->v) j->v[i] = rec.v;
        }
    }
    return NULL;
}

/* Closest hits of n rays (n x 8: o, tmin, d, tmax; tmin/tmax ignored: the reference's
 * limits F_HIT_MIN = 1e-3 and F_HIT_MAX = 1e12 apply) on `nthreads` host threads (0: all);
 * misses: id -1, t = FLT_MAX (the record's initial distance).  Returns the seconds taken. */
double oracle_refbvh_trace(void* h, const float* rays8, long n, int nthreads, int32_t* ids, float* t, float* u,
                           float* v) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    rtrace_job j = {(const rbvh*)h, rays8, n, ids, t, u, v, 0, PTHREAD_MUTEX_INITIALIZER};
    nthreads = resolve_threads(nthreads);
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (int i = 1; i < nthreads; ++i) pthread_create(&th[i], NULL, rtrace_worker, &j);
    rtrace_worker(&j);
    for (int i = 1; i < nthreads; ++i) pthread_join(th[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------- rendering */
typedef struct {
    const oracle_scene* sc;
    obvh* bvh;
    float* pos;        /* scene triangles + 2 light triangles */
    float* nrm;
    int* mat;
    long n;
    oracle_material* mats;   /* scene materials + light material */
    int light_mat;
    long light_tri0;         /* index of the first light triangle, -1 if none */
    v3 lc, la, lb, ln, le;   /* light corner, edges, unit normal, emission */
    float larea;
    v3 cam_pos, cam_cx, cam_cy, cam_cz;
    v3 cam_dir, cam_u, cam_v;  /* unit view direction and screen axes (thin lens) */
    float cam_lens, cam_focal;
    /* sun disk: direction, frame, cos of the angular radius, radiance, 1/solid angle */
    v3 sun_dir, sun_t, sun_b, sun_L;
    int sun_disk;
    float sun_cos_max, sun_pdf;
    /* spheres (Sphere, src/s3d_sphere.cpp): ids sph_base + k; the light list is the quad
       light (if any) and then the light spheres in input order */
    const float* sph;
    long n_sph, sph_base;
    int* light_sph;
    int n_light_sph, n_lights;
} rscene;

/* PinholeCamera::Update (include/s3d_camera.h:63-90) */
static void camera_update(rscene* r, const oracle_scene* sc, float aspect) {
    v3 pos = ld3(sc->cam_pos), tgt = ld3(sc->cam_target), up = ld3(sc->cam_up);
    v3 dir = unit(sub(tgt, pos));
    r->cam_cx = scl(scl(unit(cross(dir, up)), sc->cam_fov), aspect);
    r->cam_cy = scl(unit(cross(dir, r->cam_cx)), sc->cam_fov);
    r->cam_cz = add(pos, scl(dir, sc->cam_near));
    r->cam_pos = pos;
    r->cam_dir = dir;
    r->cam_u = unit(r->cam_cx);
    r->cam_v = unit(r->cam_cy);
    r->cam_lens = sc->cam_lens;
    r->cam_focal = sc->cam_focal > 0.0f ? sc->cam_focal : length(sub(tgt, pos));
}

/* ThinLensCamera::GetRay (include/s3d_camera.h:206-222) for the compat profile: the lens
 * offset lies in the world xy plane and the focal plane is z = const (the reference's
 * z-aligned view).  Physical profile: offset in the camera's screen axes, focal plane
 * perpendicular to the view direction.  Two random numbers (angle, radius). */
static void thin_lens(const rscene* r, int compat, opcg* rnd, v3* o, v3* d) {
    float th = 6.283185307179586476925286766559f * opcg_f32(rnd);
    float rad = r->cam_lens * sqrtf(fmaxf(opcg_f32(rnd), 0.0f));
    float cx = rad * cosf(th), cy = rad * sinf(th);
    v3 focus;
    if (compat) {
        focus = add(r->cam_pos, scl(*d, r->cam_focal / fabsf(d->z)));
        *o = add(r->cam_pos, mk(cx, cy, 0.0f));
    } else {
        focus = add(r->cam_pos, scl(*d, r->cam_focal / dot(*d, r->cam_dir)));
        *o = add(add(r->cam_pos, scl(r->cam_u, cx)), scl(r->cam_v, cy));
    }
    *d = unit(sub(focus, *o));
}

/* PinholeCamera::GetRay (include/s3d_camera.h:95-100) */
static v3 camera_dir(const rscene* r, float x, float y) {
    v3 p = add(add(scl(r->cam_cx, x), scl(r->cam_cy, y)), r->cam_cz);
    return unit(sub(p, r->cam_pos));
}

static void rscene_init(rscene* r, const oracle_scene* sc) {
    memset(r, 0, sizeof(*r));
    r->sc = sc;
    long n = sc->n_tris + (sc->has_light ? 2 : 0);
    r->n = n;
    r->pos = (float*)malloc(sizeof(float) * 9 * (n ? n : 1));
    r->nrm = (float*)malloc(sizeof(float) * 9 * (n ? n : 1));
    r->mat = (int*)malloc(sizeof(int) * (n ? n : 1));
    memcpy(r->pos, sc->tri_pos, sizeof(float) * 9 * sc->n_tris);
    for (long i = 0; i < sc->n_tris; ++i) {
        r->mat[i] = sc->tri_mat[i];
        if (sc->tri_nrm) {
            memcpy(r->nrm + i * 9, sc->tri_nrm + i * 9, sizeof(float) * 9);
        } else {
            const float* p = sc->tri_pos + i * 9;
            v3 g = safe_unit(cross(sub(ld3(p + 3), ld3(p)), sub(ld3(p + 6), ld3(p))));
            for (int k = 0; k < 3; ++k) { r->nrm[i * 9 + k * 3] = g.x; r->nrm[i * 9 + k * 3 + 1] = g.y; r->nrm[i * 9 + k * 3 + 2] = g.z; }
        }
    }
    r->mats = (oracle_material*)malloc(sizeof(oracle_material) * (sc->n_mats + 1));
    memcpy(r->mats, sc->mats, sizeof(oracle_material) * sc->n_mats);
    r->light_tri0 = -1;
    if (sc->has_light) {
        r->light_mat = sc->n_mats;
        oracle_material lm; memset(&lm, 0, sizeof(lm));
        lm.type = ORACLE_LAMBERT;
        for (int c = 0; c < 3; ++c) lm.emission[c] = sc->light_emission[c];
        r->mats[sc->n_mats] = lm;
        r->lc = ld3(sc->light_corner); r->la = ld3(sc->light_edge_a); r->lb = ld3(sc->light_edge_b);
        r->le = ld3(sc->light_emission);
        v3 cr = cross(r->la, r->lb);
        r->larea = sqrtf(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
        r->ln = unit(cr);
        v3 p0 = r->lc, p1 = add(r->lc, r->la), p2 = add(add(r->lc, r->la), r->lb), p3 = add(r->lc, r->lb);
        v3 tri[6] = {p0, p1, p2, p0, p2, p3};
        r->light_tri0 = sc->n_tris;
        for (int t = 0; t < 2; ++t) {
            long i = sc->n_tris + t;
            for (int k = 0; k < 3; ++k) {
                v3 q = tri[t * 3 + k];
                r->pos[i * 9 + k * 3] = q.x; r->pos[i * 9 + k * 3 + 1] = q.y; r->pos[i * 9 + k * 3 + 2] = q.z;
                r->nrm[i * 9 + k * 3] = r->ln.x; r->nrm[i * 9 + k * 3 + 1] = r->ln.y; r->nrm[i * 9 + k * 3 + 2] = r->ln.z;
            }
            r->mat[i] = r->light_mat;
        }
    }
    r->bvh = (obvh*)oracle_bvh_create(r->pos, n);
    r->sph = sc->spheres;
    r->n_sph = sc->spheres ? sc->n_spheres : 0;
    r->sph_base = n;
    r->light_sph = (int*)malloc(sizeof(int) * (r->n_sph ? r->n_sph : 1));
    for (long k = 0; k < r->n_sph; ++k)
        if (r->sph[k * 6 + 5] != 0.0f) r->light_sph[r->n_light_sph++] = (int)k;
    r->n_lights = (sc->has_light ? 1 : 0) + r->n_light_sph;
    if (sc->has_sun) {
        r->sun_dir = unit(ld3(sc->sun_dir));
        r->sun_disk = sc->sun_half_angle > 0.0f;
        r->sun_cos_max = (float)cos((double)sc->sun_half_angle);
        /* uniform cone sampling pdf 1/omega; radiance L with L pi sin^2 = sun_radiance, the
           irradiance on a surface facing the sun */
        double ca = cos((double)sc->sun_half_angle);
        double omega = 2.0 * 3.14159265358979323846 * (1.0 - ca);
        double facing = 3.14159265358979323846 * (1.0 - ca) * (1.0 + ca);
        r->sun_pdf = r->sun_disk ? (float)(1.0 / omega) : 0.0f;
        r->sun_L = r->sun_disk ? mk((float)(sc->sun_radiance[0] / facing), (float)(sc->sun_radiance[1] / facing),
                                    (float)(sc->sun_radiance[2] / facing))
                               : mk(0, 0, 0);
        tangent_space(r->sun_dir, &r->sun_t, &r->sun_b);
    }
}

static void rscene_free(rscene* r) {
    oracle_bvh_destroy(r->bvh);
    free(r->pos); free(r->nrm); free(r->mat); free(r->mats); free(r->light_sph);
}

static int is_light_tri(const rscene* r, int id) {
    return r->light_tri0 >= 0 && id >= r->light_tri0 && id < r->light_tri0 + 2;
}

/* Triangle::CalcParam (src/s3d_triangle.cpp:107-121): interpolated, SafeNormalize'd. */
/* Texture::SampleColor (src/s3d_texture.cpp:925-952): bilinear with the weights taken
 * before the wrap, indices wrapped as |i % size| */
static v3 tex_sample(const oracle_texture* t, float u, float v) {
    float fx = u * (float)(t->width - 1), fy = v * (float)(t->height - 1);
    if (!(fabsf(fx) < 1e9f)) fx = 0.0f;
    if (!(fabsf(fy) < 1e9f)) fy = 0.0f;
    int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    int x1 = x0 + 1, y1 = y0 + 1;
    float xw0 = (float)x1 - fx, xw1 = fx - (float)x0, yw0 = (float)y1 - fy, yw1 = fy - (float)y0;
    x0 = abs(x0 % t->width); x1 = abs(x1 % t->width);
    y0 = abs(y0 % t->height); y1 = abs(y1 % t->height);
    v3 c00 = ld3(t->rgb + 3 * ((long)y0 * t->width + x0)), c01 = ld3(t->rgb + 3 * ((long)y1 * t->width + x0));
    v3 c10 = ld3(t->rgb + 3 * ((long)y0 * t->width + x1)), c11 = ld3(t->rgb + 3 * ((long)y1 * t->width + x1));
    return add(scl(add(scl(c00, yw0), scl(c01, yw1)), xw0), scl(add(scl(c10, yw0), scl(c11, yw1)), xw1));
}

/* Texture::SampleColor(dir) (src/s3d_texture.cpp:957-972) */
static v3 tex_sphere(const oracle_texture* t, v3 d) {
    const float pi = 3.1415926535897932384626433832795f, two_pi = 6.283185307179586476925286766559f;
    float theta = acosf(fminf(1.0f, fmaxf(-1.0f, d.y)));
    float u = 0.0f, v = theta * (1.0f / pi);
    if (!(fabsf(d.x) <= FLT_EPSILON) && !(fabsf(d.z) <= FLT_EPSILON)) {
        float phi = atan2f(d.z, d.x);
        u = (d.z < 0.0f ? phi + two_pi : phi) * (1.0f / two_pi);
    }
    return tex_sample(t, u, v);
}

/* Scene::SampleIBL (include/s3d_scene.h:81-82): environment map or constant sky */
static v3 environment(const rscene* r, v3 d) {
    const oracle_scene* sc = r->sc;
    if (sc->ibl_map > 0) return scl(tex_sphere(&sc->textures[sc->ibl_map - 1], d), sc->ibl_scale);
    return ld3(sc->sky);
}

/* the material's colour map at the hit (Triangle::CalcParam's texture coordinate), or 1 */
static v3 color_map(const rscene* r, const oracle_material* m, int id, float b1, float b2) {
    if (m->color_map <= 0 || !r->sc->tri_uv || id >= r->sc->n_tris) return mk(1.0f, 1.0f, 1.0f);
    const float* t = r->sc->tri_uv + (long)id * 6;
    float a = 1.0f - b1 - b2;
    return tex_sample(&r->sc->textures[m->color_map - 1], t[0] * a + t[2] * b1 + t[4] * b2,
                      t[1] * a + t[3] * b1 + t[5] * b2);
}

static v3 shading_normal(const rscene* r, int id, float beta, float gamma) {
    const float* n = r->nrm + (long)id * 9;
    float alpha = 1.0f - beta - gamma;
    v3 s = mk(n[0] * alpha + n[3] * beta + n[6] * gamma,
              n[1] * alpha + n[4] * beta + n[7] * gamma,
              n[2] * alpha + n[5] * beta + n[8] * gamma);
    return safe_unit(s);
}

static v3 geometric_normal(const rscene* r, int id) {
    const float* p = r->pos + (long)id * 9;
    return safe_unit(cross(sub(ld3(p + 3), ld3(p)), sub(ld3(p + 6), ld3(p))));
}

/* Sphere::IsHit (src/s3d_sphere.cpp:66-92) with the reference's operation order: the
 * nearer root above tmin, else the farther. */
static int sph_ref(const float* c, v3 o, v3 d, float tmin, float tmax, float* t) {
    v3 po = sub(ld3(c), o);
    float b = dot(po, d);
    float D4 = b * b - dot(po, po) + c[3] * c[3];
    if (D4 < 0.0f) return 0;
    float sq = sqrtf(D4), t1 = b - sq, t2 = b + sq;
    if (t1 < tmin && t2 < tmin) return 0;
    *t = t1 > tmin ? t1 : t2;
    return *t <= tmax;
}
/* the same in double precision (physical profile): smallest root in [tmin, tmax] */
static int sph_exact(const float* c, v3 o, v3 d, float tmin, float tmax, float* t) {
    double f[3] = {(double)o.x - c[0], (double)o.y - c[1], (double)o.z - c[2]};
    double dd[3] = {d.x, d.y, d.z};
    double a = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
    double b = -(f[0] * dd[0] + f[1] * dd[1] + f[2] * dd[2]);
    double cc = f[0] * f[0] + f[1] * f[1] + f[2] * f[2] - (double)c[3] * c[3];
    double disc = b * b - a * cc;
    if (disc < 0.0) return 0;
    double sq = sqrt(disc), t0 = (b - sq) / a, t1 = (b + sq) / a;
    double tt = t0 >= tmin ? t0 : t1;
    if (!(tt >= tmin) || tt > tmax) return 0;
    *t = (float)tt;
    return 1;
}

/* closest hit over the triangles' BVH and then every sphere (equal t: the lower id) */
static int closest(const rscene* r, v3 o, v3 d, float tmin, float tmax, int mode, ohit* h) {
    float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    int hit = obvh_trace_one(r->bvh, of, df, tmin, tmax, mode, 0, 1e-3, h);
    for (long k = 0; k < r->n_sph; ++k) {
        float t;
        const float* c = r->sph + k * 6;
        int ok = mode == 0 ? sph_ref(c, o, d, tmin, tmax, &t) : sph_exact(c, o, d, tmin, tmax, &t);
        if (ok && (!hit || t < h->t)) {
            hit = 1;
            h->t = t; h->u = 0.0f; h->v = 0.0f; h->id = (int)(r->sph_base + k);
        }
    }
    return hit;
}
static int occluded(const rscene* r, v3 o, v3 d, float tmin, float tmax) {
    float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    ohit h;
    if (obvh_trace_one(r->bvh, of, df, tmin, tmax, 1, 1, 1e-3, &h)) return 1;
    for (long k = 0; k < r->n_sph; ++k) {
        float t;
        if (sph_exact(r->sph + k * 6, o, d, tmin, tmax, &t)) return 1;
    }
    return 0;
}

/* solid-angle pdf of a direction uniform in the cone sphere c subtends from x: 1 / (2 pi
 * (1 - cos theta_max)), 0 from inside */
static float sph_cone_pdf(const float* c, v3 x) {
    v3 w = sub(ld3(c), x);
    float d2 = dot(w, w), r2 = c[3] * c[3];
    if (!(d2 > r2)) return 0.0f;
    float s2 = r2 / d2, cm = sqrtf(fmaxf(0.0f, 1.0f - s2));
    return 1.0f / (6.283185307179586476925286766559f * (s2 / (1.0f + cm)));
}

/* ---- what shading needs of a hit: material, normal, texture coordinate ---- */
static int is_sph(const rscene* r, int id) { return r->n_sph > 0 && id >= r->sph_base; }
static const oracle_material* hit_mat(const rscene* r, int id) {
    if (is_sph(r, id)) return &r->mats[(int)r->sph[(id - r->sph_base) * 6 + 4]];
    return &r->mats[r->mat[id]];
}
/* Sphere::CalcParam (src/s3d_sphere.cpp:94-104): outward normal, (phi/2pi, (pi-theta)/pi) */
static v3 sph_normal(const rscene* r, int id, v3 p) {
    return safe_unit(sub(p, ld3(r->sph + (id - r->sph_base) * 6)));
}

static v3 hit_color_map(const rscene* r, const oracle_material* m, int id, float b1, float b2, v3 p) {
    if (!is_sph(r, id)) return color_map(r, m, id, b1, b2);
    if (m->color_map <= 0) return mk(1.0f, 1.0f, 1.0f);
    v3 n = sph_normal(r, id, p);
    float theta = acosf(fminf(1.0f, fmaxf(-1.0f, n.y)));
    float phi = atan2f(n.x, n.z);
    if (phi < 0.0f) phi += 6.283185307179586476925286766559f;
    return tex_sample(&r->sc->textures[m->color_map - 1], phi * (1.0f / 6.283185307179586476925286766559f),
                      (3.1415926535897932384626433832795f - theta) * (1.0f / 3.1415926535897932384626433832795f));
}

/* ---- compat profile: PathTracer::Radiance / NextEventEstimation (src/s3d_pt.cpp:182-292) */
static const float kPi = 3.1415926535897932384626433832795f;
static const float k2Pi = 6.283185307179586476925286766559f;
static const float kFHitMin = 1e-3f, kFHitMax = 1e12f;

static v3 compat_nee(const rscene* r, v3 pos, v3 n, const oracle_material* m, opcg* rnd) {
    /* Scene::GetLight (include/s3d_scene.h:84-90): u32 % (number of lights) */
    int li = (int)(opcg_u32(rnd) % (uint32_t)r->n_lights);
    v3 lp; float pdf; long want;  /* the light's point and pdf, and the id range it covers */
    const float* sp = NULL;
    if (li < r->sc->has_light) {
        float u = opcg_f32(rnd), w = opcg_f32(rnd);
        lp = add(add(r->lc, scl(r->la, u)), scl(r->lb, w));
        pdf = 1.0f / r->larea;
        want = -1;
    } else {
        /* Sphere::Sample (src/s3d_sphere.cpp:106-115): a point on the radius + 0.1 sphere */
        int k = r->light_sph[li - r->sc->has_light];
        sp = r->sph + k * 6;
        float r1 = k2Pi * opcg_f32(rnd);
        float r2 = 1.0f - 2.0f * opcg_f32(rnd);
        float r3 = sqrtf(1.0f - r2 * r2);
        lp = add(ld3(sp), scl(safe_unit(mk(r3 * cosf(r1), r3 * sinf(r1), r2)), sp[3] + 1e-1f));
        pdf = 1.0f / (4.0f * kPi * sp[3] * sp[3]);
        want = r->sph_base + k;
    }
    v3 ld = sub(lp, pos);
    float dist2 = dot(ld, ld);
    ld = safe_unit(ld);
    ohit h;
    /* accepted when the first hit is the sampled light (src/s3d_pt.cpp:274) */
    if (closest(r, pos, ld, kFHitMin, kFHitMax, 0, &h) && (want < 0 ? is_light_tri(r, h.id) : h.id == want)) {
        v3 hp = add(pos, scl(ld, h.t));
        v3 ln = want < 0 ? r->ln : sph_normal(r, h.id, hp);
        float cos_s = fabsf(dot(n, ld));
        float cos_l = fabsf(dot(ln, neg(ld)));
        v3 fs = mk(m->color[0] / kPi, m->color[1] / kPi, m->color[2] / kPi);
        float G = (cos_s * cos_l) / dist2;
        float brdf_pdf = fabsf(ld.z / kPi) * cos_l / dist2;
        float mis = pdf / (brdf_pdf + pdf);
        v3 le = ld3(hit_mat(r, h.id)->emission);
        return scl(scl(mul(le, fs), mis), G / pdf);
    }
    return mk(0, 0, 0);
}

/* SamplePhong (include/s3d_math.h:2976-2982): cos(theta) = (1 - v)^(1 / (n + 1)) */
static v3 sample_phong(float u, float v, float n) {
    float p = k2Pi * u;
    float ct = powf(1.0f - v, 1.0f / (n + 1.0f));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    return mk(st * cosf(p), st * sinf(p), ct);
}

/* Lambert::Shade (src/s3d_lambert.cpp:64-86), Mirror::Shade (src/s3d_mirror.cpp:59-71),
 * Glass::Shade (src/s3d_glass.cpp:60-128). */
static v3 compat_shade(const oracle_material* m, v3 in, v3 normal, opcg* rnd, v3* out, int* dice) {
    v3 nm = (dot(normal, in) < 0.0f) ? normal : neg(normal);
    v3 col = mk(m->color[0], m->color[1], m->color[2]);
    if (m->type == ORACLE_MIRROR) {
        *out = safe_unit(reflect(in, nm));
        *dice = 0;
        return col;
    }
    if (m->type == ORACLE_GLASS) {
        v3 refl = safe_unit(reflect(in, nm));
        int into = dot(normal, nm) > 0.0f;
        *dice = 0;
        float nc = 1.0f, nt = m->ior;
        float nnt = into ? (nc / nt) : (nt / nc);
        float ddn = dot(in, nm);
        float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
        if (cos2t < 0.0f) { *out = refl; return col; }
        float sq = cos2t > 0.0f ? sqrtf(cos2t) : 0.0f;  /* SafeSqrt */
        v3 refr = safe_unit(sub(scl(in, nnt), scl(scl(normal, into ? 1.0f : -1.0f), ddn * nnt + sq)));
        float a = nt - nc, b = nt + nc;
        float R0 = (a * a) / (b * b);
        float c = 1.0f - (into ? -ddn : dot(refr, normal));
        float c2 = c * c;
        float Re = R0 + (1.0f - R0) * (c2 * c2 * c);
        float Tr = 1.0f - Re;
        float P = 0.25f + 0.5f * Re;
        float prob = 0.5f;
        if (opcg_f32(rnd) < P) { *out = refl; return scl(col, Re / (P * prob)); }
        *out = refr;
        return scl(col, Tr / ((1.0f - P) * prob));
    }
    if (m->type == ORACLE_PHONG) {
        /* Phong::Shade (src/s3d_phong.cpp:65-88): a lobe around the mirror direction,
         * weight specular * cos(out, n), dice against max(specular, 0.01) */
        float u = opcg_f32(rnd), v = opcg_f32(rnd);
        v3 s = sample_phong(u, v, m->power);
        v3 w = safe_unit(reflect(in, nm));
        v3 t, b;
        tangent_space(w, &t, &b);
        v3 dir = safe_unit(add(add(scl(t, s.x), scl(b, s.y)), scl(w, s.z)));
        float cosine = fabsf(dot(dir, nm));
        *out = dir;
        float thr = fmaxf(fmaxf(fmaxf(m->color[0], m->color[1]), m->color[2]), 0.01f);
        *dice = opcg_f32(rnd) >= thr;
        return scl(col, cosine);
    }
    if (m->type == ORACLE_PLASTIC) {
        /* Plastic::Shade (src/s3d_plastic.cpp:71-142): Schlick R with R0 = 0.5 picks the
         * diffuse branch with P = (R + 0.5) / 2 and weights it R / P (uniform hemisphere),
         * the Phong branch (1 - R) / (1 - P) * cos; the specular dice threshold is derived
         * from the diffuse one (src/s3d_plastic.cpp:34-37) */
        float cosine = fabsf(dot(normal, in));
        float t1 = 1.0f - cosine;
        float R = 0.5f + 0.5f * t1 * t1 * t1 * t1 * t1;
        float P = (R + 0.5f) / 2.0f;
        float thr0 = fmaxf(fmaxf(fmaxf(m->color[0], m->color[1]), m->color[2]), 0.01f);
        if (opcg_f32(rnd) <= P) {
            v3 t, b;
            tangent_space(nm, &t, &b);
            float u = opcg_f32(rnd), v = opcg_f32(rnd);
            float rr = sqrtf(1.0f - u * u), p = k2Pi * v;
            v3 s = mk(rr * cosf(p), rr * sinf(p), u);
            *out = safe_unit(add(add(scl(t, s.x), scl(b, s.y)), scl(nm, s.z)));
            *dice = opcg_f32(rnd) >= thr0;
            return scl(col, R / P);
        }
        float u = opcg_f32(rnd), v = opcg_f32(rnd);
        v3 s = sample_phong(u, v, m->power);
        v3 w = safe_unit(reflect(in, nm));
        v3 t, b;
        tangent_space(w, &t, &b);
        v3 dir = safe_unit(add(add(scl(t, s.x), scl(b, s.y)), scl(w, s.z)));
        float dots = dot(dir, nm);
        *out = dir;
        *dice = opcg_f32(rnd) >= fmaxf(thr0, 0.01f);
        return scl(ld3(m->specular), dots * (1.0f - R) / (1.0f - P));
    }
    /* Lambert (GGX falls back to Lambert in the compat profile: the reference has no GGX
     * material) */
    v3 t, b;
    tangent_space(nm, &t, &b);
    float u = opcg_f32(rnd), v = opcg_f32(rnd);
    float rr = sqrtf(1.0f - u * u), p = k2Pi * v;
    v3 s = mk(rr * cosf(p), rr * sinf(p), u);     /* SampleLambert, include/s3d_math.h:2968-2973 */
    *out = safe_unit(add(add(scl(t, s.x), scl(b, s.y)), scl(nm, s.z)));
    float thr = fmaxf(fmaxf(fmaxf(m->color[0], m->color[1]), m->color[2]), 0.01f);
    *dice = opcg_f32(rnd) >= thr;
    return col;
}

static v3 compat_radiance(const rscene* r, v3 o, v3 d, int max_bounce, opcg* rnd) {
    v3 W = mk(1, 1, 1), L = mk(0, 0, 0);
    for (int depth = 0; depth < max_bounce; ++depth) {
        ohit h;
        if (!closest(r, o, d, kFHitMin, kFHitMax, 0, &h)) {
            L = add(L, mul(W, environment(r, d)));
            break;
        }
        v3 pos = add(o, scl(d, h.t));
        const oracle_material* m = hit_mat(r, h.id);
        L = add(L, mul(W, ld3(m->emission)));
        v3 n = is_sph(r, h.id) ? sph_normal(r, h.id, pos) : shading_normal(r, h.id, h.u, h.v);
        /* TexturedMaterial (src/s3d_texturedmaterial.cpp:63-87): the map scales the NEE base
         * colour and the Shade weight */
        v3 tx = hit_color_map(r, m, h.id, h.u, h.v, pos);
        oracle_material mt = *m;
        for (int c = 0; c < 3; ++c) mt.color[c] *= (c == 0 ? tx.x : c == 1 ? tx.y : tx.z);
        int delta = (m->type == ORACLE_MIRROR || m->type == ORACLE_GLASS);
        if (!delta && r->n_lights > 0 && !is_light_tri(r, h.id)) L = add(L, mul(W, compat_nee(r, pos, n, &mt, rnd)));
        v3 out; int dice = 0;
        W = mul(W, mul(compat_shade(m, d, n, rnd, &out, &dice), tx));
        if (dice) break;
        if (W.x < FLT_EPSILON && W.y < FLT_EPSILON && W.z < FLT_EPSILON) break;
        o = pos; d = out;
    }
    return L;
}

/* ---- physical profile ----
 * Cosine-weighted Lambert, mirror, smooth dielectric (exact Fresnel), GGX conductor with
 * Schlick Fresnel and separable Smith G (NDF sampling as SampleGGX, include/s3d_math.h:
 * 2985-2993, alpha = roughness^2).  NEE to the one-sided quad light with balance-heuristic
 * MIS, NEE to a delta sun, constant sky on escape, Russian roulette from rr_depth with
 * survival min(1, max W), rolled only while it is below 1.  Camera rays start at t = 1e-4, rays leaving a surface at t = 0
 * from an origin pushed off it (spawn).  Random numbers per (pixel, sample) stream,
 * consumed in this order: jitter x, y; per vertex: light point u, v (non-delta, light
 * present); BSDF (Lambert 2, glass 1, GGX 2, mirror 0, Phong 2, plastic 3); RR 1
 * (depth >= rr_depth and survival below 1). */
static const float kEps = 1e-4f;

/* Origin of a ray leaving the surface point p in direction w: p pushed off the surface along
 * the geometric normal ng (either orientation) to the side w points to, by 256 units in the
 * last place of each coordinate, or by 2^-16 near the world origin where ulps are tiny
 * (Waechter and Binder, "A Fast and Robust Method for Avoiding Self-Intersection", Ray
 * Tracing Gems, 2019).  Rays spawned this way start at t = 0. */
static float nudge(float p, float n) {
    int32_t o = (int32_t)(256.0f * n), b;
    float q;
    memcpy(&b, &p, 4);
    b += p < 0.0f ? -o : o;
    memcpy(&q, &b, 4);
    return fabsf(p) < 1.0f / 32.0f ? p + n * (1.0f / 65536.0f) : q;
}
static v3 spawn(v3 p, v3 ng, v3 w) {
    v3 n = dot(ng, w) >= 0.0f ? ng : neg(ng);
    return mk(nudge(p.x, n.x), nudge(p.y, n.y), nudge(p.z, n.z));
}

static float ggx_d(float nh, float a2) {
    float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * k * k);
}
static float ggx_g1(float nv, float a2) {
    return 2.0f * nv / (nv + sqrtf(a2 + (1.0f - a2) * nv * nv));
}
static v3 schlick(v3 f0, float c) {
    float m = 1.0f - c; float m2 = m * m; float m5 = m2 * m2 * m;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}

/* Normalised Phong lobe around the mirror direction r of wo (physical profile):
 * f = (n + 2) / (2 pi) cos^n(r, wi); sampled with pdf (n + 1) / (2 pi) cos^n(r, wi). */
static float phong_lobe(v3 n, v3 wo, v3 wi, float power, float* pdf) {
    v3 r = reflect(neg(wo), n);
    float c = dot(r, wi);
    if (c <= 0.0f) { *pdf = 0.0f; return 0.0f; }
    float cn = powf(c, power);
    *pdf = (power + 1.0f) / k2Pi * cn;
    return (power + 2.0f) / k2Pi * cn;
}
/* Plastic (physical profile): Schlick F with R0 = 0.04 at the outgoing angle splits
 * F * specular * Phong lobe + (1 - F) * diffuse / pi; sampled as a one-sample mixture that
 * takes the lobe with probability Ps = clamp(F, 0.1, 0.9). */
static float plastic_fresnel(float cos_o) {
    float m = 1.0f - fmaxf(cos_o, 0.0f), m2 = m * m;
    return 0.04f + 0.96f * m2 * m2 * m;
}
static float plastic_ps(float F) { return fminf(0.9f, fmaxf(0.1f, F)); }

/* f(wo, wi) without the cosine and the BSDF-sampling pdf, for NEE. */
static v3 phys_eval(const oracle_material* m, v3 n, v3 wo, v3 wi, float* pdf) {
    v3 col = mk(m->color[0], m->color[1], m->color[2]);
    float ni = dot(n, wi);
    if (m->type == ORACLE_PHONG) {
        float lp;
        float f = phong_lobe(n, wo, wi, m->power, &lp);
        *pdf = lp;
        return scl(col, f);
    }
    if (m->type == ORACLE_PLASTIC) {
        float lp;
        float fl = phong_lobe(n, wo, wi, m->power, &lp);
        float F = plastic_fresnel(dot(n, wo)), ps = plastic_ps(F);
        *pdf = ps * lp + (1.0f - ps) * fmaxf(ni, 0.0f) / kPi;
        return add(scl(ld3(m->specular), F * fl), scl(col, (1.0f - F) / kPi));
    }
    if (m->type == ORACLE_GGX) {
        float a = m->roughness * m->roughness, a2 = a * a;
        float no = dot(n, wo);
        v3 h = safe_unit(add(wo, wi));
        float nh = dot(n, h), oh = dot(wo, h);
        if (no <= 0.0f || ni <= 0.0f || nh <= 0.0f || oh <= 0.0f) { *pdf = 0.0f; return mk(0, 0, 0); }
        float D = ggx_d(nh, a2);
        float G = ggx_g1(no, a2) * ggx_g1(ni, a2);
        v3 F = schlick(col, oh);
        *pdf = D * nh / (4.0f * oh);
        return scl(F, D * G / (4.0f * no * ni));
    }
    *pdf = ni / kPi;
    return scl(col, 1.0f / kPi);
}

static v3 phys_radiance(const rscene* r, v3 o, v3 d, const oracle_render_opts* opt, opcg* rnd) {
    const oracle_scene* sc = r->sc;
    v3 W = mk(1, 1, 1), L = mk(0, 0, 0);
    int prev_delta = 1; float prev_pdf = 0.0f, tmin = kEps;
    for (int depth = 0; depth < opt->max_depth; ++depth) {
        ohit h;
        if (!closest(r, o, d, tmin, INFINITY, 1, &h)) {
            L = add(L, mul(W, environment(r, d)));
            if (sc->has_sun && r->sun_disk && dot(d, r->sun_dir) >= r->sun_cos_max) {
                float w = prev_delta ? 1.0f : prev_pdf / (prev_pdf + r->sun_pdf);
                L = add(L, scl(mul(W, r->sun_L), w));
            }
            break;
        }
        v3 p = add(o, scl(d, h.t));
        if (is_light_tri(r, h.id)) {
            float cos_l = dot(r->ln, neg(d));
            if (cos_l > 0.0f) {
                if (prev_delta) L = add(L, mul(W, r->le));
                else {
                    float pdf_l = (h.t * h.t) / (cos_l * r->larea * (float)r->n_lights);
                    float mis = prev_pdf / (prev_pdf + pdf_l);
                    L = add(L, scl(mul(W, r->le), mis));
                }
            }
            break;
        }
        oracle_material mtex = *hit_mat(r, h.id);
        {   /* the colour map scales the base colour */
            v3 tx = hit_color_map(r, &mtex, h.id, h.u, h.v, p);
            mtex.color[0] *= tx.x; mtex.color[1] *= tx.y; mtex.color[2] *= tx.z;
        }
        const oracle_material* m = &mtex;
        const int hs = is_sph(r, h.id) ? (int)(h.id - r->sph_base) : -1;
        if (hs >= 0 && r->sph[hs * 6 + 5] != 0.0f && !prev_delta) {
            /* a light sphere reached by BSDF sampling: MIS against its cone sampling */
            float pdf_l = sph_cone_pdf(r->sph + hs * 6, o) / (float)r->n_lights;
            L = add(L, scl(mul(W, ld3(m->emission)), prev_pdf / (prev_pdf + pdf_l)));
        } else {
            L = add(L, mul(W, ld3(m->emission)));
        }
        v3 ng = hs >= 0 ? sph_normal(r, h.id, p) : geometric_normal(r, h.id);
        int into = dot(ng, d) < 0.0f;
        v3 ngf = into ? ng : neg(ng);
        v3 ns = hs >= 0 ? ng : shading_normal(r, h.id, h.u, h.v);
        v3 nsf = (dot(ns, d) < 0.0f) ? ns : neg(ns);
        v3 wo = neg(d);
        int delta = (m->type == ORACLE_MIRROR || m->type == ORACLE_GLASS);
        if (!delta) {
            int li = 0;
            if (r->n_lights > 1) {  /* one light of the list, uniformly */
                li = (int)(opcg_f32(rnd) * (float)r->n_lights);
                if (li > r->n_lights - 1) li = r->n_lights - 1;
            }
            float psel = r->n_lights > 0 ? 1.0f / (float)r->n_lights : 0.0f;
            if (r->n_lights > 0 && li < sc->has_light) {
                float u1 = opcg_f32(rnd), u2 = opcg_f32(rnd);
                v3 lp = add(add(r->lc, scl(r->la, u1)), scl(r->lb, u2));
                v3 wi = sub(lp, p);
                float dist2 = dot(wi, wi), dist = sqrtf(dist2);
                wi = scl(wi, 1.0f / dist);
                float cos_l = dot(r->ln, neg(wi));
                float cos_s = dot(nsf, wi), cos_g = dot(ngf, wi);
                if (cos_l > 0.0f && cos_s > 0.0f && cos_g > 0.0f &&
                    !occluded(r, spawn(p, ng, wi), wi, 0.0f, dist * (1.0f - 1e-4f))) {
                    float pdf_b;
                    v3 f = phys_eval(m, nsf, wo, wi, &pdf_b);
                    float pdf_l = psel * dist2 / (cos_l * r->larea);
                    float mis = pdf_l / (pdf_l + pdf_b);
                    L = add(L, scl(mul(mul(W, f), r->le), cos_s * mis / pdf_l));
                }
            } else if (r->n_lights > 0) {
                /* a direction uniform in the cone the light sphere subtends from p */
                const float* sp = r->sph + r->light_sph[li - sc->has_light] * 6;
                float u1 = opcg_f32(rnd), u2 = opcg_f32(rnd);
                float pdf_c = sph_cone_pdf(sp, p);
                if (pdf_c > 0.0f) {
                    v3 w = sub(ld3(sp), p);
                    float dc = sqrtf(dot(w, w));
                    v3 wz = scl(w, 1.0f / dc);
                    float cos_max = sqrtf(fmaxf(0.0f, 1.0f - sp[3] * sp[3] / (dc * dc)));
                    float one_m = (1.0f - cos_max) * u1, ct = 1.0f - one_m;
                    float st = sqrtf(fmaxf(0.0f, one_m * (2.0f - one_m)));
                    v3 tx_, ty_;
                    tangent_space(wz, &tx_, &ty_);
                    v3 wi = safe_unit(add(add(scl(tx_, st * cosf(k2Pi * u2)), scl(ty_, st * sinf(k2Pi * u2))),
                                          scl(wz, ct)));
                    /* near intersection (dc^2 - r^2) / (dc cos + sqrt(r^2 - dc^2 sin^2)):
                       no cancellation at the cone's edge */
                    float dist = (dc * dc - sp[3] * sp[3]) /
                                 (dc * ct + sqrtf(fmaxf(0.0f, sp[3] * sp[3] - dc * dc * st * st)));
                    float cos_s = dot(nsf, wi), cos_g = dot(ngf, wi);
                    /* the shadow ray runs from the light point back to the surface: from
                       just outside the sphere it cannot meet the sphere itself, which a ray
                       towards a grazing point on its silhouette could, by rounding */
                    v3 q = add(p, scl(wi, dist));
                    v3 qs = spawn(q, safe_unit(sub(q, ld3(sp))), neg(wi)), ps = spawn(p, ng, wi);
                    v3 back = sub(ps, qs);
                    float blen = sqrtf(dot(back, back));
                    if (cos_s > 0.0f && cos_g > 0.0f && dist > 0.0f &&
                        !occluded(r, qs, scl(back, 1.0f / blen), 0.0f, blen * (1.0f - 1e-4f))) {
                        float pdf_b;
                        v3 f = phys_eval(m, nsf, wo, wi, &pdf_b);
                        float pdf_l = psel * pdf_c;
                        float mis = pdf_l / (pdf_l + pdf_b);
                        v3 le = ld3(r->mats[(int)sp[4]].emission);
                        L = add(L, scl(mul(mul(W, f), le), cos_s * mis / pdf_l));
                    }
                }
            }
            if (sc->has_sun) {
                v3 wi = r->sun_dir;
                if (r->sun_disk) {  /* uniform direction in the sun's cone */
                    float u1 = opcg_f32(rnd), u2 = opcg_f32(rnd);
                    float ct = 1.0f - u1 * (1.0f - r->sun_cos_max);
                    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                    float ph = k2Pi * u2;
                    wi = safe_unit(add(add(scl(r->sun_t, st * cosf(ph)), scl(r->sun_b, st * sinf(ph))), scl(wi, ct)));
                }
                float cos_s = dot(nsf, wi), cos_g = dot(ngf, wi);
                if (cos_s > 0.0f && cos_g > 0.0f && !occluded(r, spawn(p, ng, wi), wi, 0.0f, INFINITY)) {
                    float pdf_b;
                    v3 f = phys_eval(m, nsf, wo, wi, &pdf_b);
                    if (r->sun_disk) {
                        float mis = r->sun_pdf / (r->sun_pdf + pdf_b);
                        L = add(L, scl(mul(mul(W, f), r->sun_L), cos_s * mis / r->sun_pdf));
                    } else {
                        L = add(L, scl(mul(mul(W, f), ld3(sc->sun_radiance)), cos_s));
                    }
                }
            }
        }
        v3 col = mk(m->color[0], m->color[1], m->color[2]);
        v3 wi; v3 weight; float pdf = 0.0f; int is_delta = 0;
        if (m->type == ORACLE_MIRROR) {
            wi = reflect(d, nsf); weight = col; is_delta = 1;
        } else if (m->type == ORACLE_GLASS) {
            float eta = into ? 1.0f / m->ior : m->ior;
            float cosi = -dot(d, nsf);
            float sin2t = eta * eta * (1.0f - cosi * cosi);
            float F = 1.0f, cost = 0.0f;
            if (sin2t < 1.0f) {
                cost = sqrtf(1.0f - sin2t);
                float rs = (eta * cosi - cost) / (eta * cosi + cost);
                float rp = (cosi - eta * cost) / (cosi + eta * cost);
                F = 0.5f * (rs * rs + rp * rp);
            }
            float xi = opcg_f32(rnd);
            if (xi < F) wi = reflect(d, nsf);
            else wi = safe_unit(add(scl(d, eta), scl(nsf, eta * cosi - cost)));
            weight = col; is_delta = 1;
        } else if (m->type == ORACLE_GGX) {
            float a = m->roughness * m->roughness, a2 = a * a;
            float r1 = opcg_f32(rnd), r2 = opcg_f32(rnd);
            float ph = k2Pi * r1;
            float ct = sqrtf((1.0f - r2) / fmaxf(r2 * (a2 - 1.0f) + 1.0f, 1e-8f));
            float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
            v3 t, b; tangent_space(nsf, &t, &b);
            v3 hh = safe_unit(add(add(scl(t, st * cosf(ph)), scl(b, st * sinf(ph))), scl(nsf, ct)));
            wi = reflect(d, hh);
            float no = dot(nsf, wo), ni = dot(nsf, wi), nh = dot(nsf, hh), oh = dot(wo, hh);
            if (ni <= 0.0f || no <= 0.0f || oh <= 0.0f || dot(ngf, wi) <= 0.0f) break;
            float G = ggx_g1(no, a2) * ggx_g1(ni, a2);
            v3 F = schlick(col, oh);
            weight = scl(F, G * oh / (no * nh));
            pdf = ggx_d(nh, a2) * nh / (4.0f * oh);
        } else if (m->type == ORACLE_PHONG || m->type == ORACLE_PLASTIC) {
            /* random numbers: branch 1 (plastic only), direction 2 */
            int lobe = 1;
            float F = 0.0f, ps = 1.0f;
            if (m->type == ORACLE_PLASTIC) {
                F = plastic_fresnel(dot(nsf, wo));
                ps = plastic_ps(F);
                lobe = opcg_f32(rnd) < ps;
            }
            float r1 = opcg_f32(rnd), r2 = opcg_f32(rnd);
            v3 t, b;
            if (lobe) {
                v3 s = sample_phong(r1, r2, m->power);
                v3 rdir = reflect(d, nsf);
                tangent_space(rdir, &t, &b);
                wi = safe_unit(add(add(scl(t, s.x), scl(b, s.y)), scl(rdir, s.z)));
            } else {
                float rr = sqrtf(r1), ph = k2Pi * r2;
                float z = sqrtf(fmaxf(0.0f, 1.0f - r1));
                tangent_space(nsf, &t, &b);
                wi = safe_unit(add(add(scl(t, rr * cosf(ph)), scl(b, rr * sinf(ph))), scl(nsf, z)));
            }
            float ni = dot(nsf, wi);
            if (ni <= 0.0f || dot(ngf, wi) <= 0.0f) break;
            v3 f = phys_eval(m, nsf, wo, wi, &pdf);
            if (!(pdf > 0.0f)) break;
            weight = scl(f, ni / pdf);
        } else {
            float r1 = opcg_f32(rnd), r2 = opcg_f32(rnd);
            float rr = sqrtf(r1), ph = k2Pi * r2;
            float z = sqrtf(fmaxf(0.0f, 1.0f - r1));
            v3 t, b; tangent_space(nsf, &t, &b);
            wi = safe_unit(add(add(scl(t, rr * cosf(ph)), scl(b, rr * sinf(ph))), scl(nsf, z)));
            if (dot(ngf, wi) <= 0.0f) break;
            weight = col; pdf = dot(nsf, wi) / kPi;
        }
        W = mul(W, weight);
        prev_delta = is_delta; prev_pdf = pdf;
        if (W.x <= 0.0f && W.y <= 0.0f && W.z <= 0.0f) break;
        if (depth >= opt->rr_depth) {
            /* survival min(1, max W): a path whose throughput has not dropped below 1 (a
               chain of lossless mirror or glass bounces) is never cut, so its weight never
               grows beyond what the BSDFs gave it */
            float q = fminf(1.0f, maxc(W));
            if (q < 1.0f) {
                if (opcg_f32(rnd) >= q) break;
                W = scl(W, 1.0f / q);
            }
        }
        o = spawn(p, ng, wi); d = wi; tmin = 0.0f;
    }
    return L;
}

typedef struct {
    const rscene* r; const oracle_render_opts* o; double *sum, *sumsq;
    int row0, row1, next; pthread_mutex_t mu;
} render_job;

static void* render_worker(void* arg) {
    render_job* j = (render_job*)arg;
    const oracle_render_opts* o = j->o;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int y = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (y >= j->row1) break;
        for (int x = 0; x < o->width; ++x) {
            long px = (long)y * o->width + x;
            double s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
            for (int k = 0; k < o->spp; ++k) {
                opcg rnd; opcg_seed(&rnd, stream_seed(o->seed, (uint64_t)px, (uint64_t)k));
                v3 L;
                if (o->profile == ORACLE_PROFILE_COMPAT) {
                    v3 d = camera_dir(j->r, (0.5f + x) / o->width - 0.5f, (0.5f + y) / o->height - 0.5f);
                    v3 org = j->r->cam_pos;
                    if (j->r->cam_lens > 0.0f) thin_lens(j->r, 1, &rnd, &org, &d);
                    L = compat_radiance(j->r, org, d, o->max_depth, &rnd);
                } else {
                    float jx = opcg_f32(&rnd), jy = opcg_f32(&rnd);
                    v3 d = camera_dir(j->r, (jx + x) / o->width - 0.5f, (jy + y) / o->height - 0.5f);
                    v3 org = j->r->cam_pos;
                    if (j->r->cam_lens > 0.0f) thin_lens(j->r, 0, &rnd, &org, &d);
                    L = phys_radiance(j->r, org, d, o, &rnd);
                }
                s[0] += L.x; s[1] += L.y; s[2] += L.z;
                q[0] += (double)L.x * L.x; q[1] += (double)L.y * L.y; q[2] += (double)L.z * L.z;
            }
            for (int c = 0; c < 3; ++c) {
                j->sum[px * 3 + c] = s[c];
                if (j->sumsq) j->sumsq[px * 3 + c] = q[c];
            }
        }
    }
    return NULL;
}

void oracle_render(const oracle_scene* sc, const oracle_render_opts* o, double* sum, double* sumsq) {
    rscene r;
    rscene_init(&r, sc);
    camera_update(&r, sc, (float)o->width / (float)o->height);
    render_job j;
    memset(&j, 0, sizeof(j));
    j.r = &r; j.o = o; j.sum = sum; j.sumsq = sumsq;
    j.row0 = o->row_begin; j.row1 = (o->row_end > o->row_begin) ? o->row_end : o->height;
    j.next = j.row0;
    pthread_mutex_init(&j.mu, NULL);
    int nt = resolve_threads(o->nthreads);
    pthread_t th[256];
    if (nt > 256) nt = 256;
    for (int i = 1; i < nt; ++i) pthread_create(&th[i], NULL, render_worker, &j);
    render_worker(&j);
    for (int i = 1; i < nt; ++i) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&j.mu);
    rscene_free(&r);
}

/* ------------------------------------------------------- tonemapping */
/* RGBToY (src/s3d_tonemapper.cpp:31-33): Dot((0.299, 0.587, 0.114), rgb) */
static float rgb_to_y(const float* c) { return 0.299f * c[0] + 0.587f * c[1] + 0.114f * c[2]; }

/* ComputeLogarithmicAverage (src/s3d_tonemapper.cpp:38-95): sequential float sum. */
static void log_average(int w, int h, const float* px, float eps, float* ave, float* maxv) {
    int init = 0; float sum = 0.0f, mx = 0.0f;
    for (long i = 0; i < (long)w * h; ++i) {
        float lw = rgb_to_y(px + i * 3);
        if (isnan(lw)) lw = eps;
        if (lw < FLT_EPSILON) lw = eps;
        if (!init) { mx = lw; init = 1; } else mx = fmaxf(mx, lw);
        sum += logf(eps + lw);
    }
    if (isnan(sum)) sum = eps;
    sum /= (float)(w * h);
    *ave = expf(sum);
    *maxv = mx;
}

static float u2_curve(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.01f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}
static float saturate(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
static float aces_curve(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f, f = 0.665406f, g = 12.0f;
    return saturate((x * (a * x * f / g + b)) / (x * f / g * (c * x * f + d) + e));
}

void oracle_tonemap(int type, int width, int height, const float* rgb, float* out,
                    float* ave_lw, float* max_lw) {
    float ave, mx;
    log_average(width, height, rgb, 0.00001f, &ave, &mx);
    if (ave_lw) *ave_lw = ave;
    if (max_lw) *max_lw = mx;
    long n = (long)width * height;
    if (type == ORACLE_TM_UNCHARTED2) {
        float coeff = 0.18f / ave;
        float white = u2_curve(11.2f);
        for (long i = 0; i < n * 3; ++i) out[i] = u2_curve(2.0f * (rgb[i] * coeff)) / white;
    } else if (type == ORACLE_TM_ACES) {
        float coeff = 0.27f / ave;
        for (long i = 0; i < n * 3; ++i) out[i] = aces_curve(rgb[i] * coeff);
    } else {
        float coeff = 0.18f / ave;
        float m2 = mx * coeff; m2 *= m2;
        for (long i = 0; i < n * 3; ++i) {
            float L = rgb[i] * coeff;
            out[i] = L * (1.0f + (L / m2)) / (1.0f + L);
        }
    }
}

/* PathTracer::Capture (src/s3d_pt.cpp:145-171) */
void oracle_srgb8(const float* rgb, long n_px, int ref_oetf, uint8_t* out) {
    for (long i = 0; i < n_px * 3; ++i) {
        float x = rgb[i];
        if (x > 1.0f) x = 1.0f;
        if (x < 0.0f) x = 0.0f;
        if (x != x) x = 0.0f;
        if (ref_oetf) x = (x <= 0.0031308f) ? 12.92f * x : powf(1.055f * x, 1.0f / 2.4f) - 0.055f;
        else x = (x <= 0.0031308f) ? 12.92f * x : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
        out[i] = (uint8_t)(x * 255.0f + 0.5f);
    }
}

/* ------------------------------------------------------- NLM */
static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* FilterNLM (src/s3d_denoiser.cpp:19-95).  Template order: sx outer, sy inner; the
 * per-tap squared length sums the four channel products as (w + z) + (y + x), the
 * order of Vector4::LengthSq (include/s3d_math.h:1271-1274, 1349-1352). */
void oracle_nlm_ref(int width, int height, float coeff, const float* src, float* dst) {
    float ph = fmaxf(0.0001f, coeff), sigma = fmaxf(0.0001f, coeff);
    float inv_h2 = 1.0f / (ph * ph), s2 = sigma * sigma;
    const int K = 5, S = 13, hk = K / 2, hs = S / 2;
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            float sum[4] = {0, 0, 0, 0}, sw = 0.0f;
            for (int sx = x - hs; sx <= x + hs; ++sx) {
                for (int sy = y - hs; sy <= y + hs; ++sy) {
                    float acc = 0.0f;
                    for (int ax = -hk; ax <= hk; ++ax) {
                        for (int ay = -hk; ay <= hk; ++ay) {
                            const float* a = src + ((long)clampi(y + ay, 0, height - 1) * width + clampi(x + ax, 0, width - 1)) * 4;
                            const float* b = src + ((long)clampi(sy + ay, 0, height - 1) * width + clampi(sx + ax, 0, width - 1)) * 4;
                            float p0 = (a[0] - b[0]) * (a[0] - b[0]);
                            float p1 = (a[1] - b[1]) * (a[1] - b[1]);
                            float p2 = (a[2] - b[2]) * (a[2] - b[2]);
                            float p3 = (a[3] - b[3]) * (a[3] - b[3]);
                            acc += (p3 + p2) + (p1 + p0);
                        }
                    }
                    float arg = -fmaxf(acc - 2.0f * s2, 0.0f) * inv_h2;
                    float wgt = expf(arg);
                    sw += wgt;
                    const float* c = src + ((long)clampi(sy, 0, height - 1) * width + clampi(sx, 0, width - 1)) * 4;
                    for (int k = 0; k < 4; ++k) sum[k] += c[k] * wgt;
                }
            }
            float* o = dst + ((long)y * width + x) * 4;
            for (int k = 0; k < 4; ++k) o[k] = sum[k] / sw;
        }
    }
}

void oracle_nlm_var(int width, int height, int search_r, int patch_r, float k,
                    const float* rgb, const float* var, float* out) {
    const float eps = 1e-10f;
    float k2 = k * k;
    float norm = 1.0f / (3.0f * (float)((2 * patch_r + 1) * (2 * patch_r + 1)));
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            double sum[3] = {0, 0, 0}, sw = 0.0;
            for (int dy = -search_r; dy <= search_r; ++dy) {
                for (int dx = -search_r; dx <= search_r; ++dx) {
                    double d2 = 0.0;
                    for (int py = -patch_r; py <= patch_r; ++py) {
                        for (int px = -patch_r; px <= patch_r; ++px) {
                            long ia = (long)clampi(y + py, 0, height - 1) * width + clampi(x + px, 0, width - 1);
                            long ib = (long)clampi(y + dy + py, 0, height - 1) * width + clampi(x + dx + px, 0, width - 1);
                            for (int c = 0; c < 3; ++c) {
                                float a = rgb[ia * 3 + c], b = rgb[ib * 3 + c];
                                float va = var[ia * 3 + c], vb = var[ib * 3 + c];
                                float num = (a - b) * (a - b) - (va + fminf(va, vb));
                                d2 += (double)(num / (eps + k2 * (va + vb)));
                            }
                        }
                    }
                    float dd = (float)d2 * norm;
                    float wgt = expf(-fmaxf(0.0f, dd));
                    long iq = (long)clampi(y + dy, 0, height - 1) * width + clampi(x + dx, 0, width - 1);
                    sw += wgt;
                    for (int c = 0; c < 3; ++c) sum[c] += (double)wgt * rgb[iq * 3 + c];
                }
            }
            long io = (long)y * width + x;
            for (int c = 0; c < 3; ++c) out[io * 3 + c] = (float)(sum[c] / sw);
        }
    }
}
