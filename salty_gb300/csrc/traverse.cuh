// traverse.cuh -- device-side closest/any-hit traversal of the quantised BVH8.
//
// Replaces the recursive virtual walk BVH8::IsHit -> BoundingBox8::IsHit ->
// Leaf::IsHit -> Triangle::IsHit (src/s3d_bvh8.cpp:191-206, include/s3d_math.h:
// 2549-2586, src/s3d_leaf.cpp:74-87, src/s3d_triangle.cpp:73-105).  One thread per ray;
// a node is five 16-byte loads; child boxes are tested against [tmin, best t] (the
// reference tests the whole line) and visited nearest-octant first; the stack of
// pending child groups lives in shared memory.  The loop follows the compressed wide
// BVH traversal published by Ylitie, Karras and Laine (HPG 2017).
#pragma once

#include <cfloat>
#include <cstdint>

#include "internal.h"

namespace salty {

// Group stack entry: x = child base index, y = (hit bits in key order << 8) | imask.
// One more entry per thread, after the stack, holds the best hit's (u, v), which is
// written only when the best hit changes and read once at the end of the walk: two
// registers fewer for the whole walk.
struct TravStack {
    uint2* base;    // shared memory, [depth + 1][blockDim]
    int stride;     // blockDim.x
    int depth;      // stack entries per thread
    __device__ __forceinline__ uint2& at(int i) const { return base[i * stride]; }
    __device__ __forceinline__ uint2& uv() const { return base[depth * stride]; }
};

// The ray's tmax is not kept here: the walk starts with the best distance at tmax
// (TravHit::t) and only ever lowers it.
struct TravRay {
    float ox, oy, oz, dx, dy, dz;
    float ix, iy, iz;        // 1/d with zero components replaced by tiny values
    float tmin;
    unsigned oct;            // bit a set when d[a] < 0
    // watertight shear constants
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

// Best hit so far: t starts at tmax (or +inf when tmax is NaN, which bounds nothing) and
// id at -1, which compares as the largest unsigned id, so a triangle at exactly tmax is
// still taken.  (u, v) live in TravStack::uv().
struct TravHit {
    float t;
    int id;
};

struct TravCount {
    unsigned nodes, tris;
};

__device__ __forceinline__ float safe_rcp(float d) {
    float ad = fabsf(d);
    if (ad < 1e-30f) d = copysignf(1e-30f, d);
    return __frcp_rn(d);
}

__device__ __forceinline__ void make_trav_ray(TravRay& r, float ox, float oy, float oz, float tmin, float dx,
                                              float dy, float dz) {
    r.ox = ox; r.oy = oy; r.oz = oz; r.dx = dx; r.dy = dy; r.dz = dz;
    r.tmin = fmaxf(tmin, 0.0f);  // a negative tmin is treated as 0
    r.ix = safe_rcp(dx); r.iy = safe_rcp(dy); r.iz = safe_rcp(dz);
    r.oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    float ad[3] = {fabsf(dx), fabsf(dy), fabsf(dz)};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float d[3] = {dx, dy, dz};
    if (d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = __fdiv_rn(d[kx], d[kz]);
    r.Sy = __fdiv_rn(d[ky], d[kz]);
    r.Sz = __fdiv_rn(1.0f, d[kz]);
}

// ---------------------------------------------------------------- triangle tests
// The reference's test (src/s3d_triangle.cpp:73-105), operation for operation, with
// every product and sum rounded separately (no fused multiply-add) and IEEE division,
// so t, beta and gamma equal the reference's bit for bit.  The divisions are the costly
// part, so candidates are first rejected without them wherever the outcome is already
// certain: a numerator of the wrong sign (the quotient's sign is exact), or
// |nb| + |ng| clearly above |div| (beta + gamma >= 1 after every rounding), or
// |nt| clearly above |div| * tfar (t beyond the farthest useful distance).  "Clearly"
// is a relative margin of 2^-16, far above the few ulps the roundings can move.
// Candidates inside the margins take the exact path.  tfar is the current closest hit
// (or tmax): equal distances still reach the exact path, for the lowest-id tie rule.
__device__ __forceinline__ bool tri_ref(const TravRay& r, float4 a, float4 b, float4 c, float tmin, float tmax,
                                        float tfar, float& t, float& u, float& v) {
    const float e1x = __fsub_rn(b.x, a.x), e1y = __fsub_rn(b.y, a.y), e1z = __fsub_rn(b.z, a.z);
    const float e2x = __fsub_rn(c.x, a.x), e2y = __fsub_rn(c.y, a.y), e2z = __fsub_rn(c.z, a.z);
    const float s1x = __fsub_rn(__fmul_rn(r.dy, e2z), __fmul_rn(r.dz, e2y));
    const float s1y = __fsub_rn(__fmul_rn(r.dz, e2x), __fmul_rn(r.dx, e2z));
    const float s1z = __fsub_rn(__fmul_rn(r.dx, e2y), __fmul_rn(r.dy, e2x));
    const float div = __fadd_rn(__fadd_rn(__fmul_rn(s1x, e1x), __fmul_rn(s1y, e1y)), __fmul_rn(s1z, e1z));
    if (fabsf(div) <= FLT_EPSILON) return false;
    const float dvx = __fsub_rn(r.ox, a.x), dvy = __fsub_rn(r.oy, a.y), dvz = __fsub_rn(r.oz, a.z);
    const float nb = __fadd_rn(__fadd_rn(__fmul_rn(dvx, s1x), __fmul_rn(dvy, s1y)), __fmul_rn(dvz, s1z));
    if (nb == 0.0f || (__float_as_uint(nb) ^ __float_as_uint(div)) >> 31) return false;  // beta <= 0
    const float s2x = __fsub_rn(__fmul_rn(dvy, e1z), __fmul_rn(dvz, e1y));
    const float s2y = __fsub_rn(__fmul_rn(dvz, e1x), __fmul_rn(dvx, e1z));
    const float s2z = __fsub_rn(__fmul_rn(dvx, e1y), __fmul_rn(dvy, e1x));
    const float ng = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, s2x), __fmul_rn(r.dy, s2y)), __fmul_rn(r.dz, s2z));
    if (ng == 0.0f || (__float_as_uint(ng) ^ __float_as_uint(div)) >> 31) return false;  // gamma <= 0
    const float ad = fabsf(div);
    constexpr float kMargin = 1.0f + 1.0f / 65536.0f;
    if (fabsf(nb) + fabsf(ng) > ad * kMargin) return false;                             // beta + gamma >= 1
    const float nt = __fadd_rn(__fadd_rn(__fmul_rn(e2x, s2x), __fmul_rn(e2y, s2y)), __fmul_rn(e2z, s2z));
    if (fabsf(nt) > ad * (tfar * kMargin)) return false;                                 // t > tfar
    const float beta = __fdiv_rn(nb, div);
    if (beta <= 0.0f || beta >= 1.0f) return false;
    const float gamma = __fdiv_rn(ng, div);
    if (gamma <= 0.0f || __fadd_rn(beta, gamma) >= 1.0f) return false;
    const float dist = __fdiv_rn(nt, div);
    if (!(dist >= tmin) || dist > tmax) return false;
    t = dist; u = beta; v = gamma;
    return true;
}

// Watertight test (Woop, Benthin, Wald, JCGT 2013) without fused operations, so an edge
// shared by two triangles gets the same edge function with opposite sign in both.
__device__ __forceinline__ bool tri_watertight(const TravRay& r, float4 a, float4 b, float4 c, float tmin,
                                               float tmax, float& t, float& u, float& v) {
    // vertices relative to the origin, components permuted to (kx, ky, kz) with selects
    // (no dynamically indexed arrays, which would live in local memory)
    auto pick = [](float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); };
    const float a0 = __fsub_rn(a.x, r.ox), a1 = __fsub_rn(a.y, r.oy), a2 = __fsub_rn(a.z, r.oz);
    const float b0 = __fsub_rn(b.x, r.ox), b1 = __fsub_rn(b.y, r.oy), b2 = __fsub_rn(b.z, r.oz);
    const float c0 = __fsub_rn(c.x, r.ox), c1 = __fsub_rn(c.y, r.oy), c2 = __fsub_rn(c.z, r.oz);
    const float aX = pick(a0, a1, a2, r.kx), aY = pick(a0, a1, a2, r.ky), aZ = pick(a0, a1, a2, r.kz);
    const float bX = pick(b0, b1, b2, r.kx), bY = pick(b0, b1, b2, r.ky), bZ = pick(b0, b1, b2, r.kz);
    const float cX = pick(c0, c1, c2, r.kx), cY = pick(c0, c1, c2, r.ky), cZ = pick(c0, c1, c2, r.kz);
    const float Ax = __fsub_rn(aX, __fmul_rn(r.Sx, aZ)), Ay = __fsub_rn(aY, __fmul_rn(r.Sy, aZ));
    const float Bx = __fsub_rn(bX, __fmul_rn(r.Sx, bZ)), By = __fsub_rn(bY, __fmul_rn(r.Sy, bZ));
    const float Cx = __fsub_rn(cX, __fmul_rn(r.Sx, cZ)), Cy = __fsub_rn(cY, __fmul_rn(r.Sy, cZ));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.Sz, aZ), Bz = __fmul_rn(r.Sz, bZ), Cz = __fmul_rn(r.Sz, cZ);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    if (det > 0.0f) {
        if (T < __fmul_rn(tmin, det) || T > __fmul_rn(tmax, det)) return false;
    } else {
        if (T > __fmul_rn(tmin, det) || T < __fmul_rn(tmax, det)) return false;
    }
    const float rcp = __frcp_rn(det);
    t = __fmul_rn(T, rcp);
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    if (!(t >= tmin) || t > tmax) return false;
    return true;
}

// ---------------------------------------------------------------- sphere tests
// Sphere::IsHit (src/s3d_sphere.cpp:66-92) operation for operation: po = c - o,
// b = po.d, D4 = b^2 - po.po + r^2, roots b -/+ sqrt(D4); the nearer root above tmin,
// else the farther (the direction is taken as unit, as the reference does).
__device__ __forceinline__ bool sph_ref(const TravRay& r, float4 c, float rad, float tmin, float tmax, float& t) {
    const float px = __fsub_rn(c.x, r.ox), py = __fsub_rn(c.y, r.oy), pz = __fsub_rn(c.z, r.oz);
    const float b = __fadd_rn(__fadd_rn(__fmul_rn(px, r.dx), __fmul_rn(py, r.dy)), __fmul_rn(pz, r.dz));
    const float pp = __fadd_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)), __fmul_rn(pz, pz));
    const float D4 = __fadd_rn(__fsub_rn(__fmul_rn(b, b), pp), __fmul_rn(rad, rad));
    if (D4 < 0.0f) return false;
    const float sq = __fsqrt_rn(D4);
    const float t1 = __fsub_rn(b, sq), t2 = __fadd_rn(b, sq);
    if (t1 < tmin && t2 < tmin) return false;
    t = t1 > tmin ? t1 : t2;
    return t <= tmax;
}

// The same intersection without the cancellation of b^2 - po.po for small or distant
// spheres (Haines, Guenther, Akenine-Moller, "Precision Improvements for Ray/Sphere
// Intersection", Ray Tracing Gems, 2019): the discriminant from the distance between the
// centre and the ray's closest point, the roots from the stable quadratic formula; any
// direction length.
__device__ __forceinline__ bool sph_robust(const TravRay& r, float4 c, float rad, float tmin, float tmax, float& t) {
    const float fx = r.ox - c.x, fy = r.oy - c.y, fz = r.oz - c.z;
    const float a = r.dx * r.dx + r.dy * r.dy + r.dz * r.dz;
    const float b = -(fx * r.dx + fy * r.dy + fz * r.dz);  // half of -B
    const float k = b / a;
    const float lx = fx + k * r.dx, ly = fy + k * r.dy, lz = fz + k * r.dz;
    const float disc = a * (rad * rad - (lx * lx + ly * ly + lz * lz));
    if (disc < 0.0f) return false;
    // roots (b +- sqrt(disc)) / a: the one without cancellation first, the other from
    // their product cc / a
    const float cc = fx * fx + fy * fy + fz * fz - rad * rad;
    const float q = b + copysignf(sqrtf(disc), b);
    float t0 = q / a, t1 = q != 0.0f ? cc / q : t0;
    if (t0 > t1) { const float x = t0; t0 = t1; t1 = x; }
    t = t0 >= tmin ? t0 : t1;
    return t >= tmin && t <= tmax;
}

__device__ __forceinline__ float fmax4(float a, float b, float c, float d) {
    float m;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
    return fmaxf(m, d);
}
__device__ __forceinline__ float fmin4(float a, float b, float c, float d) {
    float m;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
    return fminf(m, d);
}

// Widening of the far plane (tn >= tmin >= 0): covers the rounding of the decoded
// planes, of 1/d and of the fused plane evaluation, so the quantised-box test never
// rejects a box the exact ray segment meets.
constexpr float kBoxSlackMul = 1.0f + 1.0f / (1 << 17);

// Two FP32 values in one 64-bit register pair, for the packed FP32 instructions of sm_100
// and later (add/fma .f32x2: one issue slot for two values).
__device__ __forceinline__ unsigned long long f2_pack(unsigned lo, unsigned hi) {
    unsigned long long v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "r"(lo), "r"(hi));
    return v;
}

// A child's near and far plane bytes along one axis as exact floats: each byte placed under
// the exponent of 2^23 (one byte permute each), then 2^23 taken off both with one packed
// subtraction (exact for 0..255) -- two issue slots fewer per child and axis than two
// separate subtractions.
__device__ __forceinline__ void q2(unsigned wn, unsigned wf, int k, unsigned long long off, float& qn, float& qf) {
    unsigned long long q = f2_pack(__byte_perm(wn, 0x4B000000u, 0x7540u + k),
                                   __byte_perm(wf, 0x4B000000u, 0x7540u + k));
    asm("sub.rn.f32x2 %0, %0, %1;" : "+l"(q) : "l"(off));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(qn), "=f"(qf) : "l"(q));
}

// Intersects the 8 children of node `idx`.  Returns inner-child hits in key order
// (bit slot^oct) and triangle hits relative to tri_base.
__device__ __forceinline__ void intersect_node(const Bvh8Node* __restrict__ nodes, unsigned idx, const TravRay& r,
                                               float tcull, unsigned& child_base, unsigned& imask,
                                               unsigned& inner_hits, unsigned& tri_base, unsigned& tri_hits) {
    const uint4* np = reinterpret_cast<const uint4*>(nodes + idx);
    const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    const float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    imask = w0.w >> 24;
    child_base = w1.x;
    tri_base = w1.y;
    const float ax = sx * r.ix, ay = sy * r.iy, az = sz * r.iz;
    const float bx = (px - r.ox) * r.ix, by = (py - r.oy) * r.iy, bz = (pz - r.oz) * r.iz;
    // near/far plane words by ray octant
    const unsigned nlx0 = (r.oct & 1) ? w3.z : w2.x, nlx1 = (r.oct & 1) ? w3.w : w2.y;
    const unsigned nhx0 = (r.oct & 1) ? w2.x : w3.z, nhx1 = (r.oct & 1) ? w2.y : w3.w;
    const unsigned nly0 = (r.oct & 2) ? w4.x : w2.z, nly1 = (r.oct & 2) ? w4.y : w2.w;
    const unsigned nhy0 = (r.oct & 2) ? w2.z : w4.x, nhy1 = (r.oct & 2) ? w2.w : w4.y;
    const unsigned nlz0 = (r.oct & 4) ? w4.z : w3.x, nlz1 = (r.oct & 4) ? w4.w : w3.y;
    const unsigned nhz0 = (r.oct & 4) ? w3.x : w4.z, nhz1 = (r.oct & 4) ? w3.y : w4.w;
    // Inner-child meta bytes hold 24 + slot; XOR-ing their low three bits with the ray
    // octant turns that into 24 + key, so one shift per child places inner hits in bits
    // 24..31 (key order) and leaf triangles in bits 0..23.
    const unsigned spread_lo = (((imask & 0x0fu) * 0x00204081u) & 0x01010101u) * r.oct;
    const unsigned spread_hi = ((((imask >> 4) & 0x0fu) * 0x00204081u) & 0x01010101u) * r.oct;
    const unsigned long long off = f2_pack(0x4B000000u, 0x4B000000u);  // 2^23, twice
    unsigned hits = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const unsigned lx = half ? nlx1 : nlx0, hx = half ? nhx1 : nhx0;
        const unsigned ly = half ? nly1 : nly0, hy = half ? nhy1 : nhy0;
        const unsigned lz = half ? nlz1 : nlz0, hz = half ? nhz1 : nhz0;
        const unsigned meta = half ? (w1.w ^ spread_hi) : (w1.z ^ spread_lo);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float qnx, qfx, qny, qfy, qnz, qfz;
            q2(lx, hx, k, off, qnx, qfx);
            q2(ly, hy, k, off, qny, qfy);
            q2(lz, hz, k, off, qnz, qfz);
            const float tnx = fmaf(qnx, ax, bx), tfx = fmaf(qfx, ax, bx);
            const float tny = fmaf(qny, ay, by), tfy = fmaf(qfy, ay, by);
            const float tnz = fmaf(qnz, az, bz), tfz = fmaf(qfz, az, bz);
            const float tn = fmax4(tnx, tny, tnz, r.tmin);
            const float tf = fmin4(tfx, tfy, tfz, tcull);
            if (tn <= tf * kBoxSlackMul) {
                // the slot's bit pattern shifted into place; the funnel shift takes its
                // amount modulo 32, so the meta byte needs no masking
                const unsigned m = __byte_perm(meta, 0u, 0x4440u + k);
                hits |= __funnelshift_l(0u, m >> 5, m);
            }
        }
    }
    inner_hits = hits >> 24;
    tri_hits = hits & 0x00ffffffu;
}

// ---------------------------------------------------------------- stepwise walk
// The walk of one ray as explicit state, advanced one node (and its triangles) per step,
// so a warp can keep every lane busy: finished lanes take new rays while the others
// continue (k_trace), and triangle groups can be set aside on the stack (postponed)
// while too few lanes of the warp have triangles to test.
struct TravState {
    unsigned ng_base, ng_hits, ng_imask;  // current node group (hits in key order)
    unsigned tg_base, tg_hits;            // current triangle group
    int sp;
    TravHit hit;
};

// Stack entries with this flag in .y are postponed triangle groups.
constexpr unsigned kTriGroupFlag = 0x80000000u;

// root: index of the BVH's root node (0 for one scene; a scene's offset in a batch arena)
__device__ __forceinline__ void trav_init(TravState& s, const TravRay& r, float tmax, unsigned root = 0) {
    s.ng_base = root;
    s.ng_hits = 1u << r.oct;  // a group holding only the root, in slot 0
    s.ng_imask = 1u;
    s.tg_base = 0;
    s.tg_hits = 0;
    s.sp = 0;
    s.hit.t = tmax == tmax ? tmax : INFINITY;
    s.hit.id = -1;
}

// Visits the nearest pending child of the current node group.  A full stack drops the
// remaining group and raises `overflow` (reported to the caller as an error).
// Boxes are culled beyond the best distance times (1 + cull_slack): a relative margin
// over the triangle test's rounding, so the answer never depends on what was culled.
template <bool COUNT>
__device__ __forceinline__ void trav_node_step(TravState& s, const Bvh8Node* __restrict__ nodes, const TravRay& r,
                                               TravStack st, TravCount& cnt, int& overflow, float cull_slack) {
    const unsigned key = __ffs(s.ng_hits) - 1;
    s.ng_hits &= s.ng_hits - 1;
    const unsigned slot = key ^ r.oct;
    const unsigned idx = s.ng_base + __popc(s.ng_imask & ((1u << slot) - 1u));
    if (s.ng_hits) {
        if (s.sp < st.depth) st.at(s.sp++) = make_uint2(s.ng_base, (s.ng_hits << 8) | s.ng_imask);
        else overflow = 1;
    }
    unsigned cb, im, ih, tb, th;
    intersect_node(nodes, idx, r, fmaf(cull_slack, s.hit.t, s.hit.t), cb, im, ih, tb, th);
    if (COUNT) ++cnt.nodes;
    s.ng_base = cb;
    s.ng_imask = im;
    s.ng_hits = ih;
    s.tg_base = tb;
    s.tg_hits = th;
}

// Tests the triangles of the current group.  Closest hit: smallest t, equal t to the
// lowest id, every candidate bounded by the best distance so far (tmax at first).
// Returns true when an any-hit query has its answer.
// SPH: leaf entries with ids from sph_base on are spheres, (centre, id) (radius, 0, 0, 0).
template <bool ANY, bool WATERTIGHT, bool COUNT, bool SPH = false>
__device__ __forceinline__ bool trav_tri_step(TravState& s, const float4* __restrict__ tris, const TravRay& r,
                                              TravStack st, TravCount& cnt, int id_off = 0,
                                              int sph_base = 0x7fffffff) {
    while (s.tg_hits) {
        const unsigned k = __ffs(s.tg_hits) - 1;
        s.tg_hits &= s.tg_hits - 1;
        const float4* tp = tris + (size_t)(s.tg_base + k) * kTriFloat4;
        const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (COUNT) ++cnt.tris;
        float t, u, v;
        const float tlim = s.hit.t;
        bool h;
        if (SPH && __float_as_int(a.w) >= sph_base) {
            h = WATERTIGHT ? sph_robust(r, a, b.x, r.tmin, tlim, t) : sph_ref(r, a, b.x, r.tmin, tlim, t);
            u = 0.0f;
            v = 0.0f;
        } else {
            h = WATERTIGHT ? tri_watertight(r, a, b, c, r.tmin, tlim, t, u, v)
                           : tri_ref(r, a, b, c, r.tmin, tlim, tlim, t, u, v);
        }
        if (h) {
            const int id = __float_as_int(a.w) + id_off;  // an instance's first virtual id
            if (t < s.hit.t || (t == s.hit.t && (unsigned)id < (unsigned)s.hit.id)) {
                s.hit.t = t;
                s.hit.id = id;
                st.uv() = make_uint2(__float_as_uint(u), __float_as_uint(v));
                if (ANY) return true;
            }
        }
    }
    return false;
}

// Makes a group current when both are exhausted.  Returns false when the walk is over.
__device__ __forceinline__ bool trav_pop(TravState& s, TravStack st) {
    if (s.ng_hits || s.tg_hits) return true;
    if (s.sp == 0) return false;
    const uint2 e = st.at(--s.sp);
    if (e.y & kTriGroupFlag) {
        s.tg_base = e.x;
        s.tg_hits = e.y & ~kTriGroupFlag;
    } else {
        s.ng_base = e.x;
        s.ng_hits = e.y >> 8;
        s.ng_imask = e.y & 0xffu;
    }
    return true;
}

}  // namespace salty
