// trace.cu -- closest-hit / any-hit kernels over ray arrays in HBM.
//
// Persistent warps: each warp takes a pool of consecutive rays from a global cursor, traces
// them (one thread per ray, traverse.cuh) and refills a lane as soon as its walk ends.  Rays
// are two float4 (org, tmin | dir, tmax) and hits one float4 (t, id, u, v): both read and
// written fully coalesced.  Replaces the per-pixel Scene::Intersect calls of the
// reference's OpenMP row loop (src/s3d_pt.cpp:310-333, include/s3d_scene.h:63-75).
//
// A launch walks one BVH, or a batch arena holding several scenes' BVHs back to back (then
// every ray names the root node of its scene), or a two-level BVH of instances: its top
// level's leaf entries are instances, and a ray reaching one is transformed into the
// instance's object space and walks the instance's mesh BVH, above a marker on its stack;
// popping the marker brings back the world ray and the top-level walk (instance.cu).
#include <algorithm>

#include "internal.h"
#include "traverse.cuh"

namespace salty {
namespace {

constexpr int kMaxStack = 63;  // stack entries per thread: BVHs up to 31 levels

// Rays per launch: ray indices are 32-bit in the kernel (three registers fewer than 64-bit
// ones); longer arrays are traced in consecutive launches of at most this many rays.
constexpr long long kMaxLaunchRays = 1ll << 30;

// counters: [0] ray cursor, [1] node fetches, [2] triangle fetches.  The register budget
// is set through the resident blocks asked for: 1024 / TB caps registers at 64 per thread,
// CAP's 1152 / TB at 56 for blocks of up to 128 threads (36 instead of 32 warps per SM to
// hide fetch latency, at the price of a few spilled values; 256-thread blocks stay at 64).
// The short stack lives in dynamic shared memory, `depth` entries per thread (one per BVH
// level plus one, or two per level plus one with postponing or instances; trace_launch
// sizes it) and one more for the best hit's (u, v), so shallow trees leave room for more
// resident blocks.
// Stack entry (.y) that marks where a ray entered an instance.
constexpr unsigned kInstMarker = 0x40000000u;

// SPH: leaf entries with ids from sph_base on are spheres (sphere.cu).
template <bool ANY, bool WT, bool COUNT, int TB, bool CAP, bool INST, bool SPH>
__global__ void __launch_bounds__(TB, CAP ? 1152 / TB : 1024 / TB)
k_trace(const Bvh8Node* __restrict__ nodes, const float4* __restrict__ tris, const float4* __restrict__ rays,
        const int* __restrict__ roots, long long n_arg, const int* __restrict__ n_dev, float4* __restrict__ hits,
        unsigned long long* __restrict__ counters, float cull_slack, int pool, int postpone, int depth,
        int* __restrict__ status, const InstRec* __restrict__ inst, int sph_base) {
    extern __shared__ uint2 sstack[];
    TravStack st{sstack + threadIdx.x, TB, depth};
    const int lane = threadIdx.x & 31;
    // queue length from device memory when given (wavefront queues), else the argument
    // (at most kMaxLaunchRays either way)
    const int n = n_dev ? *n_dev : (int)n_arg;
    TravCount cnt{0, 0};
    int overflow = 0;
    // Warp-uniform pool of ray indices [pool_next, pool_end), refilled `pool` at a time
    // from the global cursor; each lane holds one ray and takes a new one from the pool
    // as soon as its walk ends.  The cursor is 64-bit: warps that find the rays drained
    // may push it past 2^31.
    int pool_next = 0, pool_end = 0;
    bool drained = false;
    int rid = -1;
    TravRay r;
    TravState s;
    bool in_mesh = false;  // INST: walking an instance's mesh (else the top level)
    int vbase = 0;         // INST: virtual id of the current instance's first triangle
    for (;;) {
        const bool idle = rid < 0;
        const unsigned idle_mask = __ballot_sync(0xffffffffu, idle);
        if (idle_mask) {
            if (pool_next >= pool_end && !drained) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&counters[0], (unsigned long long)pool);
                base = __shfl_sync(0xffffffffu, base, 0);
                const long long end = (long long)base + pool;
                pool_next = (int)min((long long)base, (long long)n);
                pool_end = (int)min(end, (long long)n);
                if (end >= n) drained = true;
            }
            unsigned lt_mask;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt_mask));
            const int mine = pool_next + __popc(idle_mask & lt_mask);
            if (idle && mine < pool_end) {
                rid = mine;
                const float4 ra = __ldcs(rays + 2 * rid), rb = __ldcs(rays + 2 * rid + 1);
                make_trav_ray(r, ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z);
                trav_init(s, r, rb.w, roots ? (unsigned)__ldcs(roots + rid) : 0u);
                in_mesh = false;
                vbase = 0;
            }
            pool_next = min(pool_end, pool_next + __popc(idle_mask));
        }
        const bool active = rid >= 0;
        if (__ballot_sync(0xffffffffu, active) == 0) break;
        if (active && s.ng_hits) trav_node_step<COUNT>(s, nodes, r, st, cnt, overflow, cull_slack);
        // INST: a top-level leaf group holds instances; enter the first one, leaving the rest
        // of the group, the pending node group and a return marker on the stack
        if (INST && active && !in_mesh && s.tg_hits) {
            const unsigned k = __ffs(s.tg_hits) - 1;
            s.tg_hits &= s.tg_hits - 1;
            const int iid = __float_as_int(__ldg(tris + (size_t)(s.tg_base + k) * kTriFloat4).w);
            if (s.sp + 3 <= depth) {
                if (s.ng_hits) st.at(s.sp++) = make_uint2(s.ng_base, (s.ng_hits << 8) | s.ng_imask);
                if (s.tg_hits) st.at(s.sp++) = make_uint2(s.tg_base, s.tg_hits | kTriGroupFlag);
                st.at(s.sp++) = make_uint2(0u, kInstMarker);
                s.tg_hits = 0;
                const InstRec& R = inst[iid];
                const float* m = R.w2o;
                const float ox = fmaf(m[0], r.ox, fmaf(m[1], r.oy, fmaf(m[2], r.oz, m[3])));
                const float oy = fmaf(m[4], r.ox, fmaf(m[5], r.oy, fmaf(m[6], r.oz, m[7])));
                const float oz = fmaf(m[8], r.ox, fmaf(m[9], r.oy, fmaf(m[10], r.oz, m[11])));
                const float dx = fmaf(m[0], r.dx, fmaf(m[1], r.dy, m[2] * r.dz));
                const float dy = fmaf(m[4], r.dx, fmaf(m[5], r.dy, m[6] * r.dz));
                const float dz = fmaf(m[8], r.dx, fmaf(m[9], r.dy, m[10] * r.dz));
                make_trav_ray(r, ox, oy, oz, r.tmin, dx, dy, dz);
                s.ng_base = R.root;
                s.ng_hits = 1u << r.oct;
                s.ng_imask = 1u;
                in_mesh = true;
                vbase = R.vbase;
            } else {
                overflow = 1;
                s.ng_hits = 0;
                s.tg_hits = 0;
            }
        }
        // Triangle postponing: with too few lanes holding triangles, set the group aside
        // and keep walking nodes with the rest of the warp.
        // (postpone <= 1 never postpones: the warp-wide count is skipped)
        const bool want = active && s.tg_hits != 0 && (!INST || in_mesh);
        bool run = want;
        if (postpone > 1) {
            const unsigned want_mask = __ballot_sync(0xffffffffu, want);
            if (want && __popc(want_mask) < postpone && s.ng_hits != 0 && s.sp < depth) {
                st.at(s.sp++) = make_uint2(s.tg_base, s.tg_hits | kTriGroupFlag);
                s.tg_hits = 0;
                run = false;
            }
        }
        bool done = false;
        if (run) done = trav_tri_step<ANY, WT, COUNT, SPH>(s, tris, r, st, cnt, vbase, sph_base);
        bool more = true;
        if (INST && active && !done && !s.ng_hits && !s.tg_hits && s.sp > 0 &&
            st.at(s.sp - 1).y == kInstMarker) {
            // the instance's walk is over: back to the world ray and the top level
            --s.sp;
            const float4 ra = __ldcs(rays + 2 * rid), rb = __ldcs(rays + 2 * rid + 1);
            make_trav_ray(r, ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z);
            in_mesh = false;
            vbase = 0;
        } else if (active && !done) {
            more = trav_pop(s, st);
        }
        if (active && (done || !more)) {
            float4 h = make_float4(INFINITY, __int_as_float(-1), 0.0f, 0.0f);
            if (s.hit.id >= 0) {
                const uint2 uv = st.uv();
                h = make_float4(s.hit.t, __int_as_float(s.hit.id), __uint_as_float(uv.x), __uint_as_float(uv.y));
            }
            __stcs(hits + rid, h);
            rid = -1;
        }
    }
    if (COUNT) {
        unsigned long long a = cnt.nodes, b = cnt.tris;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (lane == 0) {
            atomicAdd(&counters[1], a);
            atomicAdd(&counters[2], b);
        }
    }
    if (overflow) atomicOr(status, 1);
}

struct Launch {
    const TraceTarget& tgt;
    const float4* rays;
    long long n;
    const int* n_dev;
    float4* hits;
    unsigned long long* counters;
    cudaStream_t st;
    float slack;
    int pool, postpone, depth;
    int* status;
};

template <bool ANY, bool WT, bool COUNT, int TB, bool CAP, bool INST, bool SPH = false>
salty_status launch(salty_ctx* ctx, const Launch& L) {
    auto kern = k_trace<ANY, WT, COUNT, TB, CAP, INST, SPH>;
    const size_t smem = (size_t)(L.depth + 1) * TB * sizeof(uint2);  // the stack and (u, v)
    if (smem > 48 * 1024)
        SALTY_TRY_CUDA(ctx->err, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SALTY_TRY_CUDA(ctx->err, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TB, smem));
    if (per_sm < 1) per_sm = 1;
    if (L.n_dev && L.n > kMaxLaunchRays)
        return ctx->err.fail(SALTY_ERR_CAPACITY, "ray queue capacity %lld exceeds %lld", L.n, kMaxLaunchRays);
    // consecutive launches of at most kMaxLaunchRays rays; each restarts the ray cursor
    for (long long off = 0; off == 0 || off < L.n; off += kMaxLaunchRays) {
        const long long n = std::min(L.n - off, kMaxLaunchRays);
        if (off > 0) SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(L.counters, 0, sizeof(unsigned long long), L.st));
        long long want = (n + TB - 1) / TB;
        long long grid = (long long)ctx->num_sms * per_sm;
        if (grid > want) grid = want;
        if (grid < 1) grid = 1;
        kern<<<(unsigned)grid, TB, smem, L.st>>>(L.tgt.nodes, L.tgt.tris, L.rays + 2 * off,
                                                 L.tgt.roots ? L.tgt.roots + off : nullptr, n, L.n_dev,
                                                 L.hits + off, L.counters, L.slack, L.pool, L.postpone, L.depth,
                                                 L.status, L.tgt.inst, L.tgt.sph_base);
        SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    }
    return SALTY_OK;
}

template <int TB, bool CAP>
salty_status dispatch_flags(salty_ctx* ctx, const Launch& L, uint32_t flags) {
    const bool any = flags & SALTY_TRACE_ANY_HIT, wt = flags & SALTY_TRACE_WATERTIGHT;
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, false, TB, CAP, false>(ctx, L)
    SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad trace flags");
}

// Two-level walks (instances), at the register budget of 64.
template <int TB>
salty_status dispatch_inst(salty_ctx* ctx, const Launch& L, uint32_t flags) {
    const bool any = flags & SALTY_TRACE_ANY_HIT, wt = flags & SALTY_TRACE_WATERTIGHT;
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, false, TB, false, true>(ctx, L)
    SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad trace flags");
}

// Scenes with spheres, at the register budget of 64.
template <int TB>
salty_status dispatch_sph(salty_ctx* ctx, const Launch& L, uint32_t flags) {
    const bool any = flags & SALTY_TRACE_ANY_HIT, wt = flags & SALTY_TRACE_WATERTIGHT;
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, false, TB, false, false, true>(ctx, L)
    SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad trace flags");
}

// Counting walks (node and triangle fetches) use the default launch shape.
salty_status dispatch_count(salty_ctx* ctx, const Launch& L, uint32_t flags) {
    const bool any = flags & SALTY_TRACE_ANY_HIT, wt = flags & SALTY_TRACE_WATERTIGHT;
    if (L.tgt.sph_base != kNoSpheres) {
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, true, 128, false, false, true>(ctx, L)
        SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    }
    if (L.tgt.inst) {
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, true, 128, false, true>(ctx, L)
        SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    }
#define SALTY_L(A, W) \
    if (any == A && wt == W) return launch<A, W, true, 128, false, false>(ctx, L)
    SALTY_L(false, false); SALTY_L(false, true); SALTY_L(true, false); SALTY_L(true, true);
#undef SALTY_L
    return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad trace flags");
}

}  // namespace

// Traces rays already resident on the device: n of them, or *n_dev when n_dev is given
// (then n is the capacity used to size the grid).  counters (3 x u64) are zeroed here.
salty_status trace_launch(salty_ctx* ctx, const TraceTarget& tgt, const TraceTuning& tune, const float4* d_rays,
                          long long n, const int* n_dev, uint32_t flags, float4* d_hits,
                          unsigned long long* d_counters, cudaStream_t st, int* d_status) {
    SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(d_counters, 0, 3 * sizeof(unsigned long long), st));
    const bool wt = flags & SALTY_TRACE_WATERTIGHT;
    // Without postponing, the walk keeps at most one pending node group per BVH level
    // (it pushes the rest of a group before descending into one of its children, and puts
    // back what is left of a group it pops); postponing adds a triangle group per level, and
    // instances their return markers.  A full stack is reported, never overrun.
    const bool two = tune.postpone > 1 || tgt.inst != nullptr;
    const int need = two ? 2 * tgt.depth + 1 : tgt.depth + 1;
    if (need > kMaxStack)
        return ctx->err.fail(SALTY_ERR_CAPACITY, "BVH depth %d needs %d traversal stack entries (at most %d)",
                             tgt.depth, need, kMaxStack);
    Launch L{tgt, d_rays, n, n_dev, d_hits, d_counters, st, wt ? (1.0f / 65536.0f) : 1e-3f,
             tune.pool >= 32 ? tune.pool : 32, tune.postpone, need, d_status};
    if (flags & SALTY_TRACE_COUNTERS) return dispatch_count(ctx, L, flags);
    if (tgt.sph_base != kNoSpheres) {
        if (tune.block == 64) return dispatch_sph<64>(ctx, L, flags);
        if (tune.block == 256) return dispatch_sph<256>(ctx, L, flags);
        return dispatch_sph<128>(ctx, L, flags);
    }
    if (tgt.inst) {
        if (tune.block == 64) return dispatch_inst<64>(ctx, L, flags);
        if (tune.block == 256) return dispatch_inst<256>(ctx, L, flags);
        return dispatch_inst<128>(ctx, L, flags);
    }
    const bool cap = tune.regs == 56;
#define SALTY_D(B) return cap ? dispatch_flags<B, true>(ctx, L, flags) : dispatch_flags<B, false>(ctx, L, flags)
    if (tune.block == 64) SALTY_D(64);
    if (tune.block == 256) SALTY_D(256);
    SALTY_D(128);
#undef SALTY_D
}

salty_status trace_launch(salty_ctx* ctx, salty_scene* sc, const float4* d_rays, long long n, const int* n_dev,
                          uint32_t flags, float4* d_hits, unsigned long long* d_counters, cudaStream_t st,
                          int* d_status) {
    TraceTarget t;
    t.nodes = sc->bvh.nodes.p;
    t.tris = sc->bvh.tris.p;
    t.depth = sc->bvh.depth;
    t.inst = sc->n_inst > 0 ? sc->inst_rec.p : nullptr;
    t.sph_base = sc->n_sph > 0 ? (int)sc->n_tris : kNoSpheres;
    return trace_launch(ctx, t, ctx->tune.trace, d_rays, n, n_dev, flags, d_hits, d_counters, st, d_status);
}

}  // namespace salty
