// trace.cu -- closest-hit / any-hit kernels over ray arrays in HBM.
//
// Persistent warps: each warp takes 32 consecutive rays from a global cursor, traces
// them (one thread per ray, traverse.cuh) and takes the next 32 when all are done.  Rays
// are two float4 (org, tmin | dir, tmax) and hits one float4 (t, id, u, v): both read and
// written fully coalesced.  Replaces the per-pixel Scene::Intersect calls of the
// reference's OpenMP row loop (src/s3d_pt.cpp:310-333, include/s3d_scene.h:63-75).
#include "internal.h"
#include "traverse.cuh"

namespace salty {
namespace {

constexpr int kTraceBlock = 128;
constexpr int kPool = 128;          // rays taken from the global cursor per refill
constexpr int kPostponeLanes = 7;   // test triangles only with at least this many lanes

// counters: [0] ray cursor, [1] node fetches, [2] triangle fetches
template <bool ANY, bool WT, bool COUNT, int DEPTH>
__global__ void __launch_bounds__(kTraceBlock)
k_trace(const Bvh8Node* __restrict__ nodes, const float4* __restrict__ tris, const float4* __restrict__ rays,
        long long n_arg, const int* __restrict__ n_dev, float4* __restrict__ hits,
        unsigned long long* __restrict__ counters, float cull_slack, int* __restrict__ status) {
    __shared__ uint2 sstack[DEPTH * kTraceBlock];
    TravStack<DEPTH> st{sstack + threadIdx.x, kTraceBlock};
    const int lane = threadIdx.x & 31;
    // queue length from device memory when given (wavefront queues), else the argument
    const long long n = n_dev ? (long long)*n_dev : n_arg;
    const unsigned lt_mask = (1u << lane) - 1u;
    TravCount cnt{0, 0};
    int overflow = 0;
    // Warp-uniform pool of ray indices [pool_next, pool_end), refilled kPool at a time
    // from the global cursor; each lane holds one ray and takes a new one from the pool
    // as soon as its walk ends.
    long long pool_next = 0, pool_end = 0;
    bool drained = false;
    long long rid = -1;
    TravRay r;
    TravState s;
    for (;;) {
        const bool idle = rid < 0;
        const unsigned idle_mask = __ballot_sync(0xffffffffu, idle);
        if (idle_mask) {
            if (pool_next >= pool_end && !drained) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&counters[0], (unsigned long long)kPool);
                base = __shfl_sync(0xffffffffu, base, 0);
                pool_next = (long long)base;
                pool_end = min((long long)base + kPool, n);
                if ((long long)base + kPool >= n) drained = true;
            }
            const long long mine = pool_next + __popc(idle_mask & lt_mask);
            if (idle && mine < pool_end) {
                rid = mine;
                const float4 ra = __ldcs(rays + 2 * rid), rb = __ldcs(rays + 2 * rid + 1);
                make_trav_ray(r, ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w);
                trav_init(s, r);
            }
            pool_next = min(pool_end, pool_next + __popc(idle_mask));
        }
        const bool active = rid >= 0;
        if (__ballot_sync(0xffffffffu, active) == 0) break;
        if (active && s.ng_hits) trav_node_step<DEPTH, COUNT>(s, nodes, r, st, cnt, overflow);
        // Triangle postponing: with too few lanes holding triangles, set the group aside
        // and keep walking nodes with the rest of the warp.
        const bool want = active && s.tg_hits != 0;
        const unsigned want_mask = __ballot_sync(0xffffffffu, want);
        bool run = want;
        if (want && __popc(want_mask) < kPostponeLanes && s.ng_hits != 0 && s.sp < DEPTH) {
            st.at(s.sp++) = make_uint2(s.tg_base, s.tg_hits | kTriGroupFlag);
            s.tg_hits = 0;
            run = false;
        }
        bool done = false;
        if (run) done = trav_tri_step<ANY, WT, COUNT>(s, tris, r, cull_slack, cnt);
        if (active && (done || !trav_pop(s, st))) {
            __stcs(hits + rid, make_float4(s.hit.t, __int_as_float(s.hit.id), s.hit.u, s.hit.v));
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

template <bool ANY, bool WT, bool COUNT, int DEPTH>
salty_status launch(salty_ctx* ctx, salty_scene* sc, const float4* rays, long long n, const int* n_dev, float4* hits,
                    unsigned long long* counters, cudaStream_t st, float cull_slack, int* status) {
    auto kern = k_trace<ANY, WT, COUNT, DEPTH>;
    int per_sm = 0;
    SALTY_TRY_CUDA(ctx->err, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTraceBlock, 0));
    if (per_sm < 1) per_sm = 1;
    long long want = (n + kTraceBlock - 1) / kTraceBlock;
    long long grid = (long long)ctx->num_sms * per_sm;
    if (grid > want) grid = want;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, kTraceBlock, 0, st>>>(sc->bvh.nodes.p, sc->bvh.tris.p, rays, n, n_dev, hits, counters,
                                                cull_slack, status);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

template <int DEPTH>
salty_status dispatch_depth(salty_ctx* ctx, salty_scene* sc, const float4* rays, long long n, const int* n_dev,
                            uint32_t flags, float4* hits, unsigned long long* counters, cudaStream_t st,
                            int* status) {
    const bool any = flags & SALTY_TRACE_ANY_HIT, wt = flags & SALTY_TRACE_WATERTIGHT,
               cnt = flags & SALTY_TRACE_COUNTERS;
    const float slack = wt ? (1.0f / 65536.0f) : 1e-3f;
#define SALTY_L(A, W, C) \
    if (any == A && wt == W && cnt == C) return launch<A, W, C, DEPTH>(ctx, sc, rays, n, n_dev, hits, counters, st, slack, status)
    SALTY_L(false, false, false); SALTY_L(false, false, true); SALTY_L(false, true, false); SALTY_L(false, true, true);
    SALTY_L(true, false, false); SALTY_L(true, false, true); SALTY_L(true, true, false); SALTY_L(true, true, true);
#undef SALTY_L
    return ctx->err.fail(SALTY_ERR_INVALID_ARG, "bad trace flags");
}

}  // namespace

// Traces rays already resident on the device: n of them, or *n_dev when n_dev is given
// (then n is the capacity used to size the grid).  counters (3 x u64) are zeroed here.
salty_status trace_launch(salty_ctx* ctx, salty_scene* sc, const float4* d_rays, long long n, const int* n_dev,
                          uint32_t flags, float4* d_hits, unsigned long long* d_counters, cudaStream_t st,
                          int* d_status) {
    SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(d_counters, 0, 3 * sizeof(unsigned long long), st));
    // Each BVH level can hold one pending node group and one postponed triangle group.
    if (2 * sc->bvh.depth + 1 <= 24)
        return dispatch_depth<24>(ctx, sc, d_rays, n, n_dev, flags, d_hits, d_counters, st, d_status);
    if (2 * sc->bvh.depth + 1 <= 48)
        return dispatch_depth<48>(ctx, sc, d_rays, n, n_dev, flags, d_hits, d_counters, st, d_status);
    return ctx->err.fail(SALTY_ERR_CAPACITY, "BVH depth %d exceeds the traversal stack (23 levels)", sc->bvh.depth);
}

}  // namespace salty
