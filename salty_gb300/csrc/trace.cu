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
    TravCount cnt{0, 0};
    int overflow = 0;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&counters[0], 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned long long)n) break;
        const long long i = (long long)base + lane;
        if (i < n) {
            const float4 ra = __ldcs(rays + 2 * i), rb = __ldcs(rays + 2 * i + 1);
            TravRay r;
            make_trav_ray(r, ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w);
            TravHit h;
            traverse<ANY, WT, COUNT, DEPTH>(nodes, tris, r, cull_slack, st, h, cnt, overflow);
            __stcs(hits + i, make_float4(h.t, __int_as_float(h.id), h.u, h.v));
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
    if (sc->bvh.depth <= 16)
        return dispatch_depth<16>(ctx, sc, d_rays, n, n_dev, flags, d_hits, d_counters, st, d_status);
    if (sc->bvh.depth <= 40)
        return dispatch_depth<40>(ctx, sc, d_rays, n, n_dev, flags, d_hits, d_counters, st, d_status);
    return ctx->err.fail(SALTY_ERR_CAPACITY, "BVH depth %d exceeds the traversal stack (40)", sc->bvh.depth);
}

}  // namespace salty
