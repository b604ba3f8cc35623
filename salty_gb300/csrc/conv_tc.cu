// conv_tc.cu -- the denoiser's 3x3 convolutions on the fifth-generation tensor cores.
//
// Implicit GEMM with the accumulators in tensor memory (TMEM).  One CTA computes a strip of
// R image rows x 128 pixels and all output channels:
//   M = 128 pixels of one image row (TMEM lane i holds pixel x0 + i),
//   N = output channels, padded to a multiple of 16 (16..256),
//   K = 9 taps x Cin, walked 16 input channels (one MMA's K) at a time.
// Operands sit in shared memory in the tensor core's K-major layout without swizzle: "core
// matrices" of 8 rows x 16 bytes (8 BF16 channels), 128 contiguous bytes each.  The
// descriptors' leading byte offset is the distance between the two 8-channel halves of K,
// the stride byte offset the distance between consecutive 8-row groups (128 B here).
//   halo  [2 channel octets][R + 2 rows][130 pixels][8 channels] -- output row r, tap
//         (ky, kx) reads the 128-pixel window starting at halo pixel (r + ky, kx), so the A
//         descriptor of every tap is the same tile with its start moved 16 B per pixel
//   wts   [9 taps][2 channel octets][Npad rows][8 channels]
// Both are staged per 16-channel chunk into one of two buffers with cp.async (zero fill
// outside the image and beyond the real output channels).  Lane 0 of each warp issues the
// chunk's MMAs for its rows (tcgen05.mma kind::f16, BF16 x BF16 -> FP32) and commits them
// to that buffer's mbarrier (4 arrivals); the loaders wait on it before refilling the
// buffer.  R x Npad <= 256
// FP32 accumulator columns are allocated per CTA.  Epilogue: tcgen05.ld of each row's
// columns, bias, ReLU, BF16, 16-byte stores.
//
// Every wait is bounded (2 s of the global timer); a wait that gives up sets
// status[0] |= 1, skips the rest of the strip, frees the CTA's TMEM and returns.
//
// k_conv3x3_tma is the same convolution for inputs held in one tensor, as a persistent,
// warp-specialised kernel (one CTA per SM looping over strips):
//   warp 0    one lane issues TMA tensor copies (cp.async.bulk.tensor): per 16-channel
//             chunk the halo (a box of 16 channels x 130 pixels x R+2 rows, the image
//             border zero-filled by the copy engine) and the weights (16 channels x Npad
//             rows x 9 taps) into a ring of up to 4 stages, each guarded by a "full"
//             (transaction bytes) and an "empty" (MMAs done) mbarrier.  A layer whose
//             weights fit in 48 KB has them copied once, before the first strip, into a
//             region of their own (its own mbarrier), and its stages hold only halos.  Both land in the
//             tensor core's 32-byte-swizzled K-major layout: one 32-byte row per pixel (or
//             weight row), the two 16-byte halves of a row exchanged where address bit 7 is
//             set.  The MMA unit undoes the exchange from the absolute shared-memory
//             address, so a tap's A operand still starts at any pixel of the halo (32-byte
//             steps, descriptor base offset 0) -- measured on this GPU with exact integer
//             products at row offsets 0-131.
//   warps 1-8 one lane each issues the MMAs of its row of the strip (r = m) and commits
//             them to the stage's "empty" barrier, and after a strip's last chunk to its
//             accumulator's barrier: one thread issues an MMA about every 100 cycles,
//             several issuing threads keep the tensor pipe fed with these small N <= 96
//             MMAs (measured: 4 issuers 1.35x faster than 1 on the 32-channel layers)
//   warps 9-12 the epilogue: TMEM -> bias, ReLU, BF16 -> global, one warp per TMEM lane
//             quarter, then release the accumulator
// Two accumulators of R x Npad columns (512 TMEM columns) let the epilogue of one strip
// overlap the MMAs of the next.  Waits are bounded as above; a wait that gives up raises
// a shared abort flag that ends every role's loop.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched from the driver at run time)
#include <cuda_bf16.h>

#include <cstdint>

#include "internal.h"
#include "unet_src.cuh"

namespace salty {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTcThreads = 128;
constexpr int kStrip = 128;              // pixels per image row of a strip (the MMA's M)
constexpr int kHaloW = kStrip + 2;       // staged pixels per halo row
constexpr int kTmemCols = 256;           // accumulator columns per CTA
constexpr int kBarBytes = 128;           // mbarriers + TMEM address at the start of shared memory
constexpr unsigned long long kWaitNs = 2000000000ull;

__host__ __device__ constexpr int halo_bytes(int R) { return 2 * (R + 2) * kHaloW * 16; }
__host__ __device__ constexpr int wts_bytes(int npad) { return 9 * 2 * npad * 16; }
__host__ __device__ constexpr int stage_bytes(int R, int npad) { return (halo_bytes(R) + wts_bytes(npad) + 127) / 128 * 128; }

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading and stride byte offsets (all >> 4), the
// descriptor version bit of this architecture (bit 46), no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try(bar, parity))
        if (global_ns() - t0 > kWaitNs) return false;
    return true;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" :: "r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TcConvArgs {
    ConvSrc src;           // the input's channels (one tensor, or [up2(coarse) | skip])
    int cin;               // cin % 16 == 0
    const bf16* wt;        // [9][wrows][cin]
    int wrows;
    const float* bias;     // [cout] or null
    bf16* out;
    int out_cs, out_co, cout;
    int npad, R;           // MMA N (cout rounded up to 16) and image rows per strip
    int N, H, W, relu;
    int* status;
};

__global__ void __launch_bounds__(kTcThreads, 1) k_conv3x3_tc(const TcConvArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);           // [2] chunk buffers consumed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 16);
    unsigned char* stage0 = smem + kBarBytes;
    const int R = a.R, npad = a.npad;
    const int sbytes = stage_bytes(R, npad), hbytes = halo_bytes(R);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const int strips_x = (a.W + kStrip - 1) / kStrip, strips_y = (a.H + R - 1) / R;
    int t = blockIdx.x;
    const int sx = t % strips_x;
    t /= strips_x;
    const int sy = t % strips_y;
    const int n = t / strips_y;
    const int x0 = sx * kStrip, y0 = sy * R;

    if (tid == 0) {  // one commit per warp's issuing thread
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(saddr(bars + 0)), "n"(kTcThreads / 32) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(saddr(bars + 1)), "n"(kTcThreads / 32) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(saddr(tmem_slot)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // stages chunk c (input channels 16c .. 16c + 15) into buffer b
    const int hrow = (R + 2) * kHaloW;
    auto load = [&](int c, int b) {
        unsigned char* hs = stage0 + b * sbytes;
        unsigned char* ws = hs + hbytes;
        const int c0 = c * 16;
        for (int i = tid; i < 2 * hrow; i += kTcThreads) {
            const int k8 = i & 1, p = i >> 1;             // neighbouring threads: the two octets of a pixel
            const int hy = p / kHaloW, hx = p - hy * kHaloW;
            const int gy = y0 - 1 + hy, gx = x0 - 1 + hx;
            const bool ok = gy >= 0 && gy < a.H && gx >= 0 && gx < a.W;
            const bf16* src = ok ? src_at(a.src, n, gy, gx, a.H, a.W, c0 + k8 * 8) : a.src.a;
            cp_async16(saddr(hs + (k8 * hrow + p) * 16), src, ok ? 16u : 0u);
        }
        const int live = a.cout < a.wrows ? a.cout : a.wrows;
        for (int i = tid; i < 9 * 2 * npad; i += kTcThreads) {
            const int k8 = i & 1, q = i >> 1;
            const int tap = q / npad, row = q - tap * npad;
            const bool ok = row < live;
            const bf16* src = ok ? a.wt + ((size_t)tap * a.wrows + row) * a.cin + c0 + k8 * 8 : a.wt;
            cp_async16(saddr(ws + ((tap * 2 + k8) * npad + row) * 16), src, ok ? 16u : 0u);
        }
    };

    const int nchunks = a.cin / 16;
    load(0, 0);
    cp_async_commit();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // barriers initialised, TMEM address written
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_bf16(kStrip, npad);
    bool failed = false;
    for (int c = 0; c < nchunks; ++c) {
        const int b = c & 1;
        if (c + 1 < nchunks) {
            bool ok = true;
            if (c >= 1) ok = mbar_wait(saddr(bars + (b ^ 1)), ((c - 1) >> 1) & 1);  // chunk c-1's MMAs are done
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            load(c + 1, b ^ 1);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async data -> tensor core reads
        __syncthreads();
        if (lane == 0) {  // four issuing threads, one per warp: rows r = warp, warp + 4, ...
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t hs = saddr(stage0 + b * sbytes), ws = hs + hbytes;
            const uint32_t lbo_a = (uint32_t)hrow * 16, lbo_b = (uint32_t)npad * 16;
            for (int tap = 0; tap < 9; ++tap) {
                const int ky = tap / 3, kx = tap - ky * 3;
                const uint64_t bd = sdesc(ws + tap * 2 * npad * 16, lbo_b, 128);
                for (int r = warp; r < R; r += kTcThreads / 32) {
                    const uint64_t ad = sdesc(hs + ((r + ky) * kHaloW + kx) * 16, lbo_a, 128);
                    umma_bf16(tmem + r * npad, ad, bd, idesc, (c > 0 || tap > 0) ? 1u : 0u);
                }
            }
            umma_commit(saddr(bars + b));
        }
    }
    cp_async_wait<0>();
    // the last commit completes when every MMA issued before it has
    bool ok = !failed && mbar_wait(saddr(bars + ((nchunks - 1) & 1)), ((nchunks - 1) >> 1) & 1);
    if (__syncthreads_or(!ok)) failed = true;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!failed) {
        const int x = x0 + warp * 32 + lane;
        for (int r = 0; r < R; ++r) {
            const int y = y0 + r;
            for (int j = 0; j < npad / 16; ++j) {
                uint32_t v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + r * npad + j * 16, v);
                if (y >= a.H || x >= a.W) continue;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int co = j * 16 + h * 8;
                    if (co >= a.cout) continue;
                    uint32_t pk[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float v0 = __uint_as_float(v[h * 8 + 2 * e]), v1 = __uint_as_float(v[h * 8 + 2 * e + 1]);
                        if (a.bias) { v0 += a.bias[co + 2 * e]; v1 += a.bias[co + 2 * e + 1]; }
                        if (a.relu) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
                        const __nv_bfloat162 p2 = __floats2bfloat162_rn(v0, v1);
                        pk[e] = *reinterpret_cast<const uint32_t*>(&p2);
                    }
                    *reinterpret_cast<uint4*>(a.out + (((size_t)n * a.H + y) * a.W + x) * a.out_cs + a.out_co + co) =
                        make_uint4(pk[0], pk[1], pk[2], pk[3]);
                }
            }
        }
    } else if (tid == 0) {
        atomicOr(a.status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTmemCols) : "memory");
}

// ---------------------------------------------------------------- persistent TMA kernel
// warp 0: TMA; warps 1..MW: MMA issue (rows r = m, m + MW, ... of a strip for MMA warp m);
// warps MW+1..MW+4: epilogue
__host__ __device__ constexpr int tma_threads(int mw) { return 32 * (mw + 5); }
constexpr int kMaxStages = 4;
constexpr int kTmaMmaWarps = 8;
constexpr int kTmaHeader = 2048;   // barriers, TMEM address, abort flag, bias
constexpr int kTmaMinSmem = 120 * 1024;  // above half an SM's shared memory: one CTA per SM owns all 512 TMEM columns
constexpr int kResidentMaxBytes = 48 * 1024;  // weights kept resident up to this size

__host__ __device__ constexpr int tma_halo(int R) { return ((R + 2) * kHaloW * 32 + 1023) / 1024 * 1024; }
__host__ __device__ constexpr int tma_wts(int npad) { return (9 * npad * 32 + 1023) / 1024 * 1024; }
__host__ __device__ constexpr int tma_stage(int R, int npad) { return tma_halo(R) + tma_wts(npad); }

// Shared-memory descriptor of a K-major operand in the 32-byte swizzle: rows of 32 bytes,
// 8-row groups 256 bytes apart (stride byte offset), leading byte offset unused (1), base
// offset 0, layout type 6 (bits 61-63).
__device__ __forceinline__ uint64_t sdesc_sw32(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(256u >> 4) << 32) | (1ull << 46) | (6ull << 61);
}

struct TmaConvArgs {
    int cin, npad, R, cout, relu, out_cs, out_co;
    int N, H, W, tiles, stages;
    int resident, wres;  // weights staged once for the whole kernel; bytes reserved for them
    const float* bias;
    bf16* out;
    int* status;
};

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar) : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar) : "memory");
}

// Bounded wait that also gives up when another role has raised the abort flag.
__device__ __forceinline__ bool wait_or_abort(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* status) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (global_ns() - t0 > kWaitNs) {
            *abort_flag = 1;
            atomicOr(status, 1);
            return false;
        }
    }
}

template <int MW>
__global__ void __launch_bounds__(tma_threads(MW), 1)
k_conv3x3_tma(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_w, const TmaConvArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kMaxStages]
    uint64_t* empty = full + kMaxStages;                 // [kMaxStages]
    uint64_t* acc_full = empty + kMaxStages;             // [2]
    uint64_t* acc_empty = acc_full + 2;                  // [2]
    uint64_t* wbar = acc_empty + 2;                      // resident weights landed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 128);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 132);
    float* sbias = reinterpret_cast<float*>(smem + 256);  // [npad]
    unsigned char* wres = smem + kTmaHeader;
    unsigned char* ring = smem + kTmaHeader + a.wres;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // TMA destinations and the descriptors below assume a 1024-byte aligned base
    if (saddr(smem) & 1023u) {
        if (tid == 0) atomicOr(a.status, 2);
        return;
    }
    const int R = a.R, npad = a.npad, S = a.stages;
    const int hbytes = tma_halo(R), sbytes = a.resident ? tma_halo(R) : tma_stage(R, npad);
    const uint32_t tx_bytes = (uint32_t)(R + 2) * kHaloW * 32u + (a.resident ? 0u : 9u * npad * 32u);
    const int nchunks = a.cin / 16;
    const int strips_x = (a.W + kStrip - 1) / kStrip, strips_y = (a.H + R - 1) / R;
    if (tid == 0) {
        for (int s = 0; s < kMaxStages; ++s) {
            mbar_init(saddr(full + s), 1);
            mbar_init(saddr(empty + s), MW);  // one commit per MMA warp
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(saddr(acc_full + b), MW);
            mbar_init(saddr(acc_empty + b), 4);  // one arrival per epilogue warp
        }
        mbar_init(saddr(wbar), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < npad; i += tma_threads(MW)) sbias[i] = (a.bias && i < a.cout) ? a.bias[i] : 0.0f;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" :: "r"(saddr(tmem_slot)) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(&tm_in)) : "memory");
            asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(&tm_w)) : "memory");
            // resident weights: every chunk's nine taps once, before the first strip
            if (a.resident) {
                mbar_expect_tx(saddr(wbar), (uint32_t)nchunks * 9u * npad * 32u);
                for (int c = 0; c < nchunks; ++c)
                    tma_load_3d(saddr(wres) + c * 9 * npad * 32, &tm_w, c * 16, 0, 0, saddr(wbar));
            }
            int k = 0;
            for (int t = blockIdx.x; t < a.tiles; t += gridDim.x) {
                int tt = t;
                const int sx = tt % strips_x;
                tt /= strips_x;
                const int sy = tt % strips_y;
                const int n = tt / strips_y;
                const int x0 = sx * kStrip, y0 = sy * R;
                bool ok = true;
                for (int c = 0; c < nchunks; ++c, ++k) {
                    const int s = k % S;
                    const uint32_t ph = (uint32_t)(k / S) & 1u;
                    if (!wait_or_abort(saddr(empty + s), ph ^ 1u, abort_flag, a.status)) { ok = false; break; }
                    const uint32_t bar = saddr(full + s);
                    mbar_expect_tx(bar, tx_bytes);
                    const uint32_t dst = saddr(ring + s * sbytes);
                    tma_load_4d(dst, &tm_in, c * 16, x0 - 1, y0 - 1, n, bar);
                    if (!a.resident) tma_load_3d(dst + hbytes, &tm_w, c * 16, 0, 0, bar);
                }
                if (!ok) break;
            }
        }
    } else if (warp <= MW) {
        const int m = warp - 1;
        if (lane == 0 && (!a.resident || wait_or_abort(saddr(wbar), 0u, abort_flag, a.status))) {
            const uint32_t idesc = idesc_bf16(kStrip, npad);
            int k = 0, i = 0;
            for (int t = blockIdx.x; t < a.tiles; t += gridDim.x, ++i) {
                const int ab = i & 1;
                if (!wait_or_abort(saddr(acc_empty + ab), ((uint32_t)(i >> 1) & 1u) ^ 1u, abort_flag, a.status)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d0 = tmem + (uint32_t)ab * 256u;
                bool ok = true;
                for (int c = 0; c < nchunks; ++c, ++k) {
                    const int s = k % S;
                    if (!wait_or_abort(saddr(full + s), (uint32_t)(k / S) & 1u, abort_flag, a.status)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t hs = saddr(ring + s * sbytes);
                    const uint32_t ws = a.resident ? saddr(wres) + c * 9 * npad * 32 : hs + hbytes;
                    for (int tap = 0; tap < 9; ++tap) {
                        const int ky = tap / 3, kx = tap - ky * 3;
                        const uint64_t bd = sdesc_sw32(ws + tap * npad * 32);
                        for (int r = m; r < R; r += MW) {
                            const uint64_t ad = sdesc_sw32(hs + ((r + ky) * kHaloW + kx) * 32);
                            umma_bf16(d0 + r * npad, ad, bd, idesc, (c > 0 || tap > 0) ? 1u : 0u);
                        }
                    }
                    umma_commit(saddr(empty + s));
                }
                if (!ok) break;
                umma_commit(saddr(acc_full + ab));
            }
        }
    } else {
        const int q = warp & 3;  // this warp's TMEM lane quarter
        int i = 0;
        for (int t = blockIdx.x; t < a.tiles; t += gridDim.x, ++i) {
            const int ab = i & 1;
            const bool got = wait_or_abort(saddr(acc_full + ab), (uint32_t)(i >> 1) & 1u, abort_flag, a.status);
            if (!__all_sync(0xffffffffu, got)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            int tt = t;
            const int sx = tt % strips_x;
            tt /= strips_x;
            const int sy = tt % strips_y;
            const int n = tt / strips_y;
            const int x = sx * kStrip + q * 32 + lane;
            for (int r = 0; r < R; ++r) {
                const int y = sy * R + r;
                for (int j = 0; j < npad / 16; ++j) {
                    uint32_t v[16];
                    tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)ab * 256u + r * npad + j * 16, v);
                    if (y >= a.H || x >= a.W) continue;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int co = j * 16 + h * 8;
                        if (co >= a.cout) continue;
                        uint32_t pk[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            float v0 = __uint_as_float(v[h * 8 + 2 * e]) + sbias[co + 2 * e];
                            float v1 = __uint_as_float(v[h * 8 + 2 * e + 1]) + sbias[co + 2 * e + 1];
                            if (a.relu) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
                            const __nv_bfloat162 p2 = __floats2bfloat162_rn(v0, v1);
                            pk[e] = *reinterpret_cast<const uint32_t*>(&p2);
                        }
                        *reinterpret_cast<uint4*>(a.out + (((size_t)n * a.H + y) * a.W + x) * a.out_cs + a.out_co + co) =
                            make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(saddr(acc_empty + ab));
        }
    }
    __syncthreads();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" :: "r"(tmem) : "memory");
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// ---------------------------------------------------------------- weight gradient
// dW[tap][co][ci] = sum over pixels p of dY[p][co] * X[p + d(tap)][ci]: per tap a GEMM on
// the tensor cores with the pixels as its K dimension,
//   M = output channels (dY transposed; 64 rows when they fit, else 128, of which cout
//       are real),
//   N = a chunk of up to 48 input channels (a CTA group's share), one accumulator of N
//       TMEM columns per tap (9 x 48 <= 512),
//   K = pixels: a strip of kWgRows image rows x 64 pixels per stage, 16 per MMA.
// A stage holds the strip's dY (boxes of 16 channels x 64 pixels x kWgRows rows) and the
// input's halo (boxes of 16 channels x 66 pixels x kWgRows + 2 rows), both copied by TMA in
// the 32-byte swizzle, which is the tensor core's MN-major layout: one 32-byte row (16
// channels) per pixel, 8-pixel groups 256 bytes apart (stride byte offset), the next 16
// channels one box further (leading byte offset).  A tap's B operand is the same halo with
// its start moved to row r + ky, pixel kx -- the copy engine has zero-filled the image
// border -- so the input is read once per strip, not once per tap.  CTAs of a group split
// the strips between them (K-split): each writes its partial sums to its own slice of a
// workspace, and k_wgrad_reduce adds the slices in order -- the result does not depend on
// scheduling, unlike atomics.
//
// Warp roles: one lane of warp 0 issues the TMA copies of each strip into a ring of
// kWgStages buffers (a "full" barrier per buffer counts the bytes), one lane of warp 1
// issues the MMAs and commits them to the buffer's "empty" barrier, and after the last
// strip to the accumulator barrier; then all four warps move the accumulators from TMEM to
// this CTA's slice.  Every wait is bounded.
constexpr int kWgStrip = 64;
constexpr int kWgRows = 2;
constexpr int kWgHaloW = kWgStrip + 2;
constexpr int kWgChunk = 48;
constexpr int kWgStages = 3;
constexpr int kWgThreads = 128;
constexpr int kWgHeader = 1024;
constexpr int kWgDyBox = kWgRows * kWgStrip * 32;                                   // 16 channels
constexpr int kWgXBox = ((kWgRows + 2) * kWgHaloW * 32 + 1023) / 1024 * 1024;  // 16 channels, padded
constexpr int kWgStage = 8 * kWgDyBox + (kWgChunk / 16) * kWgXBox;  // dY sized for M = 128 rows

// Descriptor of an MN-major operand in the 32-byte swizzle: 16-element atoms `lbo` bytes
// apart, 8-row groups 256 bytes apart, layout type 6.
__device__ __forceinline__ uint64_t sdesc_sw32_mn(uint32_t addr, uint32_t lbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)(256u >> 4) << 32) | (1ull << 46) | (6ull << 61);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both MN-major
// (transpose bits 15 and 16), N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc_bf16_mn(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

struct WgradArgs {
    int m;        // MMA rows: 128, or 64 when the output channels (cpad) fit
    int cpad, cout, cin, N, H, W;
    int strips;   // N * ceil(H / kWgRows) * ceil(W / kWgStrip)
    float* part;  // [gridDim.x slices][9][cpad][cin]
    int* status;
};

__global__ void __launch_bounds__(kWgThreads, 1)
k_wgrad_tc(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_dy, const WgradArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kWgStages]
    uint64_t* empty = full + kWgStages;                  // [kWgStages]
    uint64_t* acc = empty + kWgStages;                   // [1]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 128);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 132);
    unsigned char* stage0 = smem + kWgHeader;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (saddr(smem) & 1023u) {  // the swizzled boxes need 1 KB aligned destinations
        if (tid == 0) atomicOr(a.status, 2);
        return;
    }
    const int c0 = blockIdx.y * kWgChunk;                    // this group's input channels
    const int ch = min(kWgChunk, a.cin - c0);               // 16, 32 or 48
    const int ndy = a.cpad / 16, nx = ch / 16;
    const int sx = (a.W + kWgStrip - 1) / kWgStrip, sy = (a.H + kWgRows - 1) / kWgRows;
    const int first = blockIdx.x;
    const int count = first < a.strips ? (a.strips - 1 - first) / (int)gridDim.x + 1 : 0;

    if (tid == 0) {
        for (int k = 0; k < kWgStages; ++k) {
            mbar_init(saddr(full + k), 1);
            mbar_init(saddr(empty + k), 1);
        }
        mbar_init(saddr(acc), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" :: "r"(saddr(tmem_slot)) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    if (warp == 0 && lane == 0) {
        asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(&tm_x)) : "memory");
        asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(&tm_dy)) : "memory");
        const uint32_t tx = (uint32_t)ndy * kWgDyBox + (uint32_t)nx * ((kWgRows + 2) * kWgHaloW * 32);
        for (int it = 0; it < count; ++it) {
            const int b = it % kWgStages;
            if (!wait_or_abort(saddr(empty + b), ((uint32_t)(it / kWgStages) & 1u) ^ 1u, abort_flag, a.status)) {
                ok = false;
                break;
            }
            const int s = first + it * (int)gridDim.x;
            const int xs = s % sx, t = s / sx;
            const int y0 = (t % sy) * kWgRows, n = t / sy;
            const int x0 = xs * kWgStrip;
            const uint32_t bar = saddr(full + b);
            mbar_expect_tx(bar, tx);
            const uint32_t dyb = saddr(stage0 + b * kWgStage), xb = dyb + 8 * kWgDyBox;
            for (int k = 0; k < ndy; ++k) tma_load_4d(dyb + k * kWgDyBox, &tm_dy, k * 16, x0, y0, n, bar);
            for (int k = 0; k < nx; ++k) tma_load_4d(xb + k * kWgXBox, &tm_x, c0 + k * 16, x0 - 1, y0 - 1, n, bar);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16_mn(a.m, ch);
        for (int it = 0; it < count; ++it) {
            const int b = it % kWgStages;
            if (!wait_or_abort(saddr(full + b), (uint32_t)(it / kWgStages) & 1u, abort_flag, a.status)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t dyb = saddr(stage0 + b * kWgStage), xb = dyb + 8 * kWgDyBox;
            for (int r = 0; r < kWgRows; ++r)
                for (int k = 0; k < kWgStrip / 16; ++k) {
                    const uint64_t ad = sdesc_sw32_mn(dyb + (r * kWgStrip + 16 * k) * 32, kWgDyBox);
                    for (int tap = 0; tap < 9; ++tap) {
                        const int ky = tap / 3, kx = tap - ky * 3;
                        const uint64_t bd = sdesc_sw32_mn(xb + ((r + ky) * kWgHaloW + kx + 16 * k) * 32, kWgXBox);
                        umma_bf16(tmem + tap * ch, ad, bd, idesc, (it > 0 || r > 0 || k > 0) ? 1u : 0u);
                    }
                }
            umma_commit(saddr(empty + b));
        }
        if (ok && count > 0) umma_commit(saddr(acc));
    }
    __syncwarp();
    // epilogue: TMEM lane (warp * 32 + lane) holds output channel co for every tap
    const bool got = count == 0 || wait_or_abort(saddr(acc), 0u, abort_flag, a.status);
    if (__all_sync(0xffffffffu, got && !*abort_flag)) {  // warp-uniform: tcgen05.ld is .aligned
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // M = 128: row i in TMEM lane i.  M = 64: rows 16w..16w+15 in lanes 32w..32w+15 of
        // warp w's quarter (the upper 16 lanes of each quarter are unused)
        const int co = a.m == 128 ? warp * 32 + lane : (lane < 16 ? warp * 16 + lane : a.cpad);
        float* part = a.part + (size_t)blockIdx.x * 9 * a.cpad * a.cin;
        for (int tap = 0; tap < 9; ++tap)
            for (int j = 0; j < nx; ++j) {
                uint32_t v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + tap * ch + j * 16, v);
                if (co >= a.cout) continue;
                float4* dst = reinterpret_cast<float4*>(part + ((size_t)tap * a.cpad + co) * a.cin + c0 + j * 16);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    dst[q] = count > 0 ? make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                                     __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]))
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
            }
    } else if (lane == 0) {
        atomicOr(a.status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" :: "r"(tmem) : "memory");
}

// [up2(coarse) | skip] (a decoder convolution's input) written out as one NHWC tensor
__global__ void k_concat_src(const ConvSrc x, int cin, int N, int H, int W, bf16* __restrict__ out) {
    const int c8 = cin / 8;
    const long long n8 = (long long)N * H * W * c8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n8; i += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(i % c8);
        const long long px = i / c8;
        const int xx = (int)(px % W);
        const long long r = px / W;
        const int yy = (int)(r % H), n = (int)(r / H);
        *reinterpret_cast<uint4*>(out + px * cin + o * 8) =
            __ldg(reinterpret_cast<const uint4*>(src_at(x, n, yy, xx, H, W, o * 8)));
    }
}

// dw[tap][co][ci] += sum over slices s (in order) of part[s][tap][co][ci]
__global__ void k_wgrad_reduce(const float* __restrict__ part, int slices, int cpad, int cin, int cout,
                               float* __restrict__ dw) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;  // (tap, co, ci), ci fastest
    if (i >= 9LL * cout * cin) return;
    const int ci = (int)(i % cin);
    const long long r = i / cin;
    const int co = (int)(r % cout), tap = (int)(r / cout);
    float s = 0.0f;
    const size_t stride = (size_t)9 * cpad * cin;
    const float* p = part + ((size_t)tap * cpad + co) * cin + ci;
    for (int k = 0; k < slices; ++k) s += p[k * stride];
    dw[i] += s;
}

}  // namespace

// Image rows per strip for an output width of npad channels: R x npad accumulator columns
// fit in the CTA's 256.
int conv_tc_rows(int cout) {
    const int npad = (cout + 15) / 16 * 16;
    int R = kTmemCols / npad;
    return R > 8 ? 8 : R;
}

salty_status conv3x3_tc(salty_ctx* ctx, const ConvSrc& in, int cin, const bf16* wt, int wrows, const float* bias,
                        bf16* out, int out_cs, int out_co, int cout, int N, int H, int W, int relu, int* d_status) {
    const int npad = (cout + 15) / 16 * 16;
    if (cin % 16 || cin <= 0 || npad > 256 || npad < 16 || cout % 8 || in.a_cs % 8 || in.a_ch % 16 ||
        (in.a_ch < cin && (!in.b || in.b_cs % 8)) || out_cs % 8 || out_co % 8 || wrows < 1)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "conv3x3_tc: unsupported shape (cin %d, cout %d)", cin, cout);
    const int R = conv_tc_rows(cout);
    const size_t smem = (size_t)kBarBytes + 2 * (size_t)stage_bytes(R, npad);
    SALTY_TRY_CUDA(ctx->err, cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long tiles = (long long)N * ((H + R - 1) / R) * ((W + kStrip - 1) / kStrip);
    TcConvArgs a{in, cin, wt, wrows, bias, out, out_cs, out_co, cout, npad, R, N, H, W, relu, d_status};
    k_conv3x3_tc<<<(unsigned)tiles, kTcThreads, smem, ctx->stream>>>(a);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

salty_status conv3x3_tma(salty_ctx* ctx, const bf16* in, int in_cs, int cin, const bf16* wt, int wrows,
                         const float* bias, bf16* out, int out_cs, int out_co, int cout, int N, int H, int W, int relu,
                         int* d_status) {
    const int npad = (cout + 15) / 16 * 16;
    if (cin % 16 || cin <= 0 || cin > in_cs || in_cs % 8 || npad > 256 || npad < 16 || cout % 8 || out_cs % 8 ||
        out_co % 8 || wrows < 1 || wrows > 256 || reinterpret_cast<uintptr_t>(in) % 16 ||
        reinterpret_cast<uintptr_t>(wt) % 16)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "conv3x3_tma: unsupported shape (cin %d, cout %d)", cin, cout);
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return ctx->err.fail(SALTY_ERR_CUDA, "conv3x3_tma: cuTensorMapEncodeTiled is not available");
    const int R = conv_tc_rows(cout);
    // the layer's weights stay in shared memory for the whole kernel when they are small
    const int wbytes = (cin / 16) * 9 * npad * 32;
    const bool resident = wbytes <= kResidentMaxBytes;
    const int wres = resident ? (wbytes + 1023) / 1024 * 1024 : 0;
    const int sbytes = resident ? tma_halo(R) : tma_stage(R, npad);
    int S = (int)((227 * 1024 - kTmaHeader - wres) / sbytes);
    if (S > kMaxStages) S = kMaxStages;
    if (S < 2) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "conv3x3_tma: stage too large");
    size_t smem = (size_t)kTmaHeader + wres + (size_t)S * sbytes;
    if (smem < (size_t)kTmaMinSmem) smem = kTmaMinSmem;
    // input: 4-D (channels, x, y, image), boxes of 16 channels x 130 pixels x R + 2 rows
    CUtensorMap tm_in, tm_w;
    const cuuint64_t gdim[4] = {(cuuint64_t)in_cs, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
    const cuuint64_t gstride[3] = {(cuuint64_t)in_cs * 2, (cuuint64_t)W * in_cs * 2, (cuuint64_t)H * W * in_cs * 2};
    const cuuint32_t box[4] = {16, (cuuint32_t)kHaloW, (cuuint32_t)(R + 2), 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (enc(&tm_in, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(in), gdim, gstride, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ctx->err.fail(SALTY_ERR_CUDA, "conv3x3_tma: input tensor map");
    // weights: 3-D (input channel, row, tap), boxes of 16 channels x npad rows x 9 taps
    const cuuint64_t wdim[3] = {(cuuint64_t)cin, (cuuint64_t)wrows, 9};
    const cuuint64_t wstride[2] = {(cuuint64_t)cin * 2, (cuuint64_t)wrows * cin * 2};
    const cuuint32_t wbox[3] = {16, (cuuint32_t)npad, 9};
    if (enc(&tm_w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(wt), wdim, wstride, wbox, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ctx->err.fail(SALTY_ERR_CUDA, "conv3x3_tma: weight tensor map");
    constexpr int MW = kTmaMmaWarps;
    SALTY_TRY_CUDA(ctx->err, cudaFuncSetAttribute(k_conv3x3_tma<MW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long tiles = (long long)N * ((H + R - 1) / R) * ((W + kStrip - 1) / kStrip);
    const int grid = (int)(tiles < ctx->num_sms ? tiles : ctx->num_sms);
    TmaConvArgs a{cin, npad, R, cout, relu, out_cs, out_co, N, H, W, (int)tiles, S, resident ? 1 : 0, wres, bias, out,
                  d_status};
    k_conv3x3_tma<MW><<<grid, tma_threads(MW), smem, ctx->stream>>>(tm_in, tm_w, a);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

// Input-channel groups and strip slices for a layer: about one CTA per SM in all.
static void wgrad_plan(int num_sms, int cin, int N, int H, int W, int* groups, int* slices, int* strips) {
    *groups = (cin + kWgChunk - 1) / kWgChunk;
    const long long st = (long long)N * ((H + kWgRows - 1) / kWgRows) * ((W + kWgStrip - 1) / kWgStrip);
    long long s = num_sms / *groups;
    if (s < 1) s = 1;
    if (s > st) s = st;
    *slices = (int)s;
    *strips = (int)st;
}

size_t conv_wgrad_tc_workspace(int num_sms, int cin, int cpad, int N, int H, int W) {
    int groups, slices, strips;
    wgrad_plan(num_sms, cin, N, H, W, &groups, &slices, &strips);
    return (size_t)slices * 9 * cpad * cin;
}

salty_status conv_wgrad_tc(salty_ctx* ctx, const bf16* dy, int cpad, int cout, const ConvSrc& x, int cin, float* dw,
                           int N, int H, int W, float* ws, size_t ws_floats, bf16* cat_ws, size_t cat_elems,
                           int* d_status) {
    if (cin % 16 || cin <= 0 || cpad % 16 || cpad < 16 || cpad > 128 || cout > cpad || cout < 1 ||
        reinterpret_cast<uintptr_t>(dy) % 16 || reinterpret_cast<uintptr_t>(ws) % 16)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "conv_wgrad_tc: unsupported shape (cin %d, cout %d)", cin, cout);
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return ctx->err.fail(SALTY_ERR_CUDA, "conv_wgrad_tc: cuTensorMapEncodeTiled is not available");
    int groups, slices, strips;
    wgrad_plan(ctx->num_sms, cin, N, H, W, &groups, &slices, &strips);
    if ((size_t)slices * 9 * cpad * cin > ws_floats)
        return ctx->err.fail(SALTY_ERR_CAPACITY, "conv_wgrad_tc: workspace too small");
    // the input as one NHWC tensor: as given, or the decoder's concatenation written out
    const bf16* xin = x.a;
    int xcs = x.a_cs;
    const long long npx = (long long)N * H * W;
    if (x.a_shift != 0 || x.a_ch < cin) {
        if ((size_t)(npx * cin) > cat_elems)
            return ctx->err.fail(SALTY_ERR_CAPACITY, "conv_wgrad_tc: concatenation workspace too small");
        const long long n8 = npx * (cin / 8);
        k_concat_src<<<(unsigned)std::min<long long>((n8 + 255) / 256, (long long)ctx->num_sms * 16), 256, 0,
                       ctx->stream>>>(x, cin, N, H, W, cat_ws);
        xin = cat_ws;
        xcs = cin;
    }
    if (reinterpret_cast<uintptr_t>(xin) % 16 || xcs % 16)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "conv_wgrad_tc: input not 16-byte aligned");
    CUtensorMap tm_x, tm_dy;
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const cuuint32_t xbox[4] = {16, (cuuint32_t)kWgHaloW, (cuuint32_t)(kWgRows + 2), 1};
    const cuuint64_t xdim[4] = {(cuuint64_t)cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
    const cuuint64_t xstr[3] = {(cuuint64_t)xcs * 2, (cuuint64_t)W * xcs * 2, (cuuint64_t)H * W * xcs * 2};
    if (enc(&tm_x, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(xin), xdim, xstr, xbox, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ctx->err.fail(SALTY_ERR_CUDA, "conv_wgrad_tc: input tensor map");
    const cuuint32_t dbox[4] = {16, (cuuint32_t)kWgStrip, (cuuint32_t)kWgRows, 1};
    const cuuint64_t ddim[4] = {(cuuint64_t)cpad, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
    const cuuint64_t dstr[3] = {(cuuint64_t)cpad * 2, (cuuint64_t)W * cpad * 2, (cuuint64_t)H * W * cpad * 2};
    if (enc(&tm_dy, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(dy), ddim, dstr, dbox, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ctx->err.fail(SALTY_ERR_CUDA, "conv_wgrad_tc: gradient tensor map");
    const size_t smem = (size_t)kWgHeader + (size_t)kWgStages * kWgStage;
    SALTY_TRY_CUDA(ctx->err, cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    WgradArgs a{cpad <= 64 ? 64 : 128, cpad, cout, cin, N, H, W, strips, ws, d_status};
    k_wgrad_tc<<<dim3(slices, groups), kWgThreads, smem, ctx->stream>>>(tm_x, tm_dy, a);
    const long long outs = 9LL * cout * cin;
    k_wgrad_reduce<<<(unsigned)((outs + 255) / 256), 256, 0, ctx->stream>>>(ws, slices, cpad, cin, cout, dw);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

}  // namespace salty
