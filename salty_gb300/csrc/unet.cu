// unet.cu -- the learned denoiser: a 5-level U-Net trained and run by these kernels.
//
// The reference has an NLM filter (src/s3d_denoiser.cpp:19-95) and no learned denoiser;
// this network is new.  Input: 11 features per pixel (log(1 + colour), first-hit albedo,
// normal, 1/(1 + distance), the colour's noise level), padded to 16 channels.  Architecture (NHWC, BF16 activations):
//   enc: conv 16->32, 32->32 | pool | 32->48, 48->48 | pool | 48->64, 64->64 | pool |
//        64->80, 80->80 | pool | 80->96
//   dec: up + concat(96+80) -> 80 | up + concat(80+64) -> 64 | up + concat(64+48) -> 48 |
//        up + concat(48+32) -> 32 | conv 32->8 (channels 0..2: a correction r of the input's
//        log colour; the prediction is log(1 + colour) = x + r)
// every conv 3x3, stride 1, zero padding, ReLU except the last; 2x2 max-pool; nearest 2x
// up-sampling.  Loss: mean |x + r - log(1 + target)| (L1 in log space).  Optimiser: Adam.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16, BF16 operands,
// FP32 accumulation):
//   forward       M = pixels, N = Cout, K = 9*Cin: a CTA stages an 8x16-pixel tile plus halo
//                 in shared memory; A fragments come from it, B fragments from the weights.
//   backward data the same kernel on dY with the weights flipped and transposed.
//   backward wts  M = Cout, N = Cin, K = pixels: ldmatrix.trans turns the NHWC tiles of dY and
//                 of the shifted input into fragments with pixels along K; a CTA covers all
//                 nine taps of a 16-channel input slice (one dY fragment serves nine taps),
//                 sums its pixel tiles in registers and adds the partial into FP32 gradients.
// All three convolutions run by default on tcgen05 (conv_tc.cu: TMEM accumulators; the
// forward and backward-data ones over 128-pixel strips, inputs in one tensor staged by TMA
// in a persistent warp-specialised kernel, the decoder's two-source inputs by cp.async; the
// weight gradient over strips of 2 rows x 64 pixels with dY transposed as the MMA's A, the
// input's halo as B and the taps as descriptor offsets, summed over CTAs in a fixed order);
// the mma.sync kernels below stay selectable (salty_unet_set_conv_kernel) and are the
// reference the tcgen05 kernels are tested against.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "unet_src.cuh"

namespace salty {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTileX = 16, kTileY = 8;          // output tile of one CTA
constexpr int kHaloX = kTileX + 2, kHaloY = kTileY + 2;
constexpr int kConvThreads = 128;
constexpr int kFeatures = 11;                   // input floats per pixel

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldmatrix_x4_trans(unsigned (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}

// ---------------------------------------------------------------- conv3x3 (forward, backward data)
// in:  BF16 NHWC input channels 0..Cin-1 (Cin % 16 == 0) from one or two sources (ConvSrc)
// wt:  [9][wrows][Cin] BF16 (tap-major, input channel contiguous); output channel co reads row co
// out: [N][H][W][out_cs] BF16 at channel offset out_co (channels co < Cout written)
// NT n8-tiles per CTA; blockIdx.y selects output channels [blockIdx.y*NT*8, +NT*8).
// Shared memory: the 18x10-pixel halo tile, then one tap's weight slice [NT*8][Cin], both
// with rows padded by 8 halves so the 8 row addresses of an ldmatrix fall in distinct banks.
// Per 16-channel k-step a warp issues 2 ldmatrix.x4 for A (its two 16-pixel rows), NT/2
// ldmatrix.x4 for B and 2*NT mma.
__device__ __forceinline__ void ldmatrix_x4(unsigned (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldmatrix_x2(unsigned& r0, unsigned& r1, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(smem_addr(p)));
}

template <int NT>
__global__ void __launch_bounds__(kConvThreads) k_conv3x3(const ConvSrc in, int Cin, const bf16* __restrict__ wt, const float* __restrict__ bias,
                                                          bf16* __restrict__ out, int out_cs, int out_co, int Cout,
                                                          int N, int H, int W, int relu) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* tile = reinterpret_cast<bf16*>(smem_raw);
    const int stride = Cin + 8;  // halves per halo pixel and per weight row
    bf16* wsm = tile + kHaloX * kHaloY * stride;
    const int tiles_x = (W + kTileX - 1) / kTileX, tiles_y = (H + kTileY - 1) / kTileY;
    int t = blockIdx.x;
    const int tx = t % tiles_x;
    t /= tiles_x;
    const int ty = t % tiles_y;
    const int n = t / tiles_y;
    const int x0 = tx * kTileX, y0 = ty * kTileY;
    // stage the halo tile
    const int chunks = Cin / 8;
    for (int i = threadIdx.x; i < kHaloX * kHaloY * chunks; i += kConvThreads) {
        const int pix = i / chunks, c = i % chunks;
        const int gy = y0 - 1 + pix / kHaloX, gx = x0 - 1 + pix % kHaloX;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) v = __ldg(reinterpret_cast<const uint4*>(src_at(in, n, gy, gx, H, W, c * 8)));
        *reinterpret_cast<uint4*>(tile + pix * stride + c * 8) = v;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, tq = lane & 3;
    const int co_base = blockIdx.y * NT * 8;
    // ldmatrix lane roles: matrix lane >> 3, row lane & 7
    const int lm = lane >> 3, lr = lane & 7;
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[m][j][k] = 0.0f;
    for (int tap = 0; tap < 9; ++tap) {
        const int ky = tap / 3, kx = tap % 3;
        // this tap's weight rows [co_base, co_base + NT*8)
        __syncthreads();  // the previous tap's reads of wsm are done (and, for tap 0, the halo is in)
        const bf16* wtap = wt + ((size_t)tap * gridDim.y * NT * 8 + co_base) * Cin;
        for (int i = threadIdx.x; i < NT * 8 * chunks; i += kConvThreads) {
            const int r = i / chunks, c = i % chunks;
            *reinterpret_cast<uint4*>(wsm + r * stride + c * 8) =
                __ldg(reinterpret_cast<const uint4*>(wtap + (size_t)r * Cin + c * 8));
        }
        __syncthreads();
        for (int cb = 0; cb < Cin; cb += 16) {
            // B: n-tiles j, j+1 from one x4 (matrices: rows n, k 0-7 | n, k 8-15 | n+8, k 0-7 | n+8, k 8-15)
            unsigned b[NT][2];
#pragma unroll
            for (int j = 0; j + 1 < NT; j += 2) {
                unsigned r4[4];
                ldmatrix_x4(r4, wsm + ((j + (lm >> 1)) * 8 + lr) * stride + cb + (lm & 1) * 8);
                b[j][0] = r4[0];
                b[j][1] = r4[1];
                b[j + 1][0] = r4[2];
                b[j + 1][1] = r4[3];
            }
            if (NT & 1) ldmatrix_x2(b[NT - 1][0], b[NT - 1][1], wsm + ((NT - 1) * 8 + lr) * stride + cb + (lm & 1) * 8);
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                // A: the 16 pixels of tile row 2*warp + m (matrices: px 0-7, k 0-7 | px 8-15, k 0-7 |
                // px 0-7, k 8-15 | px 8-15, k 8-15)
                const int row = 2 * warp + m;
                unsigned a[4];
                ldmatrix_x4(a, tile + ((row + ky) * kHaloX + lr + (lm & 1) * 8 + kx) * stride + cb + (lm >> 1) * 8);
#pragma unroll
                for (int j = 0; j < NT; ++j) mma_bf16(acc[m][j], a, b[j][0], b[j][1]);
            }
        }
    }
    // epilogue: bias, ReLU, BF16
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int y = y0 + 2 * warp + m;
        if (y >= H) continue;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int co = co_base + j * 8 + 2 * tq;
            if (co >= Cout) continue;
            const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = x0 + g + 8 * h;
                if (x >= W) continue;
                float v0 = acc[m][j][2 * h] + b0, v1 = acc[m][j][2 * h + 1] + b1;
                if (relu) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
                *reinterpret_cast<__nv_bfloat162*>(out + (((size_t)n * H + y) * W + x) * out_cs + out_co + co) =
                    __floats2bfloat162_rn(v0, v1);
            }
        }
    }
}

// ---------------------------------------------------------------- conv3x3 backward weights
// dW[tap][co][ci] += sum_p dY[p][co] * X[p + (ky-1, kx-1)][ci] for all nine taps, a group of
// up to four 16-row output-channel tiles (blockIdx.y) and a 16-wide input-channel slice
// (blockIdx.z); CTAs stride over 8x16 pixel tiles (blockIdx.x).  With nm output tiles in the
// group, warp w takes tile w % nm and the tile rows s = w / nm, w / nm + 4 / nm, ... (all
// four warps busy for 1, 2 or 4 tiles).  Per tile the CTA stages its dY columns and the X halo once; per 16-pixel
// k-step a warp loads its dY^T fragment once and reuses it for the nine taps' X fragments,
// keeping 9 x 2 accumulator tiles in registers until the end, then adds them into the FP32
// gradients.  dY: [N][H][W][Cpad] (Cpad multiple of 16, zero beyond the layer's real
// outputs); rows co >= cout_real are not written.  X: the layer's input (ConvSrc),
// Cin % 16 == 0.
constexpr int kWgradCo = 64;  // output channels per CTA (4 warps x 16)
__global__ void __launch_bounds__(kConvThreads) k_conv3x3_wgrad(const bf16* __restrict__ dy, int Cpad, int cout_real,
                                                                const ConvSrc x, int Cin, float* __restrict__ dw,
                                                                int N, int H, int W) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int dstride = kWgradCo + 8;
    constexpr int xstride = 16 + 8;
    bf16* dys = reinterpret_cast<bf16*>(smem_raw);         // [128][dstride]
    bf16* xs = dys + kTileX * kTileY * dstride;            // [10*18][xstride]
    const int co0 = blockIdx.y * kWgradCo;
    const int ci0 = blockIdx.z * 16;
    const int cw = min(kWgradCo, Cpad - co0);             // this CTA's output channels (multiple of 16)
    const int tiles_x = (W + kTileX - 1) / kTileX, tiles_y = (H + kTileY - 1) / kTileY;
    const int ntiles = N * tiles_x * tiles_y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nm = cw / 16, ngrp = 4 / nm;                 // output tiles, row groups
    const int mt = warp % nm, kgrp = warp / nm;
    const bool active = kgrp < ngrp;
    float acc[9][2][4];
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[t][j][k] = 0.0f;
    const int kk = lane & 7, which = lane >> 3;  // ldmatrix: row within matrix, matrix index
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int tt = t;
        const int tx = tt % tiles_x;
        tt /= tiles_x;
        const int ty = tt % tiles_y;
        const int n = tt / tiles_y;
        const int x0 = tx * kTileX, y0 = ty * kTileY;
        __syncthreads();
        const int dchunks = cw / 8;
        for (int i = threadIdx.x; i < kTileX * kTileY * dchunks; i += kConvThreads) {
            const int pix = i / dchunks, c = i % dchunks;
            const int gy = y0 + pix / kTileX, gx = x0 + pix % kTileX;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gy < H && gx < W)
                v = __ldg(reinterpret_cast<const uint4*>(dy + (((size_t)n * H + gy) * W + gx) * Cpad + co0 + c * 8));
            *reinterpret_cast<uint4*>(dys + pix * dstride + c * 8) = v;
        }
        for (int i = threadIdx.x; i < kHaloX * kHaloY * 2; i += kConvThreads) {
            const int pix = i / 2, c = i % 2;
            const int gy = y0 - 1 + pix / kHaloX, gx = x0 - 1 + pix % kHaloX;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                v = __ldg(reinterpret_cast<const uint4*>(src_at(x, n, gy, gx, H, W, ci0 + c * 8)));
            *reinterpret_cast<uint4*>(xs + pix * xstride + c * 8) = v;
        }
        __syncthreads();
        if (!active) continue;
        // K = the tile's 128 pixels in 8 steps of 16 (one tile row each)
#pragma unroll 1
        for (int s = kgrp; s < kTileY; s += ngrp) {
            // A: output channels (rows) x pixels (k).  Matrices: 0 = (co 0-7, px 0-7),
            // 1 = (co 8-15, px 0-7), 2 = (co 0-7, px 8-15), 3 = (co 8-15, px 8-15)
            unsigned a[4];
            {
                const int px = kk + ((which & 2) ? 8 : 0);
                const int co = mt * 16 + ((which & 1) ? 8 : 0);
                ldmatrix_x4_trans(a, dys + (s * kTileX + px) * dstride + co);
            }
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
                const int ky = tap / 3, kx = tap % 3;
                // B: pixels (row s, cols 0..15) shifted by the tap x 16 input channels.  Matrices:
                // 0 = (px 0-7, ci 0-7), 1 = (px 8-15, ci 0-7), 2 = (px 0-7, ci 8-15), 3 = (px 8-15, ci 8-15)
                unsigned bq[4];
                const int px = kk + ((which & 1) ? 8 : 0);
                const int cc = (which & 2) ? 8 : 0;
                ldmatrix_x4_trans(bq, xs + ((s + ky) * kHaloX + px + kx) * xstride + cc);
                mma_bf16(acc[tap][0], a, bq[0], bq[1]);
                mma_bf16(acc[tap][1], a, bq[2], bq[3]);
            }
        }
    }
    if (!active) return;
    const int g = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int ci = ci0 + j * 8 + 2 * tq;
            const int c0 = co0 + mt * 16 + g, c1 = c0 + 8;
            if (c0 < cout_real) {
                float* r0 = dw + ((size_t)tap * cout_real + c0) * Cin + ci;
                atomicAdd(r0, acc[tap][j][0]);
                atomicAdd(r0 + 1, acc[tap][j][1]);
            }
            if (c1 < cout_real) {
                float* r1 = dw + ((size_t)tap * cout_real + c1) * Cin + ci;
                atomicAdd(r1, acc[tap][j][2]);
                atomicAdd(r1 + 1, acc[tap][j][3]);
            }
        }
}

// ---------------------------------------------------------------- elementwise / layout
// Packs 8 floats into 8 BF16 (round to nearest) in one 16-byte word.
__device__ __forceinline__ uint4 pack_bf16x8(const float (&v)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t*>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ void unpack_bf16x8(uint4 q, float (&v)[8]) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(h[k]);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}

// features (kFeatures floats per pixel: colour, albedo, normal, 1/(1+t), noise level)
// -> 16-channel BF16 input, colour as log(1 + colour)
__global__ void k_prep_input(const float* __restrict__ f, long long npx, bf16* __restrict__ x) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        const float* s = f + p * kFeatures;
        float v[16];
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = log1pf(fmaxf(__ldg(s + c), 0.0f));
#pragma unroll
        for (int c = 3; c < kFeatures; ++c) v[c] = __ldg(s + c);
#pragma unroll
        for (int c = kFeatures; c < 16; ++c) v[c] = 0.0f;
        uint32_t w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
            w[k] = *reinterpret_cast<const uint32_t*>(&h);
        }
        uint4* d = reinterpret_cast<uint4*>(x + p * 16);
        d[0] = make_uint4(w[0], w[1], w[2], w[3]);
        d[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// 2x2 max-pool: in [N][H][W][C] -> out [N][H/2][W/2][C], C % 8 == 0; one thread per output
// pixel and 8 channels (16-byte loads and store; max of BF16 values is exact)
__global__ void k_pool(const bf16* __restrict__ in, bf16* __restrict__ out, int N, int H, int W, int C) {
    const int Ho = H / 2, Wo = W / 2, G = C / 8;
    const long long total = (long long)N * Ho * Wo * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % G);
        long long p = i / G;
        const int xo = (int)(p % Wo);
        p /= Wo;
        const int yo = (int)(p % Ho);
        const int n = (int)(p / Ho);
        const bf16* s = in + (((size_t)n * H + 2 * yo) * W + 2 * xo) * C + g * 8;
        uint4 q[4] = {__ldg(reinterpret_cast<const uint4*>(s)), __ldg(reinterpret_cast<const uint4*>(s + C)),
                      __ldg(reinterpret_cast<const uint4*>(s + (size_t)W * C)),
                      __ldg(reinterpret_cast<const uint4*>(s + (size_t)W * C + C))};
        __nv_bfloat162* m = reinterpret_cast<__nv_bfloat162*>(&q[0]);
#pragma unroll
        for (int k = 1; k < 4; ++k) {
            const __nv_bfloat162* o = reinterpret_cast<const __nv_bfloat162*>(&q[k]);
#pragma unroll
            for (int e = 0; e < 4; ++e) m[e] = __hmax2(m[e], o[e]);
        }
        *reinterpret_cast<uint4*>(out + i * 8) = q[0];
    }
}

// max-pool backward: the gradient goes to the first input equal to the max (ties: first).
// One thread per output pixel and 8 channels (C % 8 == 0); din += at the chosen inputs.
__global__ void k_pool_bwd(const bf16* __restrict__ in, const float* __restrict__ dout, float* __restrict__ din, int N,
                           int H, int W, int C) {
    const int Ho = H / 2, Wo = W / 2, G = C / 8;
    const long long total = (long long)N * Ho * Wo * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % G) * 8;
        long long p = i / G;
        const long long po = p;
        const int xo = (int)(p % Wo);
        p /= Wo;
        const int yo = (int)(p % Ho);
        const int n = (int)(p / Ho);
        const size_t base = (((size_t)n * H + 2 * yo) * W + 2 * xo) * C + c;
        const size_t off[4] = {0, (size_t)C, (size_t)W * C, (size_t)W * C + C};
        float m[8], v[4][8];
        int arg[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) unpack_bf16x8(__ldg(reinterpret_cast<const uint4*>(in + base + off[k])), v[k]);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            m[e] = -INFINITY;
            arg[e] = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (v[k][e] > m[e]) { m[e] = v[k][e]; arg[e] = k; }
        }
        const float4* dp = reinterpret_cast<const float4*>(dout + po * C + c);
        const float4 d0 = __ldg(dp), d1 = __ldg(dp + 1);
        const float d[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float4* q = reinterpret_cast<float4*>(din + base + off[k]);
            float4 a = q[0], b = q[1];
            a.x += arg[0] == k ? d[0] : 0.0f; a.y += arg[1] == k ? d[1] : 0.0f;
            a.z += arg[2] == k ? d[2] : 0.0f; a.w += arg[3] == k ? d[3] : 0.0f;
            b.x += arg[4] == k ? d[4] : 0.0f; b.y += arg[5] == k ? d[5] : 0.0f;
            b.z += arg[6] == k ? d[6] : 0.0f; b.w += arg[7] == k ? d[7] : 0.0f;
            q[0] = a;
            q[1] = b;
        }
    }
}

// L1 loss in log space on channels 0..2 of the prediction y = out + x (the network predicts
// a correction of the input's log colour x, channels 0..2 of the 16-channel input [npx][16]);
// grad dout [npx][8] (FP32, zero beyond channel 2)
__global__ void k_loss(const bf16* __restrict__ out, const bf16* __restrict__ x, const float* __restrict__ target,
                       long long npx, float* __restrict__ dout, double* __restrict__ loss_sum) {
    double s = 0.0;
    const float scale = 1.0f / (3.0f * (float)npx);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < 8; ++c) {
            float g = 0.0f;
            if (c < 3) {
                const float y = __bfloat162float(out[p * 8 + c]) + __bfloat162float(x[p * 16 + c]);
                const float t = log1pf(fmaxf(target[p * 3 + c], 0.0f));
                const float d = y - t;
                s += fabsf(d);
                g = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) * scale;
            }
            dout[p * 8 + c] = g;
        }
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, s);
}

// One pass of the self-ensemble: adds weight * (the prediction of pixel (px, py), found at
// its mirrored place in the padded Wp x Hp output, or, with flip bit 2, at the transposed
// place of the Hp-wide transposed output) to rgb [H][W][3].
__global__ void k_output_flipped(const bf16* __restrict__ out, const bf16* __restrict__ x, int W, int H, int Wp,
                                 int Hp, int flip, float weight, int first, float* __restrict__ rgb) {
    const long long total = (long long)W * H;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total; p += (long long)gridDim.x * blockDim.x) {
        const int px = (int)(p % W), py = (int)(p / W);
        const int qx = (flip & 1) ? W - 1 - px : px, qy = (flip & 2) ? H - 1 - py : py;
        const long long q = (flip & 4) ? (long long)qx * Hp + qy : (long long)qy * Wp + qx;
        for (int c = 0; c < 3; ++c) {
            const float v =
                weight * fmaxf(expm1f(__bfloat162float(out[q * 8 + c]) + __bfloat162float(x[q * 16 + c])), 0.0f);
            rgb[p * 3 + c] = first ? v : rgb[p * 3 + c] + v;
        }
    }
}

// prediction (input log colour + network correction) -> linear colour
__global__ void k_output(const bf16* __restrict__ out, const bf16* __restrict__ x, long long npx,
                         float* __restrict__ rgb) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c)
            rgb[p * 3 + c] =
                fmaxf(expm1f(__bfloat162float(out[p * 8 + c]) + __bfloat162float(x[p * 16 + c])), 0.0f);
}

// ReLU backward and the bias gradient in one pass over a layer's output gradient dy:
// g = dy * (y > 0) in BF16 (the next GEMMs' operand, channels C..g_cs-1 zero), and per block
// the sums of g's BF16 values per channel in a fixed order (no atomics).  Thread t of a
// block takes 8-channel group j = t % G (G = g_cs / 8) of the pixels r = t / G, r + per,
// ... of the block's grid stride (per = blockDim / G; threads beyond per * G idle) and sums
// in registers; the per-thread sums are added in shared memory in thread order into
// part[blockIdx.x][c], and k_bias_reduce adds the blocks' partials in block order.
// dy is FP32 [npx][C], or, when dy16 is given, BF16 with dy16_cs channels per pixel (a
// backward-data GEMM's output read directly; widening it to FP32 first would be exact).
// (C, y_cs, g_cs, dy16_cs multiples of 8.)
__global__ void k_relu_bwd_bias(const bf16* __restrict__ y, int y_cs, const float* __restrict__ dy,
                                const bf16* __restrict__ dy16, int dy16_cs, int C, int relu, long long npx,
                                bf16* __restrict__ g, int g_cs, float* __restrict__ part) {
    extern __shared__ float sb[];  // [per][C]
    const int G = g_cs / 8, per = blockDim.x / G, lanes = per * G;
    if ((int)threadIdx.x < lanes) {
        const int j = threadIdx.x % G, r = threadIdx.x / G, c = j * 8;
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (long long p = (long long)blockIdx.x * per + r; p < npx; p += (long long)gridDim.x * per) {
            float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (c < C) {
                if (dy16) {
                    unpack_bf16x8(__ldg(reinterpret_cast<const uint4*>(dy16 + p * dy16_cs + c)), v);
                } else {
                    const float4* d = reinterpret_cast<const float4*>(dy + p * C + c);
                    const float4 a = __ldg(d), b = __ldg(d + 1);
                    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
                }
                if (relu) {
                    float yv[8];
                    unpack_bf16x8(__ldg(reinterpret_cast<const uint4*>(y + p * y_cs + c)), yv);
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (!(yv[k] > 0.0f)) v[k] = 0.0f;
                }
            }
            const uint4 pk = pack_bf16x8(v);
            *reinterpret_cast<uint4*>(g + p * g_cs + c) = pk;
            if (c < C) {
                float w[8];
                unpack_bf16x8(pk, w);
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] += w[k];
            }
        }
        if (c < C) {
#pragma unroll
            for (int k = 0; k < 8; ++k) sb[r * C + c + k] = s[k];
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        float t = 0.0f;
        for (int r = 0; r < per; ++r) t += sb[r * C + c];
        part[(size_t)blockIdx.x * C + c] = t;
    }
}

__global__ void k_bias_reduce(const float* __restrict__ part, int blocks, int C, float* __restrict__ db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    float t = 0.0f;
    for (int b = 0; b < blocks; ++b) t += part[(size_t)b * C + c];
    db[c] += t;
}

// BF16 activation gradient (from a backward-data GEMM) -> FP32, optionally accumulated;
// channels [off, off + C) of src [npx][Cs]
// (one thread per pixel and 8 channels; Cs, off, C multiples of 8)
__global__ void k_grad_to_f32(const bf16* __restrict__ src, int Cs, int off, int C, long long npx, float* __restrict__ dst,
                              int accumulate) {
    const int G = C / 8;
    const long long total = npx * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / G;
        const int c = (int)(i % G) * 8;
        float v[8];
        unpack_bf16x8(__ldg(reinterpret_cast<const uint4*>(src + p * Cs + off + c)), v);
        float4* d = reinterpret_cast<float4*>(dst + p * C + c);
        float4 a = make_float4(v[0], v[1], v[2], v[3]), b = make_float4(v[4], v[5], v[6], v[7]);
        if (accumulate) {
            const float4 a0 = d[0], b0 = d[1];
            a.x += a0.x; a.y += a0.y; a.z += a0.z; a.w += a0.w;
            b.x += b0.x; b.y += b0.y; b.z += b0.z; b.w += b0.w;
        }
        d[0] = a;
        d[1] = b;
    }
}

// up-sampling backward: coarse grad = sum of its 2x2 children's grads (channels [0, Cc) of dcat)
// (one thread per coarse pixel and 8 channels; Ccat, Cc multiples of 8)
__global__ void k_upsample_bwd(const bf16* __restrict__ dcat, int Ccat, float* __restrict__ dcoarse, int Cc, int N,
                               int H, int W) {
    const int Hc = H / 2, Wc = W / 2, G = Cc / 8;
    const long long total = (long long)N * Hc * Wc * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % G) * 8;
        long long p = i / G;
        const long long pc = p;
        const int x = (int)(p % Wc);
        p /= Wc;
        const int y = (int)(p % Hc);
        const int n = (int)(p / Hc);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                float v[8];
                unpack_bf16x8(__ldg(reinterpret_cast<const uint4*>(
                                  dcat + (((size_t)n * H + 2 * y + dy) * W + 2 * x + dx) * Ccat + c)),
                              v);
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] += v[k];
            }
        float4* d = reinterpret_cast<float4*>(dcoarse + pc * Cc + c);
        d[0] = make_float4(s[0], s[1], s[2], s[3]);
        d[1] = make_float4(s[4], s[5], s[6], s[7]);
    }
}

// Adam on FP32 masters, then the BF16 copies: forward layout [tap][co][ci] and the
// backward-data layout [tap][ci][co] with taps flipped (8 - tap).
struct AdamArgs {
    float lr, b1, b2, eps, c1, c2;  // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
};
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, AdamArgs a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = a.b1 * m[i] + (1.0f - a.b1) * gi;
        const float vi = a.b2 * v[i] + (1.0f - a.b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= a.lr * (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
    }
}

__global__ void k_weights_to_bf16(const float* __restrict__ w, int Cout, int Cin, int rows_fwd, int rows_bwd,
                                  int cout_pad, bf16* __restrict__ wf, bf16* __restrict__ wb) {
    const int total = 9 * Cout * Cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int ci = i % Cin, co = (i / Cin) % Cout, tap = i / (Cin * Cout);
        const bf16 v = __float2bfloat16(w[i]);
        wf[((size_t)tap * rows_fwd + co) * Cin + ci] = v;
        if (wb) wb[((size_t)(8 - tap) * rows_bwd + ci) * cout_pad + co] = v;
    }
}

// Film planes (W x H) -> network input (Wp x Hp, multiples of 16) with reflected borders:
// colour, albedo, normal, 1/(1+t), noise level mean_c sqrt(var_c) / (1 + colour_c).  With
// flip bit 0 (1) the frame is mirrored left-right (top-bottom) first; with bit 2 the input
// is the transposed frame, Hp wide and Wp tall.
__global__ void k_pack_features(const float* __restrict__ mean, const float* __restrict__ var,
                                const float* __restrict__ albedo, const float* __restrict__ normal,
                                const float* __restrict__ depth, int W, int H, int Wp, int Hp, int flip,
                                float* __restrict__ f) {
    const long long total = (long long)Wp * Hp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int x = (flip & 4) ? (int)(i / Hp) : (int)(i % Wp), y = (flip & 4) ? (int)(i % Hp) : (int)(i / Wp);
        int sx = x < W ? x : max(2 * W - 2 - x, 0), sy = y < H ? y : max(2 * H - 2 - y, 0);
        if (flip & 1) sx = W - 1 - sx;
        if (flip & 2) sy = H - 1 - sy;
        const long long p = (long long)sy * W + sx;
        float* d = f + i * kFeatures;
        float noise = 0.0f;
        for (int c = 0; c < 3; ++c) {
            const float m = mean[3 * p + c];
            d[c] = m;
            d[3 + c] = albedo[3 * p + c];
            d[6 + c] = normal[3 * p + c];
            noise += sqrtf(fmaxf(var[3 * p + c], 0.0f)) / (1.0f + fmaxf(m, 0.0f));
        }
        d[9] = depth[p];
        d[10] = noise * (1.0f / 3.0f);
    }
}

inline int gsz(long long n, int block = 256) {
    long long g = (n + block - 1) / block;
    return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

// ---------------------------------------------------------------- network
struct UnetLayer {
    int cin, cout, relu;  // cin % 16 == 0 (input padded); cout % 8 == 0
    int cout_pad;         // cout rounded up to 16 (gradient operand channels)
    long long w_off, b_off;  // parameter vector: w [9][cout][cin], then b [cout]
    int nt, rows_fwd;     // forward conv: n8 tiles per CTA, BF16 weight rows
    int nt_b, rows_bwd;   // backward-data conv (outputs cin channels)
    long long wf_off, wb_off;  // BF16 weight copies
};

// Layer table: input padded to 16 channels, output 8 channels of which 3 are used.
const int kLayers[][3] = {
    {16, 32, 1}, {32, 32, 1},   // enc0 -> e0
    {32, 48, 1}, {48, 48, 1},   // enc1 -> e1
    {48, 64, 1}, {64, 64, 1},   // enc2 -> e2
    {64, 80, 1}, {80, 80, 1},   // enc3 -> e3
    {80, 96, 1},                // bottleneck -> b
    {176, 80, 1},               // dec3: up(b) + e3 -> d3
    {144, 64, 1},               // dec2: up(d3) + e2 -> d2
    {112, 48, 1},               // dec1: up(d2) + e1 -> d1
    {80, 32, 1},                // dec0: up(d1) + e0 -> d0
    {32, 8, 0},                 // output
};
// pyramid level (resolution H >> level) each layer runs at
const int kLayerLevel[] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 3, 2, 1, 0, 0};
constexpr int kNumLayers = 14;

int pick_nt(int c) {
    if (c <= 64) return c / 8;  // the whole channel count in one CTA
    for (int nt = 6; nt >= 2; --nt)
        if (c % (nt * 8) == 0) return nt;
    return 2;
}

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

// Activation workspace (BF16), by name; sizes in elements for N x H x W inputs.
enum {
    T_X, T_A0, T_E0, T_P0, T_A1, T_E1, T_P1, T_A2, T_E2, T_P2, T_A3, T_E3, T_P3, T_B,
    T_D3, T_D2, T_D1, T_D0, T_OUT, T_G, T_G2, T_COUNT
};
// FP32 gradients, by name.
enum {
    G_OUT, G_D0, G_C0S, G_D1, G_D2, G_D3, G_B, G_E0, G_E1, G_E2, G_E3, G_P3, G_A3, G_P2, G_A2, G_P1, G_A1, G_P0,
    G_A0, G_COUNT
};

}  // namespace

struct Unet {
    std::vector<UnetLayer> layers;
    long long n_params = 0;
    DevBuf<float> params, grads, adam_m, adam_v;
    DevBuf<bf16> wf, wb;
    long long step = 0;
    int N = 0, H = 0, W = 0;
    DevBuf<bf16> act;
    DevBuf<float> gbuf;
    long long act_off[T_COUNT], g_off[G_COUNT];
    DevBuf<float> io;       // device copies of host features / targets / outputs
    DevBuf<float> film_ws;  // film planes, packed features and padded output of salty_denoise_unet
    DevBuf<double> loss;
    DevBuf<float> wg_ws;    // per-CTA partial weight and bias gradients (fixed-order sums)
    DevBuf<bf16> cat_ws;    // a decoder convolution's concatenated input, for its weight gradient
    int conv_kind = SALTY_CONV_TCGEN05;  // convolution kernels (forward, backward-data, weights)
};

namespace {

void init_layers(Unet& u) {
    u.layers.clear();
    long long off = 0, wf = 0, wb = 0;
    for (int i = 0; i < kNumLayers; ++i) {
        UnetLayer L;
        L.cin = kLayers[i][0];
        L.cout = kLayers[i][1];
        L.relu = kLayers[i][2];
        L.cout_pad = round_up(L.cout, 16);
        L.w_off = off;
        off += 9LL * L.cin * L.cout;
        L.b_off = off;
        off += L.cout;
        L.nt = pick_nt(L.cout);
        L.rows_fwd = round_up(L.cout, L.nt * 8);
        L.nt_b = pick_nt(L.cin);
        L.rows_bwd = round_up(L.cin, L.nt_b * 8);
        L.wf_off = wf;
        wf += 9LL * L.rows_fwd * L.cin;
        L.wb_off = wb;
        wb += 9LL * L.rows_bwd * L.cout_pad;
        u.layers.push_back(L);
    }
    u.n_params = off;
}

salty_status launch_conv(salty_ctx* ctx, int kind, const ConvSrc& in, int cin, const bf16* w, int rows, int nt,
                         const float* bias, bf16* out, int out_cs, int cout, int N, int H, int W, int relu) {
    if (kind == SALTY_CONV_TCGEN05 && in.a_shift == 0 && in.a_ch >= cin && rows <= 256)
        return conv3x3_tma(ctx, in.a, in.a_cs, cin, w, rows, bias, out, out_cs, 0, cout, N, H, W, relu,
                           ctx->status.p + 8);
    if (kind == SALTY_CONV_TCGEN05 || kind == SALTY_CONV_TCGEN05_CP_ASYNC)
        return conv3x3_tc(ctx, in, cin, w, rows, bias, out, out_cs, 0, cout, N, H, W, relu, ctx->status.p + 8);
    const int tiles = N * ((W + kTileX - 1) / kTileX) * ((H + kTileY - 1) / kTileY);
    dim3 grid(tiles, rows / (nt * 8));
    const size_t smem = ((size_t)kHaloX * kHaloY + (size_t)nt * 8) * (cin + 8) * sizeof(bf16);
#define SALTY_CONV_CASE(NTV)                                                                                         \
    case NTV: {                                                                                                     \
        SALTY_TRY_CUDA(ctx->err,                                                                                    \
                       cudaFuncSetAttribute(k_conv3x3<NTV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        k_conv3x3<NTV><<<grid, kConvThreads, smem, ctx->stream>>>(in, cin, w, bias, out, out_cs, 0, cout, N, H, W,   \
                                                                  relu);                                            \
        break;                                                                                                      \
    }
    switch (nt) {
        SALTY_CONV_CASE(1) SALTY_CONV_CASE(2) SALTY_CONV_CASE(4) SALTY_CONV_CASE(5) SALTY_CONV_CASE(6)
        SALTY_CONV_CASE(8)
        default:
            return ctx->err.fail(SALTY_ERR_INVALID_ARG, "unsupported conv tile %d", nt);
    }
#undef SALTY_CONV_CASE
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

salty_status launch_wgrad(salty_ctx* ctx, Unet& u, const bf16* dy, int cpad, int cout, const ConvSrc& x, int cin,
                          float* dw, int N, int H, int W) {
    if (u.conv_kind != SALTY_CONV_MMA_SYNC)
        return conv_wgrad_tc(ctx, dy, cpad, cout, x, cin, dw, N, H, W, u.wg_ws.p, u.wg_ws.cap, u.cat_ws.p,
                             u.cat_ws.cap, ctx->status.p + 8);
    const size_t smem = ((size_t)kTileX * kTileY * (kWgradCo + 8) + (size_t)kHaloX * kHaloY * 24) * sizeof(bf16);
    const int tiles = N * ((W + kTileX - 1) / kTileX) * ((H + kTileY - 1) / kTileY);
    const int mg = (cpad + kWgradCo - 1) / kWgradCo;
    // about four resident CTAs per SM over all (output-channel group, input slice) pairs
    int gx = ctx->num_sms * 4 / (mg * (cin / 16));
    if (gx < 1) gx = 1;
    if (gx > tiles) gx = tiles;
    dim3 grid(gx, mg, cin / 16);
    k_conv3x3_wgrad<<<grid, kConvThreads, smem, ctx->stream>>>(dy, cpad, cout, x, cin, dw, N, H, W);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

salty_status ensure_workspace(salty_ctx* ctx, Unet& u, int N, int H, int W) {
    if (u.N == N && u.H == H && u.W == W && u.act.p) return SALTY_OK;
    const long long P0 = (long long)N * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64, P4 = P0 / 256;
    const long long asz[T_COUNT] = {P0 * 16, P0 * 32, P0 * 32, P1 * 32, P1 * 48, P1 * 48, P2 * 48, P2 * 64, P2 * 64,
                                    P3 * 64, P3 * 80, P3 * 80, P4 * 80, P4 * 96, P3 * 80, P2 * 64, P1 * 48, P0 * 32,
                                    P0 * 8, P0 * 176, P0 * 176};
    const long long gsz_[G_COUNT] = {P0 * 8, P0 * 32, P0 * 32, P1 * 48, P2 * 64, P3 * 80, P4 * 96, P0 * 32, P1 * 48,
                                     P2 * 64, P3 * 80, P4 * 80, P3 * 80, P3 * 64, P2 * 64, P2 * 48, P1 * 48, P1 * 32,
                                     P0 * 32};
    long long o = 0;
    for (int i = 0; i < T_COUNT; ++i) { u.act_off[i] = o; o += (asz[i] + 63) / 64 * 64; }
    SALTY_TRY_CUDA(ctx->err, u.act.ensure((size_t)o));
    o = 0;
    for (int i = 0; i < G_COUNT; ++i) { u.g_off[i] = o; o += (gsz_[i] + 63) / 64 * 64; }
    SALTY_TRY_CUDA(ctx->err, u.gbuf.ensure((size_t)o));
    size_t ws = 0;
    for (int i = 0; i < kNumLayers; ++i) {
        const UnetLayer& L = u.layers[i];
        const int lv = kLayerLevel[i];
        ws = std::max(ws, conv_wgrad_tc_workspace(ctx->num_sms, L.cin, L.cout_pad, N, H >> lv, W >> lv));
    }
    // the bias gradients' per-block partials use the same workspace: up to 4 blocks per SM
    // x 128 channels
    ws = std::max(ws, (size_t)ctx->num_sms * 4 * 128);
    SALTY_TRY_CUDA(ctx->err, u.wg_ws.ensure(ws));
    size_t cat = 0;
    for (int i = 0; i < kNumLayers; ++i)
        cat = std::max(cat, (size_t)N * (H >> kLayerLevel[i]) * (W >> kLayerLevel[i]) * u.layers[i].cin);
    SALTY_TRY_CUDA(ctx->err, u.cat_ws.ensure(cat));
    u.N = N; u.H = H; u.W = W;
    return SALTY_OK;
}

salty_status refresh_bf16(salty_ctx* ctx, Unet& u) {
    for (const UnetLayer& L : u.layers)
        k_weights_to_bf16<<<gsz(9LL * L.cout * L.cin), 256, 0, ctx->stream>>>(
            u.params.p + L.w_off, L.cout, L.cin, L.rows_fwd, L.rows_bwd, L.cout_pad, u.wf.p + L.wf_off, u.wb.p + L.wb_off);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

struct Fwd {
    bf16* t[T_COUNT];
};

salty_status forward(salty_ctx* ctx, Unet& u, const float* d_feat, int N, int H, int W, Fwd& F) {
    SALTY_TRY(ensure_workspace(ctx, u, N, H, W));
    for (int i = 0; i < T_COUNT; ++i) F.t[i] = u.act.p + u.act_off[i];
    cudaStream_t st = ctx->stream;
    const long long P0 = (long long)N * H * W;
    k_prep_input<<<gsz(P0), 256, 0, st>>>(d_feat, P0, F.t[T_X]);
    auto conv = [&](int li, const ConvSrc& in, int out, int h, int w) {
        const UnetLayer& L = u.layers[li];
        return launch_conv(ctx, u.conv_kind, in, L.cin, u.wf.p + L.wf_off, L.rows_fwd, L.nt, u.params.p + L.b_off,
                           F.t[out], L.cout, L.cout, N, h, w, L.relu);
    };
    auto pool = [&](int in, int out, int h, int w, int c) {
        const long long groups = (long long)N * (h / 2) * (w / 2) * (c / 8);
        k_pool<<<gsz(groups), 256, 0, st>>>(F.t[in], F.t[out], N, h, w, c);
    };
    auto x = [&](int t, int c) { return conv_src(F.t[t], c, c); };
    // decoder inputs: [up2(coarse) | skip], read by the convolutions from both tensors
    auto cat = [&](int coarse, int cc, int skip, int cs) { return conv_src_cat(F.t[coarse], cc, F.t[skip], cs); };
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8, H4 = H / 16, W4 = W / 16;
    SALTY_TRY(conv(0, x(T_X, 16), T_A0, H, W));
    SALTY_TRY(conv(1, x(T_A0, 32), T_E0, H, W));
    pool(T_E0, T_P0, H, W, 32);
    SALTY_TRY(conv(2, x(T_P0, 32), T_A1, H1, W1));
    SALTY_TRY(conv(3, x(T_A1, 48), T_E1, H1, W1));
    pool(T_E1, T_P1, H1, W1, 48);
    SALTY_TRY(conv(4, x(T_P1, 48), T_A2, H2, W2));
    SALTY_TRY(conv(5, x(T_A2, 64), T_E2, H2, W2));
    pool(T_E2, T_P2, H2, W2, 64);
    SALTY_TRY(conv(6, x(T_P2, 64), T_A3, H3, W3));
    SALTY_TRY(conv(7, x(T_A3, 80), T_E3, H3, W3));
    pool(T_E3, T_P3, H3, W3, 80);
    SALTY_TRY(conv(8, x(T_P3, 80), T_B, H4, W4));
    SALTY_TRY(conv(9, cat(T_B, 96, T_E3, 80), T_D3, H3, W3));
    SALTY_TRY(conv(10, cat(T_D3, 80, T_E2, 64), T_D2, H2, W2));
    SALTY_TRY(conv(11, cat(T_D2, 64, T_E1, 48), T_D1, H1, W1));
    SALTY_TRY(conv(12, cat(T_D1, 48, T_E0, 32), T_D0, H, W));
    SALTY_TRY(conv(13, x(T_D0, 32), T_OUT, H, W));
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

// One conv layer backward.  dy: FP32 [npx][cout] gradient of the layer output y.  Adds the
// weight and bias gradients; leaves dL/d(input) in BF16 in F.t[T_G2] ([npx][cin]) when
// want_dx.
salty_status conv_backward(salty_ctx* ctx, Unet& u, Fwd& F, int li, const ConvSrc& x, int y, const float* dy, int N,
                           int h, int w, bool want_dx, const bf16* dy16 = nullptr, int dy16_cs = 0) {
    const UnetLayer& L = u.layers[li];
    const long long npx = (long long)N * h * w;
    cudaStream_t st = ctx->stream;
    bf16* g = F.t[T_G];
    // ReLU backward and the bias gradient's per-block partial sums in one pass (4 blocks per
    // SM), then the partials added in block order
    const int per = 256 / (L.cout_pad / 8);
    const int bias_blocks = (int)std::min<long long>((long long)ctx->num_sms * 4, (npx + per - 1) / per);
    k_relu_bwd_bias<<<bias_blocks, 256, (size_t)per * L.cout * sizeof(float), st>>>(
        F.t[y], L.cout, dy, dy16, dy16_cs, L.cout, L.relu, npx, g, L.cout_pad, u.wg_ws.p);
    k_bias_reduce<<<(L.cout + 127) / 128, 128, 0, st>>>(u.wg_ws.p, bias_blocks, L.cout, u.grads.p + L.b_off);
    SALTY_TRY(launch_wgrad(ctx, u, g, L.cout_pad, L.cout, x, L.cin, u.grads.p + L.w_off, N, h, w));
    if (want_dx)
        SALTY_TRY(launch_conv(ctx, u.conv_kind, conv_src(g, L.cout_pad, L.cout_pad), L.cout_pad, u.wb.p + L.wb_off,
                              L.rows_bwd, L.nt_b, nullptr, F.t[T_G2], L.cin, L.cin, N, h, w, 0));
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

// Loss and all gradients for the batch in F (after forward); grads are zeroed first.
salty_status backward(salty_ctx* ctx, Unet& u, Fwd& F, const float* d_target, int N, int H, int W, double* loss) {
    cudaStream_t st = ctx->stream;
    const long long P0 = (long long)N * H * W;
    float* G[G_COUNT];
    for (int i = 0; i < G_COUNT; ++i) G[i] = u.gbuf.p + u.g_off[i];
    SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(u.grads.p, 0, u.n_params * sizeof(float), st));
    SALTY_TRY_CUDA(ctx->err, u.loss.ensure(1));
    SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(u.loss.p, 0, sizeof(double), st));
    k_loss<<<gsz(P0), 256, 0, st>>>(F.t[T_OUT], F.t[T_X], d_target, P0, G[G_OUT], u.loss.p);
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8, H4 = H / 16, W4 = W / 16;
    const long long P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64, P4 = P0 / 256;
    auto x = [&](int t, int c) { return conv_src(F.t[t], c, c); };
    auto cat = [&](int coarse, int cc, int skip, int cs) { return conv_src_cat(F.t[coarse], cc, F.t[skip], cs); };
    auto to_f32 = [&](int cs, int off, int c, long long np, float* dst, int acc) {
        k_grad_to_f32<<<gsz(np * c / 8), 256, 0, st>>>(F.t[T_G2], cs, off, c, np, dst, acc);
    };
    // decoder: a conv's input gradient splits into the up-sampled part and the skip part
    auto split = [&](int cc, int cs, int h, int w, float* g_coarse, float* g_skip) {
        const long long np = (long long)N * h * w;
        k_upsample_bwd<<<gsz(np / 4 * cc / 8), 256, 0, st>>>(F.t[T_G2], cc + cs, g_coarse, cc, N, h, w);
        to_f32(cc + cs, cc, cs, np, g_skip, 0);
    };
    SALTY_TRY(conv_backward(ctx, u, F, 13, x(T_D0, 32), T_OUT, G[G_OUT], N, H, W, true));
    SALTY_TRY(conv_backward(ctx, u, F, 12, cat(T_D1, 48, T_E0, 32), T_D0, nullptr, N, H, W, true, F.t[T_G2], 32));
    split(48, 32, H, W, G[G_D1], G[G_E0]);
    SALTY_TRY(conv_backward(ctx, u, F, 11, cat(T_D2, 64, T_E1, 48), T_D1, G[G_D1], N, H1, W1, true));
    split(64, 48, H1, W1, G[G_D2], G[G_E1]);
    SALTY_TRY(conv_backward(ctx, u, F, 10, cat(T_D3, 80, T_E2, 64), T_D2, G[G_D2], N, H2, W2, true));
    split(80, 64, H2, W2, G[G_D3], G[G_E2]);
    SALTY_TRY(conv_backward(ctx, u, F, 9, cat(T_B, 96, T_E3, 80), T_D3, G[G_D3], N, H3, W3, true));
    split(96, 80, H3, W3, G[G_B], G[G_E3]);
    SALTY_TRY(conv_backward(ctx, u, F, 8, x(T_P3, 80), T_B, G[G_B], N, H4, W4, true));
    to_f32(80, 0, 80, P4, G[G_P3], 0);
    k_pool_bwd<<<gsz(P4 * 80 / 8), 256, 0, st>>>(F.t[T_E3], G[G_P3], G[G_E3], N, H3, W3, 80);
    SALTY_TRY(conv_backward(ctx, u, F, 7, x(T_A3, 80), T_E3, G[G_E3], N, H3, W3, true));
    SALTY_TRY(conv_backward(ctx, u, F, 6, x(T_P2, 64), T_A3, nullptr, N, H3, W3, true, F.t[T_G2], 80));
    to_f32(64, 0, 64, P3, G[G_P2], 0);
    k_pool_bwd<<<gsz(P3 * 64 / 8), 256, 0, st>>>(F.t[T_E2], G[G_P2], G[G_E2], N, H2, W2, 64);
    SALTY_TRY(conv_backward(ctx, u, F, 5, x(T_A2, 64), T_E2, G[G_E2], N, H2, W2, true));
    SALTY_TRY(conv_backward(ctx, u, F, 4, x(T_P1, 48), T_A2, nullptr, N, H2, W2, true, F.t[T_G2], 64));
    to_f32(48, 0, 48, P2, G[G_P1], 0);
    k_pool_bwd<<<gsz(P2 * 48 / 8), 256, 0, st>>>(F.t[T_E1], G[G_P1], G[G_E1], N, H1, W1, 48);
    SALTY_TRY(conv_backward(ctx, u, F, 3, x(T_A1, 48), T_E1, G[G_E1], N, H1, W1, true));
    SALTY_TRY(conv_backward(ctx, u, F, 2, x(T_P0, 32), T_A1, nullptr, N, H1, W1, true, F.t[T_G2], 48));
    to_f32(32, 0, 32, P1, G[G_P0], 0);
    k_pool_bwd<<<gsz(P1 * 32 / 8), 256, 0, st>>>(F.t[T_E0], G[G_P0], G[G_E0], N, H, W, 32);
    SALTY_TRY(conv_backward(ctx, u, F, 1, x(T_A0, 32), T_E0, G[G_E0], N, H, W, true));
    SALTY_TRY(conv_backward(ctx, u, F, 0, x(T_X, 16), T_A0, nullptr, N, H, W, false, F.t[T_G2], 32));
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    double l = 0.0;
    SALTY_TRY_CUDA(ctx->err, cudaMemcpyAsync(&l, u.loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(st));
    *loss = l / (3.0 * (double)P0);
    (void)P1; (void)P2; (void)P3; (void)W4; (void)H4;
    return SALTY_OK;
}

// Copies n floats of a host-or-device array to the device workspace at `off`.
salty_status stage(salty_ctx* ctx, Unet& u, const float* src, long long n, long long off, const float** out) {
    if (is_device_ptr(src)) {
        *out = src;
        return SALTY_OK;
    }
    SALTY_TRY_CUDA(ctx->err, cudaMemcpyAsync(u.io.p + off, src, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    *out = u.io.p + off;
    return SALTY_OK;
}

// The tensor-core convolutions' status word: zeroed before a call's first launch, read
// after its last synchronisation.
salty_status conv_status_reset(salty_ctx* ctx) {
    SALTY_TRY_CUDA(ctx->err, cudaMemsetAsync(ctx->status.p + 8, 0, sizeof(int), ctx->stream));
    return SALTY_OK;
}
salty_status conv_status_check(salty_ctx* ctx) {
    int s = 0;
    SALTY_TRY_CUDA(ctx->err, cudaMemcpy(&s, ctx->status.p + 8, sizeof(int), cudaMemcpyDeviceToHost));
    if (s & 1) return ctx->err.fail(SALTY_ERR_TIMEOUT, "unet: a tensor-core convolution gave up waiting");
    if (s) return ctx->err.fail(SALTY_ERR_CUDA, "unet: a tensor-core convolution found its shared memory misaligned");
    return SALTY_OK;
}

salty_status check_shape(salty_ctx* ctx, int n, int h, int w) {
    if (n <= 0 || h <= 0 || w <= 0 || h % 16 || w % 16)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "unet: n, h, w must be positive and h, w multiples of 16");
    if ((long long)n * h * w > (1ll << 26)) return ctx->err.fail(SALTY_ERR_CAPACITY, "unet: batch too large");
    return SALTY_OK;
}

}  // namespace
}  // namespace salty

struct salty_unet {
    salty::Unet net;
};

extern "C" {

salty_status salty_unet_create(salty_ctx* ctx, uint64_t seed, salty_unet** out) {
    using namespace salty;
    if (!ctx || !out) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    auto* h = new (std::nothrow) salty_unet();
    if (!h) return ctx->err.fail(SALTY_ERR_OOM, "host allocation failed");
    Unet& u = h->net;
    init_layers(u);
    long long wf = 0, wb = 0;
    for (const UnetLayer& L : u.layers) {
        wf = L.wf_off + 9LL * L.rows_fwd * L.cin;
        wb = L.wb_off + 9LL * L.rows_bwd * L.cout_pad;
    }
    auto fail = [&](salty_status s) { delete h; return s; };
    if (u.params.ensure(u.n_params) != cudaSuccess || u.grads.ensure(u.n_params) != cudaSuccess ||
        u.adam_m.ensure(u.n_params) != cudaSuccess || u.adam_v.ensure(u.n_params) != cudaSuccess ||
        u.wf.ensure(wf) != cudaSuccess || u.wb.ensure(wb) != cudaSuccess)
        return fail(ctx->err.fail(SALTY_ERR_OOM, "unet parameters"));
    // He-uniform weights from a PCG stream (seeded), zero biases
    std::vector<float> p(u.n_params, 0.0f);
    uint64_t s = seed + 1442695040888963407ull;
    auto next = [&]() {
        uint64_t old = s;
        s = old * 6364136223846793005ull + 1442695040888963407ull;
        uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27), rot = (uint32_t)(old >> 59);
        return (float)((xs >> rot) | (xs << ((~rot + 1u) & 31u))) / 4294967296.0f;
    };
    for (size_t li = 0; li < u.layers.size(); ++li) {
        const UnetLayer& L = u.layers[li];
        const int real_cin = li == 0 ? kFeatures : L.cin;
        // the output layer starts small: the initial prediction is close to the input
        const float bound = std::sqrt(6.0f / (9.0f * real_cin)) * (L.relu ? 1.0f : 0.1f);
        for (long long i = 0; i < 9LL * L.cin * L.cout; ++i) {
            const int ci = (int)(i % L.cin);
            p[L.w_off + i] = (li == 0 && ci >= kFeatures) ? 0.0f : (2.0f * next() - 1.0f) * bound;
        }
    }
    cudaStream_t st = ctx->stream;
    if (cudaMemcpyAsync(u.params.p, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(u.adam_m.p, 0, u.n_params * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(u.adam_v.p, 0, u.n_params * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(u.wf.p, 0, wf * sizeof(bf16), st) != cudaSuccess ||
        cudaMemsetAsync(u.wb.p, 0, wb * sizeof(bf16), st) != cudaSuccess)
        return fail(ctx->err.fail(SALTY_ERR_CUDA, "unet init copies"));
    if (refresh_bf16(ctx, u) != SALTY_OK) return fail(SALTY_ERR_CUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(ctx->err.fail(SALTY_ERR_CUDA, "unet init"));
    *out = h;
    return SALTY_OK;
}

void salty_unet_destroy(salty_ctx* ctx, salty_unet* net) {
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    delete net;
}

int64_t salty_unet_param_count(const salty_unet* net) { return net ? net->net.n_params : 0; }

salty_status salty_unet_get_params(salty_ctx* ctx, salty_unet* net, float* params, float* grads) {
    using namespace salty;
    if (!ctx || !net) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    if (params) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(params, u.params.p, u.n_params * sizeof(float), cudaMemcpyDefault));
    if (grads) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(grads, u.grads.p, u.n_params * sizeof(float), cudaMemcpyDefault));
    return SALTY_OK;
}

salty_status salty_unet_get_adam(salty_ctx* ctx, salty_unet* net, float* m, float* v, int64_t* step) {
    using namespace salty;
    if (!ctx || !net) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    if (m) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(m, u.adam_m.p, u.n_params * sizeof(float), cudaMemcpyDefault));
    if (v) SALTY_TRY_CUDA(ctx->err, cudaMemcpy(v, u.adam_v.p, u.n_params * sizeof(float), cudaMemcpyDefault));
    if (step) *step = u.step;
    return SALTY_OK;
}

salty_status salty_unet_set_adam(salty_ctx* ctx, salty_unet* net, const float* m, const float* v, int64_t step) {
    using namespace salty;
    if (!ctx || !net || !m || !v || step < 0) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    SALTY_TRY_CUDA(ctx->err, cudaMemcpy(u.adam_m.p, m, u.n_params * sizeof(float), cudaMemcpyDefault));
    SALTY_TRY_CUDA(ctx->err, cudaMemcpy(u.adam_v.p, v, u.n_params * sizeof(float), cudaMemcpyDefault));
    u.step = step;
    return SALTY_OK;
}

salty_status salty_unet_set_params(salty_ctx* ctx, salty_unet* net, const float* params) {
    using namespace salty;
    if (!ctx || !net || !params) return SALTY_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    SALTY_TRY_CUDA(ctx->err, cudaMemcpy(u.params.p, params, u.n_params * sizeof(float), cudaMemcpyDefault));
    SALTY_TRY(refresh_bf16(ctx, u));
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(ctx->stream));
    return SALTY_OK;
}

salty_status salty_unet_forward(salty_ctx* ctx, salty_unet* net, const float* features, int32_t n, int32_t h,
                                int32_t w, float* out_rgb) {
    using namespace salty;
    if (!ctx || !net || !features || !out_rgb) return SALTY_ERR_INVALID_ARG;
    SALTY_TRY(check_shape(ctx, n, h, w));
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    const long long P0 = (long long)n * h * w;
    SALTY_TRY_CUDA(ctx->err, u.io.ensure((size_t)P0 * 16));
    const float* df;
    SALTY_TRY(stage(ctx, u, features, P0 * kFeatures, 0, &df));
    SALTY_TRY(conv_status_reset(ctx));
    Fwd F;
    SALTY_TRY(forward(ctx, u, df, n, h, w, F));
    const bool dev_out = is_device_ptr(out_rgb);
    float* dout = dev_out ? out_rgb : u.io.p + P0 * kFeatures;
    k_output<<<gsz(P0), 256, 0, ctx->stream>>>(F.t[T_OUT], F.t[T_X], P0, dout);
    if (!dev_out)
        SALTY_TRY_CUDA(ctx->err, cudaMemcpyAsync(out_rgb, dout, P0 * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(ctx->stream));
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return conv_status_check(ctx);
}

salty_status salty_unet_train_step(salty_ctx* ctx, salty_unet* net, const float* features, const float* target_rgb,
                                   int32_t n, int32_t h, int32_t w, float lr, float* loss) {
    using namespace salty;
    if (!ctx || !net || !features || !target_rgb) return SALTY_ERR_INVALID_ARG;
    SALTY_TRY(check_shape(ctx, n, h, w));
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    const long long P0 = (long long)n * h * w;
    SALTY_TRY_CUDA(ctx->err, u.io.ensure((size_t)P0 * 16));
    const float *df, *dt;
    SALTY_TRY(stage(ctx, u, features, P0 * kFeatures, 0, &df));
    SALTY_TRY(stage(ctx, u, target_rgb, P0 * 3, P0 * kFeatures, &dt));
    SALTY_TRY(conv_status_reset(ctx));
    Fwd F;
    SALTY_TRY(forward(ctx, u, df, n, h, w, F));
    double l = 0.0;
    SALTY_TRY(backward(ctx, u, F, dt, n, h, w, &l));
    if (loss) *loss = (float)l;
    if (lr > 0.0f) {
        ++u.step;
        AdamArgs a;
        a.lr = lr;
        a.b1 = 0.9f;
        a.b2 = 0.999f;
        a.eps = 1e-8f;
        a.c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)u.step)));
        a.c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)u.step)));
        k_adam<<<gsz(u.n_params), 256, 0, ctx->stream>>>(u.params.p, u.grads.p, u.adam_m.p, u.adam_v.p, u.n_params, a);
        SALTY_TRY(refresh_bf16(ctx, u));
    }
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(ctx->stream));
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return conv_status_check(ctx);
}

salty_status salty_denoise_unet_ensemble(salty_ctx* ctx, salty_unet* net, salty_scene* scene, int32_t mirrors,
                                        float* out_rgb) {
    using namespace salty;
    if (!ctx || !net || !scene || !out_rgb) return SALTY_ERR_INVALID_ARG;
    if (mirrors != 1 && mirrors != 2 && mirrors != 4 && mirrors != 8)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "mirrors must be 1, 2, 4 or 8");
    cudaSetDevice(ctx->device);
    Unet& u = net->net;
    const Film& Fm = scene->film;
    const int W = Fm.width, H = Fm.height;
    if ((long long)W * H == 0 || Fm.samples == 0) return ctx->err.fail(SALTY_ERR_NOT_BUILT, "the film is empty");
    const int Wp = (W + 15) / 16 * 16, Hp = (H + 15) / 16 * 16;
    SALTY_TRY(check_shape(ctx, 1, Hp, Wp));
    const long long npx = (long long)W * H, npp = (long long)Wp * Hp;
    // The symmetries run as batches of images of one shape: the mirror images (up to 4) in
    // one forward pass, their transposes in a second -- each convolution launch then has
    // that many times more strips to spread over the SMs.  An image's outputs do not depend
    // on the batch it runs in (tests/test_unet_gpu.py), and the images are added to the
    // result in the order k = 0..mirrors-1, as one pass per image would add them.
    const int per = mirrors < 4 ? mirrors : 4;
    SALTY_TRY(check_shape(ctx, per, Hp, Wp));
    // [mean 3 | var 3 | albedo 3 | normal 3 | depth 1] per film pixel, then features, then the image
    SALTY_TRY_CUDA(ctx->err, u.film_ws.ensure((size_t)(npx * 16 + per * npp * kFeatures)));
    float* mean = u.film_ws.p;
    float* var = mean + npx * 3;
    float* alb = var + npx * 3;
    float* nrm = alb + npx * 3;
    float* dep = nrm + npx * 3;
    float* feat = dep + npx;
    float* img = feat + per * npp * kFeatures;
    SALTY_TRY(film_features(ctx, scene, mean, var, alb, nrm, dep));
    SALTY_TRY(conv_status_reset(ctx));
    for (int k0 = 0; k0 < mirrors; k0 += per) {
        for (int j = 0; j < per; ++j)
            k_pack_features<<<gsz(npp), 256, 0, ctx->stream>>>(mean, var, alb, nrm, dep, W, H, Wp, Hp, k0 + j,
                                                               feat + j * npp * kFeatures);
        Fwd F;
        if (k0 & 4)
            SALTY_TRY(forward(ctx, u, feat, per, Wp, Hp, F));  // the transposed frames: Hp wide, Wp tall
        else
            SALTY_TRY(forward(ctx, u, feat, per, Hp, Wp, F));
        for (int j = 0; j < per; ++j)
            k_output_flipped<<<gsz(npx), 256, 0, ctx->stream>>>(F.t[T_OUT] + j * npp * 8, F.t[T_X] + j * npp * 16, W,
                                                               H, Wp, Hp, k0 + j, 1.0f / (float)mirrors,
                                                               k0 + j == 0, img);
    }
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    SALTY_TRY_CUDA(ctx->err, cudaMemcpyAsync(out_rgb, img, (size_t)npx * 3 * sizeof(float), cudaMemcpyDefault,
                                             ctx->stream));
    SALTY_TRY_CUDA(ctx->err, cudaStreamSynchronize(ctx->stream));
    return conv_status_check(ctx);
}

salty_status salty_unet_set_conv_kernel(salty_ctx* ctx, salty_unet* net, int32_t kind) {
    if (!ctx || !net) return SALTY_ERR_INVALID_ARG;
    if (kind != SALTY_CONV_TCGEN05 && kind != SALTY_CONV_MMA_SYNC && kind != SALTY_CONV_TCGEN05_CP_ASYNC)
        return ctx->err.fail(SALTY_ERR_INVALID_ARG, "unknown convolution kernel %d", (int)kind);
    net->net.conv_kind = kind;
    return SALTY_OK;
}

salty_status salty_denoise_unet(salty_ctx* ctx, salty_unet* net, salty_scene* scene, float* out_rgb) {
    return salty_denoise_unet_ensemble(ctx, net, scene, 1, out_rgb);
}

}  // extern "C"

