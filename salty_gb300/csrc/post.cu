// post.cu -- tonemapping, sRGB8 and the NLM denoisers.
//
//   ToneMapper::Map (src/s3d_tonemapper.cpp:206-353): a log-average / max-luminance
//   reduction, then a per-pixel curve (Reinhard, Uncharted2, ACES) fused with the clamp,
//   OETF and 8-bit rounding of PathTracer::Capture (src/s3d_pt.cpp:145-171).  Both passes
//   stream the image once (HBM bound); per-pixel arithmetic keeps the reference's
//   operation order with separately rounded products.  The reduction sums log terms in
//   double, where the reference adds them one by one in single precision.
//   FilterNLM (src/s3d_denoiser.cpp:19-95): each block stages its tile plus halo in
//   shared memory and evaluates the reference's weights in the reference's order.
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "internal.h"

namespace salty {
namespace {

__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }
inline int f2o_host(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

struct LumAcc {
    double sum;
    int maxo;
    int pad;
};

// RGBToY (src/s3d_tonemapper.cpp:31-33)
__device__ __forceinline__ float rgb_to_y(float r, float g, float b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
}

constexpr int kRedBlock = 256;

__global__ void __launch_bounds__(kRedBlock) k_lum_reduce(const float* __restrict__ rgb, long long npx, LumAcc* acc) {
    const float eps = 0.00001f;
    double s = 0.0;
    float mx = -FLT_MAX;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npx;
         i += (long long)gridDim.x * blockDim.x) {
        float lw = rgb_to_y(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
        if (lw != lw) lw = eps;
        if (lw < FLT_EPSILON) lw = eps;
        mx = fmaxf(mx, lw);
        s += (double)logf(__fadd_rn(eps, lw));
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, off);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    __shared__ double ss[kRedBlock / 32];
    __shared__ float sm[kRedBlock / 32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { ss[w] = s; sm[w] = mx; }
    __syncthreads();
    if (w == 0) {
        s = l < kRedBlock / 32 ? ss[l] : 0.0;
        mx = l < kRedBlock / 32 ? sm[l] : -FLT_MAX;
        for (int off = 16; off > 0; off >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, off);
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        }
        if (l == 0) {
            atomicAdd(&acc->sum, s);
            atomicMax(&acc->maxo, f2o(mx));
        }
    }
}

__device__ __forceinline__ float u2_curve(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.01f, F = 0.30f;
    // ((x*(A*x + C*B) + D*E) / (x*(A*x + B) + D*F)) - E/F
    float num = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), __fmul_rn(C, B))), __fmul_rn(D, E));
    float den = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), B)), __fmul_rn(D, F));
    return __fsub_rn(__fdiv_rn(num, den), __fdiv_rn(E, F));
}

__device__ __forceinline__ float saturate(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// ACESFilm (src/s3d_tonemapper.cpp:117-130)
__device__ __forceinline__ float aces_curve(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f, f = 0.665406f, g = 12.0f;
    float num = __fmul_rn(x, __fadd_rn(__fdiv_rn(__fmul_rn(__fmul_rn(a, x), f), g), b));
    float den = __fadd_rn(__fmul_rn(__fdiv_rn(__fmul_rn(x, f), g), __fadd_rn(__fmul_rn(__fmul_rn(c, x), f), d)), e);
    return saturate(__fdiv_rn(num, den));
}

// 8-bit code of a tonemapped value: clamp to [0, 1], the OETF (the reference's
// 1.055^(1/2.4)-scaled variant or the standard one), then x * 255 + 0.5 truncated.  The power
// is first taken with the hardware approximation (__powf); only when the scaled value lies
// within 2^-10 of a code boundary is it recomputed with powf, so the code always equals
// the all-powf formula's: the approximation moves x * 255 + 0.5 by less than 1e-4 (from
// the documented errors of the hardware log2 and exp2 on [0.0031308, 1.055]), a tenth of
// the margin.  Most values skip powf entirely.
__device__ __forceinline__ float oetf_scaled(float x, int ref_oetf, bool exact) {
    const float b = ref_oetf ? __fmul_rn(1.055f, x) : x;
    const float p = exact ? powf(b, 1.0f / 2.4f) : __powf(b, 1.0f / 2.4f);
    const float v = ref_oetf ? __fsub_rn(p, 0.055f) : __fsub_rn(__fmul_rn(1.055f, p), 0.055f);
    return __fadd_rn(__fmul_rn(v, 255.0f), 0.5f);
}

__device__ __forceinline__ unsigned char to_srgb8(float x, int ref_oetf) {
    if (x > 1.0f) x = 1.0f;
    if (x < 0.0f) x = 0.0f;
    if (x != x) x = 0.0f;
    if (x <= 0.0031308f) return (unsigned char)__fadd_rn(__fmul_rn(__fmul_rn(12.92f, x), 255.0f), 0.5f);
    float t = oetf_scaled(x, ref_oetf, false);
    const float fr = t - floorf(t);
    if (fr < 0x1p-10f || fr > 1.0f - 0x1p-10f) t = oetf_scaled(x, ref_oetf, true);
    return (unsigned char)t;
}

struct TmParams {
    int type;
    float coeff;
    float m2;      // Reinhard (maxLw * coeff)^2
    float white;   // Uncharted2 curve at LinearWhite
    int ref_oetf;
};

__global__ void k_tonemap(const float* __restrict__ in, long long n, TmParams p, float* __restrict__ out,
                          unsigned char* __restrict__ srgb) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float x = __fmul_rn(in[i], p.coeff);
        float y;
        if (p.type == SALTY_TM_ACES) {
            y = aces_curve(x);
        } else if (p.type == SALTY_TM_UNCHARTED2) {
            y = __fdiv_rn(u2_curve(__fmul_rn(2.0f, x)), p.white);
        } else {
            // L * (1 + L / maxLw2) / (1 + L)  (src/s3d_tonemapper.cpp:256-268)
            y = __fdiv_rn(__fmul_rn(x, __fadd_rn(1.0f, __fdiv_rn(x, p.m2))), __fadd_rn(1.0f, x));
        }
        if (out) out[i] = y;
        if (srgb) srgb[i] = to_srgb8(y, p.ref_oetf);
    }
}

// ---------------------------------------------------------------- NLM (reference)
constexpr int kNlmTile = 16;
constexpr int kNlmHalo = 8;  // 13x13 search (6) + 5x5 patch (2)

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void __launch_bounds__(kNlmTile* kNlmTile) k_nlm_ref(const float4* __restrict__ src, int w, int h,
                                                                  float inv_h2, float two_s2, float4* __restrict__ dst) {
    constexpr int S = kNlmTile + 2 * kNlmHalo;
    __shared__ float4 tile[S][S];
    const int x0 = blockIdx.x * kNlmTile - kNlmHalo, y0 = blockIdx.y * kNlmTile - kNlmHalo;
    for (int i = threadIdx.y * kNlmTile + threadIdx.x; i < S * S; i += kNlmTile * kNlmTile) {
        const int ty = i / S, tx = i % S;
        tile[ty][tx] = src[(size_t)clampi(y0 + ty, 0, h - 1) * w + clampi(x0 + tx, 0, w - 1)];
    }
    __syncthreads();
    const int x = blockIdx.x * kNlmTile + threadIdx.x, y = blockIdx.y * kNlmTile + threadIdx.y;
    if (x >= w || y >= h) return;
    // tile coordinate of image pixel (ix, iy) after clamping: clamp first, then offset
    auto T = [&](int ix, int iy) -> const float4& {
        return tile[clampi(iy, 0, h - 1) - y0][clampi(ix, 0, w - 1) - x0];
    };
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    float sw = 0.0f;
    for (int sx = x - 6; sx <= x + 6; ++sx) {
        for (int sy = y - 6; sy <= y + 6; ++sy) {
            float acc = 0.0f;
            for (int ax = -2; ax <= 2; ++ax) {
                for (int ay = -2; ay <= 2; ++ay) {
                    const float4 a = T(x + ax, y + ay), b = T(sx + ax, sy + ay);
                    const float d0 = __fsub_rn(a.x, b.x), d1 = __fsub_rn(a.y, b.y), d2 = __fsub_rn(a.z, b.z),
                                d3 = __fsub_rn(a.w, b.w);
                    const float q = __fadd_rn(__fadd_rn(__fmul_rn(d3, d3), __fmul_rn(d2, d2)),
                                              __fadd_rn(__fmul_rn(d1, d1), __fmul_rn(d0, d0)));
                    acc = __fadd_rn(acc, q);
                }
            }
            const float arg = __fmul_rn(-fmaxf(__fsub_rn(acc, two_s2), 0.0f), inv_h2);
            const float wt = expf(arg);
            sw = __fadd_rn(sw, wt);
            const float4 c = T(sx, sy);
            sum.x = __fadd_rn(sum.x, __fmul_rn(c.x, wt));
            sum.y = __fadd_rn(sum.y, __fmul_rn(c.y, wt));
            sum.z = __fadd_rn(sum.z, __fmul_rn(c.z, wt));
            sum.w = __fadd_rn(sum.w, __fmul_rn(c.w, wt));
        }
    }
    dst[(size_t)y * w + x] = make_float4(__fdiv_rn(sum.x, sw), __fdiv_rn(sum.y, sw), __fdiv_rn(sum.z, sw),
                                         __fdiv_rn(sum.w, sw));
}

// ---------------------------------------------------------------- NLM (variance scaled)
// Rousselle, Knaus, Zwicker, "Adaptive rendering with non-local means filtering"
// (SIGGRAPH Asia 2012): patch distance normalised by the pixels' variances.
//
// Separable form: for one search offset (dx, dy) the patch distance of every pixel is a
// (2P+1)^2 box sum of the per-pixel term
//   D(x) = sum_c [(I_c(x) - I_c(x+d))^2 - (V_c(x) + min(V_c(x), V_c(x+d)))] / (eps + k^2 (V_c(x) + V_c(x+d)))
// (each coordinate clamped to the image), so a CTA computes D once over its tile plus the
// patch border, sums it along rows and then columns in shared memory, and every pixel reads
// its distance: O(1) work per pixel and offset instead of O(patch).  The same sums as the
// direct double loop in a different order, with quotients within 2 ulp.
constexpr int kVTile = 16;

__global__ void __launch_bounds__(kVTile* kVTile) k_nlm_var(const float* __restrict__ rgb, const float* __restrict__ var,
                                                            int w, int h, int R, int P, float k2, float norm,
                                                            float* __restrict__ out) {
    extern __shared__ float sm[];
    const int H = R + P;
    const int S = kVTile + 2 * H;   // staged halo side
    const int E = kVTile + 2 * P;   // tile plus patch border
    float* tc = sm;                 // S*S*3 colours
    float* tv = tc + S * S * 3;     // S*S*3 variances
    float* dd = tv + S * S * 3;     // E*E per-pixel terms D
    float* hs = dd + E * E;         // E rows x kVTile columns of row sums
    const int tid = threadIdx.y * kVTile + threadIdx.x, nt = kVTile * kVTile;
    const int bx = blockIdx.x * kVTile, by = blockIdx.y * kVTile;
    const int x0 = bx - H, y0 = by - H;
    for (int i = tid; i < S * S; i += nt) {
        const int ty = i / S, tx = i % S;
        const size_t g = ((size_t)clampi(y0 + ty, 0, h - 1) * w + clampi(x0 + tx, 0, w - 1)) * 3;
        for (int c = 0; c < 3; ++c) {
            tc[i * 3 + c] = rgb[g + c];
            tv[i * 3 + c] = var[g + c];
        }
    }
    __syncthreads();
    const int x = bx + threadIdx.x, y = by + threadIdx.y;
    const float eps = 1e-10f;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, sw = 0.f;
    for (int dy = -R; dy <= R; ++dy) {
        for (int dx = -R; dx <= R; ++dx) {
            // D over the tile plus its patch border (image coordinates bx - P .. bx + kVTile + P)
            for (int i = tid; i < E * E; i += nt) {
                const int u = i % E, v = i / E;
                const int ax = clampi(bx - P + u, 0, w - 1), ay = clampi(by - P + v, 0, h - 1);
                const int qx = clampi(bx - P + u + dx, 0, w - 1), qy = clampi(by - P + v + dy, 0, h - 1);
                const int ia = ((ay - y0) * S + (ax - x0)) * 3, ib = ((qy - y0) * S + (qx - x0)) * 3;
                float d = 0.0f;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float a = tc[ia + c], b = tc[ib + c], va = tv[ia + c], vb = tv[ib + c];
                    const float num = (a - b) * (a - b) - (va + fminf(va, vb));
                    d += __fdividef(num, eps + k2 * (va + vb));  // 2-ulp division: the weights need no IEEE quotient
                }
                dd[i] = d;
            }
            __syncthreads();
            // row sums over the patch width
            for (int i = tid; i < E * kVTile; i += nt) {
                const int u = i % kVTile, v = i / kVTile;
                const float* r = dd + v * E + u;
                float t = 0.0f;
                for (int k = 0; k <= 2 * P; ++k) t += r[k];
                hs[i] = t;
            }
            __syncthreads();
            // column sum over the patch height: this pixel's patch distance
            float d2 = 0.0f;
            for (int k = 0; k <= 2 * P; ++k) d2 += hs[(threadIdx.y + k) * kVTile + threadIdx.x];
            const float wt = expf(-fmaxf(0.0f, d2 * norm));
            const int iq = ((clampi(y + dy, 0, h - 1) - y0) * S + (clampi(x + dx, 0, w - 1) - x0)) * 3;
            sw += wt;
            s0 += wt * tc[iq];
            s1 += wt * tc[iq + 1];
            s2 += wt * tc[iq + 2];
        }
    }
    if (x >= w || y >= h) return;
    const size_t o = ((size_t)y * w + x) * 3;
    out[o] = s0 / sw;
    out[o + 1] = s1 / sw;
    out[o + 2] = s2 / sw;
}

}  // namespace

salty_status tonemap_device(salty_ctx* ctx, int type, int w, int h, const float* d_rgb, float* d_out,
                            uint8_t* d_srgb, int ref_oetf, float* ave, float* mx) {
    auto& E = ctx->err;
    cudaStream_t st = ctx->stream;
    const long long npx = (long long)w * h;
    LumAcc* acc = reinterpret_cast<LumAcc*>(ctx->counters.p + 32);
    LumAcc init{0.0, f2o_host(-FLT_MAX), 0};
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(acc, &init, sizeof init, cudaMemcpyHostToDevice, st));
    int grid = ctx->num_sms * 4;
    long long need = (npx + kRedBlock - 1) / kRedBlock;
    if (grid > need) grid = (int)need;
    k_lum_reduce<<<grid, kRedBlock, 0, st>>>(d_rgb, npx, acc);
    LumAcc res;
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(&res, acc, sizeof res, cudaMemcpyDeviceToHost, st));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
    // ComputeLogarithmicAverage (src/s3d_tonemapper.cpp:84-94)
    float mean = (float)(res.sum / (double)npx);
    float ave_lw = expf(mean);
    int mo = res.maxo;
    float max_lw;
    {
        int i = mo >= 0 ? mo : mo ^ 0x7fffffff;
        std::memcpy(&max_lw, &i, 4);
    }
    if (ave) *ave = ave_lw;
    if (mx) *mx = max_lw;
    TmParams p;
    p.type = type;
    p.ref_oetf = ref_oetf;
    p.coeff = (type == SALTY_TM_ACES ? 0.27f : 0.18f) / ave_lw;
    float m2 = max_lw * p.coeff;
    p.m2 = m2 * m2;
    {
        // Uncharted2Tonemap(LinearWhite = 11.2), host evaluation in the same order
        const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, Ee = 0.01f, F = 0.30f, x = 11.2f;
        float num = x * (A * x + C * B) + D * Ee;
        float den = x * (A * x + B) + D * F;
        p.white = num / den - Ee / F;
    }
    if (d_out || d_srgb) {
        const long long n = npx * 3;
        int g2 = ctx->num_sms * 8;
        long long need2 = (n + 255) / 256;
        if (g2 > need2) g2 = (int)need2;
        k_tonemap<<<g2, 256, 0, st>>>(d_rgb, n, p, d_out, d_srgb);
    }
    SALTY_TRY_CUDA(E, cudaGetLastError());
    return SALTY_OK;
}

salty_status nlm_ref_device(salty_ctx* ctx, int w, int h, float coeff, const float* d_in, float* d_out) {
    // FilterNLM parameters (src/s3d_denoiser.cpp:22-25)
    float ph = fmaxf(0.0001f, coeff), sigma = fmaxf(0.0001f, coeff);
    float inv_h2 = 1.0f / (ph * ph);
    float two_s2 = 2.0f * (sigma * sigma);
    dim3 blk(kNlmTile, kNlmTile), grd((w + kNlmTile - 1) / kNlmTile, (h + kNlmTile - 1) / kNlmTile);
    k_nlm_ref<<<grd, blk, 0, ctx->stream>>>((const float4*)d_in, w, h, inv_h2, two_s2, (float4*)d_out);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

salty_status nlm_var_device(salty_ctx* ctx, int w, int h, int search_r, int patch_r, float k, const float* d_rgb,
                            const float* d_var, float* d_out) {
    const int H = search_r + patch_r, S = kVTile + 2 * H, Eb = kVTile + 2 * patch_r;
    size_t smem = ((size_t)S * S * 6 + (size_t)Eb * Eb + (size_t)Eb * kVTile) * sizeof(float);
    if (smem > 200 * 1024) return ctx->err.fail(SALTY_ERR_CAPACITY, "NLM window too large");
    SALTY_TRY_CUDA(ctx->err, cudaFuncSetAttribute(k_nlm_var, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    float norm = 1.0f / (3.0f * (float)((2 * patch_r + 1) * (2 * patch_r + 1)));
    dim3 blk(kVTile, kVTile), grd((w + kVTile - 1) / kVTile, (h + kVTile - 1) / kVTile);
    k_nlm_var<<<grd, blk, smem, ctx->stream>>>(d_rgb, d_var, w, h, search_r, patch_r, k * k, norm, d_out);
    SALTY_TRY_CUDA(ctx->err, cudaGetLastError());
    return SALTY_OK;
}

}  // namespace salty

// ---------------------------------------------------------------- no-allocation tonemap
// salty_tonemap_noalloc: the same tonemap for callers that must not allocate device memory
// when they tonemap (see include/salty_gpu.h).  Its scratch is the fixed array below,
// part of the library image, so it exists on every device that loads the library until
// the process exits.  Layout: kNoAllocPartials partial sums (one per block of
// kNoAllocPixelsPerBlock pixels), then the tonemap parameters.  Every call overwrites what
// it reads, so nothing has to be cleared between calls; calls that overlap on the GPU share
// the array and race.
namespace salty {
namespace {

constexpr int kNoAllocPartials = 4096;
constexpr int kNoAllocPixelsPerBlock = 4096;
constexpr long long kNoAllocMaxPixels = (long long)kNoAllocPartials * kNoAllocPixelsPerBlock;

struct NoAllocScratch {
    LumAcc part[kNoAllocPartials];
    TmParams params;
    float ave_max[2];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Per-block luminance partials in a fixed pixel-to-block mapping (deterministic).
// log(eps + Lw) of one pixel, with the reference's guards, and the running maximum of Lw.
__device__ __forceinline__ float lum_log(float r, float g, float b, float& mx) {
    const float eps = 0.00001f;
    float lw = rgb_to_y(r, g, b);
    if (lw != lw) lw = eps;
    if (lw < FLT_EPSILON) lw = eps;
    mx = fmaxf(mx, lw);
    return logf(__fadd_rn(eps, lw));
}

// vec: rgb is 16-byte aligned -- four pixels (three float4) per load step, their four logs
// summed in FP32 before the FP64 running sum (a quarter of the FP64 additions).
__global__ void __launch_bounds__(kRedBlock) k_lum_partials(const float* __restrict__ rgb, long long npx,
                                                            NoAllocScratch* sc, int vec) {
    const long long b0 = (long long)blockIdx.x * kNoAllocPixelsPerBlock;
    const long long b1 = min(npx, b0 + kNoAllocPixelsPerBlock);
    double s = 0.0;
    float mx = -FLT_MAX;
    long long i0 = b0;
    if (vec) {
        const float4* q = reinterpret_cast<const float4*>(rgb);
        const long long ge = b1 / 4;  // b0 is a multiple of 4
        for (long long gi = b0 / 4 + threadIdx.x; gi < ge; gi += blockDim.x) {
            const float4 a = __ldg(q + 3 * gi), b = __ldg(q + 3 * gi + 1), c = __ldg(q + 3 * gi + 2);
            const float l4 = lum_log(a.x, a.y, a.z, mx) + lum_log(a.w, b.x, b.y, mx) + lum_log(b.z, b.w, c.x, mx) +
                             lum_log(c.y, c.z, c.w, mx);
            s += (double)l4;
        }
        i0 = ge * 4;
    }
    for (long long i = i0 + threadIdx.x; i < b1; i += blockDim.x)
        s += (double)lum_log(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], mx);
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, off);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    __shared__ double ss[kRedBlock / 32];
    __shared__ float sm[kRedBlock / 32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { ss[w] = s; sm[w] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        float m = -FLT_MAX;
        for (int k = 0; k < kRedBlock / 32; ++k) { t += ss[k]; m = fmaxf(m, sm[k]); }
        sc->part[blockIdx.x].sum = t;
        sc->part[blockIdx.x].maxo = f2o(m);
    }
}

// Reduces the partials in index order and derives the curve parameters on the device, so
// the three launches need no host round trip.  ComputeLogarithmicAverage and the
// per-operator constants: src/s3d_tonemapper.cpp:84-94, :246-250, :291-297, :331-335.
__global__ void __launch_bounds__(kRedBlock) k_lum_finalize(NoAllocScratch* sc, int nparts, long long npx, int type,
                                                            int ref_oetf) {
    double s = 0.0;
    float mx = -FLT_MAX;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        s += sc->part[i].sum;
        mx = fmaxf(mx, o2f(sc->part[i].maxo));
    }
    __shared__ double ss[kRedBlock];
    __shared__ float sm[kRedBlock];
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int h = kRedBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            ss[threadIdx.x] += ss[threadIdx.x + h];
            sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const float mean = (float)(ss[0] / (double)npx);
    const float ave = expf(mean);
    const float max_lw = sm[0];
    TmParams p;
    p.type = type;
    p.ref_oetf = ref_oetf;
    p.coeff = __fdiv_rn(type == SALTY_TM_ACES ? 0.27f : 0.18f, ave);
    const float m2 = __fmul_rn(max_lw, p.coeff);
    p.m2 = __fmul_rn(m2, m2);
    p.white = u2_curve(11.2f);
    sc->params = p;
    sc->ave_max[0] = ave;
    sc->ave_max[1] = max_lw;
}

__device__ __forceinline__ float tm_curve(float v, const TmParams& p) {
    const float x = __fmul_rn(v, p.coeff);
    if (p.type == SALTY_TM_ACES) return aces_curve(x);
    if (p.type == SALTY_TM_UNCHARTED2) return __fdiv_rn(u2_curve(__fmul_rn(2.0f, x)), p.white);
    return __fdiv_rn(__fmul_rn(x, __fadd_rn(1.0f, __fdiv_rn(x, p.m2))), __fadd_rn(1.0f, x));
}

__global__ void k_tonemap_params(const float* __restrict__ in, long long n, const NoAllocScratch* __restrict__ sc,
                                 float* __restrict__ out, unsigned char* __restrict__ srgb) {
    const TmParams p = sc->params;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float y = tm_curve(in[i], p);
        if (out) out[i] = y;
        if (srgb) srgb[i] = to_srgb8(y, p.ref_oetf);
    }
}

// The same map, four pixels (twelve values) per step: three 16-byte loads and stores and
// three 4-byte sRGB8 words.  in/out 16-byte aligned, srgb 4-byte aligned.
__global__ void k_tonemap_params4(const float4* __restrict__ in, long long groups, const NoAllocScratch* __restrict__ sc,
                                  float4* __restrict__ out, uint32_t* __restrict__ srgb) {
    const TmParams p = sc->params;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < groups;
         g += (long long)gridDim.x * blockDim.x) {
        float4 q[3] = {__ldg(in + 3 * g), __ldg(in + 3 * g + 1), __ldg(in + 3 * g + 2)};
        float* v = reinterpret_cast<float*>(q);
#pragma unroll
        for (int k = 0; k < 12; ++k) v[k] = tm_curve(v[k], p);
        if (out) {
            out[3 * g] = q[0];
            out[3 * g + 1] = q[1];
            out[3 * g + 2] = q[2];
        }
        if (srgb) {
#pragma unroll
            for (int w = 0; w < 3; ++w)
                srgb[3 * g + w] = (uint32_t)to_srgb8(v[4 * w], p.ref_oetf) |
                                  ((uint32_t)to_srgb8(v[4 * w + 1], p.ref_oetf) << 8) |
                                  ((uint32_t)to_srgb8(v[4 * w + 2], p.ref_oetf) << 16) |
                                  ((uint32_t)to_srgb8(v[4 * w + 3], p.ref_oetf) << 24);
        }
    }
}

// Device address of g_noalloc_scratch per device, looked up once per device with that
// device current (the array's name is only a host-side stand-in in host code).
constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};

cudaError_t noalloc_scratch(int device, NoAllocScratch** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    void* p = __atomic_load_n(&g_noalloc_addr[device], __ATOMIC_ACQUIRE);
    if (!p) {
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        __atomic_store_n(&g_noalloc_addr[device], p, __ATOMIC_RELEASE);
    }
    *out = static_cast<NoAllocScratch*>(p);
    return cudaSuccess;
}

// true for device memory of `device` itself, or managed memory; an array on another GPU
// would be read as peer memory (a fault without peer access), so it is refused
bool on_device(const void* p, int device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace
}  // namespace salty

extern "C" salty_status salty_tonemap_noalloc(salty_ctx* ctx, void* stream, int32_t type, int32_t width,
                                              int32_t height, const float* d_rgb, float* d_out_rgb,
                                              uint8_t* d_out_srgb8, int32_t ref_oetf) {
    using namespace salty;
    if (!ctx) return SALTY_ERR_INVALID_ARG;
    auto& E = ctx->err;
    if (width <= 0 || height <= 0) return E.fail(SALTY_ERR_INVALID_ARG, "tonemap_noalloc: bad image size");
    const long long npx = (long long)width * height;
    if (npx > kNoAllocMaxPixels)
        return E.fail(SALTY_ERR_CAPACITY, "tonemap_noalloc: %lld pixels exceed the fixed scratch limit of %lld",
                      npx, kNoAllocMaxPixels);
    if (type < SALTY_TM_REINHARD || type > SALTY_TM_ACES) return E.fail(SALTY_ERR_INVALID_ARG, "bad tonemap type");
    if (!d_out_rgb && !d_out_srgb8) return E.fail(SALTY_ERR_INVALID_ARG, "tonemap_noalloc: no output");
    SALTY_TRY_CUDA(E, cudaSetDevice(ctx->device));
    const int dv = ctx->device;
    if (!on_device(d_rgb, dv) || (d_out_rgb && !on_device(d_out_rgb, dv)) ||
        (d_out_srgb8 && !on_device(d_out_srgb8, dv)))
        return E.fail(SALTY_ERR_INVALID_ARG, "tonemap_noalloc: arrays must be device memory of the context's GPU");
    NoAllocScratch* sc = nullptr;
    SALTY_TRY_CUDA(E, noalloc_scratch(ctx->device, &sc));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const int nparts = (int)((npx + kNoAllocPixelsPerBlock - 1) / kNoAllocPixelsPerBlock);
    auto aligned = [](const void* p, uintptr_t a) { return p == nullptr || reinterpret_cast<uintptr_t>(p) % a == 0; };
    const bool vec = aligned(d_rgb, 16) && aligned(d_out_rgb, 16) && aligned(d_out_srgb8, 4);
    k_lum_partials<<<nparts, kRedBlock, 0, st>>>(d_rgb, npx, sc, aligned(d_rgb, 16) ? 1 : 0);
    k_lum_finalize<<<1, kRedBlock, 0, st>>>(sc, nparts, npx, type, ref_oetf);
    const long long n = npx * 3;
    const long long groups = vec ? npx / 4 : 0;  // whole groups of four pixels
    const long long done = groups * 12;          // channel values the vector kernel maps
    const long long cap = (long long)ctx->num_sms * 8;
    if (groups > 0) {
        const long long g4 = std::min((groups + 255) / 256, cap);
        k_tonemap_params4<<<(unsigned)g4, 256, 0, st>>>(reinterpret_cast<const float4*>(d_rgb), groups, sc,
                                                         reinterpret_cast<float4*>(d_out_rgb),
                                                         reinterpret_cast<uint32_t*>(d_out_srgb8));
    }
    if (n > done) {
        const long long g = std::min((n - done + 255) / 256, cap);
        k_tonemap_params<<<(unsigned)g, 256, 0, st>>>(d_rgb + done, n - done, sc, d_out_rgb ? d_out_rgb + done : nullptr,
                                                      d_out_srgb8 ? d_out_srgb8 + done : nullptr);
    }
    SALTY_TRY_CUDA(E, cudaGetLastError());
    return SALTY_OK;
}
