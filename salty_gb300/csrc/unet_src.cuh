// unet_src.cuh -- where a convolution's input channels come from.
//
// A decoder convolution of the U-Net reads the concatenation [up2(coarse) | skip]: channels
// [0, a_ch) are the coarse level's, nearest-up-sampled (read at (y >> 1, x >> 1) of an image
// half as tall and wide), channels [a_ch, cin) the skip connection's at (y, x).  The
// convolution kernels read both where they stage their input tiles, so the concatenated
// tensor is never written.  A plain input is source a alone (a_shift 0, a_ch = cin).
#pragma once

#include <cuda_bf16.h>

#include <cstddef>

#include "internal.h"

namespace salty {

struct ConvSrc {
    const __nv_bfloat16* a;  // [N][H >> a_shift][W >> a_shift][a_cs]
    int a_cs, a_ch, a_shift;
    const __nv_bfloat16* b;  // [N][H][W][b_cs], channels a_ch.. of the input
    int b_cs;
};

inline ConvSrc conv_src(const __nv_bfloat16* in, int cs, int ch) { return ConvSrc{in, cs, ch, 0, nullptr, 0}; }
inline ConvSrc conv_src_cat(const __nv_bfloat16* coarse, int cc, const __nv_bfloat16* skip, int cs) {
    return ConvSrc{coarse, cc, cc, 1, skip, cs};
}

// Address of input channels [ch, ch + 8) of pixel (y, x) of image n (an H x W level); the
// eight never straddle the two sources (a_ch % 8 == 0).
__device__ __forceinline__ const __nv_bfloat16* src_at(const ConvSrc& s, int n, int y, int x, int H, int W, int ch) {
    if (ch < s.a_ch) {
        const int Ha = H >> s.a_shift, Wa = W >> s.a_shift;
        return s.a + (((size_t)n * Ha + (y >> s.a_shift)) * Wa + (x >> s.a_shift)) * s.a_cs + ch;
    }
    return s.b + (((size_t)n * H + y) * W + x) * s.b_cs + (ch - s.a_ch);
}

// conv_tc.cu: 3x3 convolution, BF16 NHWC, on tcgen05 (cin % 16 == 0, source a's channel
// count % 16 == 0, cout % 8 == 0, cout <= 256); wt [9][wrows][cin]
int conv_tc_rows(int cout);
salty_status conv3x3_tc(salty_ctx* ctx, const ConvSrc& in, int cin, const __nv_bfloat16* wt, int wrows,
                        const float* bias, __nv_bfloat16* out, int out_cs, int out_co, int cout, int N, int H, int W,
                        int relu, int* d_status);
// The same for an input held in one tensor [N][H][W][in_cs] (16-byte aligned), by TMA in a
// persistent warp-specialised kernel; wrows <= 256.
salty_status conv3x3_tma(salty_ctx* ctx, const __nv_bfloat16* in, int in_cs, int cin, const __nv_bfloat16* wt,
                         int wrows, const float* bias, __nv_bfloat16* out, int out_cs, int out_co, int cout, int N,
                         int H, int W, int relu, int* d_status);

// Weight gradient of a 3x3 convolution on tcgen05, deterministic (partial sums per CTA,
// added in a fixed order): dw[9][cout][cin] += sum over pixels of dY x X(tap).  dy
// [N][H][W][cpad] (cpad = cout rounded up to 16, <= 128, zero beyond cout, 16-byte
// aligned); x the layer's input (cin % 16 == 0; a decoder's concatenation is first written
// out into cat_ws, N*H*W*cin elements); ws a workspace of at least
// conv_wgrad_tc_workspace(...) floats.
size_t conv_wgrad_tc_workspace(int num_sms, int cin, int cpad, int N, int H, int W);
salty_status conv_wgrad_tc(salty_ctx* ctx, const __nv_bfloat16* dy, int cpad, int cout, const ConvSrc& x, int cin,
                           float* dw, int N, int H, int W, float* ws, size_t ws_floats, __nv_bfloat16* cat_ws,
                           size_t cat_elems, int* d_status);

}  // namespace salty
