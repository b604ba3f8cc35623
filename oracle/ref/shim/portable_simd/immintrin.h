// Portable scalar stand-in for the x86 SSE/AVX intrinsics the Salty reference
// uses (include/s3d_math.h, include/s3d_typedef.h:276-289), so the oracle
// builds on aarch64 hosts.  ORACLE ONLY.  Each function follows Intel's
// published definition of the intrinsic lane by lane, including the x86 rules
// that matter for bit parity: MINPS/MAXPS return the SECOND operand when the
// comparison is false (NaN included), compare masks are all-ones lanes, and
// DPPS adds the four products as (p3 + p2) + (p1 + p0).  Built with
// -ffp-contract=off so no product is fused into an add.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

struct alignas(8)  __m64   { uint64_t u; };
struct alignas(16) __m128  { float f[4]; };
struct alignas(16) __m128d { double d[2]; };
struct alignas(16) __m128i { uint32_t u[4]; };
struct alignas(32) __m256  { float f[8]; };
struct alignas(32) __m256d { double d[4]; };
struct alignas(32) __m256i { uint32_t u[8]; };

#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))
#define _CMP_EQ_OQ 0x00
#define _CMP_LT_OS 0x01
#define _CMP_LE_OS 0x02
#define _CMP_NEQ_UQ 0x04
#define _CMP_GE_OS 0x0d
#define _CMP_GT_OS 0x0e

namespace salty_simd_detail {
inline float mask_lane(bool b) { uint32_t u = b ? 0xffffffffu : 0u; float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
}

// ---- 128-bit ----
inline __m128 _mm_set1_ps(float a) { __m128 r; for (int i = 0; i < 4; ++i) r.f[i] = a; return r; }
inline __m128 _mm_set_ps(float e3, float e2, float e1, float e0) { __m128 r; r.f[0] = e0; r.f[1] = e1; r.f[2] = e2; r.f[3] = e3; return r; }
inline __m128 _mm_setzero_ps() { return _mm_set1_ps(0.0f); }
#define SALTY_SIMD_BIN4(name, expr) \
    inline __m128 name(__m128 a, __m128 b) { __m128 r; for (int i = 0; i < 4; ++i) { float x = a.f[i], y = b.f[i]; r.f[i] = (expr); } return r; }
SALTY_SIMD_BIN4(_mm_add_ps, x + y)
SALTY_SIMD_BIN4(_mm_sub_ps, x - y)
SALTY_SIMD_BIN4(_mm_mul_ps, x * y)
SALTY_SIMD_BIN4(_mm_div_ps, x / y)
SALTY_SIMD_BIN4(_mm_min_ps, (x < y) ? x : y)
SALTY_SIMD_BIN4(_mm_max_ps, (x > y) ? x : y)
SALTY_SIMD_BIN4(_mm_cmpeq_ps, salty_simd_detail::mask_lane(x == y))
SALTY_SIMD_BIN4(_mm_cmpneq_ps, salty_simd_detail::mask_lane(!(x == y)))
SALTY_SIMD_BIN4(_mm_cmpge_ps, salty_simd_detail::mask_lane(x >= y))
#undef SALTY_SIMD_BIN4
inline __m128 _mm_sqrt_ps(__m128 a) { __m128 r; for (int i = 0; i < 4; ++i) r.f[i] = std::sqrt(a.f[i]); return r; }
inline __m128 _mm_shuffle_ps(__m128 a, __m128 b, int imm) {
    __m128 r;
    r.f[0] = a.f[imm & 3]; r.f[1] = a.f[(imm >> 2) & 3];
    r.f[2] = b.f[(imm >> 4) & 3]; r.f[3] = b.f[(imm >> 6) & 3];
    return r;
}
inline void _mm_store_ps(float* p, __m128 a) { for (int i = 0; i < 4; ++i) p[i] = a.f[i]; }
inline float _mm_cvtss_f32(__m128 a) { return a.f[0]; }
inline int _mm_movemask_ps(__m128 a) {
    int m = 0; for (int i = 0; i < 4; ++i) m |= (int)(salty_simd_detail::bits(a.f[i]) >> 31) << i; return m;
}
inline __m128 _mm_dp_ps(__m128 a, __m128 b, int imm) {
    float p[4];
    for (int i = 0; i < 4; ++i) p[i] = ((imm >> (4 + i)) & 1) ? a.f[i] * b.f[i] : 0.0f;
    float s = (p[3] + p[2]) + (p[1] + p[0]);
    __m128 r; for (int i = 0; i < 4; ++i) r.f[i] = ((imm >> i) & 1) ? s : 0.0f; return r;
}

// ---- 256-bit ----
inline __m256 _mm256_set1_ps(float a) { __m256 r; for (int i = 0; i < 8; ++i) r.f[i] = a; return r; }
inline __m256 _mm256_set_ps(float e7, float e6, float e5, float e4, float e3, float e2, float e1, float e0) {
    __m256 r; r.f[0] = e0; r.f[1] = e1; r.f[2] = e2; r.f[3] = e3; r.f[4] = e4; r.f[5] = e5; r.f[6] = e6; r.f[7] = e7; return r;
}
#define SALTY_SIMD_BIN8(name, expr) \
    inline __m256 name(__m256 a, __m256 b) { __m256 r; for (int i = 0; i < 8; ++i) { float x = a.f[i], y = b.f[i]; r.f[i] = (expr); } return r; }
SALTY_SIMD_BIN8(_mm256_sub_ps, x - y)
SALTY_SIMD_BIN8(_mm256_div_ps, x / y)
SALTY_SIMD_BIN8(_mm256_min_ps, (x < y) ? x : y)
SALTY_SIMD_BIN8(_mm256_max_ps, (x > y) ? x : y)
#undef SALTY_SIMD_BIN8
inline __m256 _mm256_cmp_ps(__m256 a, __m256 b, int pred) {
    __m256 r;
    for (int i = 0; i < 8; ++i) {
        float x = a.f[i], y = b.f[i]; bool v = false;
        switch (pred) {
            case _CMP_EQ_OQ: v = (x == y); break;
            case _CMP_LT_OS: v = (x < y); break;
            case _CMP_LE_OS: v = (x <= y); break;
            case _CMP_NEQ_UQ: v = !(x == y); break;
            case _CMP_GE_OS: v = (x >= y); break;
            case _CMP_GT_OS: v = (x > y); break;
            default: v = false; break;
        }
        r.f[i] = salty_simd_detail::mask_lane(v);
    }
    return r;
}
inline void _mm256_store_ps(float* p, __m256 a) { for (int i = 0; i < 8; ++i) p[i] = a.f[i]; }
inline int _mm256_movemask_ps(__m256 a) {
    int m = 0; for (int i = 0; i < 8; ++i) m |= (int)(salty_simd_detail::bits(a.f[i]) >> 31) << i; return m;
}
