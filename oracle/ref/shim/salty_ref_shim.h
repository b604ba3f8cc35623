// salty_ref_shim.h -- force-included (g++ -include) when the unmodified Salty
// reference sources are compiled as the test oracle.  TEST INFRASTRUCTURE ONLY:
// nothing in the shipped library includes this file.
//
// Salty is written for MSVC (s3d.vcxproj).  This header supplies the few MSVC
// spellings the sources rely on so that g++ (x86_64 or aarch64, -std=c++17)
// compiles them where they lie, without editing a copy:
//   * __int8/16/32/64, __forceinline, errno_t
//   * the secure CRT calls used by the loaders (fopen_s, sscanf_s, printf_s...)
//   * _aligned_malloc/_aligned_free (BVH nodes, include/s3d_bvh8.h operator new)
//   * MSVC integer-literal suffixes (0xffffffffui32 in include/s3d_math.h:2725,
//     :2804) as C++11 user-defined literals -- g++ accepts suffixes without a
//     leading underscore with a -Wliteral-suffix warning in strict -std mode.
//   * S3D_ALIGN in GNU attribute form (include/s3d_typedef.h:54-60 guards it
//     with #ifndef, so predefining it here wins)
//   * ILOG/ELOG/DLOG (include/s3d_logger.h:59-70 guard them with #ifndef), so
//     the Win32 console logger (src/s3d_logger.cpp) is not needed.
#pragma once

#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

// Macros rather than typedefs: the sources also write "unsigned __int64".
#define __int8  char
#define __int16 short
#define __int32 int
#define __int64 long long
typedef int errno_t;

// MSVC's <cmath> declares float/double overloads of abs, sqrt, exp, ... in the
// global namespace.  Under g++ an unqualified abs(float) inside namespace s3d
// finds only the C library's int abs(int) -- src/s3d_triangle.cpp:78
// `abs(div) <= FLT_EPSILON` would then truncate div to an integer and reject
// every hit with |div| < 1 -- and sqrt(float) would run in double.  Bringing
// the std overloads into the global namespace restores MSVC's overload set.
using std::abs;
using std::sqrt;
using std::exp;
using std::log;
using std::pow;
using std::sin;
using std::cos;
using std::tan;
using std::acos;
using std::asin;
using std::atan;
using std::atan2;
using std::floor;
using std::ceil;
using std::fmod;

#define __forceinline inline __attribute__((always_inline))
#define S3D_ALIGN(a) __attribute__((aligned(a)))

#define DLOG(x, ...) ((void)0)
#define ILOG(x, ...) ((void)0)
#define ELOG(x, ...) std::fprintf(stderr, "[salty-ref] " x "\n", ##__VA_ARGS__)

inline void* _aligned_malloc(size_t size, size_t alignment) {
    void* p = nullptr;
    if (alignment < sizeof(void*)) alignment = sizeof(void*);
    if (posix_memalign(&p, alignment, size ? size : alignment) != 0) return nullptr;
    return p;
}
inline void _aligned_free(void* p) { std::free(p); }

inline errno_t fopen_s(FILE** pf, const char* name, const char* mode) {
    *pf = std::fopen(name, mode);
    return *pf ? 0 : (errno ? errno : 1);
}
#define printf_s printf
#define fprintf_s fprintf
#define sscanf_s sscanf
#define vsprintf_s vsnprintf

#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wliteral-suffix"
constexpr unsigned char      operator"" ui8 (unsigned long long v) { return (unsigned char)v; }
constexpr unsigned short     operator"" ui16(unsigned long long v) { return (unsigned short)v; }
constexpr unsigned int       operator"" ui32(unsigned long long v) { return (unsigned int)v; }
constexpr unsigned long long operator"" ui64(unsigned long long v) { return v; }
constexpr signed char        operator"" i8  (unsigned long long v) { return (signed char)v; }
constexpr short              operator"" i16 (unsigned long long v) { return (short)v; }
constexpr int                operator"" i32 (unsigned long long v) { return (int)v; }
constexpr long long          operator"" i64 (unsigned long long v) { return (long long)v; }
#pragma GCC diagnostic pop
