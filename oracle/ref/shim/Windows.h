// Windows.h stand-in for compiling the Salty reference with g++ (oracle only).
// Provides the high-resolution counter used by include/s3d_timer.inl:23-80.
#pragma once
#include <chrono>
#include <cstdint>
typedef union _LARGE_INTEGER { long long QuadPart; } LARGE_INTEGER;
inline int QueryPerformanceFrequency(LARGE_INTEGER* f) { f->QuadPart = 1000000000LL; return 1; }
inline int QueryPerformanceCounter(LARGE_INTEGER* c) {
    c->QuadPart = (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::steady_clock::now().time_since_epoch()).count();
    return 1;
}
inline void OutputDebugStringA(const char*) {}
