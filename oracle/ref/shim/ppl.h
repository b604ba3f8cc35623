// ppl.h stand-in: concurrency::parallel_for over std::thread, used by
// src/s3d_pt.cpp:106,145 (buffer clear, sRGB conversion).  Oracle only.
#pragma once
#include <algorithm>
#include <thread>
#include <vector>
namespace concurrency {
template <typename T, typename F>
void parallel_for(T first, T last, const F& fn) {
    if (last <= first) return;
    unsigned hw = std::thread::hardware_concurrency();
    T n = last - first;
    T workers = (T)std::max(1u, std::min<unsigned>(hw ? hw : 1, 64));
    if ((T)workers > n) workers = n;
    T chunk = (n + workers - 1) / workers;
    std::vector<std::thread> pool;
    for (T w = 0; w < workers; ++w) {
        T b = first + w * chunk, e = std::min(last, b + chunk);
        if (b >= e) break;
        pool.emplace_back([=, &fn] { for (T i = b; i < e; ++i) fn(i); });
    }
    for (auto& t : pool) t.join();
}
}  // namespace concurrency
