// host_par.h -- host threads for the loaders and the matrix upload.
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

namespace sbx {

// All hardware threads, at most 64.
inline int host_threads()
{
    const unsigned h = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(h, 64u));
}

// Run f(t, T) on T threads (t = 0..T-1); T = 1 runs inline.
template <class F> void parallel(int T, F f)
{
    if (T <= 1) {
        f(0, 1);
        return;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)T);
    for (int t = 0; t < T; t++) th.emplace_back(f, t, T);
    for (auto &x : th) x.join();
}

}  // namespace sbx
