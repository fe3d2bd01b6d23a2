// gbarray_adapter.h -- dense copies of the reference's sparse tiled arrays
// (array2 / array3 on the tiledarray core, src/array/tiledarray3.cpp) for
// the C ABI, which takes dense arrays, x fastest.
//
// A cell of a tiled array reads (include/shiokaze/array/array3.h:796-800):
// its stored value if active, else the fill value if its tile marks it
// filled (tiledarray3.cpp:191-207), else the background value. densify()
// produces exactly those values without one operator() call per cell:
//   1. every cell <- background (plain stores, split over threads),
//   2. const_parallel_inside: filled cells <- fill value (the core visits
//      the filled cells of allocated tiles and every cell of a tile that is
//      filled as a whole, tiledarray3.cpp:291-313),
//   3. const_parallel_actives: active cells <- stored value.
// Each pass writes disjoint cells; later passes win, so the result is
// operator()'s for every cell. The cost follows the active and filled
// cells, not the grid: a narrow-band level set touches its band and its
// filled tiles, a constant array (the smoke scene's fluid) only step 1.
// Below kPassesMinCells cells the thread start-up of the passes costs more
// than a lookup per cell, and densify() reads through operator() instead
// (same values; on 8 host threads the passes take 0.8-4.9 ms per 128^3
// array against 11-35 ms of lookups, and 0.5 ms against 0.2 ms at 32^3).
#pragma once

#include <shiokaze/array/array2.h>
#include <shiokaze/array/array3.h>

#include <algorithm>
#include <cstddef>
#include <thread>
#include <vector>

namespace gbarray {

// Fills out[0, n) with v on up to `threads` threads.
inline void fill(float *out, size_t n, float v, int threads) {
    const size_t chunk = 1 << 20;
    const int t = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(threads, 1), (n + chunk - 1) / chunk));
    if (t == 1) {
        std::fill(out, out + n, v);
        return;
    }
    std::vector<std::thread> pool;
    for (int q = 0; q < t; ++q)
        pool.emplace_back([=] {
            const size_t lo = n * q / t, hi = n * (q + 1) / t;
            std::fill(out + lo, out + hi, v);
        });
    for (auto &th : pool) th.join();
}

constexpr size_t kPassesMinCells = size_t(1) << 16;

// out: s.w * s.h * s.d floats, x fastest; equals a(i, j, k) everywhere.
template <class T> void densify_passes(const shiokaze_v1::array3<T> &a, float *out) {
    const shiokaze_v1::shape3 s = a.shape();
    const size_t sx = s.w, sxy = (size_t)s.w * s.h;
    fill(out, sxy * s.d, (float)a.get_background_value(), a.get_thread_num());
    using It = typename shiokaze_v1::array3<T>::const_iterator;
    a.const_parallel_inside([&](int i, int j, int k, const It &it) { out[i + sx * j + sxy * k] = (float)it(); });
    a.const_parallel_actives([&](int i, int j, int k, const It &it) { out[i + sx * j + sxy * k] = (float)it(); });
}

// out: s.w * s.h floats, x fastest; equals a(i, j) everywhere.
template <class T> void densify_passes(const shiokaze_v1::array2<T> &a, float *out) {
    const shiokaze_v1::shape2 s = a.shape();
    const size_t sx = s.w;
    fill(out, sx * s.h, (float)a.get_background_value(), a.get_thread_num());
    using It = typename shiokaze_v1::array2<T>::const_iterator;
    a.const_parallel_inside([&](int i, int j, const It &it) { out[i + sx * j] = (float)it(); });
    a.const_parallel_actives([&](int i, int j, const It &it) { out[i + sx * j] = (float)it(); });
}

template <class T> void densify(const shiokaze_v1::array3<T> &a, float *out) {
    const shiokaze_v1::shape3 s = a.shape();
    if ((size_t)s.w * s.h * s.d >= kPassesMinCells) return densify_passes(a, out);
    size_t n = 0;
    for (int k = 0; k < (int)s.d; ++k)
        for (int j = 0; j < (int)s.h; ++j)
            for (int i = 0; i < (int)s.w; ++i) out[n++] = (float)a(i, j, k);
}

template <class T> void densify(const shiokaze_v1::array2<T> &a, float *out) {
    const shiokaze_v1::shape2 s = a.shape();
    if ((size_t)s.w * s.h >= kPassesMinCells) return densify_passes(a, out);
    size_t n = 0;
    for (int j = 0; j < (int)s.h; ++j)
        for (int i = 0; i < (int)s.w; ++i) out[n++] = (float)a(i, j);
}

}  // namespace gbarray
