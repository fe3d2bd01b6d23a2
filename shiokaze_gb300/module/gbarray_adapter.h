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
#include <atomic>
#include <cstddef>
#include <cstring>
#include <thread>
#include <vector>

#include "gbp.h"

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

// ---- bricks: the sparse form that travels to the GPU (include/gbp.h) ----
//
// to_bricks() cuts a 3D tiled array into bricks of 8^3 cells: a brick with
// an active cell, or with some but not all of its cells filled, is listed
// with its 512 values (operator()'s: stored values of active cells, the
// fill value on filled cells, the background elsewhere; cells beyond the
// extent hold the background); a brick whose cells are all filled and none
// active is GBP_BRICK_FILL; the rest GBP_BRICK_BACKGROUND. Two passes over
// the active and the filled cells (counting, then writing); the cost
// follows the band and the filled region, and nothing is written for
// background bricks.
struct Bricks {
    std::vector<int> slot;
    std::vector<float> values;
    float background = 0.0f, fill = 0.0f;
    int nbx = 0, nby = 0, nbz = 0;
    long long count() const { return (long long)(values.size() / GBP_BRICK_CELLS); }
    gbp_bricks view() const { return gbp_bricks{background, fill, slot.data(), count(), values.data()}; }
    size_t brick(int i, int j, int k) const { return (size_t)(i >> 3) + (size_t)nbx * ((j >> 3) + (size_t)nby * (k >> 3)); }
    static int offset(int i, int j, int k) { return (i & 7) + 8 * ((j & 7) + 8 * (k & 7)); }
};

template <class T> void to_bricks(const shiokaze_v1::array3<T> &a, Bricks &out) {
    const shiokaze_v1::shape3 s = a.shape();
    out.nbx = ((int)s.w + 7) / 8;
    out.nby = ((int)s.h + 7) / 8;
    out.nbz = ((int)s.d + 7) / 8;
    const size_t nb = (size_t)out.nbx * out.nby * out.nbz;
    out.background = (float)a.get_background_value();
    std::vector<std::atomic<int>> nact(nb), nfill(nb);
    std::atomic<unsigned> fill_bits{0};
    using It = typename shiokaze_v1::array3<T>::const_iterator;
    a.const_parallel_actives([&](int i, int j, int k, const It &) {
        nact[out.brick(i, j, k)].fetch_add(1, std::memory_order_relaxed);
    });
    a.const_parallel_inside([&](int i, int j, int k, const It &it) {
        nfill[out.brick(i, j, k)].fetch_add(1, std::memory_order_relaxed);
        if (!it.active()) {  // a filled cell reads the fill value
            const float f = (float)it();
            unsigned b;
            std::memcpy(&b, &f, sizeof b);
            fill_bits.store(b, std::memory_order_relaxed);
        }
    });
    const unsigned fb = fill_bits.load();
    std::memcpy(&out.fill, &fb, sizeof fb);
    out.slot.assign(nb, GBP_BRICK_BACKGROUND);
    long long count = 0;
    for (int bz = 0; bz < out.nbz; ++bz)
        for (int by = 0; by < out.nby; ++by)
            for (int bx = 0; bx < out.nbx; ++bx) {
                const size_t b = (size_t)bx + (size_t)out.nbx * (by + (size_t)out.nby * bz);
                const int cells = std::min(8, (int)s.w - 8 * bx) * std::min(8, (int)s.h - 8 * by) *
                                  std::min(8, (int)s.d - 8 * bz);
                const int na = nact[b].load(), nf = nfill[b].load();
                if (!na && !nf) continue;
                out.slot[b] = (!na && nf == cells) ? GBP_BRICK_FILL : (int)count++;
            }
    out.values.assign((size_t)count * GBP_BRICK_CELLS, out.background);
    a.const_parallel_inside([&](int i, int j, int k, const It &it) {
        const int sl = out.slot[out.brick(i, j, k)];
        if (sl >= 0 && !it.active()) out.values[(size_t)sl * GBP_BRICK_CELLS + Bricks::offset(i, j, k)] = (float)it();
    });
    a.const_parallel_actives([&](int i, int j, int k, const It &it) {
        const int sl = out.slot[out.brick(i, j, k)];
        out.values[(size_t)sl * GBP_BRICK_CELLS + Bricks::offset(i, j, k)] = (float)it();
    });
}

// Output bricks: the slots, and the values and flags gbp_project_bricks
// fills.
struct BricksOut {
    std::vector<int> slot;
    std::vector<float> values;
    std::vector<unsigned char> active;
    int nbx = 0, nby = 0;
    gbp_bricks_out view() {
        return gbp_bricks_out{slot.data(), (long long)(values.size() / GBP_BRICK_CELLS), values.data(), active.data()};
    }
    size_t index(int i, int j, int k) const {
        const size_t b = (size_t)(i >> 3) + (size_t)nbx * ((j >> 3) + (size_t)nby * (k >> 3));
        return (size_t)slot[b] * GBP_BRICK_CELLS + Bricks::offset(i, j, k);
    }
    void resize(long long count) {
        values.assign((size_t)count * GBP_BRICK_CELLS, 0.0f);
        active.assign((size_t)count * GBP_BRICK_CELLS, 0);
    }
};

}  // namespace gbarray
