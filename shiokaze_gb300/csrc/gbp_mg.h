// gbp_mg.h -- multigrid hierarchy and MGPCG launch functions (mg_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "gbp_kernels.h"

namespace gbp {

constexpr int MG_MAX_LEVELS = 16;
constexpr int MG_COARSEST_MAX = 512;  // cells of the coarsest level (held in shared memory)

// One level: operator (diag, inverse diagonal, +face couplings) and the
// right-hand side b / solution x of the V-cycle on that level.
template <class T> struct MgLevel {
    Grid g;
    const T *diag, *inv, *cx, *cy, *cz;  // cz == cy in 2D (never read)
    T *b, *x;
    // tile classes (mg_setup): one per pair tile of g (64 x 8 x tz cells,
    // the smoothing and CG items) and one per cell tile of the next coarser
    // grid (its 64 x 16 x 2tz fine cells, the restriction items); null on
    // the coarsest level
    T *tcp, *tcr;
};

// A tile class is the common value u >= 0 of every coupling that the
// stencils of the tile's cells read (each in-grid face of each cell), so the
// kernels use u instead of loading cx, cy, cz; TILE_MIXED if those
// couplings differ; TILE_EMPTY if they are all 0 and no cell of the tile
// has a nonzero diagonal (no unknown: every vector is 0 there). Couplings
// are never negative, so the two markers cannot be taken for a value.
constexpr double TILE_MIXED = -1.0;
constexpr double TILE_EMPTY = -2.0;

// Levels from `tail` down run in one single-block kernel per scene, in
// place in global memory (tail == nlevels: no such levels): the coarsest
// levels whose 7 arrays take at most MG_TAIL_BYTES_MAX, small enough that
// one block's passes beat grid-wide barriers. tail_bytes is their
// footprint (nonzero exactly when there is a tail).
constexpr int MG_TAIL_THREADS = 1024;
constexpr size_t MG_TAIL_BYTES_MAX = 200 * 1024;

template <class T> struct MgHierarchy {
    int nlevels = 0;
    int tail = 0;
    size_t tail_bytes = 0;
    bool fine_aliases_fp64 = false;  // level 0 operator is the FP64 assembly itself
    // FP32 hierarchy: the low floats of the FP64 operator against level 0's
    // diag, cx, cy, cz (the mixed refinement's float-pair products); null
    // for the FP64 hierarchy
    T *lo[4] = {nullptr, nullptr, nullptr, nullptr};
    // scratch of the tile classification (sub-box partials), or null
    void *class_parts = nullptr;
    size_t class_parts_bytes = 0;
    MgLevel<T> levels[MG_MAX_LEVELS];
};

// First level (>= 1) from which every coarser level fits the single-block
// kernel's shared memory, and the bytes needed.
template <class T> void mg_plan_tail(MgHierarchy<T> &H) {
    size_t bytes = 0;
    int tail = H.nlevels;
    for (int l = H.nlevels - 1; l >= 1; --l) {
        // 7 arrays per level, plus on the coarsest level its FP64 iterate,
        // right-hand side, inverse diagonal and couplings
        const size_t need = bytes + 7 * sizeof(T) * (size_t)H.levels[l].g.ncell +
                            (l == H.nlevels - 1 ? 16 + 6 * 8 * (size_t)H.levels[l].g.ncell : 0);
        if (need > MG_TAIL_BYTES_MAX) break;
        bytes = need;
        tail = l;
    }
    H.tail = tail;
    H.tail_bytes = bytes;
}

struct MgSettings {
    int smooth;          // red-black sweeps before and after each coarse correction
    int coarsest_pairs;  // symmetric sweep pairs on the coarsest level
    int coarsest_pairs_warp;  // the same when the coarsest level fits one warp's slots
    double alpha;        // scale of the coarse-grid correction
};

// Level 0 in T from the FP64 operator (and its inverse diagonal) unless the
// assembly wrote it (level0_done), then the Galerkin coarse operators.
template <class T>
cudaError_t mg_setup(const Grid &g0, Operator<double> A, const MgHierarchy<T> &H, bool level0_done, int grid_blocks,
                     cudaStream_t stream);

}  // namespace gbp
