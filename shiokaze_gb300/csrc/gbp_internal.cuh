// gbp_internal.cuh -- shared device/host definitions of libgbp.
//
// Data layout in HBM (one scene): every per-cell array is a dense nx*ny*nz
// array, x fastest. The operator is stored matrix-free as four per-cell
// arrays: diag (0 off the unknowns) and the coupling weight of the cell's
// +x/+y/+z face, cx/cy/cz, which is the negated off-diagonal
// -A[c][c+e_d] and is 0 unless both cells are unknowns. Vectors are dense
// with 0 off the unknowns, so A*x is the 7-point (5-point in 2D) stencil
//   (A x)_c = diag_c x_c - sum_d (cd_c x_{c+e_d} + cd_{c-e_d} x_{c-e_d}).
//
// Work is split into tiles of 32 (x) by 8 (y) by TZ (z) cells. A launch runs
// a fixed number of blocks (a multiple of the SM count); block b handles
// tiles b, b+G, b+2G, ... in order. Reductions keep one partial per block
// and the last block to finish sums them in block order, so every result is
// bitwise reproducible run to run.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbp {

constexpr int TILE_X = 32;
constexpr int TILE_Y = 8;
constexpr int BLOCK_THREADS = TILE_X * TILE_Y;  // 256
constexpr int MAX_GRID = 152 * 8;               // partial-array capacity

// Exact unsigned division by a divisor fixed at run time: one multiply-high,
// an add and two shifts instead of a division routine (Granlund and
// Montgomery, "Division by invariant integers using multiplication",
// PLDI 1994, fig. 4.1). Exact for every 32-bit dividend and divisor >= 1.
struct FastDiv {
    unsigned d, m;
    int s1, s2;
};

__host__ __device__ inline FastDiv make_fastdiv(unsigned d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1ull << l) < d) ++l;  // l = ceil(log2 d)
    f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}

__host__ __device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv &f) {
#ifdef __CUDA_ARCH__
    const unsigned t1 = __umulhi(f.m, n);
#else
    const unsigned t1 = (unsigned)(((unsigned long long)f.m * n) >> 32);
#endif
    return (t1 + ((n - t1) >> f.s1)) >> f.s2;
}

struct Grid {
    int nx, ny, nz;   // cells (nz == 1 in 2D)
    int dim;          // 2 or 3
    int tz;           // tile depth in z
    int ntx, nty, ntz;
    long long ntiles;
    long long ncell;
    // divisors of the tile decompositions: ntx (32-wide cell tiles), ntx2
    // (64-wide pair tiles), nty; and of the node grid: nx+1, (nx+1)(ny+1)
    FastDiv ftx, ftx2, fty;
    FastDiv fn1, fn2;
};

// deep_min: the fewest cells for tiles 4 planes deep. Deep tiles give a
// block more cells and the gather-first column kernels their 4 planes;
// thin ones spread small grids over all SMs. A scene's fine grid takes deep
// tiles from 2^21 cells (128^3), coarse levels only above (their 2^21-cell
// level, under a 256^3 grid, balances better in thin tiles).
constexpr long long DEEP_MIN_FINE = 1LL << 21;
constexpr long long DEEP_MIN_COARSE = (1LL << 21) + 1;
inline Grid make_grid(int dim, int nx, int ny, int nz, long long deep_min = DEEP_MIN_FINE) {
    Grid g;
    g.dim = dim;
    g.nx = nx;
    g.ny = ny;
    g.nz = dim == 3 ? nz : 1;
    g.tz = (g.nz == 1 || (long long)nx * ny * g.nz < deep_min) ? 1 : 4;
    g.ntx = (nx + TILE_X - 1) / TILE_X;
    g.nty = (ny + TILE_Y - 1) / TILE_Y;
    g.ntz = (g.nz + g.tz - 1) / g.tz;
    g.ntiles = (long long)g.ntx * g.nty * g.ntz;
    g.ncell = (long long)nx * ny * g.nz;
    g.ftx = make_fastdiv((unsigned)g.ntx);
    g.ftx2 = make_fastdiv((unsigned)((nx + 63) / 64));
    g.fty = make_fastdiv((unsigned)g.nty);
    g.fn1 = make_fastdiv((unsigned)(nx + 1));
    g.fn2 = make_fastdiv((unsigned)((nx + 1) * (ny + 1)));
    return g;
}

// Reduction scratch of one solve: per-block partials and scalars that the
// last block of a launch writes. Lives in device memory.
struct Scalars {
    double rho;      // r . z of the current iterate
    double alpha;
    double beta;
    double pap;      // p . A p
    double tol;      // absolute stopping threshold on |r|_inf
    double res0;     // |r0|_inf
    double res;      // |r|_inf of the latest iterate
    double r2;       // r . r of the latest iterate (for reporting)
    double aux[4];
    double inner_tol;   // mixed: absolute threshold of the current inner solve
    double inner_res0;  // mixed: |r_f|_inf at the start of the inner solve
    int iter;        // completed (inner) iterations
    int done;        // nonzero once the solve has stopped
    int status;      // 0 running, 1 converged, 2 max iterations, 3 breakdown (0/0 or NaN)
    int max_iter;
    int fluid_exists;
    int first;        // next preconditioned dot starts a new direction (beta = 0)
    int first_update; // next update overwrites (rather than adds to) the correction
    int inner_done;   // mixed: the current inner solve has stopped
    int inner_iter;   // mixed: iterations of the current inner solve
    int inner_max;    // mixed: iteration cap of one inner solve
    int outer_iter;   // mixed: refinement steps taken
    int pad;
    unsigned long long unknowns;
    unsigned long long bits_max;  // max of non-negative doubles through their bit patterns
    unsigned int counter[8];      // last-block tickets, one per reduction site
};

struct Partials {
    double a[MAX_GRID];
    double b[MAX_GRID];
    double c[MAX_GRID];
};

#ifdef __CUDACC__

__device__ __forceinline__ long long cell_index(const Grid &g, int i, int j, int k) {
    return (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * k);
}

// Coordinates of node t of the (nx+1)(ny+1)(nz+1) node grid, x fastest
// (node counts fit 32 bits).
__device__ __forceinline__ void node_coords(const Grid &g, long long t, int &i, int &j, int &k) {
    const unsigned tt = (unsigned)t;
    const unsigned q = fdiv(tt, g.fn1);
    const unsigned kk = fdiv(tt, g.fn2);
    i = (int)(tt - q * g.fn1.d);
    j = (int)(q - kk * (unsigned)(g.ny + 1));
    k = (int)kk;
}

// Tiles are numbered x fastest, then y, then z (tile counts fit 32 bits).
__device__ __forceinline__ void tile_origin(const Grid &g, long long t, int &i0, int &j0, int &k0) {
    const unsigned tt = (unsigned)t;
    const unsigned r = fdiv(tt, g.ftx);
    const unsigned tk = fdiv(r, g.fty);
    i0 = (int)(tt - r * (unsigned)g.ntx) * TILE_X;
    j0 = (int)(r - tk * (unsigned)g.nty) * TILE_Y;
    k0 = (int)tk * g.tz;
}

template <class T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <class T> __device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum in a fixed order; result valid in thread 0.
template <class T> __device__ __forceinline__ T block_sum(T v, T *sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = 0;
    if (wid == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : T(0);
        r = warp_sum(r);
    }
    return r;
}

template <class T> __device__ __forceinline__ T block_max(T v, T *sh) {
    v = warp_max(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = 0;
    if (wid == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : T(0);
        r = warp_max(r);
    }
    return r;
}

// Publishes this block's partial(s) and returns true in every thread of the
// block that finished last. Must be called by all threads of the block.
__device__ __forceinline__ bool last_block(unsigned int *counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int ticket = atomicAdd(counter, 1u);
        is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// Sums partial[0..n) in a fixed order (strided per thread, then the block
// tree); result valid in thread 0.
__device__ __forceinline__ double reduce_partials_sum(const double *partial, int n, double *sh) {
    double v = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) v += __ldcg(partial + t);
    return block_sum(v, sh);
}

__device__ __forceinline__ double reduce_partials_max(const double *partial, int n, double *sh) {
    double v = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) v = fmax(v, __ldcg(partial + t));
    return block_max(v, sh);
}

#endif  // __CUDACC__

}  // namespace gbp
