// cg_kernels.cu -- conjugate gradients in FP64 on the matrix-free operator,
// with the stopping rule of the reference's default solver:
// local/include/pcgsolver/pcg_solver.h:246-295, whose preconditioner
// returns its input (:379-384), so z = r and
//   x = 0, r = b, s = r, rho = r.r, tol = Residual*|b|_inf
//   loop: z = A s; alpha = rho/(s.z); x += alpha s; r -= alpha z;
//         stop if |r|_inf <= tol (iterations = it+1);
//         rho' = r.r; s = r + (rho'/rho) s; rho = rho'
//   up to MaxIterations (then iterations = MaxIterations).
// Each iteration is three launches. The stop test runs on the device: the
// last block of the update launch sets sc->done, and every later launch
// returns at once, so a host loop may enqueue (or a graph may hold) more
// iterations than are needed without changing the result.
//
// Algorithmic DRAM bytes per cell and iteration (FP64):
//   spmv    read s (8) + diag,cx,cy,cz (32), write z (8)            = 48 B
//   update  read x,s,r,z (32), write x,r (16)                       = 48 B
//   dir     read r,s (16), write s (8)                              = 24 B
#include "gbp_internal.cuh"
#include "gbp_kernels.h"

namespace gbp {
namespace {

__device__ __forceinline__ bool stopped(const Scalars *sc) { return *((volatile const int *)&sc->done) != 0; }

// (A s)_c for the 7-point (5-point) matrix-free operator.
__device__ __forceinline__ double apply_A(const Grid &g, const Operator<double> &A, const double *__restrict__ s,
                                          int i, int j, int k, long long c) {
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    double acc = __ldg(A.diag + c) * __ldg(s + c);
    if (i > 0) acc -= __ldg(A.cx + c - 1) * __ldg(s + c - 1);
    if (i + 1 < g.nx) acc -= __ldg(A.cx + c) * __ldg(s + c + 1);
    if (j > 0) acc -= __ldg(A.cy + c - sy) * __ldg(s + c - sy);
    if (j + 1 < g.ny) acc -= __ldg(A.cy + c) * __ldg(s + c + sy);
    if (g.dim == 3) {
        if (k > 0) acc -= __ldg(A.cz + c - sz) * __ldg(s + c - sz);
        if (k + 1 < g.nz) acc -= __ldg(A.cz + c) * __ldg(s + c + sz);
    }
    return acc;
}

// Iterates the cells of this block's tiles: f(i, j, k, c).
template <class F> __device__ __forceinline__ void for_each_cell(const Grid &g, F f) {
    const int tx = threadIdx.x & (TILE_X - 1), ty = threadIdx.x / TILE_X;
    for (long long t = blockIdx.x; t < g.ntiles; t += gridDim.x) {
        int i0, j0, k0;
        tile_origin(g, t, i0, j0, k0);
        const int i = i0 + tx, j = j0 + ty;
        if (i >= g.nx || j >= g.ny) continue;
        const int kend = min(k0 + g.tz, g.nz);
        for (int k = k0; k < kend; ++k) f(i, j, k, cell_index(g, i, j, k));
    }
}

__global__ void __launch_bounds__(BLOCK_THREADS, 6) cg_init_kernel(Grid g, Operator<double> A,
                                                                const double *__restrict__ b,
                                                                const double *__restrict__ prev, double *x, double *r,
                                                                double *s, Scalars *sc, Partials *pt,
                                                                double residual, int max_iter) {
    __shared__ double sh[BLOCK_THREADS / 32];
    double mx = 0.0, r2 = 0.0;
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        double rv = __ldg(b + c);
        if (prev) rv -= apply_A(g, A, prev, i, j, k, c);  // macpressuresolver3.cpp:228-229
        x[c] = 0.0;
        r[c] = rv;
        s[c] = rv;
        mx = fmax(mx, fabs(rv));
        r2 = fma(rv, rv, r2);
    });
    double bm = block_max(mx, sh);
    double bs = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        pt->a[blockIdx.x] = bm;
        pt->b[blockIdx.x] = bs;
    }
    if (last_block(&sc->counter[0])) {
        double res0 = reduce_partials_max(pt->a, gridDim.x, sh);
        double rho = reduce_partials_sum(pt->b, gridDim.x, sh);
        if (threadIdx.x == 0) {
            double tolf = residual < 1e-30 ? 1e-30 : residual;  // pcg_solver.h:51
            sc->res0 = res0;
            sc->res = res0;
            sc->tol = tolf * res0;
            sc->rho = rho;
            sc->r2 = rho;
            sc->iter = 0;
            sc->max_iter = max_iter;
            sc->alpha = sc->beta = 0.0;
            if (res0 == 0.0) {  // pcg_solver.h:65-68
                sc->done = 1;
                sc->status = 1;
            } else if (rho == 0.0 || rho != rho) {  // :74-82
                sc->done = 1;
                sc->status = 3;
            } else if (max_iter <= 0) {
                sc->done = 1;
                sc->status = 2;
            } else {
                sc->done = 0;
                sc->status = 0;
            }
            sc->counter[0] = 0;
        }
    }
}

__global__ void __launch_bounds__(BLOCK_THREADS, 6) cg_spmv_kernel(Grid g, Operator<double> A,
                                                                const double *__restrict__ s, double *z, Scalars *sc,
                                                                Partials *pt) {
    if (stopped(sc)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    double dot = 0.0;
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        double zv = apply_A(g, A, s, i, j, k, c);
        z[c] = zv;
        dot = fma(__ldg(s + c), zv, dot);
    });
    double bs = block_sum(dot, sh);
    if (threadIdx.x == 0) pt->a[blockIdx.x] = bs;
    if (last_block(&sc->counter[1])) {
        double pap = reduce_partials_sum(pt->a, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->pap = pap;
            sc->alpha = sc->rho / pap;
            sc->counter[1] = 0;
        }
    }
}

__global__ void __launch_bounds__(BLOCK_THREADS, 6) cg_update_kernel(Grid g, double *x, double *r,
                                                                  const double *__restrict__ s,
                                                                  const double *__restrict__ z, Scalars *sc,
                                                                  Partials *pt) {
    if (stopped(sc)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    const double alpha = sc->alpha;
    double mx = 0.0, r2 = 0.0;
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        x[c] = fma(alpha, __ldg(s + c), x[c]);
        double rv = fma(-alpha, __ldg(z + c), r[c]);
        r[c] = rv;
        mx = fmax(mx, fabs(rv));
        r2 = fma(rv, rv, r2);
    });
    double bm = block_max(mx, sh);
    double bs = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        pt->b[blockIdx.x] = bm;
        pt->c[blockIdx.x] = bs;
    }
    if (last_block(&sc->counter[2])) {
        double res = reduce_partials_max(pt->b, gridDim.x, sh);
        double rho_new = reduce_partials_sum(pt->c, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->res = res;
            sc->r2 = rho_new;
            sc->iter += 1;
            if (res <= sc->tol) {
                sc->done = 1;
                sc->status = 1;
            } else if (sc->iter >= sc->max_iter) {
                sc->done = 1;
                sc->status = 2;
            } else if (rho_new != rho_new || sc->alpha != sc->alpha) {
                sc->done = 1;
                sc->status = 3;
            } else {
                sc->beta = rho_new / sc->rho;
                sc->rho = rho_new;
            }
            sc->counter[2] = 0;
        }
    }
}

__global__ void __launch_bounds__(BLOCK_THREADS, 6) cg_direction_kernel(Grid g, const double *__restrict__ r,
                                                                     double *s, const Scalars *sc) {
    if (stopped(sc)) return;
    const double beta = sc->beta;
    for_each_cell(g, [&](int i, int j, int k, long long c) { s[c] = fma(beta, s[c], __ldg(r + c)); });
}

__global__ void __launch_bounds__(BLOCK_THREADS, 6) true_residual_kernel(Grid g, Operator<double> A,
                                                                      const double *__restrict__ b,
                                                                      const double *__restrict__ x,
                                                                      const double *__restrict__ prev, Scalars *sc,
                                                                      Partials *pt) {
    __shared__ double sh[BLOCK_THREADS / 32];
    double mx = 0.0, r2 = 0.0, b2 = 0.0;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    auto X = [&](long long c) { return prev ? __ldg(x + c) + __ldg(prev + c) : __ldg(x + c); };
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        double acc = __ldg(A.diag + c) * X(c);
        if (i > 0) acc -= __ldg(A.cx + c - 1) * X(c - 1);
        if (i + 1 < g.nx) acc -= __ldg(A.cx + c) * X(c + 1);
        if (j > 0) acc -= __ldg(A.cy + c - sy) * X(c - sy);
        if (j + 1 < g.ny) acc -= __ldg(A.cy + c) * X(c + sy);
        if (g.dim == 3) {
            if (k > 0) acc -= __ldg(A.cz + c - sz) * X(c - sz);
            if (k + 1 < g.nz) acc -= __ldg(A.cz + c) * X(c + sz);
        }
        // rows off the unknowns are identically 0 (diag and couplings 0, b 0)
        const double rv = __ldg(b + c) - acc;
        mx = fmax(mx, fabs(rv));
        r2 = fma(rv, rv, r2);
        double b0 = __ldg(b + c);
        if (prev) {
            double ap = __ldg(A.diag + c) * __ldg(prev + c);
            if (i > 0) ap -= __ldg(A.cx + c - 1) * __ldg(prev + c - 1);
            if (i + 1 < g.nx) ap -= __ldg(A.cx + c) * __ldg(prev + c + 1);
            if (j > 0) ap -= __ldg(A.cy + c - sy) * __ldg(prev + c - sy);
            if (j + 1 < g.ny) ap -= __ldg(A.cy + c) * __ldg(prev + c + sy);
            if (g.dim == 3) {
                if (k > 0) ap -= __ldg(A.cz + c - sz) * __ldg(prev + c - sz);
                if (k + 1 < g.nz) ap -= __ldg(A.cz + c) * __ldg(prev + c + sz);
            }
            b0 -= ap;
        }
        b2 = fma(b0, b0, b2);
    });
    double bm = block_max(mx, sh);
    double bs = block_sum(r2, sh);
    double bb = block_sum(b2, sh);
    if (threadIdx.x == 0) {
        pt->a[blockIdx.x] = bm;
        pt->b[blockIdx.x] = bs;
        pt->c[blockIdx.x] = bb;
    }
    if (last_block(&sc->counter[3])) {
        double m = reduce_partials_max(pt->a, gridDim.x, sh);
        double s2 = reduce_partials_sum(pt->b, gridDim.x, sh);
        double sb = reduce_partials_sum(pt->c, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->aux[0] = m;
            sc->aux[1] = sqrt(s2);
            sc->aux[2] = sqrt(sb);
            sc->counter[3] = 0;
        }
    }
}

int blocks_for(const Grid &g, int grid_blocks) {
    long long b = g.ntiles < grid_blocks ? g.ntiles : grid_blocks;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

cudaError_t launch_cg_init(const Grid &g, Operator<double> A, const double *b, const double *prev, double *x,
                           double *r, double *s, Scalars *sc, Partials *pt, double residual, int max_iter,
                           int grid_blocks, cudaStream_t stream) {
    cg_init_kernel<<<blocks_for(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, A, b, prev, x, r, s, sc, pt,
                                                                            residual, max_iter);
    return cudaGetLastError();
}

cudaError_t launch_cg_iteration(const Grid &g, Operator<double> A, double *x, double *r, double *s, double *z,
                                Scalars *sc, Partials *pt, int grid_blocks, cudaStream_t stream) {
    const int nb = blocks_for(g, grid_blocks);
    cg_spmv_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(g, A, s, z, sc, pt);
    cg_update_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(g, x, r, s, z, sc, pt);
    cg_direction_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(g, r, s, sc);
    return cudaGetLastError();
}

cudaError_t launch_cg_spmv(const Grid &g, Operator<double> A, const double *s, double *z, Scalars *sc, Partials *pt,
                           int grid_blocks, cudaStream_t stream) {
    cg_spmv_kernel<<<blocks_for(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, A, s, z, sc, pt);
    return cudaGetLastError();
}

cudaError_t launch_cg_update(const Grid &g, double *x, double *r, const double *s, const double *z, Scalars *sc,
                             Partials *pt, int grid_blocks, cudaStream_t stream) {
    cg_update_kernel<<<blocks_for(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, x, r, s, z, sc, pt);
    return cudaGetLastError();
}

cudaError_t launch_cg_direction(const Grid &g, const double *r, double *s, const Scalars *sc, int grid_blocks,
                                cudaStream_t stream) {
    cg_direction_kernel<<<blocks_for(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, r, s, sc);
    return cudaGetLastError();
}

cudaError_t launch_true_residual(const Grid &g, Operator<double> A, const double *b, const double *x,
                                 const double *prev, Scalars *sc, Partials *pt, int grid_blocks,
                                 cudaStream_t stream) {
    true_residual_kernel<<<blocks_for(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, A, b, x, prev, sc, pt);
    return cudaGetLastError();
}

}  // namespace gbp
