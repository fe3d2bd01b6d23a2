// csr_solver.cu -- FP64 conjugate gradients on a matrix in compressed rows
// (see csr_solver.h). One thread per row, grid-stride; each iteration is
// three launches (z = A s with s.z; the updates with |r|_inf and r.r; the new
// direction), and the stop test runs in the last block of the update launch
// (per-block partials combined in block order: reproducible run to run), so
// a CUDA graph may hold more iterations than are needed.
//
// Algorithmic DRAM bytes per iteration: spmv reads the row pointers (8 per
// row), columns and values (12 per entry: 32-bit columns) and s (8 per
// entry, mostly from cache; counted once per row), writes z (8 per row);
// update 48 and direction 24 per row.
#include "csr_solver.h"

namespace gbp {
namespace {

__device__ __forceinline__ bool stopped(const Scalars *sc) { return *((volatile const int *)&sc->done) != 0; }

template <class F> __device__ __forceinline__ void for_each_row(long long n, F f) {
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (long long)gridDim.x * blockDim.x)
        f(row);
}

// x = 0, r = s = b, |b|_inf, b.b; the threshold and the early exits of
// pcg_solver.h:250-268.
__global__ void __launch_bounds__(BLOCK_THREADS) csr_init_kernel(long long n, const double *__restrict__ b, double *x,
                                                                 double *r, double *s, Scalars *sc, Partials *pt,
                                                                 double residual, int max_iter) {
    __shared__ double sh[BLOCK_THREADS / 32];
    double mx = 0.0, r2 = 0.0;
    for_each_row(n, [&](long long row) {
        const double rv = __ldg(b + row);
        x[row] = 0.0;
        r[row] = rv;
        s[row] = rv;
        mx = fmax(mx, fabs(rv));
        r2 = fma(rv, rv, r2);
    });
    const double bm = block_max(mx, sh);
    const double bs = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        pt->a[blockIdx.x] = bm;
        pt->b[blockIdx.x] = bs;
    }
    if (last_block(&sc->counter[0])) {
        const double res0 = reduce_partials_max(pt->a, gridDim.x, sh);
        const double rho = reduce_partials_sum(pt->b, gridDim.x, sh);
        if (threadIdx.x == 0) {
            const double tolf = residual < 1e-30 ? 1e-30 : residual;  // pcg_solver.h:240
            sc->res0 = res0;
            sc->res = res0;
            sc->tol = tolf * res0;
            sc->rho = rho;
            sc->r2 = rho;
            sc->iter = 0;
            sc->max_iter = max_iter;
            sc->alpha = sc->beta = 0.0;
            if (res0 == 0.0) {  // pcg_solver.h:253-256
                sc->done = 1;
                sc->status = 1;
            } else if (rho == 0.0 || rho != rho) {  // :262-270
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

// z = A s, s.z, alpha = rho / s.z (pcg_solver.h:276-277); each row's entries
// are summed in their stored order.
__global__ void __launch_bounds__(BLOCK_THREADS) csr_spmv_kernel(long long n, const long long *__restrict__ rowstart,
                                                                 const int *__restrict__ cols,
                                                                 const double *__restrict__ vals,
                                                                 const double *__restrict__ s, double *z, Scalars *sc,
                                                                 Partials *pt) {
    if (stopped(sc)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    double dot = 0.0;
    for_each_row(n, [&](long long row) {
        const long long e0 = __ldg(rowstart + row), e1 = __ldg(rowstart + row + 1);
        double acc = 0.0;
        for (long long e = e0; e < e1; ++e) acc = fma(__ldg(vals + e), __ldg(s + __ldg(cols + e)), acc);
        z[row] = acc;
        dot = fma(__ldg(s + row), acc, dot);
    });
    const double bs = block_sum(dot, sh);
    if (threadIdx.x == 0) pt->a[blockIdx.x] = bs;
    if (last_block(&sc->counter[1])) {
        const double pap = reduce_partials_sum(pt->a, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->pap = pap;
            sc->alpha = sc->rho / pap;
            sc->counter[1] = 0;
        }
    }
}

// x += alpha s, r -= alpha z, |r|_inf and r.r; the stop test of
// pcg_solver.h:278-286, then beta = r.r / rho (:288-291).
__global__ void __launch_bounds__(BLOCK_THREADS) csr_update_kernel(long long n, double *x, double *r,
                                                                   const double *__restrict__ s,
                                                                   const double *__restrict__ z, Scalars *sc,
                                                                   Partials *pt) {
    if (stopped(sc)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    const double alpha = sc->alpha;
    double mx = 0.0, r2 = 0.0;
    for_each_row(n, [&](long long row) {
        x[row] = fma(alpha, __ldg(s + row), x[row]);
        const double rv = fma(-alpha, __ldg(z + row), r[row]);
        r[row] = rv;
        mx = fmax(mx, fabs(rv));
        r2 = fma(rv, rv, r2);
    });
    const double bm = block_max(mx, sh);
    const double bs = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        pt->b[blockIdx.x] = bm;
        pt->c[blockIdx.x] = bs;
    }
    if (last_block(&sc->counter[2])) {
        const double res = reduce_partials_max(pt->b, gridDim.x, sh);
        const double rho_new = reduce_partials_sum(pt->c, gridDim.x, sh);
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

// s = r + beta s (pcg_solver.h:290)
__global__ void __launch_bounds__(BLOCK_THREADS) csr_direction_kernel(long long n, const double *__restrict__ r,
                                                                      double *s, const Scalars *sc) {
    if (stopped(sc)) return;
    const double beta = sc->beta;
    for_each_row(n, [&](long long row) { s[row] = fma(beta, s[row], __ldg(r + row)); });
}

int blocks_for(long long n, int grid_blocks) {
    const long long b = (n + BLOCK_THREADS - 1) / BLOCK_THREADS;
    return (int)(b < 1 ? 1 : (b < grid_blocks ? b : grid_blocks));
}

constexpr int kCsrChunk = 16;  // iterations per graph replay

}  // namespace

cudaError_t csr_reserve(CsrWork &w, long long n, long long nnz) {
    cudaError_t e = cudaSuccess;
    if (!w.sc) {
        if ((e = cudaMalloc(&w.sc, sizeof(Scalars))) != cudaSuccess) return e;
        if ((e = cudaMemset(w.sc, 0, sizeof(Scalars))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w.pt, sizeof(Partials))) != cudaSuccess) return e;
        if ((e = cudaMallocHost(&w.host_sc, sizeof(Scalars))) != cudaSuccess) return e;
    }
    if (n > w.n_cap) {
        double **vecs[] = {&w.b, &w.x, &w.r, &w.s, &w.z};
        for (double **v : vecs) {
            if (*v) cudaFree(*v);
            *v = nullptr;
        }
        if (w.rowstart) cudaFree(w.rowstart);
        w.rowstart = nullptr;
        w.n_cap = 0;
        for (double **v : vecs)
            if ((e = cudaMalloc(v, sizeof(double) * (size_t)n)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w.rowstart, sizeof(long long) * (size_t)(n + 1))) != cudaSuccess) return e;
        w.n_cap = n;
        if (w.graph) cudaGraphExecDestroy(w.graph);
        w.graph = nullptr;
        w.graph_n = -1;
    }
    if (nnz > w.nnz_cap) {
        if (w.cols) cudaFree(w.cols);
        if (w.vals) cudaFree(w.vals);
        w.cols = nullptr;
        w.vals = nullptr;
        w.nnz_cap = 0;
        if ((e = cudaMalloc(&w.cols, sizeof(int) * (size_t)nnz)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w.vals, sizeof(double) * (size_t)nnz)) != cudaSuccess) return e;
        w.nnz_cap = nnz;
        if (w.graph) cudaGraphExecDestroy(w.graph);
        w.graph = nullptr;
        w.graph_n = -1;
    }
    return cudaSuccess;
}

void csr_release(CsrWork &w) {
    if (w.graph) cudaGraphExecDestroy(w.graph);
    void *d[] = {w.rowstart, w.cols, w.vals, w.b, w.x, w.r, w.s, w.z, w.sc, w.pt};
    for (void *p : d)
        if (p) cudaFree(p);
    if (w.host_sc) cudaFreeHost(w.host_sc);
    w = CsrWork{};
}

cudaError_t csr_cg_run(CsrWork &w, long long n, double residual, int max_iter, int grid_blocks,
                       cudaStream_t stream, long long *launches) {
    const int nb = blocks_for(n, grid_blocks);
    cudaError_t e;
    if ((e = cudaMemsetAsync(w.sc, 0, sizeof(Scalars), stream)) != cudaSuccess) return e;
    csr_init_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(n, w.b, w.x, w.r, w.s, w.sc, w.pt, residual, max_iter);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *launches += 1;
    if (!w.graph || w.graph_n != n || w.graph_blocks != nb) {
        if (w.graph) cudaGraphExecDestroy(w.graph);
        w.graph = nullptr;
        cudaGraph_t graph;
        if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        for (int it = 0; it < kCsrChunk; ++it) {
            csr_spmv_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(n, w.rowstart, w.cols, w.vals, w.s, w.z, w.sc, w.pt);
            csr_update_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(n, w.x, w.r, w.s, w.z, w.sc, w.pt);
            csr_direction_kernel<<<nb, BLOCK_THREADS, 0, stream>>>(n, w.r, w.s, w.sc);
        }
        const cudaError_t e1 = cudaGetLastError();
        const cudaError_t e2 = cudaStreamEndCapture(stream, &graph);
        if (e1 != cudaSuccess) return e1;
        if (e2 != cudaSuccess) return e2;
        e = cudaGraphInstantiate(&w.graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return e;
        w.graph_n = n;
        w.graph_blocks = nb;
    }
    const long long max_chunks = (long long)(max_iter > 0 ? max_iter : 0) / kCsrChunk + 2;
    for (long long k = 0; k <= max_chunks; ++k) {
        if ((e = cudaMemcpyAsync(w.host_sc, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
        if (w.host_sc->done) return cudaSuccess;
        if ((e = cudaGraphLaunch(w.graph, stream)) != cudaSuccess) return e;
        *launches += 3LL * kCsrChunk;
    }
    if ((e = cudaMemcpyAsync(w.host_sc, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
        return e;
    return cudaStreamSynchronize(stream);
}

}  // namespace gbp
