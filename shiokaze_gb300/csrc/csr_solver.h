// csr_solver.h -- conjugate gradients in FP64 on a general sparse matrix
// in compressed rows: the GPU engine behind gbp_csr_cg and the LinSolver
// plugin module, the drop-in for the reference's pcg module
// (src/linsolver/pcg.cpp:44-74). The iteration and stopping rule are those
// of local/include/pcgsolver/pcg_solver.h:246-295 with its preconditioner,
// which returns its input (:379-384): plain CG from x = 0, stop once
// |r|_inf <= Residual |b|_inf.
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

// Device arrays of one solve, grown on demand and kept between calls.
struct CsrWork {
    long long n_cap = 0, nnz_cap = 0;
    long long *rowstart = nullptr;
    int *cols = nullptr;  // column indices (32-bit: the host checks n < 2^31)
    double *vals = nullptr, *b = nullptr, *x = nullptr, *r = nullptr, *s = nullptr, *z = nullptr;
    Scalars *sc = nullptr, *host_sc = nullptr;
    Partials *pt = nullptr;
    cudaGraphExec_t graph = nullptr;  // a chunk of iterations for (graph_n, graph_blocks)
    long long graph_n = -1;
    int graph_blocks = 0;
};

cudaError_t csr_reserve(CsrWork &w, long long n, long long nnz);
void csr_release(CsrWork &w);

// Runs the solve on w's arrays (rowstart, cols, vals and b filled for n
// rows): x = 0, then iterations until the device reports done; host_sc
// holds the final scalars (status 1 converged, 2 max iterations, 3
// breakdown; res0, res, iter). *launches counts kernel launches.
cudaError_t csr_cg_run(CsrWork &w, long long n, double residual, int max_iter, int grid_blocks,
                       cudaStream_t stream, long long *launches);

}  // namespace gbp
