// gbp_solver.cpp -- allocation and the host side of the solve loop.
//
// Iterations are captured once per scene into a CUDA graph of `chunk`
// iterations (three kernels each) and replayed; after each replay the host
// reads the device scalars (one small copy) and stops when the device has
// set `done`. Iterations after the stop return immediately on the device, so
// the result and the iteration count equal those of an unchunked loop.
#include "gbp_solver.h"

#include <cstring>

namespace gbp {

namespace {
#define SOLVER_CUDA(call)                                                                              \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? GBP_ERR_OUT_OF_MEMORY : GBP_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)
}  // namespace

size_t solver_device_bytes(const Grid &g, const gbp_params &p) {
    size_t cells = (size_t)g.ncell;
    size_t fine = 8 * cells * (5 /*operator+b*/ + 4 /*x r s z*/ + (p.warm_start ? 1 : 0));
    return fine;
}

int Solver::prepare(const Grid &g, const gbp_params &p) {
    if (allocated_ && (g.nx != g_.nx || g.ny != g_.ny || g.nz != g_.nz || g.dim != g_.dim)) release();
    g_ = g;
    const size_t bytes = 8 * (size_t)g.ncell;
    if (!allocated_) {
        double **bufs[] = {&st_.diag, &st_.cx, &st_.cy, &st_.cz, &st_.b, &st_.x, &st_.r, &st_.s, &st_.z};
        for (double **b : bufs) SOLVER_CUDA(cudaMalloc(b, bytes));
        SOLVER_CUDA(cudaMemset(st_.cz, 0, bytes));
        SOLVER_CUDA(cudaMalloc(&st_.sc, sizeof(Scalars)));
        SOLVER_CUDA(cudaMemset(st_.sc, 0, sizeof(Scalars)));
        SOLVER_CUDA(cudaMalloc(&st_.pt, sizeof(Partials)));
        SOLVER_CUDA(cudaMallocHost(&st_.host_sc, sizeof(Scalars)));
        allocated_ = true;
    }
    if (p.warm_start && !have_prev_buf_) {
        SOLVER_CUDA(cudaMalloc(&st_.prev, bytes));
        SOLVER_CUDA(cudaMemset(st_.prev, 0, bytes));
        have_prev_buf_ = true;
        st_.have_prev = false;
    }
    return GBP_OK;
}

void Solver::release() {
    if (cg_graph_) {
        cudaGraphExecDestroy(cg_graph_);
        cg_graph_ = nullptr;
    }
    double **bufs[] = {&st_.diag, &st_.cx, &st_.cy, &st_.cz, &st_.b, &st_.x, &st_.r, &st_.s, &st_.z, &st_.prev};
    for (double **b : bufs) {
        if (*b) cudaFree(*b);
        *b = nullptr;
    }
    if (st_.sc) cudaFree(st_.sc);
    if (st_.pt) cudaFree(st_.pt);
    if (st_.host_sc) cudaFreeHost(st_.host_sc);
    st_ = SolverState();
    allocated_ = false;
    have_prev_buf_ = false;
}

int Solver::ensure_cg_graph(const Grid &g, int chunk, int grid_blocks, cudaStream_t stream) {
    if (cg_graph_ && cg_graph_chunk_ == chunk && cg_graph_blocks_ == grid_blocks) return GBP_OK;
    if (cg_graph_) {
        cudaGraphExecDestroy(cg_graph_);
        cg_graph_ = nullptr;
    }
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    cudaGraph_t graph;
    SOLVER_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < chunk; ++it) {
        cudaError_t e = launch_cg_iteration(g, A, st_.x, st_.r, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(stream, &graph);
            return fail(GBP_ERR_CUDA, std::string("capturing CG iterations: ") + cudaGetErrorString(e));
        }
    }
    SOLVER_CUDA(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&cg_graph_, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(GBP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    cg_graph_chunk_ = chunk;
    cg_graph_blocks_ = grid_blocks;
    cg_graph_nodes_ = 3LL * chunk;
    return GBP_OK;
}

int Solver::solve(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    *launches = 0;
    const bool warm = p.warm_start && st_.have_prev;
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    SOLVER_CUDA(launch_cg_init(g, A, st_.b, warm ? st_.prev : nullptr, st_.x, st_.r, st_.s, st_.sc, st_.pt,
                               p.residual, p.max_iterations, grid_blocks, stream));
    *launches += 1;
    const int chunk = p.iterations_per_sync > 0 ? p.iterations_per_sync : 16;
    int rc = ensure_cg_graph(g, chunk, grid_blocks, stream);
    if (rc) return rc;
    const long long max_chunks = (long long)p.max_iterations / chunk + 2;
    bool done = false;
    for (long long k = 0; k < max_chunks; ++k) {
        SOLVER_CUDA(cudaMemcpyAsync(st_.host_sc, st_.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
        SOLVER_CUDA(cudaStreamSynchronize(stream));
        if (st_.host_sc->done) {
            done = true;
            break;
        }
        SOLVER_CUDA(cudaGraphLaunch(cg_graph_, stream));
        *launches += cg_graph_nodes_;
    }
    if (!done) {
        SOLVER_CUDA(cudaMemcpyAsync(st_.host_sc, st_.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
        SOLVER_CUDA(cudaStreamSynchronize(stream));
    }
    SOLVER_CUDA(launch_true_residual(g, A, st_.b, st_.x, warm ? st_.prev : nullptr, st_.sc, st_.pt, grid_blocks,
                                     stream));
    *launches += 1;
    last_outer_ = 1;
    last_inner_total_ = st_.host_sc->iter;
    const int status = st_.host_sc->status;
    if (status == 2 || !st_.host_sc->done) return GBP_ERR_NOT_CONVERGED;
    if (status == 3) return GBP_ERR_NAN;
    return GBP_OK;
}

int Solver::bench_kernel(const Grid &g, int which, int reps, int grid_blocks, cudaStream_t stream, float *ms,
                         double *bytes) {
    if (!allocated_) return fail(GBP_ERR_INVALID_ARGUMENT, "bench_kernel: scene has not been projected yet");
    // scalars that keep every launch running: never done, alpha = 0
    Scalars h;
    std::memset(&h, 0, sizeof(h));
    h.rho = 1.0;
    h.tol = -1.0;
    h.max_iter = 1 << 30;
    h.fluid_exists = 1;
    SOLVER_CUDA(cudaMemcpyAsync(st_.sc, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    const double cells = (double)g.ncell;
    auto launch = [&]() -> cudaError_t {
        switch (which) {
        case 0: return launch_cg_spmv(g, A, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream);
        case 1: return launch_cg_update(g, st_.x, st_.r, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream);
        case 2: return launch_cg_direction(g, st_.r, st_.s, st_.sc, grid_blocks, stream);
        default: return cudaErrorInvalidValue;
        }
    };
    const double per_cell[] = {48.0, 48.0, 24.0};
    if (which < 0 || which > 2) return fail(GBP_ERR_INVALID_ARGUMENT, "bench_kernel: unknown kernel");
    *bytes = per_cell[which] * cells;
    cudaEvent_t e0, e1;
    SOLVER_CUDA(cudaEventCreate(&e0));
    SOLVER_CUDA(cudaEventCreate(&e1));
    SOLVER_CUDA(launch());
    SOLVER_CUDA(cudaEventRecord(e0, stream));
    for (int i = 0; i < reps; ++i) SOLVER_CUDA(launch());
    SOLVER_CUDA(cudaEventRecord(e1, stream));
    SOLVER_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (reps > 0 ? reps : 1);
    return GBP_OK;
}

void Solver::fill_stats(const Scalars &h, gbp_stats *s) const {
    s->iterations = last_inner_total_;
    s->outer_iterations = last_outer_;
    s->converged = h.status == 1;
    s->b_inf = h.res0;
    s->reresid = h.res0 > 0 ? h.res / h.res0 : 0.0;
    s->true_resid_inf = h.res0 > 0 ? h.aux[0] / h.res0 : 0.0;
    s->true_resid_l2 = h.aux[2] > 0 ? h.aux[1] / h.aux[2] : 0.0;
}

}  // namespace gbp
