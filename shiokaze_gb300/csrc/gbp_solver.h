// gbp_solver.h -- device state and solve loop of one scene.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbp.h"
#include "gbp_kernels.h"

namespace gbp {

struct SolverState {
    // fine-level FP64 operator and right-hand side
    double *diag = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr, *b = nullptr;
    // CG vectors (x is the correction to prev under warm start)
    double *x = nullptr, *r = nullptr, *s = nullptr, *z = nullptr;
    // warm-start pressure kept per cell
    double *prev = nullptr;
    bool have_prev = false;
    Scalars *sc = nullptr;
    Partials *pt = nullptr;
    Scalars *host_sc = nullptr;  // pinned
};

size_t solver_device_bytes(const Grid &g, const gbp_params &p);

class Solver {
public:
    Solver() = default;
    ~Solver() { release(); }
    Solver(const Solver &) = delete;
    Solver &operator=(const Solver &) = delete;

    // Allocates what a solve of grid g with params p needs (idempotent).
    int prepare(const Grid &g, const gbp_params &p);
    // Solves A x = b - A prev on `stream` after assembly filled diag/c?/b.
    // Returns GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN or an error.
    int solve(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches);
    void fill_stats(const Scalars &h, gbp_stats *st) const;
    // Times reps launches of one solver kernel (see gbp_bench_kernel).
    int bench_kernel(const Grid &g, int which, int reps, int grid_blocks, cudaStream_t stream, float *ms,
                     double *bytes);
    void release();
    SolverState &state() { return st_; }
    const char *error() const { return err_.c_str(); }

private:
    int fail(int code, const std::string &m) {
        err_ = m;
        return code;
    }
    int ensure_cg_graph(const Grid &g, int chunk, int grid_blocks, cudaStream_t stream);

    SolverState st_;
    Grid g_{};
    bool allocated_ = false;
    bool have_prev_buf_ = false;
    std::string err_;
    cudaGraphExec_t cg_graph_ = nullptr;
    int cg_graph_chunk_ = 0;
    int cg_graph_blocks_ = 0;
    long long cg_graph_nodes_ = 0;
    int last_outer_ = 1;
    int last_inner_total_ = 0;
};

}  // namespace gbp
