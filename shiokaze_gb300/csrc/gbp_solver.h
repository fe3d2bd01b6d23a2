// gbp_solver.h -- device state and solve loop of one scene.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbp.h"
#include "gbp_kernels.h"
#include "gbp_batch.h"
#include "gbp_mg.h"

namespace gbp {

struct SolverState {
    // fine-level FP64 operator and right-hand side
    double *diag = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr, *b = nullptr;
    // FP64 vectors: x (the correction to prev under warm start), r, and the
    // CG directions s, z (= A s for plain CG; z = M r for MGPCG) and q
    double *x = nullptr, *r = nullptr, *s = nullptr, *z = nullptr, *q = nullptr;
    // warm-start pressure kept per cell
    double *prev = nullptr;
    bool have_prev = false;
    // mixed precision: FP32 inner vectors
    float *rf = nullptr, *zf = nullptr, *pf = nullptr, *qf = nullptr, *df = nullptr;
    Scalars *sc = nullptr;
    Partials *pt = nullptr;
    Scalars *host_sc = nullptr;  // pinned
    // per-face weights, fluxes and fractions of the face-first assembly
    FaceArrays faces{};
};

size_t solver_device_bytes(const Grid &g, const gbp_params &p);

// Grids of the multigrid levels of g (level 0 = g).
std::vector<Grid> mg_level_grids(const Grid &g, int coarsest);

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

    // Batched MGPCG: per-scene setup (level-0 operator in T, Galerkin
    // hierarchy), then this scene's entries of a batch plan.
    int setup_mg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches);
    // Level 0 of the hierarchy p's solve uses, for the fused 3D assembly to
    // write (all null for plain CG); level0_written() tells the next
    // setup_mg that the assembly did.
    Level0Out level0_out(const gbp_params &p) const;
    void level0_written() { level0_written_ = true; }
    template <class T> void add_to_plan(BatchPlan<T> &plan, const gbp_params &p) const;
    // Reads this scene's scalars after a batched solve.
    int finish_batched(const gbp_params &p, cudaStream_t stream);
    // After the solve: FP64 true residual, iteration counts, status
    // (GBP_OK / GBP_ERR_NOT_CONVERGED / GBP_ERR_NAN).
    int complete(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches);
    bool has_prev() const { return st_.have_prev; }
    // the last single-scene MGPCG solve ran the TMA-staged fine kernels
    bool staged() const { return runner_key_ >= 0 && runner_.scene_staged(0); }
    // test hook of gbp_debug_fail_wait: the next MGPCG solve's waits run out
    void set_wait_test(int what, int block, int polls) { runner_.set_wait_test(what, block, polls); }

private:
    int fail(int code, const std::string &m) {
        err_ = m;
        return code;
    }
    template <class T> int alloc(T **p, size_t n);
    template <class T> int alloc_classes(MgHierarchy<T> &H);
    int prepare_mg(const Grid &g, const gbp_params &p);
    int solve_cg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches);
    int solve_mg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches);
    int run_graph(const gbp_params &p, int chunk, cudaStream_t stream, long long *launches);

    SolverState st_;
    Grid g_{};
    bool allocated_ = false;
    bool have_prev_buf_ = false;
    std::string err_;
    std::vector<void *> owned_;  // multigrid and mixed-precision buffers
    // multigrid hierarchies (FP64 path and FP32 inner solve), built lazily
    MgHierarchy<double> h64_;
    MgHierarchy<float> h32_;
    bool mg64_ready_ = false, mg32_ready_ = false;
    bool level0_written_ = false;
    int mg_coarsest_ = 0;
    int last_precision_ = GBP_PRECISION_FP64;
    // cached graph of solver iterations
    cudaGraphExec_t graph_ = nullptr;
    long long graph_key_ = -1;
    long long graph_nodes_ = 0;
    int last_outer_ = 1;
    int last_inner_total_ = 0;
    // batch of one for the scene's own MGPCG solves
    BatchRunner runner_;
    long long runner_key_ = -1;
};

}  // namespace gbp
