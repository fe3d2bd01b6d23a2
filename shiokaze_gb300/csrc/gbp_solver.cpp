// gbp_solver.cpp -- allocation and the host side of the solve loops.
//
// Iterations are captured once per scene and configuration into a CUDA graph
// holding `chunk` iterations and replayed; after each replay the host reads
// the device scalars (one small copy) and stops when the device has set
// `done`. Launches after the stop return immediately on the device, so the
// result and the iteration count equal those of an unchunked loop.
//
//   CG     (reference solver)  init; [spmv, update, direction] x chunk
//   MGPCG  FP64                init (r = b - A prev); [V-cycle + dot,
//                              direction, spmv, update] x chunk
//   MGPCG  mixed               FP64 init; [FP32 V-cycle + dot, direction,
//                              spmv, update (inner stop), x64 += d,
//                              r64 = b - A64 x64 (outer stop)] x chunk
#include "gbp_solver.h"

#include <cstdint>

#include <algorithm>
#include <cstring>
#include <functional>

namespace gbp {

namespace {
#define SOLVER_CUDA(call)                                                                              \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? GBP_ERR_OUT_OF_MEMORY : GBP_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

int coarsest_of(const gbp_params &p) { return p.mg_coarsest > 1 ? p.mg_coarsest : 4; }
}  // namespace

std::vector<Grid> mg_level_grids(const Grid &g, int coarsest) {
    std::vector<Grid> out{g};
    while ((int)out.size() < MG_MAX_LEVELS) {
        const Grid &f = out.back();
        const int mx = std::max(f.nx, std::max(f.ny, f.nz));
        // at least two levels (the fine level always runs the global kernels)
        if (out.size() >= 2 && ((mx <= coarsest && f.ncell <= MG_COARSEST_MAX) || mx <= 1)) break;
        out.push_back(make_grid(f.dim, (f.nx + 1) / 2, (f.ny + 1) / 2, f.dim == 3 ? (f.nz + 1) / 2 : 1,
                                DEEP_MIN_COARSE));
    }
    return out;
}

static size_t face_count(const Grid &g, int d) {
    return (size_t)(g.nx + (d == 0)) * (g.ny + (d == 1)) * (g.dim == 3 ? g.nz + (d == 2) : 1);
}

size_t solver_device_bytes(const Grid &g, const gbp_params &p) {
    const size_t cells = (size_t)g.ncell;
    size_t bytes = 8 * cells * (5 /*operator+b*/ + 4 /*x r s z*/ + (p.warm_start ? 1 : 0));
    for (int d = 0; d < g.dim; ++d) bytes += 24 * face_count(g, d);  // face arrays
    if (p.solver == GBP_SOLVER_MGPCG) {
        bytes += 8 * cells;  // q
        const size_t s = p.precision == GBP_PRECISION_MIXED ? 4 : 8;
        std::vector<Grid> lv = mg_level_grids(g, coarsest_of(p));
        // level 0: inverse diagonal (+ operator copy and 5 vectors in FP32)
        bytes += s * cells * (p.precision == GBP_PRECISION_MIXED ? 14 : 1);  // mixed: + the operator's low floats
        for (size_t l = 1; l < lv.size(); ++l) bytes += s * (size_t)lv[l].ncell * 7;
        // tile classes (a value per tile; rounded up to whole allocations)
        // and the classification's sub-box partials
        for (size_t l = 0; l + 1 < lv.size(); ++l)
            bytes += s * (size_t)(((lv[l].nx + 63) / 64) * (long long)lv[l].nty * lv[l].ntz + lv[l + 1].ntiles) + 1024;
        if (lv.size() > 1) bytes += 24 * (size_t)((lv[0].nx + 63) / 64) * lv[0].nty * lv[0].nz + 1024;
    }
    return bytes;
}

template <class T> int Solver::alloc(T **p, size_t n) {
    void *d = nullptr;
    SOLVER_CUDA(cudaMalloc(&d, sizeof(T) * (n ? n : 1)));
    owned_.push_back(d);
    *p = static_cast<T *>(d);
    return GBP_OK;
}

// Tile-class arrays of every level that has a coarser one: one value per
// pair tile of the level and per cell tile of the coarser grid.
template <class T> int Solver::alloc_classes(MgHierarchy<T> &H) {
    for (int l = 0; l + 1 < H.nlevels; ++l) {
        MgLevel<T> &F = H.levels[l];
        const Grid &C = H.levels[l + 1].g;
        int rc = alloc(&F.tcp, (size_t)(((F.g.nx + 63) / 64) * (long long)F.g.nty * F.g.ntz));
        if (rc || (rc = alloc(&F.tcr, (size_t)C.ntiles))) return rc;
    }
    // the classification's sub-box partials (64 x 8 x 1 sub-boxes of level
    // 0 at most; 3 words each, 8-byte words in the FP64 hierarchy)
    if (H.nlevels > 1) {
        const Grid &F0 = H.levels[0].g;
        const size_t n = (size_t)((F0.nx + 63) / 64) * F0.nty * F0.nz;
        double *d = nullptr;
        if (int rc = alloc(&d, 3 * n)) return rc;
        H.class_parts = d;
        H.class_parts_bytes = 3 * n * sizeof(double);
    }
    return GBP_OK;
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
        for (int d = 0; d < 3; ++d) {
            const size_t nf = d < g.dim ? face_count(g, d) : 1;
            SOLVER_CUDA(cudaMalloc(&st_.faces.rho[d], 4 * nf));
            SOLVER_CUDA(cudaMalloc(&st_.faces.area[d], 4 * nf));
            SOLVER_CUDA(cudaMalloc(&st_.faces.w[d], 8 * nf));
            SOLVER_CUDA(cudaMalloc(&st_.faces.q[d], 8 * nf));
        }
        allocated_ = true;
    }
    if (p.warm_start && !have_prev_buf_) {
        SOLVER_CUDA(cudaMalloc(&st_.prev, bytes));
        SOLVER_CUDA(cudaMemset(st_.prev, 0, bytes));
        have_prev_buf_ = true;
        st_.have_prev = false;
    }
    if (p.solver == GBP_SOLVER_MGPCG) return prepare_mg(g, p);
    return GBP_OK;
}

int Solver::prepare_mg(const Grid &g, const gbp_params &p) {
    const int coarsest = coarsest_of(p);
    if ((mg64_ready_ || mg32_ready_) && coarsest != mg_coarsest_) {
        // a different depth: drop the hierarchies (kept buffers are freed with them)
        for (void *d : owned_) cudaFree(d);
        owned_.clear();
        mg64_ready_ = mg32_ready_ = false;
        st_.q = nullptr;
        st_.rf = st_.zf = st_.pf = st_.qf = st_.df = nullptr;
        if (graph_) {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
            graph_key_ = -1;
        }
    }
    mg_coarsest_ = coarsest;
    const size_t n = (size_t)g.ncell;
    if (!st_.q) {
        int rc = alloc(&st_.q, n);
        if (rc) return rc;
    }
    std::vector<Grid> lv = mg_level_grids(g, coarsest);
    if (lv.back().ncell > MG_COARSEST_MAX) return fail(GBP_ERR_INVALID_ARGUMENT, "multigrid: coarsest level too big");
    int rc = GBP_OK;
    if (p.precision == GBP_PRECISION_FP64 && !mg64_ready_) {
        MgHierarchy<double> &H = h64_;
        H.nlevels = (int)lv.size();
        H.fine_aliases_fp64 = true;
        double *inv;
        if ((rc = alloc(&inv, n))) return rc;
        H.levels[0] = MgLevel<double>{g, st_.diag, inv, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy, st_.r, st_.z};
        for (int l = 1; l < H.nlevels; ++l) {
            const size_t m = (size_t)lv[l].ncell;
            double *d, *iv, *x1, *y1, *z1, *b, *x;
            if ((rc = alloc(&d, m)) || (rc = alloc(&iv, m)) || (rc = alloc(&x1, m)) || (rc = alloc(&y1, m)) ||
                (rc = alloc(&z1, m)) || (rc = alloc(&b, m)) || (rc = alloc(&x, m)))
                return rc;
            H.levels[l] = MgLevel<double>{lv[l], d, iv, x1, y1, lv[l].dim == 3 ? z1 : y1, b, x};
        }
        if ((rc = alloc_classes(H))) return rc;
        mg_plan_tail(H);
        mg64_ready_ = true;
    }
    if (p.precision == GBP_PRECISION_MIXED && !mg32_ready_) {
        MgHierarchy<float> &H = h32_;
        H.nlevels = (int)lv.size();
        H.fine_aliases_fp64 = false;
        if ((rc = alloc(&st_.rf, n)) || (rc = alloc(&st_.zf, n)) || (rc = alloc(&st_.pf, n)) ||
            (rc = alloc(&st_.qf, n)) || (rc = alloc(&st_.df, n)))
            return rc;
        for (int l = 0; l < H.nlevels; ++l) {
            const size_t m = (size_t)lv[l].ncell;
            float *d, *iv, *x1, *y1, *z1, *b = nullptr, *x = nullptr;
            if ((rc = alloc(&d, m)) || (rc = alloc(&iv, m)) || (rc = alloc(&x1, m)) || (rc = alloc(&y1, m)) ||
                (rc = alloc(&z1, m)))
                return rc;
            if (l == 0) {
                b = st_.rf;
                x = st_.zf;
            } else if ((rc = alloc(&b, m)) || (rc = alloc(&x, m))) {
                return rc;
            }
            H.levels[l] = MgLevel<float>{lv[l], d, iv, x1, y1, lv[l].dim == 3 ? z1 : y1, b, x};
        }
        for (int q = 0; q < 4; ++q)
            if ((rc = alloc(&H.lo[q], n))) return rc;
        if ((rc = alloc_classes(H))) return rc;
        mg_plan_tail(H);
        mg32_ready_ = true;
    }
    return GBP_OK;
}

void Solver::release() {
    if (graph_) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        graph_key_ = -1;
    }
    double **bufs[] = {&st_.diag, &st_.cx, &st_.cy, &st_.cz, &st_.b, &st_.x, &st_.r, &st_.s, &st_.z, &st_.prev};
    for (double **b : bufs) {
        if (*b) cudaFree(*b);
        *b = nullptr;
    }
    for (void *d : owned_) cudaFree(d);
    owned_.clear();
    if (st_.sc) cudaFree(st_.sc);
    if (st_.pt) cudaFree(st_.pt);
    if (st_.host_sc) cudaFreeHost(st_.host_sc);
    for (int d = 0; d < 3; ++d) {
        if (st_.faces.w[d]) cudaFree(st_.faces.w[d]);
        if (st_.faces.q[d]) cudaFree(st_.faces.q[d]);
        if (st_.faces.rho[d]) cudaFree(st_.faces.rho[d]);
        if (st_.faces.area[d]) cudaFree(st_.faces.area[d]);
    }
    st_ = SolverState();
    allocated_ = false;
    have_prev_buf_ = false;
    mg64_ready_ = mg32_ready_ = false;
}

// Replays the cached graph until the device reports done.
int Solver::run_graph(const gbp_params &p, int chunk, cudaStream_t stream, long long *launches) {
    const long long max_chunks = (long long)p.max_iterations / chunk + 64;
    for (long long k = 0; k < max_chunks; ++k) {
        SOLVER_CUDA(cudaMemcpyAsync(st_.host_sc, st_.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
        SOLVER_CUDA(cudaStreamSynchronize(stream));
        if (st_.host_sc->done) return GBP_OK;
        SOLVER_CUDA(cudaGraphLaunch(graph_, stream));
        *launches += graph_nodes_;
    }
    SOLVER_CUDA(cudaMemcpyAsync(st_.host_sc, st_.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
    SOLVER_CUDA(cudaStreamSynchronize(stream));
    return GBP_OK;
}

int Solver::solve(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    *launches = 0;
    int rc = p.solver == GBP_SOLVER_MGPCG ? solve_mg(g, p, grid_blocks, stream, launches)
                                          : solve_cg(g, p, grid_blocks, stream, launches);
    if (rc) return rc;
    return complete(g, p, grid_blocks, stream, launches);
}

int Solver::complete(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    const bool warm = p.warm_start && st_.have_prev;
    // A mixed MGPCG solve that stopped on its refinement check has the
    // residual of its solution already (that check updates it, see
    // refine_update_pair); every other solve gets a separate FP64 pass.
    const bool have_true = p.solver == GBP_SOLVER_MGPCG && p.precision == GBP_PRECISION_MIXED &&
                           (st_.host_sc->status == 1 || st_.host_sc->status == 2);
    if (!have_true) {
        Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
        SOLVER_CUDA(launch_true_residual(g, A, st_.b, st_.x, warm ? st_.prev : nullptr, st_.sc, st_.pt, grid_blocks,
                                         stream));
        *launches += 1;
    }
    last_inner_total_ = st_.host_sc->iter;
    last_outer_ = p.precision == GBP_PRECISION_MIXED ? st_.host_sc->outer_iter : 1;
    last_precision_ = p.precision;
    const int status = st_.host_sc->status;
    if (status == 3) return GBP_ERR_NAN;
    if (status == 2 || !st_.host_sc->done) return GBP_ERR_NOT_CONVERGED;
    return GBP_OK;
}

int Solver::solve_cg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    const bool warm = p.warm_start && st_.have_prev;
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    SOLVER_CUDA(launch_cg_init(g, A, st_.b, warm ? st_.prev : nullptr, st_.x, st_.r, st_.s, st_.sc, st_.pt,
                               p.residual, p.max_iterations, grid_blocks, stream));
    *launches += 1;
    const int chunk = p.iterations_per_sync > 0 ? p.iterations_per_sync : 16;
    const long long key = ((long long)chunk << 20) | ((long long)grid_blocks << 4) | 0;
    if (!graph_ || graph_key_ != key) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        cudaGraph_t graph;
        SOLVER_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int it = 0; it < chunk && e == cudaSuccess; ++it)
            e = launch_cg_iteration(g, A, st_.x, st_.r, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream);
        cudaError_t e2 = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess)
            return fail(GBP_ERR_CUDA, std::string("capturing CG iterations: ") +
                                          cudaGetErrorString(e != cudaSuccess ? e : e2));
        e = cudaGraphInstantiate(&graph_, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(GBP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        graph_key_ = key;
        graph_nodes_ = 3LL * chunk;
    }
    return run_graph(p, chunk, stream, launches);
}

Level0Out Solver::level0_out(const gbp_params &p) const {
    Level0Out o{};
    if (p.solver != GBP_SOLVER_MGPCG) return o;
    if (p.precision == GBP_PRECISION_MIXED && mg32_ready_) {
        const MgLevel<float> &L = h32_.levels[0];
        o.diag = const_cast<float *>(L.diag);
        o.inv = const_cast<float *>(L.inv);
        o.cx = const_cast<float *>(L.cx);
        o.cy = const_cast<float *>(L.cy);
        o.cz = const_cast<float *>(L.cz);
        o.diag_lo = h32_.lo[0];
        o.cx_lo = h32_.lo[1];
        o.cy_lo = h32_.lo[2];
        o.cz_lo = h32_.lo[3];
    } else if (p.precision == GBP_PRECISION_FP64 && mg64_ready_) {
        o.inv64 = const_cast<double *>(h64_.levels[0].inv);
    }
    return o;
}

int Solver::setup_mg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    const bool level0 = level0_written_;
    level0_written_ = false;
    if (p.precision == GBP_PRECISION_MIXED) {
        SOLVER_CUDA(mg_setup<float>(g, A, h32_, level0, grid_blocks, stream));
        *launches += h32_.nlevels - (level0 ? 1 : 0);
    } else {
        SOLVER_CUDA(mg_setup<double>(g, A, h64_, level0, grid_blocks, stream));
        *launches += h64_.nlevels - (level0 ? 1 : 0);
    }
    return GBP_OK;
}

template <class T> void Solver::add_to_plan(BatchPlan<T> &plan, const gbp_params &p) const {
    const MgHierarchy<T> &H = *reinterpret_cast<const MgHierarchy<T> *>(
        sizeof(T) == 4 ? static_cast<const void *>(&h32_) : static_cast<const void *>(&h64_));
    const int s = plan.nscenes++;
    const bool warm = p.warm_start && st_.have_prev;
    const int G = H.tail;  // levels [0, G) run the global kernels; [G, L) the tail
    BScene<T> sc{};
    sc.g = H.levels[0].g;
    if (sizeof(T) == 4) {
        sc.x = reinterpret_cast<T *>(st_.df);
        sc.r = reinterpret_cast<T *>(st_.rf);
        sc.z = reinterpret_cast<T *>(st_.zf);
        sc.p = reinterpret_cast<T *>(st_.pf);
        sc.q = reinterpret_cast<T *>(st_.qf);
    } else {
        sc.x = reinterpret_cast<T *>(st_.x);
        sc.r = reinterpret_cast<T *>(st_.r);
        sc.z = reinterpret_cast<T *>(st_.z);
        sc.p = reinterpret_cast<T *>(st_.s);
        sc.q = reinterpret_cast<T *>(st_.q);
    }
    sc.A = Operator<double>{st_.diag, st_.cx, st_.cy, sc.g.dim == 3 ? st_.cz : st_.cy};
    if (sizeof(T) == 4)
        sc.lo = Operator<float>{h32_.lo[0], h32_.lo[1], h32_.lo[2], sc.g.dim == 3 ? h32_.lo[3] : h32_.lo[2]};
    sc.b = st_.b;
    sc.prev = warm ? st_.prev : nullptr;
    sc.x64 = st_.x;
    sc.r64 = st_.r;
    sc.sc = st_.sc;
    sc.levels = H.nlevels;
    sc.tail = G;
    plan.scenes.push_back(sc);
    if ((int)plan.pair.size() < G) {
        plan.pair.resize(G);
        plan.restrict_.resize(G);
        plan.n_pair.resize(G, 0);
        plan.n_restrict.resize(G, 0);
    }
    plan.max_global = std::max(plan.max_global, G);
    const int base = (int)plan.levels.size();
    for (int l = 0; l < G; ++l) {
        const MgLevel<T> &F = H.levels[l], &C = H.levels[l + 1];
        // 2-wide accesses need an even row length and 2-element alignment of
        // every array that moves in pairs (on level 0 also the scene's
        // vectors and FP64 operator and refinement arrays)
        auto al = [](const void *ptr, size_t bytes) { return ptr == nullptr || (uintptr_t)ptr % bytes == 0; };
        bool vec = F.g.nx % 2 == 0;
        for (const void *ptr : {(const void *)F.diag, (const void *)F.inv, (const void *)F.cx, (const void *)F.cy,
                                (const void *)F.cz, (const void *)F.b, (const void *)F.x})
            vec = vec && al(ptr, 2 * sizeof(T));
        if (l == 0) {
            for (const void *ptr : {(const void *)sc.x, (const void *)sc.r, (const void *)sc.z, (const void *)sc.p,
                                    (const void *)sc.q})
                vec = vec && al(ptr, 2 * sizeof(T));
            for (const void *ptr : {(const void *)sc.A.diag, (const void *)sc.A.cx, (const void *)sc.A.cy,
                                    (const void *)sc.A.cz, (const void *)sc.b, (const void *)sc.prev,
                                    (const void *)sc.x64, (const void *)sc.r64})
                vec = vec && al(ptr, 2 * sizeof(double));
            for (const void *ptr : {(const void *)sc.lo.diag, (const void *)sc.lo.cx, (const void *)sc.lo.cy,
                                    (const void *)sc.lo.cz})
                vec = vec && al(ptr, 2 * sizeof(float));
        }
        if (l == 0) plan.fine_ref.push_back((int)plan.levels.size());
        plan.levels.push_back(
            BLevel<T>{F.g, F.diag, F.inv, F.cx, F.cy, F.cz, F.b, F.x, C.x, C.b, C.g, s, vec ? 1 : 0, nullptr,
                      p.tile_classes ? F.tcp : nullptr, p.tile_classes ? F.tcr : nullptr});
        plan.scene_of.push_back(s);
        auto add = [&](std::vector<BSeg> &list, int &items, long long tiles, long long cells_per_tile) {
            const int m = (int)std::max(1LL, BITEM_CELLS / cells_per_tile);
            const int count = (int)((tiles + m - 1) / m);
            list.push_back(BSeg{base + l, items, count, m, (int)tiles});
            items += count;
        };
        add(plan.pair[l], plan.n_pair[l], pair_tiles(F.g), 64LL * TILE_Y * F.g.tz);
        // a restriction item's work is its 8x as many fine cells
        add(plan.restrict_[l], plan.n_restrict[l], cell_tiles(C.g), 8LL * TILE_X * TILE_Y * C.g.tz);
        if (l == 0) add(plan.fine_pairs, plan.n_fine_pairs, pair_tiles(F.g), 64LL * TILE_Y * F.g.tz);
    }
    BTail<T> tail{};
    tail.nt = H.nlevels - G;
    for (int l = G; l < H.nlevels; ++l) tail.lv[l - G] = H.levels[l];
    plan.tails.push_back(tail);
    plan.tail_bytes = std::max(plan.tail_bytes, H.tail_bytes);
}

template void Solver::add_to_plan<double>(BatchPlan<double> &, const gbp_params &) const;
template void Solver::add_to_plan<float>(BatchPlan<float> &, const gbp_params &) const;

int Solver::finish_batched(const gbp_params &p, cudaStream_t stream) {
    SOLVER_CUDA(cudaMemcpyAsync(st_.host_sc, st_.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
    SOLVER_CUDA(cudaStreamSynchronize(stream));
    return GBP_OK;
}

int Solver::solve_mg(const Grid &g, const gbp_params &p, int grid_blocks, cudaStream_t stream, long long *launches) {
    const bool mixed = p.precision == GBP_PRECISION_MIXED;
    const bool warm = p.warm_start && st_.have_prev;
    int rc = setup_mg(g, p, grid_blocks, stream, launches);
    if (rc) return rc;
    // a batch of one: the same kernels and reductions as a batched solve
    const long long key = (mixed ? 1 : 0) | (warm ? 2 : 0) | (p.tma_staging ? 4 : 0) | (p.tile_classes ? 0 : 8) |
                          ((long long)grid_blocks << 4) | ((long long)mg_coarsest_ << 24);
    if (runner_key_ != key) {
        if (mixed) {
            BatchPlan<float> plan;
            add_to_plan<float>(plan, p);
            rc = runner_.build<float>(plan, grid_blocks, p.tma_staging, stream);
        } else {
            BatchPlan<double> plan;
            add_to_plan<double>(plan, p);
            rc = runner_.build<double>(plan, grid_blocks, 0, stream);
        }
        if (rc) return fail(rc, runner_.error());
        runner_key_ = key;
    }
    rc = mixed ? runner_.solve<float>(p, stream, launches) : runner_.solve<double>(p, stream, launches);
    if (rc) return fail(rc, runner_.error());
    return finish_batched(p, stream);
}

namespace {
// Fine cells of level 0 by tile class, for the byte counts of the
// multigrid kernels: [0] over the pair tiles (tcp), [1] over the
// restriction tiles (tcr); classes mixed, uniform, empty. Without classes
// every cell counts as mixed.
template <class T> void class_cells(const MgHierarchy<T> &H, double out[2][3]) {
    for (int a = 0; a < 2; ++a) out[a][0] = out[a][1] = out[a][2] = 0.0;
    const MgLevel<T> &F = H.levels[0];
    const Grid &g = F.g;
    if (H.nlevels < 2 || !F.tcp || !F.tcr) {
        out[0][0] = out[1][0] = (double)g.ncell;
        return;
    }
    const Grid &C = H.levels[1].g;
    const long long ntx2 = (g.nx + 63) / 64, np = ntx2 * g.nty * g.ntz, nr = C.ntiles;
    std::vector<T> cp((size_t)np), cr((size_t)nr);
    if (cudaMemcpy(cp.data(), F.tcp, sizeof(T) * np, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cr.data(), F.tcr, sizeof(T) * nr, cudaMemcpyDeviceToHost) != cudaSuccess) {
        out[0][0] = out[1][0] = (double)g.ncell;
        return;
    }
    auto cls = [](T v) { return v == T(TILE_EMPTY) ? 2 : (v >= T(0) && sizeof(T) == 4 ? 1 : 0); };
    for (long long t = 0; t < np; ++t) {
        const long long tx = t % ntx2, r = t / ntx2, ty = r % g.nty, tk = r / g.nty;
        const double n = (double)std::min<long long>(64, g.nx - 64 * tx) * std::min<long long>(TILE_Y, g.ny - TILE_Y * ty) *
                         std::min<long long>(g.tz, g.nz - g.tz * tk);
        out[0][cls(cp[(size_t)t])] += n;
    }
    for (long long t = 0; t < nr; ++t) {
        const long long tx = t % C.ntx, r = t / C.ntx, ty = r % C.nty, tk = r / C.nty;
        const long long i0 = 2 * TILE_X * tx, j0 = 2 * TILE_Y * ty, k0 = g.dim == 3 ? 2LL * C.tz * tk : 0;
        const long long bz = g.dim == 3 ? 2LL * C.tz : 1;
        const double n = (double)std::max(0LL, std::min<long long>(2 * TILE_X, g.nx - i0)) *
                         std::max(0LL, std::min<long long>(2 * TILE_Y, g.ny - j0)) *
                         std::max(0LL, std::min<long long>(bz, g.nz - k0));
        out[1][cls(cr[(size_t)t])] += n;
    }
}
}  // namespace

int Solver::bench_kernel(const Grid &g, int which, int reps, int grid_blocks, cudaStream_t stream, float *ms,
                         double *bytes) {
    if (!allocated_) return fail(GBP_ERR_INVALID_ARGUMENT, "bench_kernel: scene has not been projected yet");
    // scalars that keep every launch running: never done, alpha = 0
    Scalars h;
    std::memset(&h, 0, sizeof(h));
    h.rho = 1.0;
    h.tol = -1.0;
    h.inner_tol = -1.0;
    h.max_iter = 1 << 30;
    h.inner_max = 1 << 30;
    h.fluid_exists = 1;
    SOLVER_CUDA(cudaMemcpyAsync(st_.sc, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
    Operator<double> A{st_.diag, st_.cx, st_.cy, g.dim == 3 ? st_.cz : st_.cy};
    const double cells = (double)g.ncell;
    const bool mixed = last_precision_ == GBP_PRECISION_MIXED;
    const double s = mixed ? 4.0 : 8.0;
    double per_cell = 0.0;
    std::function<cudaError_t()> launch;
    switch (which) {
    case GBP_KERNEL_CG_SPMV:
        per_cell = 48.0;
        launch = [&]() { return launch_cg_spmv(g, A, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream); };
        break;
    case GBP_KERNEL_CG_UPDATE:
        per_cell = 48.0;
        launch = [&]() { return launch_cg_update(g, st_.x, st_.r, st_.s, st_.z, st_.sc, st_.pt, grid_blocks, stream); };
        break;
    case GBP_KERNEL_CG_DIRECTION:
        per_cell = 24.0;
        launch = [&]() { return launch_cg_direction(g, st_.r, st_.s, st_.sc, grid_blocks, stream); };
        break;
    case GBP_KERNEL_MG_PRESMOOTH:
    case GBP_KERNEL_MG_RESTRICT:
    case GBP_KERNEL_MG_POST_BLACK:
    case GBP_KERNEL_MG_RED_DOT:
    case GBP_KERNEL_PCG_DIRECTION:
    case GBP_KERNEL_PCG_SPMV:
    case GBP_KERNEL_PCG_UPDATE: {
        if (runner_key_ < 0) return fail(GBP_ERR_INVALID_ARGUMENT, "bench_kernel: no multigrid solve yet");
        static const int map[8] = {0, -1, 1, 2, 3, 4, 5, 6};
        // compulsory bytes per fine cell in units of the word size, for
        // tiles of mixed couplings / uniform couplings (no coupling loads;
        // FP32 only) / no unknown (zeros written or nothing)
        static const double pc[8][3] = {{6.0, 3.0, 1.0},     {7.0, 4.0, 0.0},   {6.125, 3.125, 0.125},
                                        {7.125, 4.125, 0.0}, {7.0, 4.0, 0.0},   {3.0, 3.0, 0.0},
                                        {6.0, 3.0, 0.0},     {6.0, 6.0, 0.0}};
        const int k = which - GBP_KERNEL_MG_PRESMOOTH;
        double cc[2][3];
        if (mixed) class_cells(h32_, cc);
        else class_cells(h64_, cc);
        const int a = which == GBP_KERNEL_MG_RESTRICT ? 1 : 0;
        *bytes = s * (pc[k][0] * cc[a][0] + pc[k][1] * cc[a][1] + pc[k][2] * cc[a][2]);
        const int rk = map[k];
        int rc = mixed ? runner_.bench<float>(rk, reps, stream, ms) : runner_.bench<double>(rk, reps, stream, ms);
        if (rc) return fail(rc, runner_.error());
        return GBP_OK;
    }
    default: return fail(GBP_ERR_INVALID_ARGUMENT, "bench_kernel: unknown kernel");
    }
    *bytes = per_cell * cells;
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
