// gbp_api.cpp -- the C ABI of libgbp (include/gbp.h): contexts, scenes and
// the projection call that sequences the device kernels.
//
// One projection (replacing macpressuresolver3::project,
// src/projection/macpressuresolver3.cpp:50-272) is, on the scene's stream:
//   assemble   face fractions, labels, operator, right-hand side
//   solve      CG or MGPCG (FP64 or mixed), iterations captured in a CUDA
//              graph and replayed in chunks; the host reads the device's
//              stop flag between chunks
//   pressure   float pressure (+ warm-start copy)
//   velocity   pressure-gradient update of every face
#include "gbp.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "advect.h"
#include "brick_kernels.h"
#include "csr_solver.h"
#include "gbp_kernels.h"
#include "gbp_solver.h"

using namespace gbp;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define GBP_CUDA(call)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            return fail(e_ == cudaErrorMemoryAllocation ? GBP_ERR_OUT_OF_MEMORY : GBP_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
        }                                                                                              \
    } while (0)

}  // namespace

namespace gbp {
// Message for gbp_strerror from code outside this file.
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace gbp

struct gbp_ctx {
    int device = 0;
    int sm_count = 0;
    int grid_blocks = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // the host-array call's second stream: the pressure's copy back runs
    // there while the velocity update runs on the first
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_pressure = nullptr;
    long long launches = 0;
    CsrWork csr;  // device arrays of gbp_csr_cg
    AdvectWork adv;  // device scratch of gbp_advect3*
    // staging of the host-array advection call, grown on demand
    float *adv_stage = nullptr;
    long long adv_stage_floats = 0;
};

struct gbp_scene {
    gbp_ctx *ctx = nullptr;
    Grid g{};
    double dx = 0.0;
    // staging for the host-array call
    float *d_solid = nullptr, *d_fluid = nullptr, *d_u = nullptr, *d_v = nullptr, *d_w = nullptr,
          *d_p = nullptr;
    // active sets of the last gbp_project_active call (unknown cells, kept faces)
    unsigned char *d_unknown = nullptr, *d_on[3] = {nullptr, nullptr, nullptr};
    // volume correction state (macpressuresolver3.cpp:316-318)
    double current_volume = 0.0, target_volume = 0.0, y_prev = 0.0;
    Solver *solver = nullptr;
    // device copies of gbp_project_bricks' brick lists (5 in, 4 out: slots
    // or slot-to-brick maps, values, flags), grown on demand
    struct DevBuf {
        void *p = nullptr;
        size_t cap = 0;
    };
    DevBuf brick_buf[9][3];
};

extern "C" {

void gbp_params_default(gbp_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->residual = 1e-4;
    p->max_iterations = 30000;
    p->warm_start = 0;
    p->eps_fluid = 1e-2;
    p->eps_solid = 1e-2;
    p->second_order_fluid = 1;
    p->second_order_solid = 1;
    p->gain = 1.0;
    p->solver = GBP_SOLVER_CG;
    p->precision = GBP_PRECISION_FP64;
    p->mg_smooth = 1;
    p->mg_coarsest = 7;  // coarsest level 4^3 for power-of-two grids, 6^3 / 5^3 / ... for the others
    p->inner_tolerance = 1e-3;
    p->iterations_per_sync = 16;
    p->surface_tension = 0.0;
    p->tma_staging = 0;
    p->tile_classes = 1;
}

const char *gbp_strerror(int status) {
    switch (status) {
    case GBP_OK: return "ok";
    case GBP_ERR_INVALID_ARGUMENT: return g_last_error.empty() ? "invalid argument" : g_last_error.c_str();
    case GBP_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case GBP_ERR_OUT_OF_MEMORY: return g_last_error.empty() ? "out of device memory" : g_last_error.c_str();
    case GBP_ERR_NOT_CONVERGED: return "linear solve stopped at max_iterations";
    case GBP_ERR_NAN: return "linear solve broke down (NaN or zero curvature)";
    case GBP_ERR_NO_DEVICE: return g_last_error.empty() ? "no CUDA device" : g_last_error.c_str();
    case GBP_ERR_BUDGET: return "device memory budget exceeded";
    case GBP_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

int gbp_create(int device, gbp_ctx **out) {
    if (!out) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_create: out is NULL");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
        cudaGetLastError();
        return fail(GBP_ERR_NO_DEVICE, "gbp_create: CUDA device " + std::to_string(device) + " not available");
    }
    GBP_CUDA(cudaSetDevice(device));
    auto *c = new (std::nothrow) gbp_ctx();
    if (!c) return fail(GBP_ERR_OUT_OF_MEMORY, "gbp_create: host allocation");
    c->device = device;
    cudaDeviceProp prop;
    GBP_CUDA(cudaGetDeviceProperties(&prop, device));
    c->sm_count = prop.multiProcessorCount;
    c->grid_blocks = c->sm_count * 6;
    if (c->grid_blocks > MAX_GRID) c->grid_blocks = MAX_GRID;
    GBP_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    GBP_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (auto &e : c->ev) GBP_CUDA(cudaEventCreate(&e));
    GBP_CUDA(cudaEventCreateWithFlags(&c->ev_pressure, cudaEventDisableTiming));
    *out = c;
    return GBP_OK;
}

void gbp_destroy(gbp_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    csr_release(c->csr);
    advect_release(c->adv);
    if (c->adv_stage) cudaFree(c->adv_stage);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->ev_pressure) cudaEventDestroy(c->ev_pressure);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

long long gbp_launch_count(gbp_ctx *c) { return c ? c->launches : 0; }

int gbp_csr_cg(gbp_ctx *c, long long n, const long long *rowstart, const long long *cols, const double *vals,
               const double *b, double *x, double residual, int max_iterations, gbp_csr_stats *stats) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!c || n < 0 || (n > 0 && (!rowstart || !b || !x)))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: bad argument");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) {
        if (stats) stats->converged = 1;
        return GBP_OK;
    }
    // the structure is checked on the host: no index reaches the device
    // unless it lies inside the arrays
    if (rowstart[0] != 0) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: rowstart[0] != 0");
    for (long long r = 0; r < n; ++r)
        if (rowstart[r + 1] < rowstart[r]) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: rowstart decreases");
    const long long nnz = rowstart[n];
    if (nnz > 0 && (!cols || !vals)) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: NULL cols or vals");
    if (n >= (1LL << 31) || nnz > (1LL << 40)) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: too large");
    // checked and narrowed to the device's 32-bit column indices in one pass
    std::vector<int> cols32((size_t)(nnz > 0 ? nnz : 1));
    for (long long e = 0; e < nnz; ++e) {
        if (cols[e] < 0 || cols[e] >= n) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_csr_cg: column out of range");
        cols32[(size_t)e] = (int)cols[e];
    }
    GBP_CUDA(cudaSetDevice(c->device));
    GBP_CUDA(csr_reserve(c->csr, n, nnz > 0 ? nnz : 1));
    CsrWork &w = c->csr;
    cudaStream_t st = c->stream;
    GBP_CUDA(cudaMemcpyAsync(w.rowstart, rowstart, sizeof(long long) * (size_t)(n + 1), cudaMemcpyHostToDevice, st));
    if (nnz > 0) {
        GBP_CUDA(cudaMemcpyAsync(w.cols, cols32.data(), sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, st));
        GBP_CUDA(cudaMemcpyAsync(w.vals, vals, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
    }
    GBP_CUDA(cudaMemcpyAsync(w.b, b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaEventRecord(c->ev[0], st));
    long long launches = 0;
    GBP_CUDA(csr_cg_run(w, n, residual, max_iterations, c->grid_blocks, st, &launches));
    GBP_CUDA(cudaEventRecord(c->ev[1], st));
    GBP_CUDA(cudaMemcpyAsync(x, w.x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launches;
    const Scalars &h = *w.host_sc;
    if (stats) {
        stats->iterations = h.iter;
        stats->converged = h.status == 1;
        stats->reresid = h.res0 > 0.0 ? h.res / h.res0 : 0.0;  // pcg_solver.h:284, :294
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        stats->ms_solve = ms;
        stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (h.status == 3) return fail(GBP_ERR_NAN, "gbp_csr_cg: breakdown (NaN or zero curvature)");
    if (h.status != 1) return fail(GBP_ERR_NOT_CONVERGED, "gbp_csr_cg: not converged");
    return GBP_OK;
}

size_t gbp_scene_device_bytes(int dim, int nx, int ny, int nz, const gbp_params *params) {
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    Grid g = make_grid(dim, nx, ny, nz);
    size_t cells = (size_t)g.ncell;
    size_t nodes = (size_t)(nx + 1) * (ny + 1) * (dim == 3 ? nz + 1 : 1);
    size_t faces = (size_t)(nx + 1) * ny * g.nz + (size_t)nx * (ny + 1) * g.nz + (dim == 3 ? (size_t)nx * ny * (nz + 1) : 0);
    size_t staging = 4 * (nodes + cells + faces + cells);
    return staging + solver_device_bytes(g, p) + sizeof(Scalars) + sizeof(Partials);
}

int gbp_scene_create(gbp_ctx *c, int dim, int nx, int ny, int nz, double dx, gbp_scene **out) {
    if (!c || !out) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_scene_create: NULL argument");
    *out = nullptr;
    if ((dim != 2 && dim != 3) || nx < 1 || ny < 1 || (dim == 3 && nz < 1) || !(dx > 0.0))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_scene_create: bad shape or dx");
    if ((long long)nx * ny * (dim == 3 ? nz : 1) > (1LL << 31))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_scene_create: more than 2^31 cells");
    auto *s = new (std::nothrow) gbp_scene();
    if (!s) return fail(GBP_ERR_OUT_OF_MEMORY, "gbp_scene_create: host allocation");
    s->ctx = c;
    s->g = make_grid(dim, nx, ny, nz);
    s->dx = dx;
    s->solver = new (std::nothrow) Solver();
    if (!s->solver) {
        delete s;
        return fail(GBP_ERR_OUT_OF_MEMORY, "gbp_scene_create: host allocation");
    }
    *out = s;
    return GBP_OK;
}

void gbp_scene_destroy(gbp_scene *s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    for (float *p : {s->d_solid, s->d_fluid, s->d_u, s->d_v, s->d_w, s->d_p})
        if (p) cudaFree(p);
    for (unsigned char *m : {s->d_unknown, s->d_on[0], s->d_on[1], s->d_on[2]})
        if (m) cudaFree(m);
    for (auto &row : s->brick_buf)
        for (auto &b : row)
            if (b.p) cudaFree(b.p);
    if (s->solver) {
        s->solver->release();
        delete s->solver;
    }
    delete s;
}

int gbp_scene_set_target_volume(gbp_scene *s, double current_volume, double target_volume) {
    if (!s) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_scene_set_target_volume: NULL scene");
    s->current_volume = current_volume;
    s->target_volume = target_volume;
    return GBP_OK;
}

}  // extern "C"

namespace {

size_t n_nodes(const Grid &g) { return (size_t)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1); }
size_t n_face(const Grid &g, int d) {
    return (size_t)(g.nx + (d == 0)) * (g.ny + (d == 1)) * (g.dim == 3 ? g.nz + (d == 2) : 1);
}

int ensure_staging(gbp_scene *s) {
    const Grid &g = s->g;
    if (!s->d_solid) GBP_CUDA(cudaMalloc(&s->d_solid, 4 * n_nodes(g)));
    if (!s->d_fluid) GBP_CUDA(cudaMalloc(&s->d_fluid, 4 * (size_t)g.ncell));
    if (!s->d_u) GBP_CUDA(cudaMalloc(&s->d_u, 4 * n_face(g, 0)));
    if (!s->d_v) GBP_CUDA(cudaMalloc(&s->d_v, 4 * n_face(g, 1)));
    if (g.dim == 3 && !s->d_w) GBP_CUDA(cudaMalloc(&s->d_w, 4 * n_face(g, 2)));
    if (!s->d_p) GBP_CUDA(cudaMalloc(&s->d_p, 4 * (size_t)g.ncell));
    return GBP_OK;
}

// Volume-correction constant (macpressuresolver3.cpp:204-217); advances the
// controller's integral state once per projection.
// Face fractions, operator and right-hand side of one scene (the face pass
// and the cell pass), and level 0 of the solver's hierarchy o names.
cudaError_t launch_setup(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                         const float *fluid, const float *u, const float *v, const float *w, SolverState &st,
                         Level0Out o, int grid_blocks, cudaStream_t stream, long long *launches) {
    cudaError_t e = launch_faces(g, dt, dx, sp, solid, fluid, u, v, w, st.faces, grid_blocks, stream);
    if (e == cudaSuccess)
        e = launch_assemble_faces(g, dt, dx, sp, fluid, u, v, w, st.faces, st.diag, st.cx, st.cy, st.cz, st.b, o,
                                  st.sc, grid_blocks, stream);
    *launches += 2;
    return e;
}

// launch_setup for a solve: level 0 of the solver's hierarchy comes with it
int setup_for_solve(gbp_scene *s, const Grid &g, double dt, const SetupParams &sp, const gbp_params &p,
                    const float *solid, const float *fluid, const float *u, const float *v, const float *w,
                    int grid_blocks, cudaStream_t stream, long long *launches) {
    const Level0Out o = s->solver->level0_out(p);
    GBP_CUDA(launch_setup(g, dt, s->dx, sp, solid, fluid, u, v, w, s->solver->state(), o, grid_blocks, stream,
                          launches));
    if (o.diag || o.inv64) s->solver->level0_written();
    return GBP_OK;
}

double volume_correction(gbp_scene *s, double dt, const gbp_params &p) {
    if (!(p.gain && s->target_volume)) return 0.0;
    double x = (s->current_volume - s->target_volume) / s->target_volume;
    double y = s->y_prev + x * dt;
    s->y_prev = y;
    double kp = p.gain * 2.3 / (25.0 * 0.01);
    double ki = kp * kp / 16.0;
    return -(kp * x + ki * y) / (x + 1.0);
}

}  // namespace

namespace gbp {
// Parameter checks shared by every projection entry point.
int validate_params(const gbp_params &p) {
    if (!(p.residual >= 0.0) || p.max_iterations < 0 || !(p.eps_fluid >= 0.0) || !(p.eps_solid >= 0.0))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_params: negative residual, eps or max_iterations");
    if (p.solver != GBP_SOLVER_CG && p.solver != GBP_SOLVER_MGPCG)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_params: unknown solver");
    if (p.precision != GBP_PRECISION_FP64 && p.precision != GBP_PRECISION_MIXED)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_params: unknown precision");
    if (p.precision == GBP_PRECISION_MIXED && p.solver != GBP_SOLVER_MGPCG)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_params: mixed precision needs the MGPCG solver");
    return GBP_OK;
}
}  // namespace gbp

namespace {

int ensure_active_sets(gbp_scene *s) {
    const Grid &g = s->g;
    if (!s->d_unknown) GBP_CUDA(cudaMalloc(&s->d_unknown, (size_t)g.ncell));
    for (int d = 0; d < g.dim; ++d)
        if (!s->d_on[d]) GBP_CUDA(cudaMalloc(&s->d_on[d], n_face(g, d)));
    return GBP_OK;
}

// pressure_host (host-array calls): the pressure is copied there on the
// context's copy stream while the velocity update (which only reads it)
// runs on `stream`; both streams are synchronised before the return.
int project_device(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                   const gbp_params &p, float *pressure, gbp_stats *stats, cudaStream_t stream,
                   bool active_sets = false, float *pressure_host = nullptr) {
    gbp_ctx *c = s->ctx;
    const Grid &g = s->g;
    int rc = gbp::validate_params(p);
    if (rc) return rc;
    if (!solid || !fluid || !u || !v || (g.dim == 3 && !w) || !pressure)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project: NULL array");
    GBP_CUDA(cudaSetDevice(c->device));
    rc = s->solver->prepare(g, p);
    if (rc) return fail(rc, s->solver->error());
    SolverState &st = s->solver->state();

    SetupParams sp{p.eps_solid, p.eps_fluid, p.second_order_solid, p.second_order_fluid, 0.0};
    sp.rhs_correct = volume_correction(s, dt, p);

    GBP_CUDA(cudaEventRecord(c->ev[0], stream));
    GBP_CUDA(cudaMemsetAsync(st.sc, 0, sizeof(Scalars), stream));
    if (p.surface_tension != 0.0) {
        GBP_CUDA(launch_surface_tension(g, dt, s->dx, sp, p.surface_tension, fluid, u, v, w, c->grid_blocks, stream));
        c->launches += 1;
    }
    rc = setup_for_solve(s, g, dt, sp, p, solid, fluid, u, v, w, c->grid_blocks, stream, &c->launches);
    if (rc) return rc;
    GBP_CUDA(cudaEventRecord(c->ev[1], stream));

    long long launched = 0;
    rc = s->solver->solve(g, p, c->grid_blocks, stream, &launched);
    c->launches += launched;
    if (rc != GBP_OK && rc != GBP_ERR_NOT_CONVERGED && rc != GBP_ERR_NAN) return fail(rc, s->solver->error());
    int solve_status = rc;
    GBP_CUDA(cudaEventRecord(c->ev[2], stream));

    GBP_CUDA(launch_pressure(g, st.diag, st.x, p.warm_start && st.have_prev ? st.prev : nullptr, pressure,
                             p.warm_start ? st.prev : nullptr, c->grid_blocks, stream));
    if (pressure_host) GBP_CUDA(cudaEventRecord(c->ev_pressure, stream));
    if (active_sets) {
        GBP_CUDA(launch_active_sets(g, st.faces, fluid, u, v, w, st.diag, s->d_unknown, s->d_on[0], s->d_on[1],
                                    s->d_on[2], st.sc, c->grid_blocks, stream));
        c->launches += 1;
    }
    GBP_CUDA(launch_velocity_faces(g, dt, s->dx, sp, pressure, st.faces, u, v, w, st.sc, c->grid_blocks, stream));
    c->launches += 2;
    if (p.warm_start) st.have_prev = true;
    GBP_CUDA(cudaEventRecord(c->ev[3], stream));
    if (pressure_host) {
        // enqueued after the velocity update, so that the host, which a copy
        // into pageable memory holds until it is done, has launched it first
        GBP_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_pressure, 0));
        GBP_CUDA(cudaMemcpyAsync(pressure_host, pressure, 4 * (size_t)g.ncell, cudaMemcpyDeviceToHost,
                                 c->copy_stream));
        GBP_CUDA(cudaStreamSynchronize(c->copy_stream));
    }
    GBP_CUDA(cudaStreamSynchronize(stream));

    if (stats) {
        Scalars h;
        GBP_CUDA(cudaMemcpy(&h, st.sc, sizeof(Scalars), cudaMemcpyDeviceToHost));
        s->solver->fill_stats(h, stats);
        stats->unknowns = (long long)h.unknowns;
        stats->tma_staged = p.solver == GBP_SOLVER_MGPCG && s->solver->staged() ? 1 : 0;
        cudaEventElapsedTime(&stats->ms_assemble, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&stats->ms_solve, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&stats->ms_update, c->ev[2], c->ev[3]);
    }
    return solve_status;
}

// The host-array calls: inputs copied to the scene's device staging, the
// projection, results copied back; with unknown != NULL also the active sets.
int project_host(const char *who, gbp_scene *s, double dt, const float *solid, const float *fluid, float *u,
                 float *v, float *w, const gbp_params *params, float *pressure, gbp_stats *stats,
                 unsigned char *unknown, unsigned char *u_active, unsigned char *v_active,
                 unsigned char *w_active) {
    if (!s) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL scene");
    auto t0 = std::chrono::steady_clock::now();
    const Grid &g = s->g;
    if (!solid || !fluid || !u || !v || (g.dim == 3 && !w))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL array");
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    GBP_CUDA(cudaSetDevice(s->ctx->device));
    int rc = ensure_staging(s);
    if (rc) return rc;
    const bool sets = unknown != nullptr;
    if (sets && (rc = ensure_active_sets(s))) return rc;
    cudaStream_t st = s->ctx->stream;
    GBP_CUDA(cudaMemcpyAsync(s->d_solid, solid, 4 * n_nodes(g), cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(s->d_fluid, fluid, 4 * (size_t)g.ncell, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(s->d_u, u, 4 * n_face(g, 0), cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(s->d_v, v, 4 * n_face(g, 1), cudaMemcpyHostToDevice, st));
    if (g.dim == 3) GBP_CUDA(cudaMemcpyAsync(s->d_w, w, 4 * n_face(g, 2), cudaMemcpyHostToDevice, st));
    rc = project_device(s, dt, s->d_solid, s->d_fluid, s->d_u, s->d_v, s->d_w, p, s->d_p, stats, st, sets, pressure);
    if (rc != GBP_OK && rc != GBP_ERR_NOT_CONVERGED && rc != GBP_ERR_NAN) return rc;
    GBP_CUDA(cudaMemcpyAsync(u, s->d_u, 4 * n_face(g, 0), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaMemcpyAsync(v, s->d_v, 4 * n_face(g, 1), cudaMemcpyDeviceToHost, st));
    if (g.dim == 3) GBP_CUDA(cudaMemcpyAsync(w, s->d_w, 4 * n_face(g, 2), cudaMemcpyDeviceToHost, st));
    if (sets) {
        unsigned char *out[3] = {u_active, v_active, w_active};
        GBP_CUDA(cudaMemcpyAsync(unknown, s->d_unknown, (size_t)g.ncell, cudaMemcpyDeviceToHost, st));
        for (int d = 0; d < g.dim; ++d)
            GBP_CUDA(cudaMemcpyAsync(out[d], s->d_on[d], n_face(g, d), cudaMemcpyDeviceToHost, st));
    }
    GBP_CUDA(cudaStreamSynchronize(st));
    if (stats)
        stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

}  // namespace

extern "C" {

int gbp_project_device(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v,
                       float *w, const gbp_params *params, float *pressure, gbp_stats *stats, void *stream) {
    if (!s) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device: NULL scene");
    auto t0 = std::chrono::steady_clock::now();
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    if (!stream) {
        // The caller's work sits on the legacy default stream, which does not
        // order against the context's non-blocking stream: wait for it.
        GBP_CUDA(cudaSetDevice(s->ctx->device));
        GBP_CUDA(cudaEventRecord(s->ctx->ev[0], cudaStreamLegacy));
        GBP_CUDA(cudaStreamWaitEvent(st, s->ctx->ev[0], 0));
    }
    int rc = GBP_OK;
    if (!pressure) {
        rc = ensure_staging(s);
        if (rc) return rc;
        pressure = s->d_p;
    }
    rc = project_device(s, dt, solid, fluid, u, v, w, p, pressure, stats, st);
    if (stats)
        stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int gbp_project(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                const gbp_params *params, float *pressure, gbp_stats *stats) {
    return project_host("gbp_project", s, dt, solid, fluid, u, v, w, params, pressure, stats, nullptr, nullptr,
                        nullptr, nullptr);
}

int gbp_project_active(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                       const gbp_params *params, float *pressure, gbp_stats *stats, unsigned char *unknown,
                       unsigned char *u_active, unsigned char *v_active, unsigned char *w_active) {
    if (s && (!unknown || !u_active || !v_active || (s->g.dim == 3 && !w_active)))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_active: NULL active-set array");
    return project_host("gbp_project_active", s, dt, solid, fluid, u, v, w, params, pressure, stats, unknown,
                        u_active, v_active, w_active);
}

}  // extern "C"

// ---- sparse arrays in bricks -------------------------------------------------------

namespace {

size_t brick_count(int nx, int ny, int nz) {
    return (size_t)((nx + 7) / 8) * (size_t)((ny + 7) / 8) * (size_t)((nz + 7) / 8);
}

int grow(gbp_scene::DevBuf &b, size_t bytes) {
    if (bytes <= b.cap) return GBP_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    GBP_CUDA(cudaMalloc(&b.p, bytes));
    b.cap = bytes;
    return GBP_OK;
}

// Every slot is a brick kind or a listed slot, so no expansion reads
// outside `values`.
int check_bricks(const char *who, const char *what, const gbp_bricks *b, size_t nb) {
    if (!b || !b->slot || b->count < 0 || (b->count > 0 && !b->values))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": bad " + what + " bricks");
    for (size_t q = 0; q < nb; ++q) {
        const int sl = b->slot[q];
        if (sl < GBP_BRICK_FILL || sl >= b->count)
            return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": " + what + " brick " + std::to_string(q) +
                                                      " has slot " + std::to_string(sl));
    }
    return GBP_OK;
}

// brick_of[s] for the output slots; each slot 0 .. count-1 names exactly
// one brick.
int output_map(const char *who, const char *what, const gbp_bricks_out *o, size_t nb, std::vector<long long> &brick_of) {
    if (!o->slot || o->count < 0 || (o->count > 0 && !o->values))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": bad " + what + " output bricks");
    brick_of.assign((size_t)o->count, -1);
    for (size_t q = 0; q < nb; ++q) {
        const int sl = o->slot[q];
        if (sl < 0) continue;
        if (sl >= o->count || brick_of[(size_t)sl] >= 0)
            return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": " + what + " output slot " +
                                                      std::to_string(sl) + " out of range or repeated");
        brick_of[(size_t)sl] = (long long)q;
    }
    for (long long b : brick_of)
        if (b < 0) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": " + what + " output slot unused");
    return GBP_OK;
}

// Uploads one brick list into buf[0] (slots) and buf[1] (values) and
// expands it into dense.
int expand_on(gbp_ctx *c, int nx, int ny, int nz, const gbp_bricks *in, gbp_scene::DevBuf *buf, float *dense,
              cudaStream_t st) {
    const size_t nb = brick_count(nx, ny, nz);
    int rc;
    if ((rc = grow(buf[0], 4 * nb)) || (rc = grow(buf[1], 4 * (size_t)in->count * GBP_BRICK_CELLS))) return rc;
    GBP_CUDA(cudaMemcpyAsync(buf[0].p, in->slot, 4 * nb, cudaMemcpyHostToDevice, st));
    if (in->count)
        GBP_CUDA(cudaMemcpyAsync(buf[1].p, in->values, 4 * (size_t)in->count * GBP_BRICK_CELLS,
                                 cudaMemcpyHostToDevice, st));
    GBP_CUDA(launch_brick_expand(nx, ny, nz, in->background, in->fill, static_cast<const int *>(buf[0].p),
                                 static_cast<const float *>(buf[1].p), dense, c->grid_blocks, st));
    c->launches += 1;
    return GBP_OK;
}

}  // namespace

extern "C" {

int gbp_bricks_expand(gbp_ctx *c, int nx, int ny, int nz, const gbp_bricks *in, float *dense, void *stream) {
    const char *who = "gbp_bricks_expand";
    if (!c || !dense || nx < 1 || ny < 1 || nz < 1) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": bad arguments");
    int rc = check_bricks(who, "input", in, brick_count(nx, ny, nz));
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    gbp_scene::DevBuf buf[2];
    rc = expand_on(c, nx, ny, nz, in, buf, dense, st);
    cudaError_t e = cudaStreamSynchronize(st);
    for (auto &b : buf)
        if (b.p) cudaFree(b.p);
    if (rc) return rc;
    GBP_CUDA(e);
    return GBP_OK;
}

int gbp_project_bricks(gbp_scene *s, double dt, const gbp_bricks *solid, const gbp_bricks *fluid, const gbp_bricks *u,
                       const gbp_bricks *v, const gbp_bricks *w, const gbp_params *params, gbp_bricks_out *pressure,
                       gbp_bricks_out *u_out, gbp_bricks_out *v_out, gbp_bricks_out *w_out, gbp_stats *stats) {
    const char *who = "gbp_project_bricks";
    if (!s) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL scene");
    auto t0 = std::chrono::steady_clock::now();
    const Grid &g = s->g;
    if (g.dim != 3) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": 3D scenes only");
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    // extents of solid (nodes), fluid (cells), u, v, w (faces)
    const int ext[5][3] = {{nx + 1, ny + 1, nz + 1}, {nx, ny, nz}, {nx + 1, ny, nz}, {nx, ny + 1, nz}, {nx, ny, nz + 1}};
    const gbp_bricks *in[5] = {solid, fluid, u, v, w};
    const char *names[5] = {"solid", "fluid", "u", "v", "w"};
    int rc;
    for (int a = 0; a < 5; ++a)
        if ((rc = check_bricks(who, names[a], in[a], brick_count(ext[a][0], ext[a][1], ext[a][2])))) return rc;
    gbp_bricks_out *outs[4] = {pressure, u_out, v_out, w_out};
    const int oext[4] = {1, 2, 3, 4};  // extents of the outputs: fluid's, u's, v's, w's
    std::vector<long long> brick_of[4];
    bool sets = false;
    for (int o = 0; o < 4; ++o) {
        if (!outs[o]) continue;
        const int *e = ext[oext[o]];
        if ((rc = output_map(who, names[oext[o]], outs[o], brick_count(e[0], e[1], e[2]), brick_of[o]))) return rc;
        sets = sets || outs[o]->active;
    }
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    GBP_CUDA(cudaSetDevice(s->ctx->device));
    if ((rc = ensure_staging(s))) return rc;
    if (sets && (rc = ensure_active_sets(s))) return rc;
    cudaStream_t st = s->ctx->stream;
    float *dense[5] = {s->d_solid, s->d_fluid, s->d_u, s->d_v, s->d_w};
    for (int a = 0; a < 5; ++a)
        if ((rc = expand_on(s->ctx, ext[a][0], ext[a][1], ext[a][2], in[a], s->brick_buf[a], dense[a], st))) return rc;
    rc = project_device(s, dt, s->d_solid, s->d_fluid, s->d_u, s->d_v, s->d_w, p, s->d_p, stats, st, sets);
    if (rc != GBP_OK && rc != GBP_ERR_NOT_CONVERGED && rc != GBP_ERR_NAN) return rc;
    const float *src[4] = {s->d_p, s->d_u, s->d_v, s->d_w};
    const unsigned char *flags[4] = {s->d_unknown, s->d_on[0], s->d_on[1], s->d_on[2]};
    for (int o = 0; o < 4; ++o) {
        gbp_bricks_out *out = outs[o];
        if (!out || out->count == 0) continue;
        gbp_scene::DevBuf *buf = s->brick_buf[5 + o];
        const size_t cells = (size_t)out->count * GBP_BRICK_CELLS;
        int r2;
        if ((r2 = grow(buf[0], 8 * (size_t)out->count)) || (r2 = grow(buf[1], 4 * cells)) ||
            (out->active && (r2 = grow(buf[2], cells))))
            return r2;
        GBP_CUDA(cudaMemcpyAsync(buf[0].p, brick_of[o].data(), 8 * (size_t)out->count, cudaMemcpyHostToDevice, st));
        const int *e = ext[oext[o]];
        GBP_CUDA(launch_brick_gather(e[0], e[1], e[2], static_cast<const long long *>(buf[0].p), out->count, src[o],
                                     out->active ? flags[o] : nullptr, static_cast<float *>(buf[1].p),
                                     out->active ? static_cast<unsigned char *>(buf[2].p) : nullptr,
                                     s->ctx->grid_blocks, st));
        s->ctx->launches += 1;
        GBP_CUDA(cudaMemcpyAsync(out->values, buf[1].p, 4 * cells, cudaMemcpyDeviceToHost, st));
        if (out->active) GBP_CUDA(cudaMemcpyAsync(out->active, buf[2].p, cells, cudaMemcpyDeviceToHost, st));
    }
    GBP_CUDA(cudaStreamSynchronize(st));
    if (stats)
        stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

}  // extern "C"

struct gbp_batch {
    gbp_ctx *ctx = nullptr;
    std::vector<gbp_scene *> scenes;
    BatchRunner runner;
    long long key = -1;
};

extern "C" {

int gbp_batch_create(gbp_ctx *c, int count, gbp_scene *const *scenes, gbp_batch **out) {
    if (!c || !out || count < 1 || !scenes) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_batch_create: bad argument");
    *out = nullptr;
    for (int i = 0; i < count; ++i)
        if (!scenes[i] || scenes[i]->ctx != c)
            return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_batch_create: scene missing or from another context");
    auto *b = new (std::nothrow) gbp_batch();
    if (!b) return fail(GBP_ERR_OUT_OF_MEMORY, "gbp_batch_create: host allocation");
    b->ctx = c;
    b->scenes.assign(scenes, scenes + count);
    *out = b;
    return GBP_OK;
}

void gbp_batch_destroy(gbp_batch *b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
}

int gbp_batch_project_device(gbp_batch *b, const double *dt, const float *const *solid, const float *const *fluid,
                             float *const *u, float *const *v, float *const *w, const gbp_params *params,
                             float *const *pressure, gbp_stats *stats, void *stream) {
    if (!b || !dt || !solid || !fluid || !u || !v) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_batch_project_device: NULL");
    auto t0 = std::chrono::steady_clock::now();
    gbp_ctx *c = b->ctx;
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    int rc = gbp::validate_params(p);
    if (rc) return rc;
    if (p.solver != GBP_SOLVER_MGPCG) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_batch_project_device: MGPCG only");
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    const int n = (int)b->scenes.size();
    for (int i = 0; i < n; ++i) {
        const Grid &g = b->scenes[i]->g;
        if (!solid[i] || !fluid[i] || !u[i] || !v[i] || (g.dim == 3 && (!w || !w[i])))
            return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_batch_project_device: NULL array");
    }
    GBP_CUDA(cudaEventRecord(c->ev[0], st));
    // per scene: assembly and multigrid setup
    long long launched = 0;
    bool warm_key = false;
    for (int i = 0; i < n; ++i) {
        gbp_scene *s = b->scenes[i];
        const Grid &g = s->g;
        rc = s->solver->prepare(g, p);
        if (rc) return fail(rc, s->solver->error());
        if (!pressure || !pressure[i]) {
            rc = ensure_staging(s);
            if (rc) return rc;
        }
        SolverState &ss = s->solver->state();
        SetupParams sp{p.eps_solid, p.eps_fluid, p.second_order_solid, p.second_order_fluid, 0.0};
        sp.rhs_correct = volume_correction(s, dt[i], p);
        GBP_CUDA(cudaMemsetAsync(ss.sc, 0, sizeof(Scalars), st));
        if (p.surface_tension != 0.0) {
            GBP_CUDA(launch_surface_tension(g, dt[i], s->dx, sp, p.surface_tension, fluid[i], u[i], v[i],
                                            g.dim == 3 ? w[i] : nullptr, c->grid_blocks, st));
            launched += 1;
        }
        rc = setup_for_solve(s, g, dt[i], sp, p, solid[i], fluid[i], u[i], v[i], g.dim == 3 ? w[i] : nullptr,
                             c->grid_blocks, st, &launched);
        if (rc) return rc;
        rc = s->solver->setup_mg(g, p, c->grid_blocks, st, &launched);
        if (rc) return fail(rc, s->solver->error());
        warm_key = warm_key || (p.warm_start && s->solver->has_prev());
    }
    GBP_CUDA(cudaEventRecord(c->ev[1], st));
    // the batched solve
    const bool mixed = p.precision == GBP_PRECISION_MIXED;
    long long key = (mixed ? 1 : 0) | (p.warm_start ? 2 : 0) | (p.tma_staging ? 4 : 0) | (p.tile_classes ? 0 : 8) |
                    ((long long)c->grid_blocks << 4) | ((long long)(p.mg_coarsest > 1 ? p.mg_coarsest : 4) << 24);
    for (int i = 0; i < n; ++i) key = key * 31 + (b->scenes[i]->solver->has_prev() ? 1 : 0);
    if (b->key != key) {
        if (mixed) {
            BatchPlan<float> plan;
            for (gbp_scene *s : b->scenes) s->solver->add_to_plan<float>(plan, p);
            rc = b->runner.build<float>(plan, c->grid_blocks, p.tma_staging, st);
        } else {
            BatchPlan<double> plan;
            for (gbp_scene *s : b->scenes) s->solver->add_to_plan<double>(plan, p);
            rc = b->runner.build<double>(plan, c->grid_blocks, 0, st);
        }
        if (rc) return fail(rc, b->runner.error());
        b->key = key;
    }
    rc = mixed ? b->runner.solve<float>(p, st, &launched) : b->runner.solve<double>(p, st, &launched);
    if (rc) return fail(rc, b->runner.error());
    GBP_CUDA(cudaEventRecord(c->ev[2], st));
    // per scene: residual report, pressure, velocity
    int first_bad = GBP_OK;
    for (int i = 0; i < n; ++i) {
        gbp_scene *s = b->scenes[i];
        const Grid &g = s->g;
        SolverState &ss = s->solver->state();
        rc = s->solver->finish_batched(p, st);
        if (rc) return fail(rc, s->solver->error());
        int status = s->solver->complete(g, p, c->grid_blocks, st, &launched);
        if (status != GBP_OK && status != GBP_ERR_NOT_CONVERGED && status != GBP_ERR_NAN)
            return fail(status, s->solver->error());
        if (status != GBP_OK && first_bad == GBP_OK) first_bad = status;
        float *pout = pressure && pressure[i] ? pressure[i] : s->d_p;
        SetupParams sp{p.eps_solid, p.eps_fluid, p.second_order_solid, p.second_order_fluid, 0.0};
        GBP_CUDA(launch_pressure(g, ss.diag, ss.x, p.warm_start && ss.have_prev ? ss.prev : nullptr, pout,
                                 p.warm_start ? ss.prev : nullptr, c->grid_blocks, st));
        GBP_CUDA(launch_velocity_faces(g, dt[i], s->dx, sp, pout, ss.faces, u[i], v[i], g.dim == 3 ? w[i] : nullptr,
                                       ss.sc, c->grid_blocks, st));
        launched += 2;
        if (p.warm_start) ss.have_prev = true;
    }
    GBP_CUDA(cudaEventRecord(c->ev[3], st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    if (stats) {
        float ms_a = 0, ms_s = 0, ms_u = 0;
        cudaEventElapsedTime(&ms_a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&ms_s, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&ms_u, c->ev[2], c->ev[3]);
        const float total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        for (int i = 0; i < n; ++i) {
            Scalars h;
            GBP_CUDA(cudaMemcpy(&h, b->scenes[i]->solver->state().sc, sizeof(Scalars), cudaMemcpyDeviceToHost));
            std::memset(&stats[i], 0, sizeof(gbp_stats));
            b->scenes[i]->solver->fill_stats(h, &stats[i]);
            stats[i].unknowns = (long long)h.unknowns;
            stats[i].tma_staged = b->runner.scene_staged(i) ? 1 : 0;
            stats[i].ms_assemble = ms_a;
            stats[i].ms_solve = ms_s;
            stats[i].ms_update = ms_u;
            stats[i].ms_total = total;
        }
    }
    return first_bad;
}

int gbp_bench_kernel(gbp_scene *s, int which, int reps, void *stream, float *ms_per_launch,
                     double *bytes_per_launch) {
    if (!s || !ms_per_launch || !bytes_per_launch || reps < 1)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_bench_kernel: bad argument");
    GBP_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    int rc = s->solver->bench_kernel(s->g, which, reps, s->ctx->grid_blocks, st, ms_per_launch, bytes_per_launch);
    if (rc) return fail(rc, s->solver->error());
    s->ctx->launches += reps + 1;
    return GBP_OK;
}

int gbp_debug_fail_wait(gbp_scene *s, int what, int block, int polls) {
    if (!s || !s->solver) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_debug_fail_wait: NULL scene");
    if ((what != GBP_WAIT_GRID_BARRIER && what != GBP_WAIT_TILE) || block < 0 || polls < 1 || polls > (1 << 24))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_debug_fail_wait: what must be GBP_WAIT_GRID_BARRIER or "
                                              "GBP_WAIT_TILE, block >= 0 and polls in [1, 2^24]");
    s->solver->set_wait_test(what, block, polls);
    return GBP_OK;
}

int gbp_debug_assemble(gbp_scene *s, double dt, const float *solid, const float *fluid, const float *u,
                       const float *v, const float *w, const gbp_params *params, double *diag, double *cx,
                       double *cy, double *cz, double *b) {
    if (!s || !solid || !fluid || !u || !v || !diag || !cx || !cy || !b)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_debug_assemble: NULL argument");
    const Grid &g = s->g;
    if (g.dim == 3 && (!w || !cz)) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_debug_assemble: NULL w/cz in 3D");
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    int rc = gbp::validate_params(p);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(s->ctx->device));
    rc = ensure_staging(s);
    if (rc) return rc;
    rc = s->solver->prepare(g, p);
    if (rc) return fail(rc, s->solver->error());
    SolverState &st = s->solver->state();
    cudaStream_t str = s->ctx->stream;
    GBP_CUDA(cudaMemcpyAsync(s->d_solid, solid, 4 * n_nodes(g), cudaMemcpyHostToDevice, str));
    GBP_CUDA(cudaMemcpyAsync(s->d_fluid, fluid, 4 * (size_t)g.ncell, cudaMemcpyHostToDevice, str));
    GBP_CUDA(cudaMemcpyAsync(s->d_u, u, 4 * n_face(g, 0), cudaMemcpyHostToDevice, str));
    GBP_CUDA(cudaMemcpyAsync(s->d_v, v, 4 * n_face(g, 1), cudaMemcpyHostToDevice, str));
    if (g.dim == 3) GBP_CUDA(cudaMemcpyAsync(s->d_w, w, 4 * n_face(g, 2), cudaMemcpyHostToDevice, str));
    SetupParams sp{p.eps_solid, p.eps_fluid, p.second_order_solid, p.second_order_fluid, 0.0};
    GBP_CUDA(cudaMemsetAsync(st.sc, 0, sizeof(Scalars), str));
    if (p.surface_tension != 0.0)
        GBP_CUDA(launch_surface_tension(g, dt, s->dx, sp, p.surface_tension, s->d_fluid, s->d_u, s->d_v, s->d_w,
                                        s->ctx->grid_blocks, str));
    GBP_CUDA(launch_setup(g, dt, s->dx, sp, s->d_solid, s->d_fluid, s->d_u, s->d_v, s->d_w, st, Level0Out{},
                          s->ctx->grid_blocks, str, &s->ctx->launches));
    const size_t bytes = 8 * (size_t)g.ncell;
    GBP_CUDA(cudaMemcpyAsync(diag, st.diag, bytes, cudaMemcpyDeviceToHost, str));
    GBP_CUDA(cudaMemcpyAsync(cx, st.cx, bytes, cudaMemcpyDeviceToHost, str));
    GBP_CUDA(cudaMemcpyAsync(cy, st.cy, bytes, cudaMemcpyDeviceToHost, str));
    if (g.dim == 3) GBP_CUDA(cudaMemcpyAsync(cz, st.cz, bytes, cudaMemcpyDeviceToHost, str));
    GBP_CUDA(cudaMemcpyAsync(b, st.b, bytes, cudaMemcpyDeviceToHost, str));
    GBP_CUDA(cudaStreamSynchronize(str));
    return GBP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// MAC advection (macadvection3, src/advection/macadvection3.cpp)

namespace {

int advect_check(const char *who, gbp_ctx *c, int nx, int ny, int nz, double dx, double dt,
                 const gbp_advect_params *params, const float *u, const float *v, const float *w,
                 const float *fluid, const float *q, gbp_advect_params *out) {
    if (!c) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL context");
    gbp_advect_params_default(out);
    if (params) *out = *params;
    if (nx < 2 || ny < 2 || nz < 2)
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": every grid edge must be at least 2 cells");
    if ((long long)(nx + 1) * ny * nz >= (1LL << 31) || (long long)nx * (ny + 1) * nz >= (1LL << 31) ||
        (long long)nx * ny * (nz + 1) >= (1LL << 31))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": 2^31 faces or more in one component");
    if (!(dx > 0.0) || !std::isfinite(dx) || !std::isfinite(dt))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": dx must be positive and finite, dt finite");
    if (out->trim_narrowband < 0)
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": trim_narrowband must be >= 0");
    if (!fluid || !u || !v || !w) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL array");
    if (!out->advect_velocity && !q)
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": nothing to advect (no scalar, velocity off)");
    return GBP_OK;
}

AdvectArgs advect_args(int nx, int ny, int nz, double dx, double dt, const gbp_advect_params &p, float *u, float *v,
                       float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    AdvectArgs a{};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.dx = dx;
    a.dt = dt;
    a.maccormack = p.maccormack ? 1 : 0;
    a.trim_narrowband = p.trim_narrowband;
    a.u = u;
    a.v = v;
    a.w = w;
    a.fluid = fluid;
    a.q = q;
    a.q_mask = q_mask;
    a.q_bg = q_bg;
    a.velocity = p.advect_velocity ? 1 : 0;
    return a;
}

}  // namespace

extern "C" {

void gbp_advect_params_default(gbp_advect_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->maccormack = 1;
    p->trim_narrowband = 1;
    p->advect_velocity = 1;
}

int gbp_advect3_device(gbp_ctx *c, int nx, int ny, int nz, double dx, double dt, const gbp_advect_params *params,
                       float *u, float *v, float *w, const float *fluid, float *q, const unsigned char *q_mask,
                       float q_bg, void *stream) {
    gbp_advect_params p;
    int rc = advect_check("gbp_advect3_device", c, nx, ny, nz, dx, dt, params, u, v, w, fluid, q, &p);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (!stream) {
        GBP_CUDA(cudaEventRecord(c->ev[0], cudaStreamLegacy));
        GBP_CUDA(cudaStreamWaitEvent(st, c->ev[0], 0));
    }
    long long launched = 0;
    GBP_CUDA(advect_run(c->adv, advect_args(nx, ny, nz, dx, dt, p, u, v, w, fluid, q, q_mask, q_bg), st, &launched));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

int gbp_advect3(gbp_ctx *c, int nx, int ny, int nz, double dx, double dt, const gbp_advect_params *params, float *u,
                float *v, float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    gbp_advect_params p;
    int rc = advect_check("gbp_advect3", c, nx, ny, nz, dx, dt, params, u, v, w, fluid, q, &p);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    const size_t cells = (size_t)nx * ny * nz;
    const size_t nf[3] = {(size_t)(nx + 1) * ny * nz, (size_t)nx * (ny + 1) * nz, (size_t)nx * ny * (nz + 1)};
    const size_t mask_floats = q && q_mask ? (cells + 3) / 4 : 0;
    const long long need = (long long)(nf[0] + nf[1] + nf[2] + cells + (q ? cells : 0) + mask_floats);
    if (need > c->adv_stage_floats) {
        if (c->adv_stage) cudaFree(c->adv_stage);
        c->adv_stage = nullptr;
        c->adv_stage_floats = 0;
        GBP_CUDA(cudaMalloc(&c->adv_stage, sizeof(float) * (size_t)need));
        c->adv_stage_floats = need;
    }
    float *du = c->adv_stage, *dv = du + nf[0], *dw = dv + nf[1], *df = dw + nf[2];
    float *dq = q ? df + cells : nullptr;
    unsigned char *dm = mask_floats ? (unsigned char *)(df + 2 * cells) : nullptr;
    cudaStream_t st = c->stream;
    GBP_CUDA(cudaMemcpyAsync(du, u, 4 * nf[0], cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dv, v, 4 * nf[1], cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dw, w, 4 * nf[2], cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(df, fluid, 4 * cells, cudaMemcpyHostToDevice, st));
    if (dq) GBP_CUDA(cudaMemcpyAsync(dq, q, 4 * cells, cudaMemcpyHostToDevice, st));
    if (dm) GBP_CUDA(cudaMemcpyAsync(dm, q_mask, cells, cudaMemcpyHostToDevice, st));
    long long launched = 0;
    GBP_CUDA(advect_run(c->adv, advect_args(nx, ny, nz, dx, dt, p, du, dv, dw, df, dq, dm, q_bg), st, &launched));
    if (p.advect_velocity) {
        GBP_CUDA(cudaMemcpyAsync(u, du, 4 * nf[0], cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaMemcpyAsync(v, dv, 4 * nf[1], cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaMemcpyAsync(w, dw, 4 * nf[2], cudaMemcpyDeviceToHost, st));
    }
    if (dq) GBP_CUDA(cudaMemcpyAsync(q, dq, 4 * cells, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

// The 2D step: advect_check with nz = 2 and w = u stands for the 2D checks
// (edges of at least 2 cells, sizes, arrays, parameters).
int gbp_advect2_device(gbp_ctx *c, int nx, int ny, double dx, double dt, const gbp_advect_params *params, float *u,
                       float *v, const float *fluid, float *q, const unsigned char *q_mask, float q_bg,
                       void *stream) {
    gbp_advect_params p;
    int rc = advect_check("gbp_advect2_device", c, nx, ny, 2, dx, dt, params, u, v, u, fluid, q, &p);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (!stream) {
        GBP_CUDA(cudaEventRecord(c->ev[0], cudaStreamLegacy));
        GBP_CUDA(cudaStreamWaitEvent(st, c->ev[0], 0));
    }
    long long launched = 0;
    GBP_CUDA(advect_run2(c->adv, advect_args(nx, ny, 1, dx, dt, p, u, v, nullptr, fluid, q, q_mask, q_bg), st,
                         &launched));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

int gbp_advect2(gbp_ctx *c, int nx, int ny, double dx, double dt, const gbp_advect_params *params, float *u, float *v,
                const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    gbp_advect_params p;
    int rc = advect_check("gbp_advect2", c, nx, ny, 2, dx, dt, params, u, v, u, fluid, q, &p);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    const size_t cells = (size_t)nx * ny;
    const size_t nf[2] = {(size_t)(nx + 1) * ny, (size_t)nx * (ny + 1)};
    const size_t mask_floats = q && q_mask ? (cells + 3) / 4 : 0;
    const long long need = (long long)(nf[0] + nf[1] + cells + (q ? cells : 0) + mask_floats);
    if (need > c->adv_stage_floats) {
        if (c->adv_stage) cudaFree(c->adv_stage);
        c->adv_stage = nullptr;
        c->adv_stage_floats = 0;
        GBP_CUDA(cudaMalloc(&c->adv_stage, sizeof(float) * (size_t)need));
        c->adv_stage_floats = need;
    }
    float *du = c->adv_stage, *dv = du + nf[0], *df = dv + nf[1];
    float *dq = q ? df + cells : nullptr;
    unsigned char *dm = mask_floats ? (unsigned char *)(df + 2 * cells) : nullptr;
    cudaStream_t st = c->stream;
    GBP_CUDA(cudaMemcpyAsync(du, u, 4 * nf[0], cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dv, v, 4 * nf[1], cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(df, fluid, 4 * cells, cudaMemcpyHostToDevice, st));
    if (dq) GBP_CUDA(cudaMemcpyAsync(dq, q, 4 * cells, cudaMemcpyHostToDevice, st));
    if (dm) GBP_CUDA(cudaMemcpyAsync(dm, q_mask, cells, cudaMemcpyHostToDevice, st));
    long long launched = 0;
    GBP_CUDA(advect_run2(c->adv, advect_args(nx, ny, 1, dx, dt, p, du, dv, nullptr, df, dq, dm, q_bg), st,
                         &launched));
    if (p.advect_velocity) {
        GBP_CUDA(cudaMemcpyAsync(u, du, 4 * nf[0], cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaMemcpyAsync(v, dv, 4 * nf[1], cudaMemcpyDeviceToHost, st));
    }
    if (dq) GBP_CUDA(cudaMemcpyAsync(q, dq, 4 * cells, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Solid constraint of the velocity (macutility3::constrain_velocity,
// src/utility/macutility3.cpp:61-86)

namespace {

int constrain_check(const char *who, gbp_ctx *c, int nx, int ny, int nz, double dx, const float *solid,
                    const float *u, const float *v, const float *w) {
    if (!c) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL context");
    if (nx < 2 || ny < 2 || nz < 2)
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": every grid edge must be at least 2 cells");
    if ((long long)(nx + 1) * (ny + 1) * (nz + 1) >= (1LL << 31))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": 2^31 nodes or more");
    if (!(dx > 0.0) || !std::isfinite(dx))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": dx must be positive and finite");
    if (!solid || !u || !v || !w) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL array");
    return GBP_OK;
}

ConstrainArgs constrain_args(int nx, int ny, int nz, double dx, const float *solid, float *u, float *v, float *w,
                             const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    ConstrainArgs a{};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.dx = dx;
    a.solid = solid;
    a.u = u;
    a.v = v;
    a.w = w;
    a.mu = mu;
    a.mv = mv;
    a.mw = mw;
    return a;
}

}  // namespace

extern "C" {

int gbp_constrain_velocity3_device(gbp_ctx *c, int nx, int ny, int nz, double dx, const float *solid, float *u,
                                   float *v, float *w, const unsigned char *mu, const unsigned char *mv,
                                   const unsigned char *mw, void *stream) {
    int rc = constrain_check("gbp_constrain_velocity3_device", c, nx, ny, nz, dx, solid, u, v, w);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (!stream) {
        GBP_CUDA(cudaEventRecord(c->ev[0], cudaStreamLegacy));
        GBP_CUDA(cudaStreamWaitEvent(st, c->ev[0], 0));
    }
    long long launched = 0;
    GBP_CUDA(constrain_run(c->adv, constrain_args(nx, ny, nz, dx, solid, u, v, w, mu, mv, mw), st, &launched));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

int gbp_constrain_velocity3(gbp_ctx *c, int nx, int ny, int nz, double dx, const float *solid, float *u, float *v,
                            float *w, const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    int rc = constrain_check("gbp_constrain_velocity3", c, nx, ny, nz, dx, solid, u, v, w);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    const size_t nodes = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    const size_t nf[3] = {(size_t)(nx + 1) * ny * nz, (size_t)nx * (ny + 1) * nz, (size_t)nx * ny * (nz + 1)};
    const unsigned char *masks[3] = {mu, mv, mw};
    size_t mask_floats = 0;
    for (int d = 0; d < 3; ++d)
        if (masks[d]) mask_floats += (nf[d] + 3) / 4;
    const long long need = (long long)(nodes + nf[0] + nf[1] + nf[2] + mask_floats);
    if (need > c->adv_stage_floats) {
        if (c->adv_stage) cudaFree(c->adv_stage);
        c->adv_stage = nullptr;
        c->adv_stage_floats = 0;
        GBP_CUDA(cudaMalloc(&c->adv_stage, sizeof(float) * (size_t)need));
        c->adv_stage_floats = need;
    }
    cudaStream_t st = c->stream;
    float *ds = c->adv_stage, *dc[3];
    dc[0] = ds + nodes;
    dc[1] = dc[0] + nf[0];
    dc[2] = dc[1] + nf[1];
    float *next = dc[2] + nf[2];
    const unsigned char *dm[3] = {nullptr, nullptr, nullptr};
    float *hc[3] = {u, v, w};
    GBP_CUDA(cudaMemcpyAsync(ds, solid, 4 * nodes, cudaMemcpyHostToDevice, st));
    for (int d = 0; d < 3; ++d) {
        GBP_CUDA(cudaMemcpyAsync(dc[d], hc[d], 4 * nf[d], cudaMemcpyHostToDevice, st));
        if (masks[d]) {
            GBP_CUDA(cudaMemcpyAsync(next, masks[d], nf[d], cudaMemcpyHostToDevice, st));
            dm[d] = (const unsigned char *)next;
            next += (nf[d] + 3) / 4;
        }
    }
    long long launched = 0;
    GBP_CUDA(constrain_run(c->adv, constrain_args(nx, ny, nz, dx, ds, dc[0], dc[1], dc[2], dm[0], dm[1], dm[2]), st,
                           &launched));
    for (int d = 0; d < 3; ++d) GBP_CUDA(cudaMemcpyAsync(hc[d], dc[d], 4 * nf[d], cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Extrapolation (array_extrapolator3::extrapolate, array_extrapolator3.h:
// 36-73) and macutility3::extrapolate_and_constrain_velocity
// (src/utility/macutility3.cpp:88-92)

namespace {

int extrapolate_check(const char *who, gbp_ctx *c, int w, int h, int d, const void *a, const void *m, int count) {
    if (!c) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL context");
    if (w < 1 || h < 1 || d < 1 || (long long)w * h * d >= (1LL << 31))
        return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": bad shape (each edge >= 1, fewer than 2^31 cells)");
    if (count < 0) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": negative count");
    if (!a || !m) return fail(GBP_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL array");
    return GBP_OK;
}

// device staging of the host-array calls, kept in the context
int stage_floats(gbp_ctx *c, long long need) {
    if (need > c->adv_stage_floats) {
        if (c->adv_stage) cudaFree(c->adv_stage);
        c->adv_stage = nullptr;
        c->adv_stage_floats = 0;
        GBP_CUDA(cudaMalloc(&c->adv_stage, sizeof(float) * (size_t)need));
        c->adv_stage_floats = need;
    }
    return GBP_OK;
}

}  // namespace

extern "C" {

int gbp_extrapolate3_device(gbp_ctx *c, int w, int h, int d, float *a, unsigned char *active, int count,
                            long long *activated, void *stream) {
    int rc = extrapolate_check("gbp_extrapolate3_device", c, w, h, d, a, active, count);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (!stream) {
        GBP_CUDA(cudaEventRecord(c->ev[0], cudaStreamLegacy));
        GBP_CUDA(cudaStreamWaitEvent(st, c->ev[0], 0));
    }
    unsigned long long added = 0;
    long long launched = 0;
    GBP_CUDA(extrapolate_run(c->adv, w, h, d, a, active, count, st, &launched, activated ? &added : nullptr));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    if (activated) *activated = (long long)added;
    return GBP_OK;
}

int gbp_extrapolate3(gbp_ctx *c, int w, int h, int d, float *a, unsigned char *active, int count,
                     long long *activated) {
    int rc = extrapolate_check("gbp_extrapolate3", c, w, h, d, a, active, count);
    if (rc) return rc;
    GBP_CUDA(cudaSetDevice(c->device));
    const size_t n = (size_t)w * h * d;
    if ((rc = stage_floats(c, (long long)(n + (n + 3) / 4)))) return rc;
    float *da = c->adv_stage;
    unsigned char *dm = reinterpret_cast<unsigned char *>(da + n);
    cudaStream_t st = c->stream;
    GBP_CUDA(cudaMemcpyAsync(da, a, 4 * n, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dm, active, n, cudaMemcpyHostToDevice, st));
    unsigned long long added = 0;
    long long launched = 0;
    GBP_CUDA(extrapolate_run(c->adv, w, h, d, da, dm, count, st, &launched, activated ? &added : nullptr));
    GBP_CUDA(cudaMemcpyAsync(a, da, 4 * n, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaMemcpyAsync(active, dm, n, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    if (activated) *activated = (long long)added;
    return GBP_OK;
}

int gbp_extrapolate_constrain_velocity3(gbp_ctx *c, int nx, int ny, int nz, double dx, const float *solid, float *u,
                                        float *v, float *w, unsigned char *mu, unsigned char *mv, unsigned char *mw,
                                        int width) {
    int rc = constrain_check("gbp_extrapolate_constrain_velocity3", c, nx, ny, nz, dx, solid, u, v, w);
    if (rc) return rc;
    if (width < 0) return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_extrapolate_constrain_velocity3: negative width");
    if ((mu != nullptr) != (mv != nullptr) || (mu != nullptr) != (mw != nullptr))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_extrapolate_constrain_velocity3: give all three masks or none");
    GBP_CUDA(cudaSetDevice(c->device));
    const size_t nodes = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    const size_t nf[3] = {(size_t)(nx + 1) * ny * nz, (size_t)nx * (ny + 1) * nz, (size_t)nx * ny * (nz + 1)};
    const bool masked = mu != nullptr;
    const size_t mask_floats = masked ? (nf[0] + 3) / 4 + (nf[1] + 3) / 4 + (nf[2] + 3) / 4 : 0;
    if ((rc = stage_floats(c, (long long)(nodes + nf[0] + nf[1] + nf[2] + mask_floats)))) return rc;
    cudaStream_t st = c->stream;
    float *ds = c->adv_stage, *dc[3];
    dc[0] = ds + nodes;
    dc[1] = dc[0] + nf[0];
    dc[2] = dc[1] + nf[1];
    float *next = dc[2] + nf[2];
    unsigned char *dm[3] = {nullptr, nullptr, nullptr};
    float *hc[3] = {u, v, w};
    unsigned char *hm[3] = {mu, mv, mw};
    GBP_CUDA(cudaMemcpyAsync(ds, solid, 4 * nodes, cudaMemcpyHostToDevice, st));
    for (int d = 0; d < 3; ++d) {
        GBP_CUDA(cudaMemcpyAsync(dc[d], hc[d], 4 * nf[d], cudaMemcpyHostToDevice, st));
        if (masked) {
            dm[d] = reinterpret_cast<unsigned char *>(next);
            GBP_CUDA(cudaMemcpyAsync(dm[d], hm[d], nf[d], cudaMemcpyHostToDevice, st));
            next += (nf[d] + 3) / 4;
        }
    }
    long long launched = 0;
    // macarray_extrapolator3::extrapolate: each component on its own
    // (macarray_extrapolator3.h:44-48); with every face active nothing grows
    if (masked)
        for (int d = 0; d < 3; ++d)
            GBP_CUDA(extrapolate_run(c->adv, nx + (d == 0), ny + (d == 1), nz + (d == 2), dc[d], dm[d], width, st,
                                     &launched, nullptr));
    GBP_CUDA(constrain_run(c->adv, constrain_args(nx, ny, nz, dx, ds, dc[0], dc[1], dc[2], dm[0], dm[1], dm[2]), st,
                           &launched));
    for (int d = 0; d < 3; ++d) {
        GBP_CUDA(cudaMemcpyAsync(hc[d], dc[d], 4 * nf[d], cudaMemcpyDeviceToHost, st));
        if (masked) GBP_CUDA(cudaMemcpyAsync(hm[d], dm[d], nf[d], cudaMemcpyDeviceToHost, st));
    }
    GBP_CUDA(cudaStreamSynchronize(st));
    c->launches += launched;
    return GBP_OK;
}

}  // extern "C"
