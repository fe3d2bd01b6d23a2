// gbp_noalloc.cu -- gbp_project_device_static: the plain-CG projection of
// gbp_project_device for callers that cannot allocate device memory.
//
// Some callers of a pressure projection cannot call cudaMalloc: a host
// application whose device memory is handed out by its own allocator (or a
// memory pool sized up front), a plugin running inside a process that caps
// or forbids further allocations, or code that must not hit the allocator
// on its per-step path. This entry point takes the caller's inputs and
// outputs and keeps everything else it needs -- operator, CG vectors,
// reduction partials and scalars -- in one file-scope device array,
// g_static_scratch, of GBP_STATIC_SCRATCH_BYTES. Every GPU that loads the
// library holds that array until the process exits. It calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// Limits: at most GBP_STATIC_MAX_CELLS cells; plain CG in FP64 only (the
// reference's solver); no warm start and no volume correction (both need
// state kept between calls). All calls share the one array: calls that
// overlap on the GPU (two streams, two host threads) race on it, so the
// caller serialises them. What must start at zero (the scalars block with
// the reduction tickets) is cleared by every call.
#include <cstring>
#include <string>

#include "gbp.h"
#include "gbp_internal.cuh"
#include "gbp_kernels.h"

namespace gbp {
void set_last_error(const std::string &msg);   // gbp_api.cpp
int validate_params(const gbp_params &p);      // gbp_api.cpp: the checks of every projection entry point
}

namespace {

using namespace gbp;

// operator (diag, cx, cy, cz), b, and CG vectors x, r, s, z: 9 doubles per
// cell, then the partials and the scalars, each block 256-byte aligned
constexpr size_t align256(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t kVecBytes = align256(sizeof(double) * GBP_STATIC_MAX_CELLS);
constexpr size_t kScratchBytes = 9 * kVecBytes + align256(sizeof(Partials)) + align256(sizeof(Scalars));
static_assert(kScratchBytes <= GBP_STATIC_SCRATCH_BYTES, "static scratch too small");

static __device__ __align__(256) unsigned char g_static_scratch[GBP_STATIC_SCRATCH_BYTES];

int fail(int code, const std::string &m) {
    gbp::set_last_error(m);  // reported by gbp_strerror(code)
    return code;
}

#define NOALLOC_CUDA(call)                                                                             \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(GBP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device address of g_static_scratch on the current device. The host-side
// name is only a stand-in, not a device address, so the address is looked
// up on every call (cheap, and it allocates nothing): a cached one would go
// stale if the device's context were reset and the module loaded again.
int scratch_for_device(int device, unsigned char **addr, int *sms) {
    void *p = nullptr;
    NOALLOC_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
    int n = 0;
    NOALLOC_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device));
    *addr = static_cast<unsigned char *>(p);
    *sms = n;
    return GBP_OK;
}

}  // namespace

extern "C" int gbp_project_device_static(int dim, int nx, int ny, int nz, double dx, double dt, const float *solid,
                                         const float *fluid, float *u, float *v, float *w, const gbp_params *params,
                                         float *pressure, gbp_stats *stats, void *stream) {
    if ((dim != 2 && dim != 3) || nx < 1 || ny < 1 || (dim == 3 && nz < 1) || !(dx > 0.0))
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device_static: bad shape or dx");
    const long long cells = (long long)nx * ny * (dim == 3 ? nz : 1);
    if (cells > GBP_STATIC_MAX_CELLS)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device_static: " + std::to_string(cells) +
                                                  " cells exceed the static scratch limit of " +
                                                  std::to_string(GBP_STATIC_MAX_CELLS) + " cells");
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    int rc = gbp::validate_params(p);
    if (rc) return rc;
    if (p.solver != GBP_SOLVER_CG || p.precision != GBP_PRECISION_FP64)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device_static: only the plain FP64 CG solver");
    if (p.warm_start)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device_static: warm start needs a scene (gbp_scene_create)");
    if (!solid || !fluid || !u || !v || (dim == 3 && !w) || !pressure)
        return fail(GBP_ERR_INVALID_ARGUMENT, "gbp_project_device_static: NULL array");

    int device = 0;
    NOALLOC_CUDA(cudaGetDevice(&device));
    unsigned char *base = nullptr;
    int sms = 0;
    rc = scratch_for_device(device, &base, &sms);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    const Grid g = make_grid(dim, nx, ny, nz);
    double *vec[9];
    for (int i = 0; i < 9; ++i) vec[i] = reinterpret_cast<double *>(base + (size_t)i * kVecBytes);
    double *diag = vec[0], *cx = vec[1], *cy = vec[2], *cz = vec[3], *b = vec[4];
    double *x = vec[5], *r = vec[6], *s = vec[7], *z = vec[8];
    Partials *pt = reinterpret_cast<Partials *>(base + 9 * kVecBytes);
    Scalars *sc = reinterpret_cast<Scalars *>(base + 9 * kVecBytes + align256(sizeof(Partials)));
    int grid_blocks = sms * 6;
    if (grid_blocks > MAX_GRID) grid_blocks = MAX_GRID;

    // the scalars block (tickets, flags, counters) must start at zero
    NOALLOC_CUDA(cudaMemsetAsync(sc, 0, sizeof(Scalars), st));
    SetupParams sp{p.eps_solid, p.eps_fluid, p.second_order_solid, p.second_order_fluid, 0.0};
    if (p.surface_tension != 0.0)
        NOALLOC_CUDA(launch_surface_tension(g, dt, dx, sp, p.surface_tension, fluid, u, v, w, grid_blocks, st));
    NOALLOC_CUDA(launch_assemble(g, dt, dx, sp, solid, fluid, u, v, w, diag, cx, cy, cz, b, sc, grid_blocks, st));
    Operator<double> A{diag, cx, cy, dim == 3 ? cz : cy};
    NOALLOC_CUDA(launch_cg_init(g, A, b, nullptr, x, r, s, sc, pt, p.residual, p.max_iterations, grid_blocks, st));
    const int chunk = p.iterations_per_sync > 0 ? p.iterations_per_sync : 16;
    Scalars h;
    std::memset(&h, 0, sizeof(h));
    const long long max_chunks = (long long)p.max_iterations / chunk + 2;
    for (long long k = 0; k < max_chunks; ++k) {
        NOALLOC_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        NOALLOC_CUDA(cudaStreamSynchronize(st));
        if (h.done) break;
        for (int it = 0; it < chunk; ++it)
            NOALLOC_CUDA(launch_cg_iteration(g, A, x, r, s, z, sc, pt, grid_blocks, st));
    }
    NOALLOC_CUDA(launch_true_residual(g, A, b, x, nullptr, sc, pt, grid_blocks, st));
    NOALLOC_CUDA(launch_pressure(g, diag, x, nullptr, pressure, nullptr, grid_blocks, st));
    NOALLOC_CUDA(launch_velocity(g, dt, dx, sp, solid, fluid, pressure, u, v, w, sc, grid_blocks, st));
    NOALLOC_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    NOALLOC_CUDA(cudaStreamSynchronize(st));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->iterations = h.iter;
        stats->outer_iterations = 1;
        stats->converged = h.status == 1;
        stats->b_inf = h.res0;
        stats->reresid = h.res0 > 0 ? h.res / h.res0 : 0.0;
        stats->true_resid_inf = h.res0 > 0 ? h.aux[0] / h.res0 : 0.0;
        stats->true_resid_l2 = h.aux[2] > 0 ? h.aux[1] / h.aux[2] : 0.0;
        stats->unknowns = (long long)h.unknowns;
    }
    if (h.status == 3) return GBP_ERR_NAN;
    if (h.status == 2 || !h.done) return GBP_ERR_NOT_CONVERGED;
    return GBP_OK;
}
