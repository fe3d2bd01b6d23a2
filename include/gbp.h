/*
 * gbp.h -- C ABI of the GB300 pressure-projection library (libgbp.so).
 *
 * One call projects a MAC velocity field onto its divergence-free part the
 * way Shiokaze's pressure projection does it: face fractions from the solid
 * and fluid level sets, the variational ghost-fluid Poisson system, its
 * solve, and the pressure-gradient velocity update. It replaces
 *
 *   macproject3_interface::project(dt, velocity, solid, fluid, ...)
 *     include/shiokaze/projection/macproject3_interface.h:67-72
 *   macproject2_interface::project(...)
 *     include/shiokaze/projection/macproject2_interface.h:67-72
 *   as implemented by src/projection/macpressuresolver3.cpp:50-272 and
 *   src/projection/macpressuresolver2.cpp:48-238,
 *
 * with get_pressure() (macproject3_interface.h:79) returned through the
 * pressure output and set_target_volume() (:50) as its own call.
 *
 * Arrays are dense, x fastest (index i + nx*(j + ny*k)):
 *   solid     nodal level set   (nx+1)*(ny+1)*(nz+1)   [(nx+1)*(ny+1) in 2D]
 *   fluid     cell level set    nx*ny*nz               [nx*ny]
 *   u, v, w   face velocities   (nx+1)*ny*nz, nx*(ny+1)*nz, nx*ny*(nz+1)
 *                               (in/out; w is ignored in 2D)
 *   pressure  cell pressure     nx*ny*nz, 0 off the unknowns (out, optional)
 * Level sets are the values the reference reads through its narrow-band
 * arrays (outside the band they read +-band). Every face is updated.
 *
 * Errors are reported as int status codes (GBP_OK == 0). The reference has
 * no error returns (it asserts or exits); a solve that stops at
 * max_iterations still writes its last iterate and the velocity update, as
 * the reference does, and returns GBP_ERR_NOT_CONVERGED.
 *
 * Threading: a context and its scenes belong to one host thread at a time.
 */
#ifndef GBP_H
#define GBP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBP_OK 0
#define GBP_ERR_INVALID_ARGUMENT 1
#define GBP_ERR_CUDA 2
#define GBP_ERR_OUT_OF_MEMORY 3
#define GBP_ERR_NOT_CONVERGED 4
#define GBP_ERR_NAN 5
#define GBP_ERR_NO_DEVICE 6
#define GBP_ERR_BUDGET 7
#define GBP_ERR_TIMEOUT 8

/* Linear solver. GBP_SOLVER_CG is the reference's default "pcg" module,
 * whose preconditioner returns its input (local/include/pcgsolver/
 * pcg_solver.h:379-384): plain CG, x0 = 0, stop at |r|_inf <= residual*|b|_inf
 * on the recursively updated residual. GBP_SOLVER_MGPCG is CG preconditioned
 * by a geometric multigrid V-cycle, same stopping rule. */
#define GBP_SOLVER_CG 0
#define GBP_SOLVER_MGPCG 1

/* Arithmetic. FP64: every vector and operator in double.
 * MIXED: outer iterative refinement in FP64 storage (x and r in double,
 * FP64 norms and stopping rule) around an FP32 MGPCG inner solve (FP32
 * stencil, smoother and transfers). After each inner solve with correction
 * d: x += d and r -= A d, the product with the FP64 operator formed in
 * float pairs (each coupling as its float rounding plus the float of the
 * remainder, 48 bits; products split exactly by FMA, TwoSum sums; within
 * about 2^-47 |A||d|) and subtracted in FP64: three FP64 additions per cell
 * instead of the eight FP64 operations of b - A x. The inner solve's dot
 * products and norms are not FP64 per term: each thread sums its n terms in
 * float-float (the product split exactly by an FMA, TwoSum, renormalised
 * after every term), within gamma_n^2 sum |a_i b_i| of the exact value
 * (gamma_n = n u / (1 - n u), u = 2^-24; about 1.6e-11 sum |a_i b_i| for the
 * 72 terms a thread sums at 256^3), and the threads' partials add in FP64.
 * That is far below the inner solve's own tolerance (1e-3), and the outer
 * refinement's residual, norms and stopping rule are FP64 throughout. */
#define GBP_PRECISION_FP64 0
#define GBP_PRECISION_MIXED 1

typedef struct gbp_ctx gbp_ctx;
typedef struct gbp_scene gbp_scene;

typedef struct gbp_params {
    double residual;        /* "Residual", src/linsolver/pcg.cpp:40 (default 1e-4) */
    int max_iterations;     /* "MaxIterations", pcg.cpp:43 (default 30000) */
    int warm_start;         /* "WarmStart", macpressuresolver3.cpp:278 (default 0) */
    double eps_fluid;       /* "EpsFluid", src/utility/macutility3.cpp:408 (default 1e-2) */
    double eps_solid;       /* "EpsSolid", macutility3.cpp:409 (default 1e-2) */
    int second_order_fluid; /* "SecondOrderAccurateFluid", macpressuresolver3.cpp:275 (default 1) */
    int second_order_solid; /* "SecondOrderAccurateSolid", macpressuresolver3.cpp:276 (default 1) */
    double gain;            /* "Gain", macpressuresolver3.cpp:277 (default 1) */
    int solver;             /* GBP_SOLVER_* (default GBP_SOLVER_CG) */
    int precision;          /* GBP_PRECISION_* (default GBP_PRECISION_FP64) */
    int mg_smooth;          /* red-black sweeps before and after each coarse correction (default 1) */
    int mg_coarsest;        /* coarsen while any edge exceeds this (default 7) */
    double inner_tolerance; /* MIXED: relative residual of each inner solve (default 1e-3) */
    int iterations_per_sync;/* CG iterations between host checks of convergence (default 16) */
    double surface_tension; /* the surface_tension argument of macproject3_interface::project
                               (macpressuresolver3.cpp:85-115); 0 (default) leaves the velocity as is */
    int tma_staging;        /* MGPCG MIXED: nonzero runs the fine level's four stencil passes with their
                               tiles staged in shared memory by TMA where the grid allows it (3D, at least
                               2^21 cells, nx % 8 == 0); 0 (default) uses the direct-load kernels, which
                               compute every cell alike and measure faster over a whole solve on GB300 */
    int tile_classes;       /* MGPCG: nonzero (default) lets the multigrid and CG kernels use the tile classes of
                               each level: in the FP32 kernels a tile whose couplings all share one value reads
                               that value instead of the coupling arrays, and a tile with no unknown writes zeros
                               without loading; the results equal those with 0, which reads every array */
} gbp_params;

typedef struct gbp_stats {
    int iterations;         /* CG iterations (summed over refinement steps for MIXED) */
    int outer_iterations;   /* refinement steps (1 unless MIXED) */
    int converged;          /* stopping rule met */
    double reresid;         /* |r|_inf / |b|_inf at exit, r the solver's residual (pcg_solver.h:292) */
    double true_resid_inf;  /* |b - A x|_inf / |b|_inf at exit: recomputed in FP64, or for MIXED MGPCG the
                               refinement's residual, updated r -= A d after each inner solve with float-pair
                               products (within about 2^-47 |A||x| of the recomputed value) */
    double true_resid_l2;   /* |b - A x|_2 / |b|_2 */
    double b_inf;           /* |b|_inf of the system solved (after warm-start shift) */
    long long unknowns;     /* pressure unknowns (cells in the linear system) */
    float ms_assemble;      /* device time, face fractions + labelling + operator + rhs */
    float ms_solve;         /* device time, the linear solve */
    float ms_update;        /* device time, velocity update + pressure write */
    float ms_total;         /* host wall time of the call */
    int tma_staged;         /* the fine level ran the TMA-staged kernels (see gbp_params.tma_staging) */
} gbp_stats;

/* Result of gbp_csr_cg. */
typedef struct gbp_csr_stats {
    int iterations;         /* CG iterations, as pcg_solver.h:283-293 counts them */
    int converged;          /* stopping rule met (or b == 0) */
    double reresid;         /* |r|_inf / |b|_inf at exit: the residual the reference's pcg module returns */
    float ms_solve;         /* device time of the iterations */
    float ms_total;         /* host wall time of the call, copies included */
} gbp_csr_stats;

/* Fills *p with the reference's defaults (and CG / FP64). */
void gbp_params_default(gbp_params *p);

/* Solves A x = b on the GPU for a symmetric positive (semi)definite matrix
 * of n < 2^31 rows in compressed rows (host arrays: rowstart[0..n], rowstart[0] = 0;
 * column indices cols[rowstart[r]..rowstart[r+1]) in [0, n) and values vals
 * alike; duplicate entries of a row add up), with the reference's LinSolver
 * "pcg" (src/linsolver/pcg.cpp:44-74; local/include/pcgsolver/pcg_solver.h:
 * 246-295): plain CG from x = 0 in FP64 until |r|_inf <= residual |b|_inf
 * or max_iterations. x (n values) receives the solution (the last iterate
 * if not converged). Returns GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN
 * (breakdown) or an argument / CUDA error; stats may be NULL. The matrix
 * and vectors are copied to the device on every call; the context keeps the
 * device arrays between calls of up to the same sizes. */
int gbp_csr_cg(gbp_ctx *ctx, long long n, const long long *rowstart, const long long *cols, const double *vals,
               const double *b, double *x, double residual, int max_iterations, gbp_csr_stats *stats);

/* Context on CUDA device `device`: stream, events, graph cache. */
int gbp_create(int device, gbp_ctx **out);
void gbp_destroy(gbp_ctx *ctx);

/* A scene holds the device state of one grid: operator, solver vectors,
 * multigrid hierarchy and warm-start pressure. It replaces a
 * macpressuresolver{2,3} instance after initialize(shape, dx)
 * (macpressuresolver3.cpp:281-291). dim is 2 or 3 (nz ignored in 2D). */
int gbp_scene_create(gbp_ctx *ctx, int dim, int nx, int ny, int nz, double dx, gbp_scene **out);
void gbp_scene_destroy(gbp_scene *scene);

/* Device bytes a scene of this shape holds once projected with `params`
 * (used for admission against a memory budget). */
size_t gbp_scene_device_bytes(int dim, int nx, int ny, int nz, const gbp_params *params);

/* macproject3_interface::set_target_volume (macproject3_interface.h:50,
 * macpressuresolver3.cpp:45-48): arms the volume-correction term. */
int gbp_scene_set_target_volume(gbp_scene *scene, double current_volume, double target_volume);

/* One projection with HOST arrays (copied in and out on the context's
 * stream). params may be NULL (defaults); pressure and stats may be NULL. */
int gbp_project(gbp_scene *scene, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                const gbp_params *params, float *pressure, gbp_stats *stats);

/* gbp_project plus the active sets the reference leaves on its sparse
 * arrays, for callers that keep them (the Shiokaze plugin modules):
 *   unknown   nx*ny*nz: 1 on the cells whose pressure the reference sets --
 *             every unknown, a pressure of 0 included
 *             (macpressuresolver3.cpp:245-248) -- 0 elsewhere;
 *   u_active, v_active, w_active  per face: 1 on the faces the reference's
 *             velocity update keeps active (open faces, and closed faces on
 *             the domain boundary next to a fluid cell; in 2D only where the
 *             velocity before the update points out of the domain), 0 on the
 *             faces it deactivates with set_off (macpressuresolver3.cpp:
 *             252-267; macpressuresolver2.cpp:221-236). Those read 0.
 * Host arrays; w_active is ignored in 2D. Otherwise as gbp_project. */
int gbp_project_active(gbp_scene *scene, double dt, const float *solid, const float *fluid, float *u, float *v,
                       float *w, const gbp_params *params, float *pressure, gbp_stats *stats, unsigned char *unknown,
                       unsigned char *u_active, unsigned char *v_active, unsigned char *w_active);

/* The same with DEVICE arrays, on `stream` (a cudaStream_t; NULL = the
 * context's stream). Returns after the solve has finished on the device. */
int gbp_project_device(gbp_scene *scene, double dt, const float *solid, const float *fluid, float *u, float *v,
                       float *w, const gbp_params *params, float *pressure, gbp_stats *stats, void *stream);

/* ---- sparse 3D arrays in bricks -------------------------------------------
 * The reference's arrays are tiled and sparse (src/array/tiledarray3.cpp:
 * tiles allocated where cells are active or partly filled; a cell reads its
 * value if active, else the fill value if filled, else the background,
 * include/shiokaze/array/array3.h:796-800). A gbp_bricks carries such an
 * array of extent nx x ny x nz (cells, nodes or faces) in bricks of
 * GBP_BRICK^3 cells: brick (bx, by, bz) holds cells [8 bx, 8 bx + 8) x
 * [8 by, ..) x [8 bz, ..) and is numbered bx + nbx (by + nby bz), nbx =
 * ceil(nx / 8) (nby, nbz likewise). slot[b] says what brick b holds:
 *   GBP_BRICK_BACKGROUND  every cell reads `background`;
 *   GBP_BRICK_FILL        every cell reads `fill`;
 *   s >= 0                its cells read values[s * GBP_BRICK_CELLS + x +
 *                         8 (y + 8 z)] (cells beyond the extent ignored).
 * Only the listed bricks travel to the GPU, which expands them; the
 * outputs come back the same way, for the bricks a gbp_bricks_out lists. */
#define GBP_BRICK 8
#define GBP_BRICK_CELLS 512
#define GBP_BRICK_BACKGROUND (-1)
#define GBP_BRICK_FILL (-2)
typedef struct gbp_bricks {
    float background, fill;
    const int *slot;      /* one per brick */
    long long count;      /* bricks with a slot >= 0; their slots are 0 .. count-1 */
    const float *values;  /* count * GBP_BRICK_CELLS */
} gbp_bricks;

typedef struct gbp_bricks_out {
    const int *slot;        /* one per brick: s >= 0 copies the brick out to slot s, < 0 skips it */
    long long count;        /* bricks copied out; their slots are 0 .. count-1 */
    float *values;          /* count * GBP_BRICK_CELLS, written */
    unsigned char *active;  /* count * GBP_BRICK_CELLS (or NULL): the active sets of gbp_project_active */
} gbp_bricks_out;

/* gbp_project_active with its inputs and outputs in bricks (3D scenes):
 * solid (nodes), fluid (cells), u, v, w (faces) in; pressure with the
 * unknown cells, and u, v, w with the faces the reference keeps active, out
 * for the listed bricks (any output may be NULL). The velocities are
 * updated on the GPU in the expanded arrays; only the listed output bricks
 * are copied back. Equal, cell for cell, to gbp_project_active on the
 * expanded arrays. */
int gbp_project_bricks(gbp_scene *scene, double dt, const gbp_bricks *solid, const gbp_bricks *fluid,
                       const gbp_bricks *u, const gbp_bricks *v, const gbp_bricks *w, const gbp_params *params,
                       gbp_bricks_out *pressure, gbp_bricks_out *u_out, gbp_bricks_out *v_out, gbp_bricks_out *w_out,
                       gbp_stats *stats);

/* The expansion alone: `dense` (a DEVICE array of nx*ny*nz floats, x
 * fastest) receives the cell values of `in`, on `stream` (NULL = the
 * context's stream; returns after the copy has finished). */
int gbp_bricks_expand(gbp_ctx *ctx, int nx, int ny, int nz, const gbp_bricks *in, float *dense, void *stream);

/* Batched projection: many independent scenes of uneven sizes solved
 * together. Every kernel of the multigrid-preconditioned CG iteration runs
 * once per iteration for the whole batch, over a work list of tiles of all
 * scenes, and the iterations are replayed from one CUDA graph; each scene
 * stops on its own stopping rule, and its reductions are its own (per
 * scene, in a fixed order for a given batch): its result matches its
 * single-scene solve up to the grouping of its dot-product partials. Replaces a loop of macpressuresolver3::project calls over
 * independent scenes. Scenes belong to `ctx`; the batch refers to them (it
 * does not own them) and keeps their per-scene state (warm start, volume
 * correction). params->solver must be GBP_SOLVER_MGPCG. */
typedef struct gbp_batch gbp_batch;
int gbp_batch_create(gbp_ctx *ctx, int count, gbp_scene *const *scenes, gbp_batch **out);
void gbp_batch_destroy(gbp_batch *batch);
/* DEVICE arrays, one per scene (dt per scene); stats may be NULL or hold
 * `count` entries. Returns GBP_OK, or the first scene's non-OK status. */
int gbp_batch_project_device(gbp_batch *batch, const double *dt, const float *const *solid,
                             const float *const *fluid, float *const *u, float *const *v, float *const *w,
                             const gbp_params *params, float *const *pressure, gbp_stats *stats, void *stream);

/* Operator and right-hand side as assembled on the device, copied to host
 * arrays (each nx*ny*nz doubles): diagonal, coupling weight of each cell's
 * +x/+y/+z face (the negated off-diagonal, 0 unless both cells are
 * unknowns), and b. For checking the assembly against the reference
 * (macpressuresolver3.cpp:163-199). cz may be NULL in 2D. */
int gbp_debug_assemble(gbp_scene *scene, double dt, const float *solid, const float *fluid, const float *u,
                       const float *v, const float *w, const gbp_params *params, double *diag, double *cx,
                       double *cy, double *cz, double *b);

/* Test hook for the bounded device waits (no counterpart in the reference):
 * in the scene's next MGPCG solve, block `block` of the kernels named by
 * `what` leaves out its part -- GBP_WAIT_GRID_BARRIER: its arrival at the
 * grid-wide barriers of the cooperative coarse-level kernels;
 * GBP_WAIT_TILE: the copies of its first tile in the TMA-staged fine-level
 * kernels (gbp_params.tma_staging) -- and every bounded wait polls at most
 * `polls` times (1..2^24; the defaults are 2^24 and 2^22 polls, about a
 * second). The waits of the other blocks (or of that block) then run out,
 * the kernels record it and return, and the solve returns GBP_ERR_CUDA with
 * a message naming the wait; the context stays usable and the next solve
 * runs normally. Nothing faults and nothing waits without a limit. */
#define GBP_WAIT_GRID_BARRIER 1
#define GBP_WAIT_TILE 2
int gbp_debug_fail_wait(gbp_scene *scene, int what, int block, int polls);

/* Benchmark hook: times `reps` back-to-back launches of one kernel on the
 * scene's last assembled system with CUDA events on `stream` (NULL = the
 * context's stream), after one untimed launch. which: GBP_KERNEL_*. Writes
 * the mean milliseconds per launch and the algorithmic DRAM bytes one launch
 * moves (compulsory traffic over the dense grid). The scene's solver vectors
 * are overwritten; the next gbp_project recomputes them. No counterpart in
 * the reference (its timers are per phase, src/core/scoped_timer.cpp). */
#define GBP_KERNEL_CG_SPMV 0
#define GBP_KERNEL_CG_UPDATE 1
#define GBP_KERNEL_CG_DIRECTION 2
/* multigrid kernels on the fine level of the scene's last MGPCG solve */
#define GBP_KERNEL_MG_PRESMOOTH 10
#define GBP_KERNEL_MG_SWEEP 11
#define GBP_KERNEL_MG_RESTRICT 12
#define GBP_KERNEL_MG_POST_BLACK 13
#define GBP_KERNEL_MG_RED_DOT 14
/* CG kernels of the scene's last MGPCG solve (FP64, or FP32 inner) */
#define GBP_KERNEL_PCG_DIRECTION 15
#define GBP_KERNEL_PCG_SPMV 16
#define GBP_KERNEL_PCG_UPDATE 17
int gbp_bench_kernel(gbp_scene *scene, int which, int reps, void *stream, float *ms_per_launch,
                     double *bytes_per_launch);

/* Allocation-free projection, for callers that cannot call cudaMalloc: a
 * host whose device memory comes from its own allocator or a pool sized up
 * front, a plugin in a process that forbids further device allocations, or
 * a per-step path that must never reach the allocator. It is the plain FP64
 * CG projection of gbp_project_device (the reference's solver), but keeps
 * its scratch -- operator, CG vectors, reduction partials and scalars -- in
 * one static device array of GBP_STATIC_SCRATCH_BYTES that every GPU loading
 * the library holds until exit, and calls no cudaMalloc, cudaFree or
 * allocating library routine. Inputs and outputs are the caller's DEVICE
 * arrays, as for gbp_project_device; `stream` is a cudaStream_t (NULL = the
 * legacy default stream) and the call returns once the work is done.
 * At most GBP_STATIC_MAX_CELLS cells (larger grids return
 * GBP_ERR_INVALID_ARGUMENT; gbp_strerror gives the reason); params->solver
 * must be GBP_SOLVER_CG with GBP_PRECISION_FP64, and warm start and volume
 * correction are not available (they need a scene's state). Every call
 * looks up the array's device address on the current device (the host-side
 * name of a __device__ array is not a device address); the first call on a
 * device also loads the library's module there, so make that first call
 * before any stream capture on that device. Every call shares the one
 * array, which keeps the last call's contents: calls that overlap on the
 * GPU race, so callers must serialise them. No counterpart in the reference,
 * whose projection allocates on the host on every call. */
#define GBP_STATIC_MAX_CELLS 32768
#define GBP_STATIC_SCRATCH_BYTES (2400 * 1024)
int gbp_project_device_static(int dim, int nx, int ny, int nz, double dx, double dt, const float *solid,
                              const float *fluid, float *u, float *v, float *w, const gbp_params *params,
                              float *pressure, gbp_stats *stats, void *stream);

/* MAC advection, the neighbouring step of the projection in a smoke time
 * step: replaces the reference's advection module
 *   macadvection3_interface::advect_scalar / advect_vector
 *     include/shiokaze/advection/macadvection3_interface.h:52-72
 *   as implemented by src/advection/macadvection3.cpp:38-54 (advect_cell
 *   :234-282, advect_u :136-180) with bilinear interpolation (WENO off),
 * called in macsmoke3::idle's order (src/smoke/macsmoke3.cpp:270-281): the
 * cell scalar q, if not NULL, is carried by u, v, w; then, if
 * advect_velocity, u, v, w are carried by themselves. Results equal the
 * reference's bit for bit. Every face of the velocity is active (a smoke
 * velocity); q is active where q_mask is nonzero (all cells if q_mask is
 * NULL) and reads q_bg elsewhere, where it is also written as q_bg.
 * fluid is the cell level set that decides the narrow band in which the
 * MacCormack limiter falls back to the forward value. Arrays are dense, x
 * fastest, shapes as for gbp_project; at least 2 cells per edge. */
typedef struct gbp_advect_params {
    int maccormack;      /* "MacCormack" key: 1 (default) MacCormack, 0 one semi-Lagrangian pass */
    int trim_narrowband; /* "TrimNarrowBand" key (default 1) */
    int advect_velocity; /* 1 (default): also advect u, v, w by themselves */
} gbp_advect_params;
void gbp_advect_params_default(gbp_advect_params *p);
/* DEVICE arrays, on `stream` (NULL = the context's stream, ordered after the
 * legacy default stream); returns when the step has finished. */
int gbp_advect3_device(gbp_ctx *ctx, int nx, int ny, int nz, double dx, double dt, const gbp_advect_params *params,
                       float *u, float *v, float *w, const float *fluid, float *q, const unsigned char *q_mask,
                       float q_bg, void *stream);
/* HOST arrays, copied in and out on the context's stream. */
int gbp_advect3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, double dt, const gbp_advect_params *params, float *u,
                float *v, float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg);
/* The 2D step: replaces macadvection2_interface::advect_scalar /
 * advect_vector (include/shiokaze/advection/macadvection2_interface.h:
 * 52-71) as implemented by src/advection/macadvection2.cpp (bilinear), in
 * macsmoke2's order (src/smoke/macsmoke2.cpp:244-254). u (nx+1)*ny,
 * v nx*(ny+1), fluid and q nx*ny, x fastest; otherwise as gbp_advect3. */
int gbp_advect2_device(gbp_ctx *ctx, int nx, int ny, double dx, double dt, const gbp_advect_params *params, float *u,
                       float *v, const float *fluid, float *q, const unsigned char *q_mask, float q_bg, void *stream);
int gbp_advect2(gbp_ctx *ctx, int nx, int ny, double dx, double dt, const gbp_advect_params *params, float *u,
                float *v, const float *fluid, float *q, const unsigned char *q_mask, float q_bg);

/* Solid constraint of the velocity, the step after the projection in the
 * liquid and smoke solvers (src/liquid/macliquid3.cpp:316,
 * src/smoke/macsmoke3.cpp:294): replaces
 *   macutility3_interface::constrain_velocity(solid, velocity)
 *     include/shiokaze/utility/macutility3_interface.h
 *   as implemented by src/utility/macutility3.cpp:61-86.
 * If the nodal solid level set has a negative value, every active face
 * inside the solid (interpolated solid < 0) loses the velocity's component
 * into the solid (the saved velocity, interpolated at the face, minus its
 * projection on the solid gradient, when that projection is negative), and
 * faces on the domain walls keep no outflow. Results equal the reference's
 * bit for bit. solid is nodal (nx+1)(ny+1)(nz+1); u, v, w in/out, holding
 * the velocity's background (0) on inactive faces; mu, mv, mw mark the
 * active faces (NULL: all). The reference tests for a negative solid value
 * over the solid array's active values; this call over all values (the
 * same answer for a narrow-band level set). */
int gbp_constrain_velocity3_device(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid, float *u,
                                   float *v, float *w, const unsigned char *mu, const unsigned char *mv,
                                   const unsigned char *mw, void *stream);
int gbp_constrain_velocity3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid, float *u, float *v,
                            float *w, const unsigned char *mu, const unsigned char *mv, const unsigned char *mw);

/* Extrapolation of an array into its inactive cells: replaces
 *   array_extrapolator3::extrapolate(array, count)
 *     include/shiokaze/array/array_extrapolator3.h:36-73
 *   as the reference's tiled array runs it (array3::dilate,
 *   src/array/dilate3.h:43-95).
 * `count` rounds; each activates every inactive in-bounds 6-neighbour of an
 * active cell with the float mean of its active neighbours (summed in the
 * order +x, -x, +y, -y, -z, +z), all values of a round computed from the
 * state before it. a (w*h*d floats, x fastest) and active (1 = active) are
 * in/out; *activated (may be NULL) receives the number of cells activated,
 * the count the reference returns. Results equal the reference's bit for
 * bit. */
int gbp_extrapolate3_device(gbp_ctx *ctx, int w, int h, int d, float *a, unsigned char *active, int count,
                            long long *activated, void *stream);
int gbp_extrapolate3(gbp_ctx *ctx, int w, int h, int d, float *a, unsigned char *active, int count,
                     long long *activated);

/* The velocity extrapolated by `width` rounds, component by component, then
 * the solid constraint: replaces
 *   macutility3_interface::extrapolate_and_constrain_velocity(solid, velocity, width)
 *   as implemented by src/utility/macutility3.cpp:88-92
 *   (macarray_extrapolator3::extrapolate, macarray_extrapolator3.h:44-48,
 *   then constrain_velocity over the grown active set).
 * HOST arrays as for gbp_constrain_velocity3, inactive faces holding 0;
 * mu, mv, mw mark the active faces and are updated to the grown sets (all
 * three NULL: every face is active and only the constraint acts). Results
 * equal the reference's bit for bit. */
int gbp_extrapolate_constrain_velocity3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid,
                                        float *u, float *v, float *w, unsigned char *mu, unsigned char *mv,
                                        unsigned char *mw, int width);

/* Number of kernel launches this context has issued (graph nodes count one
 * each). */
long long gbp_launch_count(gbp_ctx *ctx);

const char *gbp_strerror(int status);

#ifdef __cplusplus
}
#endif

#endif /* GBP_H */
