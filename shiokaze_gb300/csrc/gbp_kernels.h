// gbp_kernels.h -- host-side launch functions of libgbp's kernels.
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

struct SetupParams {
    double eps_solid, eps_fluid;
    int second_order_solid, second_order_fluid;
    double rhs_correct;  // volume-correction constant added to every row's b
};

// Operator arrays of one grid level, in precision T.
template <class T> struct Operator {
    const T *diag, *cx, *cy, *cz;  // cz == cy in 2D (never read)
};

// Per-face results of the face-first assembly, one array per face
// direction, sized like that direction's face velocities.
struct FaceArrays {
    float *rho[3];   // rho of open faces, -1 if only rho closes the face, 0 if area == 0
    float *area[3];  // open (solid) fraction, 0 on the domain boundary
    // written only where the cell pass cannot form them from rho, area and
    // the face velocity: the weight dt*area/(dx^2 rho) of an open face that
    // is not area = rho = 1, the flux area*u/dx of a face with 0 < area and
    // not (area = 1 with dx a power of two)
    double *w[3];
    double *q[3];
};

// Level-0 arrays of a multigrid hierarchy that the fused 3D assembly writes
// with the FP64 operator: the mixed solver's FP32 operator and inverse
// diagonal, or the FP64 hierarchy's inverse diagonal (unused ones null).
struct Level0Out {
    float *diag, *inv, *cx, *cy, *cz;
    // the low floats of the FP64 operator against diag, cx, cy, cz (each
    // FP64 value = high + low within 2^-48): the mixed refinement's products
    float *diag_lo, *cx_lo, *cy_lo, *cz_lo;
    double *inv64;
};

// ---- setup (setup_kernels.cu) ------------------------------------------------
// Face-first path: faces, then cells; velocity update from the faces.
// Surface-tension increment of the face velocities, in place (kappa != 0).
cudaError_t launch_surface_tension(const Grid &g, double dt, double dx, const SetupParams &sp, double kappa,
                                   const float *fluid, float *u, float *v, float *w, int grid_blocks,
                                   cudaStream_t stream);
cudaError_t launch_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                         const float *fluid, const float *u, const float *v, const float *w, FaceArrays fa,
                         int grid_blocks, cudaStream_t stream);
// The cell pass; also writes level 0 of the hierarchy o names (null
// pointers: nothing).
cudaError_t launch_assemble_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *fluid,
                                  const float *u, const float *v, const float *w, FaceArrays fa, double *diag,
                                  double *cx, double *cy, double *cz, double *b, Level0Out o, Scalars *sc,
                                  int grid_blocks, cudaStream_t stream);
cudaError_t launch_velocity_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *p,
                                  FaceArrays fa, float *u, float *v, float *w, const Scalars *sc, int grid_blocks,
                                  cudaStream_t stream);
// Active sets the reference leaves: unknown cells (diag != 0) and the faces
// its velocity update keeps active; on the velocity before the update.
cudaError_t launch_active_sets(const Grid &g, FaceArrays fa, const float *fluid, const float *u, const float *v,
                               const float *w, const double *diag, unsigned char *unknown, unsigned char *on_u,
                               unsigned char *on_v, unsigned char *on_w, const Scalars *sc, int grid_blocks,
                               cudaStream_t stream);
// Single-pass path (per cell, fractions recomputed per cell).
cudaError_t launch_assemble(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                            const float *fluid, const float *u, const float *v, const float *w, double *diag,
                            double *cx, double *cy, double *cz, double *b, Scalars *sc, int grid_blocks,
                            cudaStream_t stream);
cudaError_t launch_pressure(const Grid &g, const double *diag, const double *x, const double *prev, float *p,
                            double *keep, int grid_blocks, cudaStream_t stream);
cudaError_t launch_velocity(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                            const float *fluid, const float *p, float *u, float *v, float *w, const Scalars *sc,
                            int grid_blocks, cudaStream_t stream);

// ---- plain CG in FP64 (cg_kernels.cu) ---------------------------------------
// r = b - A prev (prev may be NULL), x = 0, s = r; stopping threshold.
cudaError_t launch_cg_init(const Grid &g, Operator<double> A, const double *b, const double *prev, double *x,
                           double *r, double *s, Scalars *sc, Partials *pt, double residual, int max_iter,
                           int grid_blocks, cudaStream_t stream);
// One CG iteration: z = A s; alpha; x += alpha s; r -= alpha z; stop test;
// beta; s = r + beta s. Three launches; all return at once after the stop.
cudaError_t launch_cg_iteration(const Grid &g, Operator<double> A, double *x, double *r, double *s, double *z,
                                Scalars *sc, Partials *pt, int grid_blocks, cudaStream_t stream);
// The three launches of an iteration, one at a time (benchmarking).
cudaError_t launch_cg_spmv(const Grid &g, Operator<double> A, const double *s, double *z, Scalars *sc, Partials *pt,
                           int grid_blocks, cudaStream_t stream);
cudaError_t launch_cg_update(const Grid &g, double *x, double *r, const double *s, const double *z, Scalars *sc,
                             Partials *pt, int grid_blocks, cudaStream_t stream);
cudaError_t launch_cg_direction(const Grid &g, const double *r, double *s, const Scalars *sc, int grid_blocks,
                                cudaStream_t stream);
// |b - A (x + prev)|_inf and _2, |b - A prev|_2 into sc->aux[0..2].
cudaError_t launch_true_residual(const Grid &g, Operator<double> A, const double *b, const double *x,
                                 const double *prev, Scalars *sc, Partials *pt, int grid_blocks,
                                 cudaStream_t stream);

}  // namespace gbp
