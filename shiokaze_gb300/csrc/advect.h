// advect.h -- the MAC advection step on the GPU: the engine behind
// gbp_advect3 / gbp_advect3_device, the drop-in for the reference's
// macadvection3 module (src/advection/macadvection3.cpp: advect_scalar
// :38-45 and advect_vector :47-54 with bilinear interpolation) in the order
// macsmoke3::idle calls them (src/smoke/macsmoke3.cpp:270-281): a scalar
// carried by the velocity, then the velocity carried by itself.
#pragma once

#include <cuda_runtime.h>

#include "advect_core.cuh"

namespace gbp {

// Device scratch of the advection step, grown on demand and kept between
// calls: the forward values and the limiter's bounds of the faces and cells.
struct AdvectWork {
    long long face_cap = 0, cell_cap = 0;
    float *v0 = nullptr;   // forward velocity, the three face arrays back to back
    gba::MinMax *vmm = nullptr;  // limiter record per face
    float *q0 = nullptr;   // forward scalar
    gba::MinMax *qmm = nullptr;  // limiter record per cell
    int *flag = nullptr;         // the solid constraint's levelset_exist flag
    // extrapolation: the second value and mask buffers of a dilation round,
    // and the counter of cells it activated
    long long ext_cap = 0;
    float *ext_a = nullptr;
    unsigned char *ext_m = nullptr;
    unsigned long long *ext_count = nullptr;
};

cudaError_t advect_reserve(AdvectWork &w, long long faces, long long cells);
void advect_release(AdvectWork &w);

struct AdvectArgs {
    int nx, ny, nz;
    double dx, dt;
    int maccormack;       // MacCormack (the reference's default) or one semi-Lagrangian pass
    int trim_narrowband;  // TrimNarrowBand: bands of the fluid level set kept first order
    float *u, *v, *w;     // device face velocities, in/out
    const float *fluid;   // device cell level set
    float *q;             // device cell scalar, in/out (may be NULL: velocity only)
    const unsigned char *q_mask;  // active cells of q (NULL: all)
    float q_bg;           // the value q reads off its active cells
    int velocity;         // also carry u, v, w by themselves (advect_vector)
};

// Enqueues the step on `stream`; *launches counts kernel launches.
cudaError_t advect_run(AdvectWork &w, const AdvectArgs &a, cudaStream_t stream, long long *launches);
// The 2D step (src/advection/macadvection2.cpp, macsmoke2's order): nz and
// w unused, u (nx+1)*ny, v nx*(ny+1), fluid and q nx*ny.
cudaError_t advect_run2(AdvectWork &w, const AdvectArgs &a, cudaStream_t stream, long long *launches);

// The solid constraint of the velocity (macutility3::constrain_velocity,
// src/utility/macutility3.cpp:61-86) on device arrays: solid nodal, u, v, w
// in/out, masks of active faces (NULL: all). Enqueued on `stream`.
struct ConstrainArgs {
    int nx, ny, nz;
    double dx;
    const float *solid;
    float *u, *v, *w;
    const unsigned char *mu, *mv, *mw;
};
cudaError_t constrain_run(AdvectWork &w, const ConstrainArgs &a, cudaStream_t stream, long long *launches);

// array_extrapolator3::extrapolate (include/shiokaze/array/
// array_extrapolator3.h:36-73) on a dense W x H x D device array a with its
// active mask m, as the reference's tiled array runs it (array3::dilate,
// src/array/dilate3.h:43-95): `count` rounds, each activating every
// inactive in-bounds 6-neighbour of an active cell with the float mean of
// its active neighbours, summed in the order +x, -x, +y, -y, -z, +z, all
// computed from the state before the round. One launch per round into the
// second buffers (held in w), then the roles swap; the result ends in a and
// m. When activated_host is not null, the number of cells activated is
// copied there (valid once the stream is synchronised).
cudaError_t extrapolate_run(AdvectWork &w, int W, int H, int D, float *a, unsigned char *m, int count,
                            cudaStream_t stream, long long *launches, unsigned long long *activated_host);

}  // namespace gbp
