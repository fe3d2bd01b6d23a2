// setup_kernels.cu -- face fractions, labelling, operator and right-hand
// side assembly, and the pressure-gradient velocity update.
//
// Built with --fmad=false: every expression here rounds like the reference's
// scalar C++ (no fused multiply-add), so the operator, the right-hand side
// and the velocity update are bit-identical to the reference's given the
// same pressure.
//
// Algorithmic DRAM bytes per cell (3D): assemble reads fluid (4) + solid
// nodes (4) + u,v,w (12) and writes diag, cx, cy, cz, b (40) = 60 B;
// velocity update reads solid (4) + fluid (4) + pressure (4) + u,v,w (12)
// and writes u,v,w (12) = 36 B.
#include <cfloat>
#include <cmath>

#include "gbp_convert.cuh"
#include "gbp_exact.cuh"
#include "gbp_internal.cuh"
#include "gbp_kernels.h"

namespace gbp {
namespace {

// utility::fraction, include/shiokaze/utility/utility.h:162-170.
__device__ double fraction(double phi0, double phi1) {
    if (phi0 * phi1 >= 0.0) {
        if (phi0 < 0.0 || phi1 < 0.0) return 1.0;
        return 0.0;
    }
    double mn = phi0 < phi1 ? phi0 : phi1;
    double d = fabs(phi1 - phi0);
    return -mn / (d > DBL_MIN ? d : DBL_MIN);
}

// utility::get_area, utility.h:179-214: area of {phi < 0} in the unit square
// with corner values v0..v3 at (0,0),(1,0),(1,1),(0,1): the marching-squares
// polygon (corners inside, then edge crossings, in corner order) and its
// shoelace area.
__device__ double solid_area(double v0, double v1, double v2, double v3) {
    // Uniform squares: no corner inside gives an empty polygon (area 0);
    // all four inside give the unit square (shoelace sum 2, area 1). Both
    // are what the general path computes, exactly.
    if (v0 >= 0.0 && v1 >= 0.0 && v2 >= 0.0 && v3 >= 0.0) return 0.0;
    if (v0 < 0.0 && v1 < 0.0 && v2 < 0.0 && v3 < 0.0) return 1.0;
    const double v[4] = {v0, v1, v2, v3};
    const double qx[4] = {0.0, 1.0, 1.0, 0.0};
    const double qy[4] = {0.0, 0.0, 1.0, 1.0};
    double px[8], py[8];
    int pnum = 0;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        const int m = (n + 1) & 3;
        if (v[n] < 0.0) {
            px[pnum] = qx[n];
            py[pnum] = qy[n];
            pnum++;
        }
        if (v[n] * v[m] < 0) {
            double y0 = v[n], y1 = v[m];
            if (y0 - y1) {
                double a = y0 / (y0 - y1);
                px[pnum] = (1.0 - a) * qx[n] + a * qx[m];
                py[pnum] = (1.0 - a) * qy[n] + a * qy[m];
                pnum++;
            }
        }
    }
    double sum = 0.0;
    for (int q = 0; q < pnum; ++q) {
        int r = (q + 1 == pnum) ? 0 : q + 1;
        sum += px[q] * py[r] - py[q] * px[r];
    }
    return 0.5 * sum;
}

struct FaceParams {
    double eps_solid, eps_fluid;
    int second_order_solid, second_order_fluid;
    // When dx is a power of two, 1/dx and 1/dx^2 are exact, and x/dx and
    // x*(1/dx) are both the correctly rounded value of the same real number:
    // multiplying gives the bit-identical result without an FP64 division.
    int dx_pow2;
    double inv_dx, inv_dx2;
    double w_unit;  // dt*1/(dx*dx*1), the weight of a face with area = rho = 1 (host-evaluated)
    int inv_dx_exp;  // 1/dx = 2^inv_dx_exp when dx_pow2
    double dt_inv_dx;  // dt * (1/dx), exact when dx_pow2
    // eps_solid <= 1 (eps_fluid <= 1): a fraction of exactly 0 or 1 is never
    // clamped, so uniform faces skip the FP64 clamp and conversion
    int eps_solid_le1, eps_fluid_le1;
    // w_sum[n]: 0 + w_unit + ... + w_unit (n terms) in FP64, the diagonal
    // of a cell whose n open faces all have area = rho = 1; inv_sum[n] its
    // reciprocal (host-evaluated, the same IEEE operations)
    double w_sum[7], inv_sum[7];
    // the FP32 level-0 operator of such a cell, from the same conversions
    // the kernel applies (host-evaluated): sum_hi[n] = d2f_rn(w_sum[n]),
    // sum_lo[n] = split_lo(w_sum[n], sum_hi[n]), sum_inv[n] = 1 / sum_hi[n]
    // rounded to nearest (0 for n = 0), unit_hi / unit_lo the pair of w_unit
    float sum_hi[7], sum_lo[7], sum_inv[7];
    float unit_hi, unit_lo;
    // dt for the velocity update's dt dp / dx by integer instructions
    // (gbp_exact.cuh), with 1/dx as its power of two
    MulConst dt_mul;
};

// a[n] for n in [0, 7) by selects (an indexed kernel parameter would be
// copied to local memory)
template <class T> __device__ __forceinline__ T pick7(const T (&a)[7], int n) {
    T r = a[0];
#pragma unroll
    for (int q = 1; q < 7; ++q) r = n == q ? a[q] : r;
    return r;
}

// x / dx, bit-identical either way (see FaceParams::dx_pow2)
__device__ __forceinline__ double div_dx(double x, double dx, const FaceParams &fp) {
    return fp.dx_pow2 ? x * fp.inv_dx : x / dx;
}

// dt * area / (dx * dx * rho), as the reference evaluates it
// (macpressuresolver3.cpp:185); with rho == 1, dx*dx*rho == dx*dx exactly.
__device__ __forceinline__ double face_weight(double dt, double area, double rho, double dx, const FaceParams &fp) {
    const double num = dt * area;
    if (fp.dx_pow2 && rho == 1.0) return num * fp.inv_dx2;
    return num / (dx * dx * rho);
}

// face_weight and the flux area*u/dx of a cut face, not inlined (see
// area3_fp64): the same operations as face_weight and div_dx.
__device__ __noinline__ double face_weight_fp64(double dt, float area, float rho, double dx, int dx_pow2,
                                                double inv_dx2) {
    const double num = dt * (double)area;
    if (dx_pow2 && (double)rho == 1.0) return num * inv_dx2;
    return num / (dx * dx * (double)rho);
}
__device__ __noinline__ double face_flux_fp64(float area, float uf, double dx, int dx_pow2, double inv_dx) {
    const double x = (double)area * (double)uf;
    return dx_pow2 ? x * inv_dx : x / dx;
}

// face_area of an interior 3D face from its four corner levels (q00, q10,
// q11, q01 in the corner order of face_area).
// The FP64 tail of area3 (a cut square, or eps_solid above 1): not inlined,
// so that the compiler cannot issue its FP64 instructions speculatively for
// the uniform squares that return early.
__device__ __noinline__ float area3_fp64(float q00, float q10, float q11, float q01, bool uniform, double eps_solid,
                                         int second_order_solid) {
    double area = uniform ? 1.0 : 1.0 - solid_area(q00, q10, q11, q01);
    if (area && area < eps_solid) area = eps_solid;
    float a = (float)area;
    if (!second_order_solid && a) a = 1.0f;  // macpressuresolver3.cpp:76-80
    return a;
}

__device__ __forceinline__ float area3(float q00, float q10, float q11, float q01, const FaceParams &fp) {
    // uniform squares decided in float (the same comparisons as in double);
    // their fraction (1 or 0) is final unless eps_solid exceeds 1
    if (q00 >= 0.0f && q10 >= 0.0f && q11 >= 0.0f && q01 >= 0.0f) {
        if (fp.eps_solid_le1) return 1.0f;
        return area3_fp64(q00, q10, q11, q01, true, fp.eps_solid, fp.second_order_solid);
    }
    if (q00 < 0.0f && q10 < 0.0f && q11 < 0.0f && q01 < 0.0f) return 0.0f;
    return area3_fp64(q00, q10, q11, q01, false, fp.eps_solid, fp.second_order_solid);
}

// Open (non-solid) fraction of face (i,j,k) normal to d
// (src/utility/macutility3.cpp:117-143; 2D macutility2.cpp:100-105).
// Domain-boundary faces read 0; their value never reaches the outputs.
__device__ float face_area(const Grid &g, const float *__restrict__ solid, int d, int i, int j, int k,
                           const FaceParams &fp) {
    const int p[3] = {i, j, k};
    const int n[3] = {g.nx, g.ny, g.nz};
    double area;
    if (p[d] == 0 || p[d] == n[d]) {
        return 0.0f;  // 0 is never clamped, and the first-order override keeps it
    } else if (g.dim == 3) {
        const long long sx = g.nx + 1, sxy = sx * (g.ny + 1);
        auto S = [&](int a, int b, int c) { return __ldg(solid + a + sx * b + sxy * c); };
        float q00, q10, q11, q01;
        if (d == 0) {
            q00 = S(i, j, k); q10 = S(i, j + 1, k); q11 = S(i, j + 1, k + 1); q01 = S(i, j, k + 1);
        } else if (d == 1) {
            q00 = S(i, j, k); q10 = S(i + 1, j, k); q11 = S(i + 1, j, k + 1); q01 = S(i, j, k + 1);
        } else {
            q00 = S(i, j, k); q10 = S(i + 1, j, k); q11 = S(i + 1, j + 1, k); q01 = S(i, j + 1, k);
        }
        return area3(q00, q10, q11, q01, fp);
    } else {
        const long long sx = g.nx + 1;
        double s0 = __ldg(solid + i + sx * j);
        double s1 = d == 0 ? __ldg(solid + i + sx * (j + 1)) : __ldg(solid + (i + 1) + sx * j);
        area = 1.0 - fraction(s0, s1);
    }
    if (area && area < fp.eps_solid) area = fp.eps_solid;
    float a = (float)area;
    if (!fp.second_order_solid && a) a = 1.0f;  // macpressuresolver3.cpp:76-80
    return a;
}

// face_rho of a face between cells of levels f0 and f1, with fluid present.
// The FP64 tail of rho_of (a cut face, or eps_fluid above 1), not inlined
// (see area3_fp64).
__device__ __noinline__ float rho_fp64(float f0, float f1, bool uniform, double eps_fluid, int second_order_fluid) {
    double rho = uniform ? 1.0 : fraction(f0, f1);
    if (rho && rho < eps_fluid) rho = eps_fluid;
    float r = (float)rho;
    if (!second_order_fluid && r) r = 1.0f;  // macpressuresolver3.cpp:70-74
    return r;
}

__device__ __forceinline__ float rho_of(float f0, float f1, const FaceParams &fp) {
    // Same sign (or a zero): fraction() returns 1 or 0. The double product
    // of two floats never underflows to 0, so its sign test equals this
    // float sign test.
    if (!((f0 < 0.0f && f1 > 0.0f) || (f0 > 0.0f && f1 < 0.0f))) {
        // 1 or 0, final unless eps_fluid exceeds 1
        const bool wet = f0 < 0.0f || f1 < 0.0f;
        if (!wet || fp.eps_fluid_le1) {
            float r = wet ? 1.0f : 0.0f;
            if (!fp.second_order_fluid && r) r = 1.0f;
            return r;
        }
        return rho_fp64(f0, f1, true, fp.eps_fluid, fp.second_order_fluid);
    }
    return rho_fp64(f0, f1, false, fp.eps_fluid, fp.second_order_fluid);
}

// Liquid fraction of face (i,j,k) normal to d, between the clamped cells
// (i,j,k) and (i,j,k)-e_d (macutility3.cpp:178-184). With no fluid anywhere
// the reference fills every fraction with 1 (macutility3.cpp:190-192).
__device__ float face_rho(const Grid &g, const float *__restrict__ fluid, int d, int i, int j, int k,
                          const FaceParams &fp, int fluid_exists) {
    float r;
    if (!fluid_exists) {
        r = 1.0f;
    } else {
        int a0 = min(max(i, 0), g.nx - 1), a1 = min(max(j, 0), g.ny - 1), a2 = min(max(k, 0), g.nz - 1);
        int b0 = min(max(i - (d == 0), 0), g.nx - 1), b1 = min(max(j - (d == 1), 0), g.ny - 1),
            b2 = min(max(k - (d == 2), 0), g.nz - 1);
        const float f0 = __ldg(fluid + a0 + (long long)g.nx * (a1 + (long long)g.ny * a2));
        const float f1 = __ldg(fluid + b0 + (long long)g.nx * (b1 + (long long)g.ny * b2));
        return rho_of(f0, f1, fp);
    }
    if (!fp.second_order_fluid && r) r = 1.0f;  // macpressuresolver3.cpp:70-74
    return r;
}

__device__ __forceinline__ long long face_index(const Grid &g, int d, int i, int j, int k) {
    const long long fx = g.nx + (d == 0), fy = g.ny + (d == 1);
    return i + fx * (j + fy * (long long)k);
}

// Curvature of cell (i, j, k) as the surface-tension term computes it
// (macpressuresolver3.cpp:93-101, macpressuresolver2.cpp:79-88): the level
// set at the clamped neighbours summed in float in the order -x, +x, -y,
// +y[, -z, +z], then minus 6 (4 in 2D) times the cell's value in double,
// over dx^2, rounded to float as the reference stores it.
__device__ float st_curvature(const Grid &g, const float *__restrict__ fluid, int i, int j, int k, double dx) {
    auto F = [&](int a, int b, int c) {
        a = min(max(a, 0), g.nx - 1);
        b = min(max(b, 0), g.ny - 1);
        c = min(max(c, 0), g.nz - 1);
        return __ldg(fluid + a + (long long)g.nx * (b + (long long)g.ny * c));
    };
    float s = F(i - 1, j, k) + F(i + 1, j, k);
    s = s + F(i, j - 1, k);
    s = s + F(i, j + 1, k);
    double value;
    if (g.dim == 3) {
        s = s + F(i, j, k - 1);
        s = s + F(i, j, k + 1);
        value = ((double)s - 6.0 * (double)F(i, j, k)) / (dx * dx);
    } else {
        value = ((double)s - 4.0 * (double)F(i, j, k)) / (dx * dx);
    }
    return (float)value;
}

// Surface tension (macpressuresolver3.cpp:85-115, macpressuresolver2.cpp:
// 76-105), in place on the face velocities before anything reads them:
// every face with 0 < rho < 1 gets -sgn dt/(dx rho) kappa face_c added, sgn
// the sign of the level set on the face's + side, theta = rho (1 - rho for
// sgn < 0) and face_c = theta c+ + (1 - theta) c- from the curvatures of the
// two cells; the increment is rounded to float and added in float, as the
// reference's iterator increment does.
__global__ void __launch_bounds__(BLOCK_THREADS) surface_tension_kernel(Grid g, double dt, double dx, double kappa,
                                                                        FaceParams fp, const float *__restrict__ fluid,
                                                                        float *u, float *v, float *w) {
    const long long NX = g.nx + 1, NY = g.ny + 1, NZ = g.dim == 3 ? g.nz + 1 : 1;
    const long long total = NX * NY * NZ;
    float *vel[3] = {u, v, w};
    const int n[3] = {g.nx, g.ny, g.nz};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_coords(g, t, i, j, k);
        const int pi[3] = {i, j, k};
        for (int d = 0; d < g.dim; ++d) {
            bool exists = true;
            for (int e = 0; e < g.dim; ++e)
                if (e != d && pi[e] >= n[e]) exists = false;
            if (!exists) continue;
            const double rho = face_rho(g, fluid, d, i, j, k, fp, 1);
            if (!(rho && rho < 1.0)) continue;
            const int a0 = min(max(i, 0), g.nx - 1), a1 = min(max(j, 0), g.ny - 1), a2 = min(max(k, 0), g.nz - 1);
            const int b0 = min(max(i - (d == 0), 0), g.nx - 1), b1 = min(max(j - (d == 1), 0), g.ny - 1),
                      b2 = min(max(k - (d == 2), 0), g.nz - 1);
            const float fa = __ldg(fluid + a0 + (long long)g.nx * (a1 + (long long)g.ny * a2));
            const double sgn = fa < 0.0 ? -1.0 : 1.0;
            const double theta = sgn < 0 ? 1.0 - rho : rho;
            const double face_c = theta * (double)st_curvature(g, fluid, a0, a1, a2, dx) +
                                  (1.0 - theta) * (double)st_curvature(g, fluid, b0, b1, b2, dx);
            const float inc = (float)(-sgn * dt / (dx * rho) * kappa * face_c);
            const long long f = face_index(g, d, i, j, k);
            vel[d][f] = vel[d][f] + inc;
        }
    }
}

// One thread per cell: labels the cell, assembles its row of the operator
// and its right-hand side (macpressuresolver3.cpp:121-199,
// macpressuresolver2.cpp:111-179). A cell is an unknown iff it is fluid and
// has a fluid in-bounds neighbour across a face with area > 0 and rho > 0;
// since that neighbour is then an unknown too, the +d coupling of a cell is
// that face's weight whenever both cells are fluid and the face is open.
__global__ void __launch_bounds__(BLOCK_THREADS) assemble_kernel(
    Grid g, double dt, double dx, FaceParams fp, double rhs_correct, const float *__restrict__ solid,
    const float *__restrict__ fluid, const float *__restrict__ u, const float *__restrict__ v,
    const float *__restrict__ w, double *__restrict__ diag, double *__restrict__ cx, double *__restrict__ cy,
    double *__restrict__ cz, double *__restrict__ b, Scalars *sc) {
    __shared__ unsigned long long sh_count[BLOCK_THREADS / 32];
    const int tx = threadIdx.x & (TILE_X - 1), ty = threadIdx.x / TILE_X;
    unsigned long long my_count = 0;
    int my_fluid = 0;
    const float *vel[3] = {u, v, w};
    double *cp[3] = {cx, cy, cz};
    for (long long t = blockIdx.x; t < g.ntiles; t += gridDim.x) {
        int i0, j0, k0;
        tile_origin(g, t, i0, j0, k0);
        const int i = i0 + tx, j = j0 + ty;
        if (i >= g.nx || j >= g.ny) continue;
        for (int kk = 0; kk < g.tz; ++kk) {
            const int k = k0 + kk;
            if (k >= g.nz) break;
            const long long c = cell_index(g, i, j, k);
            const float fc = __ldg(fluid + c);
            double dg = 0.0, rhs = 0.0, cpl[3] = {0.0, 0.0, 0.0};
            bool unknown = false;
            if (fc < 0.0f) {
                my_fluid = 1;
                const int n[3] = {g.nx, g.ny, g.nz};
                for (int nq = 0; nq < 2 * g.dim; ++nq) {
                    const int d = nq >> 1;
                    const bool plus = (nq & 1) == 0;
                    const int sgn = plus ? 1 : -1;
                    int q[3] = {i, j, k};
                    q[d] += sgn;
                    if (q[d] < 0 || q[d] >= n[d]) continue;
                    int f[3] = {i, j, k};
                    if (plus) f[d] += 1;
                    const double area = face_area(g, solid, d, f[0], f[1], f[2], fp);
                    const float uf = __ldg(vel[d] + face_index(g, d, f[0], f[1], f[2]));
                    if (area) {
                        const double rho = face_rho(g, fluid, d, f[0], f[1], f[2], fp, 1);
                        if (rho) {
                            const double value = face_weight(dt, area, rho, dx, fp);
                            if (__ldg(fluid + cell_index(g, q[0], q[1], q[2])) < 0.0f) {
                                unknown = true;
                                if (plus) cpl[d] = value;
                            }
                            dg += value;
                        }
                        if (g.dim == 3) rhs += div_dx(-sgn * area * (double)uf, dx, fp);
                    }
                    if (g.dim == 2) rhs += div_dx(-sgn * area * (double)uf, dx, fp);
                }
            }
            if (unknown) {
                my_count++;
                if (rhs_correct) rhs += rhs_correct;  // macpressuresolver3.cpp:212-214
            } else {
                dg = 0.0;
                rhs = 0.0;
                cpl[0] = cpl[1] = cpl[2] = 0.0;
            }
            diag[c] = dg;
            b[c] = rhs;
            for (int d = 0; d < g.dim; ++d) cp[d][c] = cpl[d];
        }
    }
    // unknown count and "any fluid" flag
    unsigned long long wsum = my_count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_down_sync(0xffffffffu, wsum, o);
    if ((threadIdx.x & 31) == 0) sh_count[threadIdx.x >> 5] = wsum;
    int any_fluid = __syncthreads_or(my_fluid);
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int q = 0; q < BLOCK_THREADS / 32; ++q) s += sh_count[q];
        if (s) atomicAdd(&sc->unknowns, s);
        if (any_fluid) atomicOr(&sc->fluid_exists, 1);
    }
}

// Float pressure of every cell (0 off the unknowns, macpressuresolver3.cpp:
// 245-248). With warm start the solve found the correction x to the kept
// pressure prev; the result is x + prev (:239-242), which is kept again.
template <bool WARM>
__global__ void __launch_bounds__(BLOCK_THREADS) pressure_kernel(Grid g, const double *__restrict__ diag,
                                                                 const double *__restrict__ x,
                                                                 const double *prev, float *__restrict__ p,
                                                                 double *keep) {
    // WARM (prev != NULL) is a template argument so that the FP64 addition
    // is not issued, predicated off, for every cell of a cold start
    const long long n = g.ncell;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const bool unk = nonzero_bits(__ldg(diag + c));  // diag != 0, as integers
        double xv = unk ? __ldg(x + c) : 0.0;
        if (WARM && unk) xv = xv + prev[c];
        p[c] = d2f_rn(xv);  // (float)xv, by integer instructions
        if (keep) keep[c] = xv;
    }
}

// Velocity update, one thread per node of the (nx+1)(ny+1)(nz+1) lattice,
// handling the x-, y- and z-face with that lower corner
// (macpressuresolver3.cpp:252-268, macpressuresolver2.cpp:221-237). Open
// faces (area > 0, rho > 0) inside the domain get
//   u -= (float)(dt * (float)(p_c - p_{c-e_d}) / (rho * dx));
// domain-boundary faces and closed faces end at 0 (set to 0, or
// deactivated, which reads back as the background 0).
__global__ void __launch_bounds__(BLOCK_THREADS) velocity_kernel(Grid g, double dt, double dx, FaceParams fp,
                                                                 const float *__restrict__ solid,
                                                                 const float *__restrict__ fluid,
                                                                 const float *__restrict__ p, float *__restrict__ u,
                                                                 float *__restrict__ v, float *__restrict__ w,
                                                                 const Scalars *__restrict__ sc) {
    const int fluid_exists = sc->fluid_exists;
    const long long NX = g.nx + 1, NY = g.ny + 1, NZ = g.dim == 3 ? g.nz + 1 : 1;
    const long long total = NX * NY * NZ;
    float *vel[3] = {u, v, w};
    const int n[3] = {g.nx, g.ny, g.nz};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_coords(g, t, i, j, k);
        const int pi[3] = {i, j, k};
        for (int d = 0; d < g.dim; ++d) {
            // face (i,j,k) of dimension d exists if the other indices are cells
            bool exists = true;
            for (int e = 0; e < g.dim; ++e)
                if (e != d && pi[e] >= n[e]) exists = false;
            if (!exists) continue;
            const long long f = face_index(g, d, i, j, k);
            const float area = face_area(g, solid, d, i, j, k, fp);
            const float rho = face_rho(g, fluid, d, i, j, k, fp, fluid_exists);
            float out;
            if (area && rho) {
                if (pi[d] == 0 || pi[d] == n[d]) {
                    out = 0.0f;
                } else {
                    int m[3] = {i, j, k};
                    m[d] -= 1;
                    const float pc = __ldg(p + cell_index(g, i, j, k));
                    const float pm = __ldg(p + cell_index(g, m[0], m[1], m[2]));
                    const float dp = pc - pm;
                    // rho * dx == dx exactly when rho == 1
                    const double val = rho == 1.0f ? div_dx(dt * (double)dp, dx, fp)
                                                   : dt * (double)dp / ((double)rho * dx);
                    out = vel[d][f] - (float)val;
                }
            } else {
                out = 0.0f;
            }
            vel[d][f] = out;
        }
    }
}


// ---- face-first assembly ----------------------------------------------------------
//
// Pass 1, one thread per node of the (nx+1)(ny+1)(nz+1) lattice, for the x-,
// y- and z-face with that lower corner: the face's fractions, computed once
// per face, stored as
//   rho  = rho if the face is open (area > 0, rho > 0), -1 if area > 0 but
//          rho == 0, 0 if area == 0
//   area = the open fraction
// and, only where pass 2 cannot form them from these and the face velocity
// (cut faces, or dx not a power of two), the FP64 weight dt*area/(dx*dx*rho)
// and flux area*u/dx. Pass 2, one thread per cell, forms its row from its
// faces in the reference's order (+x, -x, +y, -y, +z, -z): weight w_unit on
// faces with area = rho = 1, flux u 2^k when area = 1 and 1/dx = 2^k (an
// exact double), and the sums in integers where they are exact
// (gbp_exact.cuh), so diag, couplings and b are bit-identical to the
// single-pass assemble_kernel (and to the reference); it also writes level 0
// of the multigrid hierarchy (the FP32 operator of the mixed solver, or the
// FP64 inverse diagonal) from the same registers.
// DIM is a template argument: the 3D instantiation holds no FP64 code of
// the 2D path, which the compiler would otherwise issue predicated off for
// every node (a predicated-off FP64 instruction still takes its FP64-pipe
// slot on this GPU).
// Faces whose fractions need the FP64 forms (a cut square, a cut face,
// eps above 1) are few and scattered: one per warp would take the warp
// through the FP64 path with one lane active, and on this GPU every FP64
// warp instruction costs its pipe slots however few lanes it has. The 3D
// kernel therefore queues them in shared memory and computes them
// together, a full warp at a time, when the queue fills and at the end.
constexpr int FACE_QUEUE = 1024;
struct FaceQueue {
    long long f[FACE_QUEUE];
    float q[4][FACE_QUEUE];  // the square's corners (area3's order)
    float fa[FACE_QUEUE], fb[FACE_QUEUE], uf[FACE_QUEUE];
    unsigned char tag[FACE_QUEUE];  // d | interior << 2
};

// area3 needs area3_fp64 (corners neither all >= 0 with eps_solid <= 1
// nor all < 0)
__device__ __forceinline__ bool area3_slow(float q00, float q10, float q11, float q01, const FaceParams &fp) {
    if (q00 >= 0.0f && q10 >= 0.0f && q11 >= 0.0f && q01 >= 0.0f) return !fp.eps_solid_le1;
    return !(q00 < 0.0f && q10 < 0.0f && q11 < 0.0f && q01 < 0.0f);
}
// rho_of needs rho_fp64 (a cut face, or a wet face with eps_fluid > 1)
__device__ __forceinline__ bool rho_slow(float f0, float f1, const FaceParams &fp) {
    if ((f0 < 0.0f && f1 > 0.0f) || (f0 > 0.0f && f1 < 0.0f)) return true;
    return (f0 < 0.0f || f1 < 0.0f) && !fp.eps_fluid_le1;
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK_THREADS) faces_kernel(Grid g, double dt, double dx, FaceParams fp,
                                                              const float *__restrict__ solid,
                                                              const float *__restrict__ fluid,
                                                              const float *__restrict__ u,
                                                              const float *__restrict__ v,
                                                              const float *__restrict__ w, FaceArrays fa) {
    const long long NX = g.nx + 1, NY = g.ny + 1, NZ = g.dim == 3 ? g.nz + 1 : 1;
    const long long total = NX * NY * NZ;
    const float *vel[3] = {u, v, w};
    const int n[3] = {g.nx, g.ny, g.nz};
    // One face's outputs from its fractions and velocity.
    auto emit = [&](int d, long long f, float area, float rho, float uf) {
        const bool open = area && rho;
        fa.rho[d][f] = open ? rho : (area ? -1.0f : 0.0f);
        fa.area[d][f] = area;
        // the FP64 weight and flux only where the cell pass cannot form them
        if (open && !(area == 1.0f && rho == 1.0f))
            fa.w[d][f] = face_weight_fp64(dt, area, rho, dx, fp.dx_pow2, fp.inv_dx2);
        if (area != 0.0f && !(area == 1.0f && fp.dx_pow2)) fa.q[d][f] = face_flux_fp64(area, uf, dx, fp.dx_pow2, fp.inv_dx);
    };
    __shared__ FaceQueue Q;
    __shared__ int qn;
    if (threadIdx.x == 0) qn = 0;
    __syncthreads();
    // the queued faces, a thread each; the fractions by the same functions
    // the direct path uses
    auto flush = [&]() {
        __syncthreads();
        const int cnt = qn;
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int d = Q.tag[e] & 3;
            const float area = (Q.tag[e] >> 2) ? area3(Q.q[0][e], Q.q[1][e], Q.q[2][e], Q.q[3][e], fp) : 0.0f;
            emit(d, Q.f[e], area, rho_of(Q.fa[e], Q.fb[e], fp), Q.uf[e]);
        }
        __syncthreads();
        if (threadIdx.x == 0) qn = 0;
        __syncthreads();
    };
    // block-uniform trip count (the queue's flushes are block-wide)
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total; base += (long long)gridDim.x * blockDim.x) {
        const long long t = base + threadIdx.x;
        // room for this iteration's faces (at most 3 per thread): the barrier's
        // OR includes the last pusher's own reading, which is the count
        if (DIM == 3 && __syncthreads_or(qn > FACE_QUEUE - 3 * BLOCK_THREADS)) flush();
        if (t >= total) continue;
        int i, j, k;
        node_coords(g, t, i, j, k);
        if constexpr (DIM == 3) {
            // The node's three faces with every load issued first (the
            // per-face form waits for each face's loads in turn: its stores
            // could alias the next face's inputs). A face exists when its
            // other two indices are cells; its area comes from its corners
            // unless it lies on the domain boundary (area 0).
            const bool ci = i < g.nx, cj = j < g.ny, ck = k < g.nz;
            const bool ex[3] = {cj && ck, ci && ck, ci && cj};
            const bool in[3] = {ex[0] && i > 0 && ci, ex[1] && j > 0 && cj, ex[2] && k > 0 && ck};
            const long long sx = NX, sxy = NX * NY;
            const float *s0 = solid + i + sx * j + sxy * k;
            const float S000 = (in[0] || in[1] || in[2]) ? __ldg(s0) : 0.0f;
            const float S010 = (in[0] || in[2]) ? __ldg(s0 + sx) : 0.0f;
            const float S001 = (in[0] || in[1]) ? __ldg(s0 + sxy) : 0.0f;
            const float S011 = in[0] ? __ldg(s0 + sx + sxy) : 0.0f;
            const float S100 = (in[1] || in[2]) ? __ldg(s0 + 1) : 0.0f;
            const float S101 = in[1] ? __ldg(s0 + 1 + sxy) : 0.0f;
            const float S110 = in[2] ? __ldg(s0 + 1 + sx) : 0.0f;
            // the face's cells, clamped as face_rho clamps them
            const int a0 = min(i, g.nx - 1), a1 = min(j, g.ny - 1), a2 = min(k, g.nz - 1);
            const long long ca = cell_index(g, a0, a1, a2);
            const bool any = ex[0] || ex[1] || ex[2];
            const float fA = any ? __ldg(fluid + ca) : 0.0f;
            const float fB0 = ex[0] ? __ldg(fluid + cell_index(g, min(max(i - 1, 0), g.nx - 1), a1, a2)) : 0.0f;
            const float fB1 = ex[1] ? __ldg(fluid + cell_index(g, a0, min(max(j - 1, 0), g.ny - 1), a2)) : 0.0f;
            const float fB2 = ex[2] ? __ldg(fluid + cell_index(g, a0, a1, min(max(k - 1, 0), g.nz - 1))) : 0.0f;
            long long f[3];
            float uf[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                f[d] = face_index(g, d, i, j, k);
                uf[d] = ex[d] ? __ldg(vel[d] + f[d]) : 0.0f;
            }
            // fractions of 0 or 1 here; a face that needs the FP64 forms is
            // queued with its inputs
            auto face = [&](int d, float q00, float q10, float q11, float q01, float fB) {
                if (in[d] ? area3_slow(q00, q10, q11, q01, fp) || rho_slow(fA, fB, fp) : rho_slow(fA, fB, fp)) {
                    const int e = atomicAdd(&qn, 1);
                    Q.f[e] = f[d];
                    Q.q[0][e] = q00;
                    Q.q[1][e] = q10;
                    Q.q[2][e] = q11;
                    Q.q[3][e] = q01;
                    Q.fa[e] = fA;
                    Q.fb[e] = fB;
                    Q.uf[e] = uf[d];
                    Q.tag[e] = (unsigned char)(d | (in[d] ? 4 : 0));
                    return;
                }
                emit(d, f[d], in[d] ? area3(q00, q10, q11, q01, fp) : 0.0f, rho_of(fA, fB, fp), uf[d]);
            };
            if (ex[0]) face(0, S000, S010, S011, S001, fB0);
            if (ex[1]) face(1, S000, S100, S101, S001, fB1);
            if (ex[2]) face(2, S000, S100, S110, S010, fB2);
        } else {
            const int pi[3] = {i, j, k};
            for (int d = 0; d < 2; ++d) {
                bool exists = true;
                for (int e = 0; e < 2; ++e)
                    if (e != d && pi[e] >= n[e]) exists = false;
                if (!exists) continue;
                const long long f = face_index(g, d, i, j, k);
                emit(d, f, face_area(g, solid, d, i, j, k, fp), face_rho(g, fluid, d, i, j, k, fp, 1),
                     __ldg(vel[d] + f));
            }
        }
    }
    if (DIM == 3) flush();
}

// The FP64 fallbacks of the cell pass, out of line (see faces_kernel):
// the diagonal as the sequential sum of the open faces' weights, and the
// right-hand side as the sequential sum of -+area*u/dx, in the order +x,
// -x, +y, -y, +z, -z, for a cell the integer forms leave.
__device__ __noinline__ double diag_fp64(const Grid g, const FaceArrays fa, int i, int j, int k, double w_unit) {
    const int n[3] = {g.nx, g.ny, g.nz};
    double dg = 0.0;
    for (int nq = 0; nq < 2 * g.dim; ++nq) {
        const int d = nq >> 1;
        int q[3] = {i, j, k}, f[3] = {i, j, k};
        q[d] += (nq & 1) == 0 ? 1 : -1;
        if (q[d] < 0 || q[d] >= n[d]) continue;
        if ((nq & 1) == 0) f[d] += 1;
        const long long fi = face_index(g, d, f[0], f[1], f[2]);
        const float r = fa.rho[d][fi], a = fa.area[d][fi];
        if (r > 0.0f) dg += (a == 1.0f && r == 1.0f) ? w_unit : fa.w[d][fi];
    }
    return dg;
}
__device__ __noinline__ double rhs_fp64(const Grid g, const FaceArrays fa, const float *u, const float *v,
                                        const float *w, int i, int j, int k, int dx_pow2, double inv_dx) {
    const int n[3] = {g.nx, g.ny, g.nz};
    const float *vel[3] = {u, v, w};
    double rhs = 0.0;
    for (int nq = 0; nq < 2 * g.dim; ++nq) {
        const int d = nq >> 1;
        int q[3] = {i, j, k}, f[3] = {i, j, k};
        q[d] += (nq & 1) == 0 ? 1 : -1;
        if (q[d] < 0 || q[d] >= n[d]) continue;
        if ((nq & 1) == 0) f[d] += 1;
        const long long fi = face_index(g, d, f[0], f[1], f[2]);
        const float a = fa.area[d][fi];
        double qv = 0.0;
        if (a == 1.0f && dx_pow2) qv = (double)vel[d][fi] * inv_dx;  // u / dx, exact
        else if (a != 0.0f) qv = fa.q[d][fi];
        rhs += (nq & 1) == 0 ? -qv : qv;
    }
    return rhs;
}
__device__ __noinline__ double add_fp64(double a, double b) { return a + b; }
__device__ __noinline__ double recip_fp64(double a) { return 1.0 / a; }

// RC: a volume-correction constant is added to every unknown's b (a
// template argument, so that no FP64 addition is issued predicated off).
// Four blocks per SM (64 registers, a few spilled): the pass is bound by
// instruction issue, and more warps measured 40 us faster at 256^3 than
// three blocks at 80 registers.
template <bool RC>
__global__ void __launch_bounds__(BLOCK_THREADS, 4) assemble_faces_kernel(
    Grid g, double dt, double dx, FaceParams fp, double rhs_correct, const float *__restrict__ fluid,
    const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w, FaceArrays fa,
    double *__restrict__ diag, double *__restrict__ cx, double *__restrict__ cy, double *__restrict__ cz,
    double *__restrict__ b, Level0Out o, Scalars *sc) {
    __shared__ unsigned long long sh_count[BLOCK_THREADS / 32];
    const int tx = threadIdx.x & (TILE_X - 1), ty = threadIdx.x / TILE_X;
    unsigned long long my_count = 0;
    int my_fluid = 0;
    double *cp[3] = {cx, cy, cz};
    const float *vel[3] = {u, v, w};
    for (long long t = blockIdx.x; t < g.ntiles; t += gridDim.x) {
        int i0, j0, k0;
        tile_origin(g, t, i0, j0, k0);
        const int i = i0 + tx, j = j0 + ty;
        if (i >= g.nx || j >= g.ny) continue;
        for (int kk = 0; kk < g.tz; ++kk) {
            const int k = k0 + kk;
            if (k >= g.nz) break;
            const long long c = cell_index(g, i, j, k);
            double dg = 0.0, rhs = 0.0, cpl[3] = {0.0, 0.0, 0.0};
            bool unknown = false, unit = true;
            int nopen = 0;
            // every load of the cell's row first (its own level, and per face
            // in the order +x, -x, +y, -y, +z, -z: fraction, area, velocity
            // and the neighbour's level), then the row in that order
            const int n[3] = {g.nx, g.ny, g.nz};
            const float fc = __ldg(fluid + c);
            float fr[6], ar[6], uv[6], fq[6];
            bool has[6];
            // the index of face nq from the cell's: the -x face of cell c is
            // c + j + ny k, the -y face c + nx k, the -z face c; the + faces
            // one step further (face_index, without its multiplications)
            auto findex = [&](int nq) {
                const int d = nq >> 1;
                const long long base = c + (d == 0 ? (long long)j + (long long)g.ny * k
                                                   : (d == 1 ? (long long)g.nx * k : 0ll));
                const long long step = d == 0 ? 1ll : (d == 1 ? (long long)g.nx : (long long)g.nx * g.ny);
                return (nq & 1) == 0 ? base + step : base;
            };
#pragma unroll
            for (int nq = 0; nq < 6; ++nq) {
                const int d = nq >> 1;
                const bool plus = (nq & 1) == 0;
                int q[3] = {i, j, k};
                q[d] += plus ? 1 : -1;
                has[nq] = d < g.dim && q[d] >= 0 && q[d] < n[d];
                const long long fi = has[nq] ? findex(nq) : 0;
                fr[nq] = has[nq] ? __ldg(fa.rho[d] + fi) : 0.0f;
                ar[nq] = has[nq] ? __ldg(fa.area[d] + fi) : 0.0f;
                uv[nq] = has[nq] ? __ldg(vel[d] + fi) : 0.0f;
                fq[nq] = has[nq] ? __ldg(fluid + cell_index(g, q[0], q[1], q[2])) : 0.0f;
            }
            // the weight of an open face
            auto wface = [&](int nq) {
                return (ar[nq] == 1.0f && fr[nq] == 1.0f) ? fp.w_unit : __ldg(fa.w[nq >> 1] + findex(nq));
            };
            if (fc < 0.0f) {
                my_fluid = 1;
                // the right-hand side's terms -+u/dx by face (0 where a face
                // has no term or area 0: adding +-0 changes no sum)
                float terms[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                bool qexact = fp.dx_pow2 != 0;
#pragma unroll
                for (int nq = 0; nq < 6; ++nq) {
                    if (!has[nq]) continue;
                    if (fr[nq] > 0.0f) {  // open face
                        nopen++;
                        unit = unit && ar[nq] == 1.0f && fr[nq] == 1.0f;
                        if (fq[nq] < 0.0f) {
                            unknown = true;
                            if ((nq & 1) == 0) cpl[nq >> 1] = wface(nq);
                        }
                    }
                    if (ar[nq] == 1.0f) terms[nq] = uv[nq];
                    else if (ar[nq] != 0.0f) qexact = false;
                }
                if (unknown) {
                    dg = unit ? pick7(fp.w_sum, nopen) : diag_fp64(g, fa, i, j, k, fp.w_unit);
                    // 0x15: the + faces' terms are negated
                    if (!(qexact && exact_sum(terms, 6, 0x15u, fp.inv_dx_exp, rhs)))
                        rhs = rhs_fp64(g, fa, u, v, w, i, j, k, fp.dx_pow2, fp.inv_dx);
                }
            }
            if (unknown) {
                my_count++;
                if constexpr (RC) rhs = add_fp64(rhs, rhs_correct);  // macpressuresolver3.cpp:212-214
            } else {
                dg = 0.0;
                rhs = 0.0;
                cpl[0] = cpl[1] = cpl[2] = 0.0;
                unit = true;  // the zero row: table entry 0
                nopen = 0;
            }
            diag[c] = dg;
            b[c] = rhs;
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (d < g.dim) cp[d][c] = cpl[d];
            if (o.diag) {
                float d32, i32, x32, y32, z32, dlo, xlo, ylo, zlo;
                if (unit) {
                    // every open face unit (or no unknown: all zero): the
                    // conversions of the table values, computed on the host
                    d32 = pick7(fp.sum_hi, nopen);
                    dlo = pick7(fp.sum_lo, nopen);
                    i32 = pick7(fp.sum_inv, nopen);
                    const bool bx = nonzero_bits(cpl[0]), by = nonzero_bits(cpl[1]), bz = nonzero_bits(cpl[2]);
                    x32 = bx ? fp.unit_hi : 0.0f;
                    xlo = bx ? fp.unit_lo : 0.0f;
                    y32 = by ? fp.unit_hi : 0.0f;
                    ylo = by ? fp.unit_lo : 0.0f;
                    z32 = bz ? fp.unit_hi : 0.0f;
                    zlo = bz ? fp.unit_lo : 0.0f;
                } else {
                    d32 = d2f_rn(dg);
                    x32 = d2f_rn(cpl[0]);
                    y32 = d2f_rn(cpl[1]);
                    z32 = d2f_rn(cpl[2]);
                    i32 = positive_bits(dg) ? __frcp_rn(d32) : 0.0f;
                    dlo = split_lo(dg, d32);
                    xlo = split_lo(cpl[0], x32);
                    ylo = split_lo(cpl[1], y32);
                    zlo = split_lo(cpl[2], z32);
                }
                o.diag[c] = d32;
                o.inv[c] = i32;
                o.cx[c] = x32;
                o.cy[c] = y32;
                if (o.diag_lo) {
                    o.diag_lo[c] = dlo;
                    o.cx_lo[c] = xlo;
                    o.cy_lo[c] = ylo;
                }
                if (g.dim == 3) {
                    o.cz[c] = z32;
                    if (o.diag_lo) o.cz_lo[c] = zlo;
                }
            }
            if (o.inv64) o.inv64[c] = positive_bits(dg) ? (unit ? pick7(fp.inv_sum, nopen) : recip_fp64(dg)) : 0.0;
        }
    }
    unsigned long long wsum = my_count;
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) wsum += __shfl_down_sync(0xffffffffu, wsum, q);
    if ((threadIdx.x & 31) == 0) sh_count[threadIdx.x >> 5] = wsum;
    int any_fluid = __syncthreads_or(my_fluid);
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int q = 0; q < BLOCK_THREADS / 32; ++q) s += sh_count[q];
        if (s) atomicAdd(&sc->unknowns, s);
        if (any_fluid) atomicOr(&sc->fluid_exists, 1);
    }
}

// The new velocity of one face from its stored fraction (fr), the pressures
// on its two sides and its velocity; interior: not on the domain boundary.
// Open faces get u - (float)(dt (pc - pm) / (rho dx)), every other face 0.
__device__ __forceinline__ float face_update(float fr, bool interior, float pc, float pm, float uf,
                                             int fluid_exists, double dt, double dx, const FaceParams &fp) {
    const bool open = fluid_exists ? fr > 0.0f : fr != 0.0f;
    const float rho = fluid_exists ? fr : 1.0f;
    if (!open || !interior) return 0.0f;
    const float dp = pc - pm;
    // rho * dx == dx exactly when rho == 1; (float)(dt dp / dx) by integer
    // instructions where they decide (gbp_exact.cuh)
    float vv;
    if (rho == 1.0f && mul_round(fp.dt_mul, dp, vv)) return uf - vv;
    const double val = rho == 1.0f ? div_dx(dt * (double)dp, dx, fp) : dt * (double)dp / ((double)rho * dx);
    return uf - (float)val;
}

// Velocity update from the stored face fractions (same rule as
// velocity_kernel): open faces inside the domain get the pressure gradient,
// every other face 0; with no fluid anywhere every face with area > 0 is open
// with rho = 1 (macutility3.cpp:190-192).
__global__ void __launch_bounds__(BLOCK_THREADS) velocity_faces_kernel(Grid g, double dt, double dx, FaceParams fp,
                                                                       const float *__restrict__ p, FaceArrays fa,
                                                                       float *__restrict__ u, float *__restrict__ v,
                                                                       float *__restrict__ w,
                                                                       const Scalars *__restrict__ sc) {
    const int fluid_exists = sc->fluid_exists;
    const long long NX = g.nx + 1, NY = g.ny + 1, NZ = g.dim == 3 ? g.nz + 1 : 1;
    const long long total = NX * NY * NZ;
    float *vel[3] = {u, v, w};
    const int n[3] = {g.nx, g.ny, g.nz};
    auto update = [&](float fr, bool interior, float pc, float pm, float uf) {
        return face_update(fr, interior, pc, pm, uf, fluid_exists, dt, dx, fp);
    };
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_coords(g, t, i, j, k);
        const int pi[3] = {i, j, k};
        bool ex[3], in[3];
        long long f[3];
        float fr[3], pm[3], uf[3];
        bool any_in = false;
        // every load of the node's faces first, then the updates (the
        // per-face form waits for each face's loads in turn)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            ex[d] = d < g.dim;
#pragma unroll
            for (int e = 0; e < 3; ++e)
                if (e < g.dim && e != d && pi[e] >= n[e]) ex[d] = false;
            in[d] = ex[d] && pi[d] > 0 && pi[d] < n[d];
            any_in = any_in || in[d];
            f[d] = ex[d] ? face_index(g, d, i, j, k) : 0;
            fr[d] = ex[d] ? __ldg(fa.rho[d] + f[d]) : 0.0f;
            uf[d] = in[d] ? vel[d][f[d]] : 0.0f;
            pm[d] = in[d] ? __ldg(p + cell_index(g, i - (d == 0), j - (d == 1), k - (d == 2))) : 0.0f;
        }
        const float pc = any_in ? __ldg(p + cell_index(g, i, j, k)) : 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (ex[d]) vel[d][f[d]] = update(fr[d], in[d], pc, pm[d], uf[d]);
    }
}

// The active sets the reference leaves behind (macpressuresolver3.cpp:
// 245-266; 2D macpressuresolver2.cpp:214-236), for callers that keep sparse
// arrays: unknown[c] = 1 on the cells whose pressure the reference sets (the
// unknowns, diag != 0 as pressure_kernel decides), on[d][f] = 1 on the faces
// its velocity update keeps active: open faces (area > 0 and rho > 0) and
// closed faces on the domain boundary next to a fluid cell (in 2D only where
// the velocity points out of the domain: u < 0 on the low wall, u > 0 on the
// high one). Every other face is deactivated (set_off) by the reference.
// Runs before the velocity update, on the velocity it is given.
__global__ void __launch_bounds__(BLOCK_THREADS) active_sets_kernel(Grid g, FaceArrays fa,
                                                                    const float *__restrict__ fluid,
                                                                    const float *__restrict__ u,
                                                                    const float *__restrict__ v,
                                                                    const float *__restrict__ w,
                                                                    const double *__restrict__ diag,
                                                                    unsigned char *__restrict__ unknown,
                                                                    unsigned char *on0, unsigned char *on1,
                                                                    unsigned char *on2,
                                                                    const Scalars *__restrict__ sc) {
    const int fluid_exists = sc->fluid_exists;
    const long long NX = g.nx + 1, NY = g.ny + 1, NZ = g.dim == 3 ? g.nz + 1 : 1;
    const long long total = NX * NY * NZ;
    const float *vel[3] = {u, v, w};
    unsigned char *on[3] = {on0, on1, on2};
    const int n[3] = {g.nx, g.ny, g.nz};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_coords(g, t, i, j, k);
        const int pi[3] = {i, j, k};
        if (i < g.nx && j < g.ny && (g.dim == 2 || k < g.nz)) {
            const long long c = cell_index(g, i, j, k);
            unknown[c] = nonzero_bits(__ldg(diag + c)) ? 1 : 0;
        }
        for (int d = 0; d < g.dim; ++d) {
            bool exists = true;
            for (int e = 0; e < g.dim; ++e)
                if (e != d && pi[e] >= n[e]) exists = false;
            if (!exists) continue;
            const long long f = face_index(g, d, i, j, k);
            const float fr = __ldg(fa.rho[d] + f);
            bool keep = fluid_exists ? fr > 0.0f : fr != 0.0f;
            if (!keep && pi[d] == 0) {
                keep = __ldg(fluid + cell_index(g, i, j, k)) < 0.0f && (g.dim == 3 || __ldg(vel[d] + f) < 0.0f);
            } else if (!keep && pi[d] == n[d]) {
                keep = __ldg(fluid + cell_index(g, i - (d == 0), j - (d == 1), k - (d == 2))) < 0.0f &&
                       (g.dim == 3 || __ldg(vel[d] + f) > 0.0f);
            }
            on[d][f] = keep ? 1 : 0;
        }
    }
}

FaceParams face_params(const SetupParams &sp, double dx, double dt) {
    FaceParams fp{sp.eps_solid, sp.eps_fluid, sp.second_order_solid, sp.second_order_fluid, 0, 0.0, 0.0, 0.0, 0, 0.0,
                  0, 0};
    fp.eps_solid_le1 = sp.eps_solid <= 1.0;
    fp.eps_fluid_le1 = sp.eps_fluid <= 1.0;
    int e = 0;
    const double m = std::frexp(dx, &e);
    if (m == 0.5 && e > -500 && e < 500) {  // dx == 2^(e-1)
        fp.dx_pow2 = 1;
        fp.inv_dx = std::ldexp(1.0, 1 - e);
        fp.inv_dx_exp = 1 - e;
        fp.dt_inv_dx = dt * fp.inv_dx;  // a power-of-two scaling: exact
        fp.inv_dx2 = std::ldexp(1.0, 2 * (1 - e));
    }
    // the device's face_weight(dt, 1, 1, dx) evaluated here with the same
    // IEEE operations (no additions, so no contraction can change it)
    const double num = dt * 1.0;
    volatile double denom = dx * dx;
    fp.w_unit = fp.dx_pow2 ? num * fp.inv_dx2 : num / (denom * 1.0);
    volatile double acc = 0.0;
    for (int n = 0; n < 7; ++n) {
        fp.w_sum[n] = acc;
        fp.inv_sum[n] = n ? 1.0 / acc : 0.0;
        fp.sum_hi[n] = d2f_rn(fp.w_sum[n]);
        fp.sum_lo[n] = split_lo(fp.w_sum[n], fp.sum_hi[n]);
        volatile float one = 1.0f;
        fp.sum_inv[n] = n ? one / fp.sum_hi[n] : 0.0f;  // IEEE division: __frcp_rn's value
        acc = acc + fp.w_unit;
    }
    fp.unit_hi = d2f_rn(fp.w_unit);
    fp.unit_lo = split_lo(fp.w_unit, fp.unit_hi);
    fp.dt_mul = make_mul_const(dt, fp.dx_pow2 ? fp.inv_dx_exp : 0);
    fp.dt_mul.ok = fp.dt_mul.ok && fp.dx_pow2;
    return fp;
}

}  // namespace

cudaError_t launch_assemble(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                            const float *fluid, const float *u, const float *v, const float *w, double *diag,
                            double *cx, double *cy, double *cz, double *b, Scalars *sc, int grid_blocks,
                            cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    int blocks = (int)(g.ntiles < grid_blocks ? g.ntiles : grid_blocks);
    if (blocks < 1) blocks = 1;
    assemble_kernel<<<blocks, BLOCK_THREADS, 0, stream>>>(g, dt, dx, fp, sp.rhs_correct, solid, fluid, u, v, w, diag,
                                                          cx, cy, g.dim == 3 ? cz : cy, b, sc);
    return cudaGetLastError();
}

static int node_blocks(const Grid &g, int grid_blocks) {
    const long long total = (long long)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1);
    const long long need = (total + BLOCK_THREADS - 1) / BLOCK_THREADS;
    const long long b = need < grid_blocks ? need : grid_blocks;
    return b < 1 ? 1 : (int)b;
}

cudaError_t launch_surface_tension(const Grid &g, double dt, double dx, const SetupParams &sp, double kappa,
                                   const float *fluid, float *u, float *v, float *w, int grid_blocks,
                                   cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    surface_tension_kernel<<<node_blocks(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, dt, dx, kappa, fp, fluid, u, v,
                                                                                       w);
    return cudaGetLastError();
}

cudaError_t launch_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                         const float *fluid, const float *u, const float *v, const float *w, FaceArrays fa,
                         int grid_blocks, cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    if (g.dim == 3)
        faces_kernel<3><<<node_blocks(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, dt, dx, fp, solid, fluid, u, v, w,
                                                                                   fa);
    else
        faces_kernel<2><<<node_blocks(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, dt, dx, fp, solid, fluid, u, v, w,
                                                                                   fa);
    return cudaGetLastError();
}

cudaError_t launch_assemble_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *fluid,
                                  const float *u, const float *v, const float *w, FaceArrays fa, double *diag,
                                  double *cx, double *cy, double *cz, double *b, Level0Out o, Scalars *sc,
                                  int grid_blocks, cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    int blocks = (int)(g.ntiles < grid_blocks ? g.ntiles : grid_blocks);
    if (blocks < 1) blocks = 1;
    if (sp.rhs_correct != 0.0)
        assemble_faces_kernel<true><<<blocks, BLOCK_THREADS, 0, stream>>>(
            g, dt, dx, fp, sp.rhs_correct, fluid, u, v, g.dim == 3 ? w : v, fa, diag, cx, cy, g.dim == 3 ? cz : cy, b, o,
            sc);
    else
        assemble_faces_kernel<false><<<blocks, BLOCK_THREADS, 0, stream>>>(
            g, dt, dx, fp, sp.rhs_correct, fluid, u, v, g.dim == 3 ? w : v, fa, diag, cx, cy, g.dim == 3 ? cz : cy, b, o,
            sc);
    return cudaGetLastError();
}

cudaError_t launch_velocity_faces(const Grid &g, double dt, double dx, const SetupParams &sp, const float *p,
                                  FaceArrays fa, float *u, float *v, float *w, const Scalars *sc, int grid_blocks,
                                  cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    velocity_faces_kernel<<<node_blocks(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, dt, dx, fp, p, fa, u, v, w, sc);
    return cudaGetLastError();
}

cudaError_t launch_active_sets(const Grid &g, FaceArrays fa, const float *fluid, const float *u, const float *v,
                               const float *w, const double *diag, unsigned char *unknown, unsigned char *on_u,
                               unsigned char *on_v, unsigned char *on_w, const Scalars *sc, int grid_blocks,
                               cudaStream_t stream) {
    active_sets_kernel<<<node_blocks(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, fa, fluid, u, v, w, diag, unknown,
                                                                                  on_u, on_v, on_w, sc);
    return cudaGetLastError();
}

cudaError_t launch_pressure(const Grid &g, const double *diag, const double *x, const double *prev, float *p,
                            double *keep, int grid_blocks, cudaStream_t stream) {
    long long need = (g.ncell + BLOCK_THREADS - 1) / BLOCK_THREADS;
    int blocks = (int)(need < grid_blocks ? need : grid_blocks);
    if (blocks < 1) blocks = 1;
    if (prev) pressure_kernel<true><<<blocks, BLOCK_THREADS, 0, stream>>>(g, diag, x, prev, p, keep);
    else pressure_kernel<false><<<blocks, BLOCK_THREADS, 0, stream>>>(g, diag, x, prev, p, keep);
    return cudaGetLastError();
}

cudaError_t launch_velocity(const Grid &g, double dt, double dx, const SetupParams &sp, const float *solid,
                            const float *fluid, const float *p, float *u, float *v, float *w, const Scalars *sc,
                            int grid_blocks, cudaStream_t stream) {
    const FaceParams fp = face_params(sp, dx, dt);
    long long total = (long long)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1);
    long long need = (total + BLOCK_THREADS - 1) / BLOCK_THREADS;
    int blocks = (int)(need < grid_blocks ? need : grid_blocks);
    if (blocks < 1) blocks = 1;
    velocity_kernel<<<blocks, BLOCK_THREADS, 0, stream>>>(g, dt, dx, fp, solid, fluid, p, u, v, w, sc);
    return cudaGetLastError();
}

}  // namespace gbp
