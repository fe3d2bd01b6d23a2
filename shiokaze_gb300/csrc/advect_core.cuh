// advect_core.cuh -- per-face and per-cell arithmetic of the MAC advection
// step (MacCormack or semi-Lagrangian, trilinear interpolation), shared by
// the kernels in advect_kernels.cu.
//
// It follows src/advection/macadvection3.cpp (WENO off, the module's
// default) with the reference's types, so that every result rounds as the
// reference's scalar C++ does (the including translation unit is compiled
// with --fmad=false):
//   face trace   (i,j,k) - dt*u/dx with u a float vector: dt*u and /dx are
//                each rounded to float, the difference taken in double
//                (advect_semiLagrangian_u, :82-89)
//   min/max      the same trace in double, the eight interpolation corners'
//                min/max from DBL_MAX / DBL_MIN, and the narrow-band test
//                on the fluid level set at the traced face position
//                (:97-131)
//   cell trace   (i,j,k) - dt*u/dx in double (:188-203); min/max from
//                FLT_MAX / FLT_MIN (:212-227)
//   correction   0.5*(float)(in - backward), clamped to [min, max] outside
//                the narrow band (:150-167, :256-269)
//   interpolation include/shiokaze/array/array_interpolator3.h:50-104:
//                clamp to the array, corner weights as products of the three
//                axis weights, skip zero weights, accumulate in float with
//                double products
//   full vectors  include/shiokaze/array/macarray3.h:305-371: the other two
//                components at a face as the mean of four clamped faces
//                (double sum / 4), at a cell as 0.5*(lo + hi) faces
// Every face of the velocity is active (the smoke scene's velocity,
// src/smoke/macsmoke3.cpp:115); a scalar's inactive cells read its
// background value.
#pragma once

#include <cfloat>
#include <cmath>

#ifdef __CUDACC__
#define GBA_HD __host__ __device__ __forceinline__
// out of line on the device: the compiler cannot issue the FP64 work of a
// rare path speculatively (predicated off) for every element
#define GBA_HD_OUTLINE __host__ __device__ __noinline__
#else
#define GBA_HD inline
#define GBA_HD_OUTLINE inline
#endif

namespace gba {

struct Shape {
    int w, h, d;
};

struct Dims {
    int nx, ny, nz;
    double dx;      // grid spacing
    double inv_dx;  // 1/dx; used only when dx is a power of two (then exact)
    float inv_dx_f;
    int pow2;       // dx is a power of two: divisions by dx are exact multiplications
    double limit;   // -dx * TrimNarrowBand
};

GBA_HD Shape face_shape(const Dims &g, int dim) {
    return Shape{g.nx + (dim == 0), g.ny + (dim == 1), g.nz + (dim == 2)};
}

GBA_HD long long at(const Shape &s, int i, int j, int k) {
    return (long long)i + (long long)s.w * ((long long)j + (long long)s.h * k);
}

// std::min / std::max with the reference's argument order
GBA_HD double smin(double a, double b) { return (b < a) ? b : a; }
GBA_HD double smax(double a, double b) { return (a < b) ? b : a; }

// corner of the interpolation cell and the three axis positions
// (array_interpolator3::interpolate_coef, array_interpolator3.h:50-73)
struct Corner {
    int i, j, k;
    double x, y, z;
};

GBA_HD Corner corner(const Shape &s, double px, double py, double pz) {
    Corner c;
    c.x = smax(0.0, smin(s.w - 1., px));
    c.y = smax(0.0, smin(s.h - 1., py));
    c.z = smax(0.0, smin(s.d - 1., pz));
    c.i = (int)smin(c.x, s.w - 2.);
    c.j = (int)smin(c.y, s.h - 2.);
    c.k = (int)smin(c.z, s.d - 2.);
    return c;
}

// array_interpolator3::interpolate<float> (:86-104) of a dense float array;
// Read(x) returns the array's value at a flat index.
template <class Read>
GBA_HD float interp(const Shape &s, double px, double py, double pz, Read read) {
    const Corner c = corner(s, px, py, pz);
    const double ax0 = c.i + 1 - c.x, ax1 = c.x - c.i;
    const double ay0 = c.j + 1 - c.y, ay1 = c.y - c.j;
    const double az0 = c.k + 1 - c.z, az1 = c.z - c.k;
    // coef[n] = az * ax * ay, multiplied left to right as the reference does
    const double zx00 = az0 * ax0, zx01 = az0 * ax1, zx10 = az1 * ax0, zx11 = az1 * ax1;
    const double coef[8] = {zx00 * ay0, zx01 * ay0, zx00 * ay1, zx01 * ay1,
                            zx10 * ay0, zx11 * ay0, zx10 * ay1, zx11 * ay1};
    const long long base = at(s, c.i, c.j, c.k);
    const long long sy = s.w, sz = (long long)s.w * s.h;
    const long long off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
    float value = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n)
        if (coef[n]) value = (float)((double)value + (double)read(base + off[n]) * coef[n]);
    return value;
}

// min and max of the eight corners' values (the MacCormack limiter's
// bounds), starting from `lo0` and `hi0`. The reference compares in double
// from DBL_MAX / DBL_MIN (faces) or FLT_MAX / FLT_MIN (cells); the same
// comparisons on the floats themselves give the same answers (a float's
// double image is exact and ordered alike), and the double start values are
// replaced by floats with the same outcome: DBL_MAX by +inf (only +inf and
// NaN fail `v < start`, and DBL_MAX rounds to +inf in the end), DBL_MIN by
// +0 (`DBL_MIN < v` holds for a float v exactly when `0 < v`, and DBL_MIN
// rounds to +0). So the whole search runs on FP32, bit-exact.
template <class Read>
GBA_HD void corner_minmax(const Shape &s, double px, double py, double pz, float lo0, float hi0, Read read,
                          float &lo, float &hi) {
    const Corner c = corner(s, px, py, pz);
    const long long base = at(s, c.i, c.j, c.k);
    const long long sy = s.w, sz = (long long)s.w * s.h;
    const long long off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
    float l = lo0, h = hi0;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float v = read(base + off[n]);
        l = (v < l) ? v : l;
        h = (h < v) ? v : h;
    }
    lo = l;
    hi = h;
}

// How interp(s, p, a) compares with `limit`: -1 below, 1 above, 0 equal,
// 2 unordered (NaN). The eight corners' range [mn, mx] usually decides it:
// the weights are nonnegative and sum to 1 within 16 double ulps, and each
// of the eight float accumulations of interp rounds by at most 2^-24 of a
// partial sum bounded by M = max|a|, so the interpolant lies in
// [mn - d, mx + d] for d = 2^-20 M + 1e-38 (twice the bound, plus the
// subnormal spacing eight times over). When the limit falls inside that
// band, or a value is not finite, the interpolant itself is compared;
// either way the answer is the reference's.
GBA_HD int compare_interp(const Shape &s, double px, double py, double pz, const float *a, double limit) {
    const Corner c = corner(s, px, py, pz);
    const long long base = at(s, c.i, c.j, c.k);
    const long long sy = s.w, sz = (long long)s.w * s.h;
    const long long off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
    float v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = a[base + off[n]];
    float mn = v[0], mx = v[0], sum = v[0];
#pragma unroll
    for (int n = 1; n < 8; ++n) {
        mn = v[n] < mn ? v[n] : mn;
        mx = mx < v[n] ? v[n] : mx;
        sum += v[n];
    }
    if (sum - sum == 0.0f) {  // every value finite (a NaN or an infinity makes this false)
        const float am = (-mn < mx) ? mx : -mn;
        const double d = (double)am * 9.5367431640625e-07 + 1e-38;
        if ((double)mx + d < limit) return -1;
        if ((double)mn - d > limit) return 1;
    }
    // the interpolant, as interp forms it (same corner, weights and order)
    const double ax0 = c.i + 1 - c.x, ax1 = c.x - c.i;
    const double ay0 = c.j + 1 - c.y, ay1 = c.y - c.j;
    const double az0 = c.k + 1 - c.z, az1 = c.z - c.k;
    const double zx00 = az0 * ax0, zx01 = az0 * ax1, zx10 = az1 * ax0, zx11 = az1 * ax1;
    const double coef[8] = {zx00 * ay0, zx01 * ay0, zx00 * ay1, zx01 * ay1,
                            zx10 * ay0, zx11 * ay0, zx10 * ay1, zx11 * ay1};
    float value = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n)
        if (coef[n]) value = (float)((double)value + (double)v[n] * coef[n]);
    const double x = value;
    return x < limit ? -1 : (x > limit ? 1 : (x == limit ? 0 : 2));
}

// interp(s, p, a) > limit, the narrow-band test
GBA_HD bool above_limit(const Shape &s, double px, double py, double pz, const float *a, double limit) {
    return compare_interp(s, px, py, pz, a, limit) == 1;
}

// the full velocity at face (i,j,k) of component `dim` (macarray3.h:350-371):
// its own component, and each other component as the mean of the four faces
// around it, indices clamped to that component's shape
GBA_HD void face_full(const Dims &g, const float *const comp[3], int dim, int i, int j, int k, float u[3]) {
    const int pi[3] = {i - (dim == 0), j - (dim == 1), k - (dim == 2)};
#pragma unroll
    for (int ud = 0; ud < 3; ++ud) {
        if (ud == dim) {
            u[ud] = comp[ud][at(face_shape(g, ud), i, j, k)];
            continue;
        }
        const Shape s = face_shape(g, ud);
        double sum = 0.0;
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
            for (int jj = 0; jj < 2; ++jj) {
                int q[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) q[c] = pi[c] + ii * (dim == c) + jj * (ud == c);
                // shape3::clamp (include/shiokaze/math/shape.h:790-797)
                q[0] = q[0] < 0 ? 0 : (q[0] > s.w - 1 ? s.w - 1 : q[0]);
                q[1] = q[1] < 0 ? 0 : (q[1] > s.h - 1 ? s.h - 1 : q[1]);
                q[2] = q[2] < 0 ? 0 : (q[2] > s.d - 1 ? s.d - 1 : q[2]);
                sum += comp[ud][at(s, q[0], q[1], q[2])];
            }
        u[ud] = (float)(sum / 4.0);
    }
}

// the full velocity at cell (i,j,k) (macarray3.h:305-343)
GBA_HD void cell_full(const Dims &g, const float *const comp[3], int i, int j, int k, float u[3]) {
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        const Shape s = face_shape(g, dim);
        double value = 0.0;
        value += comp[dim][at(s, i, j, k)];
        value += comp[dim][at(s, i + (dim == 0), j + (dim == 1), k + (dim == 2))];
        u[dim] = (float)(0.5 * value);
    }
}

// dt*u/dx of one float velocity component as the float vector arithmetic
// forms it: (float)(u*dt), then (float)(t/dx)
GBA_HD float trace_f(const Dims &g, float u, double dt) {
    const float t = (float)((double)u * dt);
    return g.pow2 ? t * g.inv_dx_f : (float)((double)t / g.dx);
}

// u*dt/dx in double
GBA_HD double trace_d(const Dims &g, double u, double dt) {
    return g.pow2 ? (u * dt) * g.inv_dx : (u * dt) / g.dx;
}

// the MacCormack limiter's record for one face or cell: within the narrow
// band (take the forward value) or the [lo, hi] clamp bounds. `within` is
// kept as a NaN in lo: lo is a min over values starting from a finite bound,
// and a NaN never wins std::min's comparison, so lo is never NaN otherwise.
struct alignas(8) MinMax {
    float lo, hi;
};

GBA_HD bool mm_within(const MinMax &m) { return m.lo != m.lo; }

// the final MacCormack value (macadvection3.cpp:150-167, :256-269)
GBA_HD float maccormack(const MinMax &m, float in, float fwd, float bwd) {
    if (mm_within(m)) return fwd;
    const double lo = m.lo, hi = m.hi, x0 = fwd;
    const double corr = 0.5 * (double)(float)(in - bwd);
    if (x0 + corr < lo) return (float)lo;
    if (x0 + corr > hi) return (float)hi;
    return (float)(x0 + corr);
}

GBA_HD float nan_mark() {
    union {
        unsigned u;
        float f;
    } b{0x7fc00000u};
    return b.f;
}

struct Idx {
    int i, j, k;
};

GBA_HD Idx decode(const Shape &s, unsigned f) {
    const unsigned t = f / (unsigned)s.w;
    return Idx{(int)(f - t * (unsigned)s.w), (int)(t % (unsigned)s.h), (int)(t / (unsigned)s.h)};
}

GBA_HD unsigned count(const Shape &s) { return (unsigned)s.w * (unsigned)s.h * (unsigned)s.d; }

// Arguments of the four passes. Face scratch (v0, vmm) holds the three
// components back to back at offsets 0, off1, off2.
struct StepArgs {
    Dims g;
    double dt;
    float *u, *v, *w;  // velocity, in/out
    const float *fluid;
    float *q;  // scalar, in/out
    const unsigned char *mask;
    float bg;
    float *v0;
    MinMax *vmm;
    long long off1, off2;
    float *q0;
    MinMax *qmm;
};

// forward semi-Lagrangian pass at face f of component dim
// (advect_semiLagrangian_u, macadvection3.cpp:70-134): the forward value
// and, for MacCormack, the limiter record
template <bool MAC>
GBA_HD void face_forward(const StepArgs &a, int dim, unsigned f) {
    const Dims &g = a.g;
    const Shape fs = face_shape(g, dim);
    if (f >= count(fs)) return;
    const Idx x = decode(fs, f);
    const int ip[3] = {x.i, x.j, x.k};
    const float *const comp[3] = {a.u, a.v, a.w};
    const float *src = dim == 0 ? a.u : (dim == 1 ? a.v : a.w);
    const long long o = dim == 0 ? 0 : (dim == 1 ? a.off1 : a.off2);
    auto rd = [src](long long n) { return src[n]; };
    float uf[3];
    face_full(g, comp, dim, x.i, x.j, x.k, uf);
    const bool moving = uf[0] != 0.0f || uf[1] != 0.0f || uf[2] != 0.0f;
    float out;
    if (moving) {
        double p[3];
        for (int c = 0; c < 3; ++c) p[c] = (double)ip[c] - (double)trace_f(g, uf[c], a.dt);
        out = interp(fs, p[0], p[1], p[2], rd);
    } else {
        out = src[f];
    }
    a.v0[o + f] = out;
    if (!MAC) return;
    MinMax m;
    double fp[3];
    if (moving) {
        double p[3];
        for (int c = 0; c < 3; ++c) {
            const double disp = trace_d(g, (double)uf[c], a.dt);
            p[c] = (double)ip[c] - disp;
            fp[c] = (ip[c] + 0.5 * (dim != c)) - disp;
        }
        corner_minmax(fs, p[0], p[1], p[2], INFINITY, 0.0f, rd, m.lo, m.hi);  // DBL_MAX, DBL_MIN
    } else {
        for (int c = 0; c < 3; ++c) fp[c] = ip[c] + 0.5 * (dim != c);
        m.lo = m.hi = src[f];
    }
    const Shape cs{g.nx, g.ny, g.nz};
    const float *fl = a.fluid;
    const bool within = above_limit(cs, fp[0] - 0.5, fp[1] - 0.5, fp[2] - 0.5, fl, g.limit);
    if (within) m.lo = nan_mark();
    a.vmm[o + f] = m;
}

// backward pass from the forward values (advect_semiLagrangian_u with -dt)
// and the limited MacCormack correction (macadvection3.cpp:150-167), written
// over the input face (the only read of the input in this pass)
GBA_HD void face_backward(const StepArgs &a, int dim, unsigned f) {
    const Dims &g = a.g;
    const Shape fs = face_shape(g, dim);
    if (f >= count(fs)) return;
    const Idx x = decode(fs, f);
    const int ip[3] = {x.i, x.j, x.k};
    const float *const comp[3] = {a.v0, a.v0 + a.off1, a.v0 + a.off2};
    const float *src = dim == 0 ? comp[0] : (dim == 1 ? comp[1] : comp[2]);
    float *io = dim == 0 ? a.u : (dim == 1 ? a.v : a.w);
    const long long o = dim == 0 ? 0 : (dim == 1 ? a.off1 : a.off2);
    float uf[3];
    face_full(g, comp, dim, x.i, x.j, x.k, uf);
    const bool moving = uf[0] != 0.0f || uf[1] != 0.0f || uf[2] != 0.0f;
    float bwd;
    if (moving) {
        double p[3];
        for (int c = 0; c < 3; ++c) p[c] = (double)ip[c] - (double)trace_f(g, uf[c], -a.dt);
        bwd = interp(fs, p[0], p[1], p[2], [src](long long n) { return src[n]; });
    } else {
        bwd = src[f];
    }
    io[f] = maccormack(a.vmm[o + f], io[f], src[f], bwd);
}

// forward semi-Lagrangian pass at cell c (advect_semiLagrangian_cell,
// macadvection3.cpp:182-232); inactive cells take the background
template <bool MAC>
GBA_HD void cell_forward(const StepArgs &a, unsigned c) {
    const Dims &g = a.g;
    const Shape cs{g.nx, g.ny, g.nz};
    if (c >= count(cs)) return;
    const unsigned char *mask = a.mask;
    const float bg = a.bg;
    if (mask && !mask[c]) {
        a.q0[c] = bg;
        return;
    }
    const Idx x = decode(cs, c);
    const int ip[3] = {x.i, x.j, x.k};
    const float *const comp[3] = {a.u, a.v, a.w};
    const float *q = a.q;
    auto rq = [q, mask, bg](long long n) { return (mask && !mask[n]) ? bg : q[n]; };
    float uc[3];
    cell_full(g, comp, x.i, x.j, x.k, uc);
    const bool moving = uc[0] != 0.0f || uc[1] != 0.0f || uc[2] != 0.0f;
    double p[3] = {0.0, 0.0, 0.0};
    if (moving)
        for (int d = 0; d < 3; ++d) p[d] = (double)ip[d] - trace_d(g, (double)uc[d], a.dt);
    const float qc = q[c];
    a.q0[c] = moving ? interp(cs, p[0], p[1], p[2], rq) : qc;
    if (!MAC) return;
    MinMax m;
    bool within;
    const float *fl = a.fluid;
    if (moving) {
        corner_minmax(cs, p[0], p[1], p[2], FLT_MAX, FLT_MIN, rq, m.lo, m.hi);
        within = above_limit(cs, p[0], p[1], p[2], fl, g.limit);
    } else {
        m.lo = m.hi = qc;
        within = (double)fl[c] > g.limit;
    }
    if (within) m.lo = nan_mark();
    a.qmm[c] = m;
}

// backward pass and limited correction at cell c (macadvection3.cpp:
// 256-269), written over the input scalar (its only read in this pass)
GBA_HD void cell_backward(const StepArgs &a, unsigned c) {
    const Dims &g = a.g;
    const Shape cs{g.nx, g.ny, g.nz};
    if (c >= count(cs)) return;
    if (a.mask && !a.mask[c]) {
        a.q[c] = a.bg;
        return;
    }
    const Idx x = decode(cs, c);
    const int ip[3] = {x.i, x.j, x.k};
    const float *const comp[3] = {a.u, a.v, a.w};
    float uc[3];
    cell_full(g, comp, x.i, x.j, x.k, uc);
    const bool moving = uc[0] != 0.0f || uc[1] != 0.0f || uc[2] != 0.0f;
    const float *q0 = a.q0;
    float bwd;
    if (moving) {
        double p[3];
        for (int d = 0; d < 3; ++d) p[d] = (double)ip[d] - trace_d(g, (double)uc[d], -a.dt);
        bwd = interp(cs, p[0], p[1], p[2], [q0](long long n) { return q0[n]; });
    } else {
        bwd = q0[c];
    }
    a.q[c] = maccormack(a.qmm[c], a.q[c], q0[c], bwd);
}

// ---------------------------------------------------------------------------
// The 2D step, src/advection/macadvection2.cpp (WENO off): the same passes
// on (nx, ny) grids with bilinear interpolation (include/shiokaze/array/
// array_interpolator2.h:50-89: weights (i+1-x)(j+1-y), (x-i)(j+1-y),
// (i+1-x)(y-j), (x-i)(y-j)) and the full vectors of macarray2.h:302-367 (the
// face's other component summed over its four faces with x outer, y inner).
// Every face of the velocity is active (src/smoke/macsmoke2.cpp:106).

struct Shape2 {
    int w, h;
};

GBA_HD Shape2 face_shape2(const Dims &g, int dim) { return Shape2{g.nx + (dim == 0), g.ny + (dim == 1)}; }

GBA_HD long long at2(const Shape2 &s, int i, int j) { return (long long)i + (long long)s.w * j; }

struct Corner2 {
    int i, j;
    double x, y;
};

GBA_HD Corner2 corner2(const Shape2 &s, double px, double py) {
    Corner2 c;
    c.x = smax(0.0, smin(s.w - 1., px));
    c.y = smax(0.0, smin(s.h - 1., py));
    c.i = (int)smin(c.x, s.w - 2.);
    c.j = (int)smin(c.y, s.h - 2.);
    return c;
}

GBA_HD void coef2(const Corner2 &c, double coef[4]) {
    coef[0] = (c.i + 1 - c.x) * (c.j + 1 - c.y);
    coef[1] = (c.x - c.i) * (c.j + 1 - c.y);
    coef[2] = (c.i + 1 - c.x) * (c.y - c.j);
    coef[3] = (c.x - c.i) * (c.y - c.j);
}

// array_interpolator2::interpolate<float> (:77-89)
template <class Read>
GBA_HD float interp2(const Shape2 &s, double px, double py, Read read) {
    const Corner2 c = corner2(s, px, py);
    double coef[4];
    coef2(c, coef);
    const long long base = at2(s, c.i, c.j);
    const long long off[4] = {0, 1, s.w, (long long)s.w + 1};
    float value = 0.0f;
#pragma unroll
    for (int n = 0; n < 4; ++n)
        if (coef[n]) value = (float)((double)value + (double)read(base + off[n]) * coef[n]);
    return value;
}

// the four corners' min and max (see corner_minmax)
template <class Read>
GBA_HD void corner_minmax2(const Shape2 &s, double px, double py, float lo0, float hi0, Read read, float &lo,
                           float &hi) {
    const Corner2 c = corner2(s, px, py);
    const long long base = at2(s, c.i, c.j);
    const long long off[4] = {0, 1, s.w, (long long)s.w + 1};
    float l = lo0, h = hi0;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        const float v = read(base + off[n]);
        l = (v < l) ? v : l;
        h = (h < v) ? v : h;
    }
    lo = l;
    hi = h;
}

// interp2(s, p, a) > limit (the bound of compare_interp holds for four
// corners as for eight)
GBA_HD bool above_limit2(const Shape2 &s, double px, double py, const float *a, double limit) {
    const Corner2 c = corner2(s, px, py);
    const long long base = at2(s, c.i, c.j);
    const long long off[4] = {0, 1, s.w, (long long)s.w + 1};
    float v[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) v[n] = a[base + off[n]];
    float mn = v[0], mx = v[0], sum = v[0];
#pragma unroll
    for (int n = 1; n < 4; ++n) {
        mn = v[n] < mn ? v[n] : mn;
        mx = mx < v[n] ? v[n] : mx;
        sum += v[n];
    }
    if (sum - sum == 0.0f) {
        const float am = (-mn < mx) ? mx : -mn;
        const double d = (double)am * 9.5367431640625e-07 + 1e-38;
        if ((double)mx + d < limit) return false;
        if ((double)mn - d > limit) return true;
    }
    double coef[4];
    coef2(c, coef);
    float value = 0.0f;
#pragma unroll
    for (int n = 0; n < 4; ++n)
        if (coef[n]) value = (float)((double)value + (double)v[n] * coef[n]);
    return (double)value > limit;
}

// the full velocity at face (i,j) of component dim (macarray2.h:347-367)
GBA_HD void face_full2(const Dims &g, const float *const comp[2], int dim, int i, int j, float u[2]) {
    const int ud = 1 - dim;
    const Shape2 s = face_shape2(g, ud);
    const int p0 = i - (dim == 0), p1 = j - (dim == 1);
    double sum = 0.0;
#pragma unroll
    for (int ii = 0; ii < 2; ++ii)
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            int q0 = p0 + ii, q1 = p1 + jj;
            // shape2::clamp
            q0 = q0 < 0 ? 0 : (q0 > s.w - 1 ? s.w - 1 : q0);
            q1 = q1 < 0 ? 0 : (q1 > s.h - 1 ? s.h - 1 : q1);
            sum += comp[ud][at2(s, q0, q1)];
        }
    u[dim] = comp[dim][at2(face_shape2(g, dim), i, j)];
    u[ud] = (float)(sum / 4.0);
}

// the full velocity at cell (i,j) (macarray2.h:302-340)
GBA_HD void cell_full2(const Dims &g, const float *const comp[2], int i, int j, float u[2]) {
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const Shape2 s = face_shape2(g, dim);
        double value = 0.0;
        value += comp[dim][at2(s, i, j)];
        value += comp[dim][at2(s, i + (dim == 0), j + (dim == 1))];
        u[dim] = (float)(0.5 * value);
    }
}

GBA_HD Idx decode2(const Shape2 &s, unsigned f) {
    const unsigned t = f / (unsigned)s.w;
    return Idx{(int)(f - t * (unsigned)s.w), (int)t, 0};
}

GBA_HD unsigned count2(const Shape2 &s) { return (unsigned)s.w * (unsigned)s.h; }

// the 2D passes take StepArgs with w unused and off2 = 0

// forward pass at face f of component dim (advect_semiLagrangian_u,
// macadvection2.cpp:66-131)
template <bool MAC>
GBA_HD void face_forward2(const StepArgs &a, int dim, unsigned f) {
    const Dims &g = a.g;
    const Shape2 fs = face_shape2(g, dim);
    if (f >= count2(fs)) return;
    const Idx x = decode2(fs, f);
    const int ip[2] = {x.i, x.j};
    const float *const comp[2] = {a.u, a.v};
    const float *src = dim == 0 ? a.u : a.v;
    const long long o = dim == 0 ? 0 : a.off1;
    auto rd = [src](long long n) { return src[n]; };
    float uf[2];
    face_full2(g, comp, dim, x.i, x.j, uf);
    const bool moving = uf[0] != 0.0f || uf[1] != 0.0f;
    float out;
    if (moving) {
        double p[2];
        for (int c = 0; c < 2; ++c) p[c] = (double)ip[c] - (double)trace_f(g, uf[c], a.dt);
        out = interp2(fs, p[0], p[1], rd);
    } else {
        out = src[f];
    }
    a.v0[o + f] = out;
    if (!MAC) return;
    MinMax m;
    double fp[2];
    if (moving) {
        double p[2];
        for (int c = 0; c < 2; ++c) {
            const double disp = trace_d(g, (double)uf[c], a.dt);
            p[c] = (double)ip[c] - disp;
            fp[c] = (ip[c] + 0.5 * (dim != c)) - disp;
        }
        corner_minmax2(fs, p[0], p[1], INFINITY, 0.0f, rd, m.lo, m.hi);  // DBL_MAX, DBL_MIN
    } else {
        for (int c = 0; c < 2; ++c) fp[c] = ip[c] + 0.5 * (dim != c);
        m.lo = m.hi = src[f];
    }
    const Shape2 cs{g.nx, g.ny};
    if (above_limit2(cs, fp[0] - 0.5, fp[1] - 0.5, a.fluid, g.limit)) m.lo = nan_mark();
    a.vmm[o + f] = m;
}

// backward pass and the limited correction at face f (macadvection2.cpp:
// 133-165), over the input face
GBA_HD void face_backward2(const StepArgs &a, int dim, unsigned f) {
    const Dims &g = a.g;
    const Shape2 fs = face_shape2(g, dim);
    if (f >= count2(fs)) return;
    const Idx x = decode2(fs, f);
    const int ip[2] = {x.i, x.j};
    const float *const comp[2] = {a.v0, a.v0 + a.off1};
    const float *src = dim == 0 ? comp[0] : comp[1];
    float *io = dim == 0 ? a.u : a.v;
    const long long o = dim == 0 ? 0 : a.off1;
    float uf[2];
    face_full2(g, comp, dim, x.i, x.j, uf);
    const bool moving = uf[0] != 0.0f || uf[1] != 0.0f;
    float bwd;
    if (moving) {
        double p[2];
        for (int c = 0; c < 2; ++c) p[c] = (double)ip[c] - (double)trace_f(g, uf[c], -a.dt);
        bwd = interp2(fs, p[0], p[1], [src](long long n) { return src[n]; });
    } else {
        bwd = src[f];
    }
    io[f] = maccormack(a.vmm[o + f], io[f], src[f], bwd);
}

// forward pass at cell c (advect_semiLagrangian_cell, macadvection2.cpp:
// 167-217); inactive cells take the background
template <bool MAC>
GBA_HD void cell_forward2(const StepArgs &a, unsigned c) {
    const Dims &g = a.g;
    const Shape2 cs{g.nx, g.ny};
    if (c >= count2(cs)) return;
    const unsigned char *mask = a.mask;
    const float bg = a.bg;
    if (mask && !mask[c]) {
        a.q0[c] = bg;
        return;
    }
    const Idx x = decode2(cs, c);
    const int ip[2] = {x.i, x.j};
    const float *const comp[2] = {a.u, a.v};
    const float *q = a.q;
    auto rq = [q, mask, bg](long long n) { return (mask && !mask[n]) ? bg : q[n]; };
    float uc[2];
    cell_full2(g, comp, x.i, x.j, uc);
    const bool moving = uc[0] != 0.0f || uc[1] != 0.0f;
    double p[2] = {0.0, 0.0};
    if (moving)
        for (int d = 0; d < 2; ++d) p[d] = (double)ip[d] - trace_d(g, (double)uc[d], a.dt);
    const float qc = q[c];
    a.q0[c] = moving ? interp2(cs, p[0], p[1], rq) : qc;
    if (!MAC) return;
    MinMax m;
    bool within;
    if (moving) {
        corner_minmax2(cs, p[0], p[1], FLT_MAX, FLT_MIN, rq, m.lo, m.hi);
        within = above_limit2(cs, p[0], p[1], a.fluid, g.limit);
    } else {
        m.lo = m.hi = qc;
        within = (double)a.fluid[c] > g.limit;
    }
    if (within) m.lo = nan_mark();
    a.qmm[c] = m;
}

// backward pass and the limited correction at cell c (macadvection2.cpp:
// 219-249), over the input scalar
GBA_HD void cell_backward2(const StepArgs &a, unsigned c) {
    const Dims &g = a.g;
    const Shape2 cs{g.nx, g.ny};
    if (c >= count2(cs)) return;
    if (a.mask && !a.mask[c]) {
        a.q[c] = a.bg;
        return;
    }
    const Idx x = decode2(cs, c);
    const int ip[2] = {x.i, x.j};
    const float *const comp[2] = {a.u, a.v};
    float uc[2];
    cell_full2(g, comp, x.i, x.j, uc);
    const bool moving = uc[0] != 0.0f || uc[1] != 0.0f;
    const float *q0 = a.q0;
    float bwd;
    if (moving) {
        double p[2];
        for (int d = 0; d < 2; ++d) p[d] = (double)ip[d] - trace_d(g, (double)uc[d], -a.dt);
        bwd = interp2(cs, p[0], p[1], [q0](long long n) { return q0[n]; });
    } else {
        bwd = q0[c];
    }
    a.q[c] = maccormack(a.qmm[c], a.q[c], q0[c], bwd);
}

// ---------------------------------------------------------------------------
// The solid constraint of the velocity, macutility3::constrain_velocity
// (src/utility/macutility3.cpp:61-86), per face.

// array_derivative3::derivative (include/shiokaze/array/array_derivative3.h:
// 51-95, 107-116): the trilinear gradient in index space, every corner
// included, accumulated in float with double products
GBA_HD void derivative(const Shape &s, const double p[3], const float *a, float out[3]) {
    const Corner c = corner(s, p[0], p[1], p[2]);
    const int i = c.i, j = c.j, k = c.k;
    const double x = c.x, y = c.y, z = c.z;
    const double cf[3][8] = {
        {-(k + 1 - z) * (j + 1 - y), (k + 1 - z) * (j + 1 - y), -(k + 1 - z) * (y - j), (k + 1 - z) * (y - j),
         -(z - k) * (j + 1 - y), (z - k) * (j + 1 - y), -(z - k) * (y - j), (z - k) * (y - j)},
        {-(k + 1 - z) * (i + 1 - x), -(k + 1 - z) * (x - i), (k + 1 - z) * (i + 1 - x), (k + 1 - z) * (x - i),
         -(z - k) * (i + 1 - x), -(z - k) * (x - i), (z - k) * (i + 1 - x), (z - k) * (x - i)},
        {-(i + 1 - x) * (j + 1 - y), -(x - i) * (j + 1 - y), -(i + 1 - x) * (y - j), -(x - i) * (y - j),
         (i + 1 - x) * (j + 1 - y), (x - i) * (j + 1 - y), (i + 1 - x) * (y - j), (x - i) * (y - j)}};
    const long long base = at(s, i, j, k);
    const long long sy = s.w, sz = (long long)s.w * s.h;
    const long long off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
    float v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = a[base + off[n]];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float r = 0.0f;
#pragma unroll
        for (int n = 0; n < 8; ++n) r = (float)((double)r + cf[d][n] * (double)v[n]);
        out[d] = r;
    }
}

struct ConstrainArgs {
    Dims g;
    const float *solid;     // nodal level set (nx+1)(ny+1)(nz+1)
    const float *save;      // the input velocity, three components back to back at 0, off1, off2
    long long off1, off2;
    float *u, *v, *w;       // velocity, written where a face changes
    const unsigned char *mu, *mv, *mw;  // active faces (NULL: all)
    const int *exists;      // the solid has a negative value (levelset_exist)
};

// compare_interp(s, p, a, 0.0) from float comparisons alone when the eight
// corners lie clearly on one side of 0: -1 (all below) or 1 (all above),
// else 2 (the full test decides). p2 holds twice the position: whole and
// half nodes, as the faces' positions are. The corners and the float
// min/max/sum are compare_interp's; its range test is decided here when
// |the corner nearest 0| >= max(2^-19 am, 2^-100), am the largest
// magnitude, which exceeds its margin d = 2^-20 am + 1e-38 (so the double
// test gives the same answer).
GBA_HD int sign_corners_fast(const Shape &s, const int p2[3], const float *a) {
    auto cell = [](int v2, int w) {
        v2 = v2 < 0 ? 0 : (v2 > 2 * (w - 1) ? 2 * (w - 1) : v2);
        const int c = v2 >> 1;
        return c < w - 2 ? c : w - 2;
    };
    const int i = cell(p2[0], s.w), j = cell(p2[1], s.h), k = cell(p2[2], s.d);
    const long long base = at(s, i, j, k);
    const long long sy = s.w, sz = (long long)s.w * s.h;
    const long long off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
    float v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = a[base + off[n]];
    float mn = v[0], mx = v[0], sum = v[0];
#pragma unroll
    for (int n = 1; n < 8; ++n) {
        mn = v[n] < mn ? v[n] : mn;
        mx = mx < v[n] ? v[n] : mx;
        sum += v[n];
    }
    if (!(sum - sum == 0.0f)) return 2;
    const float am = (-mn < mx) ? mx : -mn;
    const float margin = am * 0x1p-19f;
    if (mx < 0.0f && -mx >= margin && -mx >= 0x1p-100f) return -1;
    if (mn > 0.0f && mn >= margin && mn >= 0x1p-100f) return 1;
    return 2;
}

// The solid branch of one face (macutility3.cpp:70-80): the saved velocity
// interpolated at the face minus its projection on the solid's gradient
// when that projection is negative; `in` otherwise.
GBA_HD_OUTLINE float constrain_solid(const ConstrainArgs a, int dim, int i, int j, int k, float in, int side) {
    const Dims &g = a.g;
    const int ip[3] = {i, j, k};
    const float *save[3] = {a.save, a.save + a.off1, a.save + a.off2};
    const double p[3] = {ip[0] + 0.5 * (dim != 0), ip[1] + 0.5 * (dim != 1), ip[2] + 0.5 * (dim != 2)};
    float val = in;
    const Shape ns{g.nx + 1, g.ny + 1, g.nz + 1};
    if (side == 2) side = compare_interp(ns, p[0], p[1], p[2], a.solid, 0.0);
    if (side == -1) {
        float dr[3];
        derivative(ns, p, a.solid, dr);
        double nrm[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) nrm[c] = (double)dr[c] / g.dx;
        double n2 = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) n2 += nrm[c] * nrm[c];
        if (n2 != 0.0) {
            // macarray_interpolator3::interpolate (macarray_interpolator3.h:49-56)
            double uu[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float *sc = save[c];
                uu[c] = interp(face_shape(g, c), p[0] - 0.5 * (c != 0), p[1] - 0.5 * (c != 1), p[2] - 0.5 * (c != 2),
                               [sc](long long n) { return sc[n]; });
            }
            double dot = 0.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) dot += uu[c] * nrm[c];
            if (dot < 0.0) val = (float)((dim == 0 ? uu[0] : (dim == 1 ? uu[1] : uu[2])) -
                                         (dim == 0 ? nrm[0] : (dim == 1 ? nrm[1] : nrm[2])) * dot);
        }
    }
    return val;
}

// One face. The reference runs its face loop three times over the same
// saved velocity (macutility3.cpp:68); the loop is idempotent (the solid
// branch sets the same value from the saved velocity each time, and the
// wall clamps are idempotent), so one pass gives its result. Faces whose
// solid corners are all clearly positive skip the FP64 work.
GBA_HD void constrain_face(const ConstrainArgs &a, int dim, unsigned f) {
    const Dims &g = a.g;
    const Shape fs = face_shape(g, dim);
    if (f >= count(fs) || !*a.exists) return;
    const unsigned char *mask = dim == 0 ? a.mu : (dim == 1 ? a.mv : a.mw);
    if (mask && !mask[f]) return;
    const Idx x = decode(fs, f);
    const int ip[3] = {x.i, x.j, x.k};
    const float in = (dim == 0 ? a.save : (dim == 1 ? a.save + a.off1 : a.save + a.off2))[f];
    float val = in;
    const Shape ns{g.nx + 1, g.ny + 1, g.nz + 1};
    const int p2[3] = {2 * ip[0] + (dim != 0), 2 * ip[1] + (dim != 1), 2 * ip[2] + (dim != 2)};
    const int side = sign_corners_fast(ns, p2, a.solid);
    if (side != 1) val = constrain_solid(a, dim, ip[0], ip[1], ip[2], in, side);
    const int n_dim = dim == 0 ? g.nx : (dim == 1 ? g.ny : g.nz);
    if (ip[dim] == 0 && val < 0.0f) val = 0.0f;
    if (ip[dim] == n_dim && val > 0.0f) val = 0.0f;
    float *io = dim == 0 ? a.u : (dim == 1 ? a.v : a.w);
    union {
        float f;
        unsigned u;
    } b0{in}, b1{val};
    if (b0.u != b1.u) io[f] = val;
}

}  // namespace gba
