/*
 * advect_oracle.c -- CPU restatement of the reference's MAC advection on
 * dense 3D grids. TEST INFRASTRUCTURE: part of the oracle (liboracle.so).
 * Only tests/, the smoke check and bench.py's CPU-baseline leg load it, to
 * check or time against; the shipped GPU library never calls it.
 *
 * It restates src/advection/macadvection3.cpp with bilinear (trilinear)
 * interpolation (the module's default, WENO off):
 *   advect_vector  :47-53, advect_u :136-180, advect_semiLagrangian_u :72-134
 *   advect_scalar  :39-45, advect_cell :234-274, advect_semiLagrangian_cell :182-232
 * and the helpers they call:
 *   MAC -> full vector at faces  include/shiokaze/array/macarray3.h:350-371
 *   MAC -> full vector at cells  macarray3.h:305-343
 *   trilinear interpolation      include/shiokaze/array/array_interpolator3.h:50-104
 *   vector arithmetic            include/shiokaze/math/vec.h:177-260, 353-380, 401
 *
 * Scope: every velocity face active (the smoke scene's velocity,
 * src/smoke/macsmoke3.cpp:115); the scalar may have any active set (mask),
 * its inactive cells reading the background value. Inputs are the dense
 * values the reference reads through operator().
 *
 * Arithmetic follows the reference's types: Real = float storage; in the
 * face trace p = (i,j,k) - dt*u/dx is formed from a float vector (each
 * product and quotient rounded to float), in the min/max trace and the
 * cell trace from a double vector; interpolation accumulates in float with
 * double products; the max search starts from DBL_MIN (faces) or FLT_MIN
 * (cells) as the reference's numeric_limits<>::min() does.
 *
 * Build: compiled into liboracle.so with gbp_oracle.c (-ffp-contract=off).
 */
#include <float.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int w, h, d;
} shp3;

static shp3 face_shape(int nx, int ny, int nz, int dim) {
    shp3 s = {nx + (dim == 0), ny + (dim == 1), nz + (dim == 2)};
    return s;
}

static long long at(shp3 s, int i, int j, int k) { return i + (long long)s.w * (j + (long long)s.h * k); }

/* std::min / std::max as the reference calls them: (b < a) ? b : a and
 * (a < b) ? b : a */
static double smin(double a, double b) { return (b < a) ? b : a; }
static double smax(double a, double b) { return (a < b) ? b : a; }

/* array_interpolator3::interpolate_coef (array_interpolator3.h:50-73) */
static void interp_coef(shp3 s, const double p[3], int idx[8][3], double coef[8]) {
    const double x = smax(0.0, smin(s.w - 1., p[0]));
    const double y = smax(0.0, smin(s.h - 1., p[1]));
    const double z = smax(0.0, smin(s.d - 1., p[2]));
    const int i = (int)smin(x, s.w - 2.);
    const int j = (int)smin(y, s.h - 2.);
    const int k = (int)smin(z, s.d - 2.);
    for (int n = 0; n < 8; ++n) {
        idx[n][0] = i + (n & 1);
        idx[n][1] = j + ((n >> 1) & 1);
        idx[n][2] = k + ((n >> 2) & 1);
    }
    coef[0] = (k + 1 - z) * (i + 1 - x) * (j + 1 - y);
    coef[1] = (k + 1 - z) * (x - i) * (j + 1 - y);
    coef[2] = (k + 1 - z) * (i + 1 - x) * (y - j);
    coef[3] = (k + 1 - z) * (x - i) * (y - j);
    coef[4] = (z - k) * (i + 1 - x) * (j + 1 - y);
    coef[5] = (z - k) * (x - i) * (j + 1 - y);
    coef[6] = (z - k) * (i + 1 - x) * (y - j);
    coef[7] = (z - k) * (x - i) * (y - j);
}

/* array_interpolator3::interpolate<float> (:86-104, only_actives false) */
static float interp(const float *a, shp3 s, const double p[3]) {
    int idx[8][3];
    double coef[8];
    interp_coef(s, p, idx, coef);
    float value = 0.0f;
    for (int n = 0; n < 8; ++n)
        if (coef[n]) value = (float)((double)value + (double)a[at(s, idx[n][0], idx[n][1], idx[n][2])] * coef[n]);
    return value;
}

/* macarray3::convert_to_full onto faces (macarray3.h:350-371), every face
 * active: full[dim][f*3 + c] */
static void face_full(const float *comp[3], int nx, int ny, int nz, float *full[3]) {
    for (int dim = 0; dim < 3; ++dim) {
        const shp3 fs = face_shape(nx, ny, nz, dim);
        for (int k = 0; k < fs.d; ++k)
            for (int j = 0; j < fs.h; ++j)
                for (int i = 0; i < fs.w; ++i) {
                    double u[3] = {0.0, 0.0, 0.0};
                    for (int ud = 0; ud < 3; ++ud) {
                        if (ud == dim) {
                            u[ud] = comp[ud][at(fs, i, j, k)];
                        } else {
                            const shp3 s = face_shape(nx, ny, nz, ud);
                            const int pi[3] = {i - (dim == 0), j - (dim == 1), k - (dim == 2)};
                            for (int ii = 0; ii < 2; ++ii)
                                for (int jj = 0; jj < 2; ++jj) {
                                    int q[3];
                                    for (int c = 0; c < 3; ++c) q[c] = pi[c] + ii * (dim == c) + jj * (ud == c);
                                    /* shape3::clamp (shape.h:790-797) */
                                    if (q[0] < 0) q[0] = 0;
                                    if (q[0] > s.w - 1) q[0] = s.w - 1;
                                    if (q[1] < 0) q[1] = 0;
                                    if (q[1] > s.h - 1) q[1] = s.h - 1;
                                    if (q[2] < 0) q[2] = 0;
                                    if (q[2] > s.d - 1) q[2] = s.d - 1;
                                    u[ud] += comp[ud][at(s, q[0], q[1], q[2])];
                                }
                            u[ud] /= 4.0;
                        }
                    }
                    float *o = full[dim] + 3 * at(fs, i, j, k);
                    for (int c = 0; c < 3; ++c) o[c] = (float)u[c];
                }
    }
}

/* one semi-Lagrangian pass over the faces (advect_semiLagrangian_u,
 * :72-91): out = v_in at p = (i,j,k) - dt*u/dx, u the full velocity of
 * v_in itself; the trace in float as vec3r arithmetic does */
static void semi_lagrangian_u(const float *vin[3], int nx, int ny, int nz, double dx, double dt, float *out[3],
                              float *full[3]) {
    face_full(vin, nx, ny, nz, full);
    for (int dim = 0; dim < 3; ++dim) {
        const shp3 fs = face_shape(nx, ny, nz, dim);
        for (int k = 0; k < fs.d; ++k)
            for (int j = 0; j < fs.h; ++j)
                for (int i = 0; i < fs.w; ++i) {
                    const long long f = at(fs, i, j, k);
                    const float *u = full[dim] + 3 * f;
                    if (u[0] || u[1] || u[2]) {
                        const int ip[3] = {i, j, k};
                        double p[3];
                        for (int c = 0; c < 3; ++c) {
                            const float t = (float)(u[c] * dt);     /* dt*u: vec<float> *= double */
                            const float t2 = (float)(t / dx);       /* /m_dx: vec<float> /= double */
                            p[c] = (double)ip[c] - (double)t2;      /* vec3d - vec3r */
                        }
                        out[dim][f] = (float)(double)interp(vin[dim], fs, p);
                    } else {
                        out[dim][f] = vin[dim][f];
                    }
                }
    }
}

typedef struct {
    float lo, hi;
    unsigned char within;
} minmax_t;

/* the forward pass's min/max and narrow-band flag per face (:93-133): the
 * trace in double (const vec3d & bound to the float vector) */
static void minmax_u(const float *vin[3], float *full[3], const float *fluid, int nx, int ny, int nz, double dx,
                     double dt, int trim, minmax_t *mm[3]) {
    const shp3 cs = {nx, ny, nz};
    const double limit = -dx * (double)trim;
    for (int dim = 0; dim < 3; ++dim) {
        const shp3 fs = face_shape(nx, ny, nz, dim);
        for (int k = 0; k < fs.d; ++k)
            for (int j = 0; j < fs.h; ++j)
                for (int i = 0; i < fs.w; ++i) {
                    const long long f = at(fs, i, j, k);
                    const float *uf = full[dim] + 3 * f;
                    const double u[3] = {uf[0], uf[1], uf[2]};
                    const int ip[3] = {i, j, k};
                    minmax_t r;
                    double fp[3];
                    if (u[0] || u[1] || u[2]) {
                        double p[3];
                        for (int c = 0; c < 3; ++c) {
                            const double disp = u[c] * dt / dx;
                            p[c] = (double)ip[c] - disp;
                            fp[c] = (ip[c] + 0.5 * (dim != c)) - disp;
                        }
                        int idx[8][3];
                        double coef[8];
                        interp_coef(fs, p, idx, coef);
                        double lo = DBL_MAX, hi = DBL_MIN;
                        for (int n = 0; n < 8; ++n) {
                            const double val = vin[dim][at(fs, idx[n][0], idx[n][1], idx[n][2])];
                            lo = smin(lo, val);
                            hi = smax(hi, val);
                        }
                        r.lo = (float)lo;
                        r.hi = (float)hi;
                    } else {
                        for (int c = 0; c < 3; ++c) fp[c] = ip[c] + 0.5 * (dim != c);
                        r.lo = r.hi = vin[dim][f];
                    }
                    double cp[3];
                    for (int c = 0; c < 3; ++c) cp[c] = fp[c] - 0.5;
                    r.within = (double)interp(fluid, cs, cp) > limit;
                    mm[dim][f] = r;
                }
    }
}

/* advect_u (:136-180): MacCormack, or one semi-Lagrangian pass */
static void advect_u(float *vel[3], int nx, int ny, int nz, double dx, double dt, int maccormack, int trim,
                     const float *fluid) {
    long long nf[3];
    float *vin[3], *v0[3], *v1[3], *full[3];
    minmax_t *mm[3];
    for (int d = 0; d < 3; ++d) {
        const shp3 fs = face_shape(nx, ny, nz, d);
        nf[d] = (long long)fs.w * fs.h * fs.d;
        vin[d] = (float *)malloc(sizeof(float) * nf[d]);
        memcpy(vin[d], vel[d], sizeof(float) * nf[d]);
        v0[d] = (float *)malloc(sizeof(float) * nf[d]);
        v1[d] = (float *)malloc(sizeof(float) * nf[d]);
        full[d] = (float *)malloc(sizeof(float) * 3 * nf[d]);
        mm[d] = (minmax_t *)malloc(sizeof(minmax_t) * nf[d]);
    }
    const float *cvin[3] = {vin[0], vin[1], vin[2]};
    if (!maccormack) {
        semi_lagrangian_u(cvin, nx, ny, nz, dx, dt, vel, full);
    } else {
        semi_lagrangian_u(cvin, nx, ny, nz, dx, dt, v0, full);
        minmax_u(cvin, full, fluid, nx, ny, nz, dx, dt, trim, mm);
        const float *cv0[3] = {v0[0], v0[1], v0[2]};
        semi_lagrangian_u(cv0, nx, ny, nz, dx, -dt, v1, full);
        for (int d = 0; d < 3; ++d)
            for (long long f = 0; f < nf[d]; ++f) {
                if (mm[d][f].within) {
                    vel[d][f] = v0[d][f];
                } else {
                    const double lo = mm[d][f].lo, hi = mm[d][f].hi, x0 = v0[d][f];
                    const double corr = 0.5 * (float)(vin[d][f] - v1[d][f]);
                    if (x0 + corr < lo) vel[d][f] = (float)lo;
                    else if (x0 + corr > hi) vel[d][f] = (float)hi;
                    else vel[d][f] = (float)(x0 + corr);
                }
            }
    }
    for (int d = 0; d < 3; ++d) {
        free(vin[d]);
        free(v0[d]);
        free(v1[d]);
        free(full[d]);
        free(mm[d]);
    }
}

/* macarray3::convert_to_full onto cells (macarray3.h:305-343), every face
 * active so every cell is valid: full[c*3 + dim] */
static void cell_full(const float *comp[3], int nx, int ny, int nz, float *full) {
    const shp3 cs = {nx, ny, nz};
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                float *o = full + 3 * at(cs, i, j, k);
                for (int dim = 0; dim < 3; ++dim) {
                    const shp3 fs = face_shape(nx, ny, nz, dim);
                    double value = 0.0;
                    value += comp[dim][at(fs, i, j, k)];
                    value += comp[dim][at(fs, i + (dim == 0), j + (dim == 1), k + (dim == 2))];
                    o[dim] = (float)(0.5 * value);
                }
            }
}

/* advect_semiLagrangian_cell (:182-232) on the active cells, the rest the
 * background; the trace in double */
static void semi_lagrangian_cell(const float *qin, const float *full, const unsigned char *mask, float bg, int nx,
                                 int ny, int nz, double dx, double dt, float *out, minmax_t *mm, const float *fluid,
                                 int trim) {
    const shp3 cs = {nx, ny, nz};
    const double limit = -dx * (double)trim;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long long c = at(cs, i, j, k);
                if (mask && !mask[c]) {
                    out[c] = bg;
                    continue;
                }
                const float *uf = full + 3 * c;
                const double u[3] = {uf[0], uf[1], uf[2]};
                const int ip[3] = {i, j, k};
                const int moving = u[0] || u[1] || u[2];
                double p[3];
                if (moving)
                    for (int d = 0; d < 3; ++d) p[d] = (double)ip[d] - u[d] * dt / dx;
                out[c] = moving ? (float)(double)interp(qin, cs, p) : qin[c];
                if (!mm) continue;
                minmax_t r;
                if (moving) {
                    int idx[8][3];
                    double coef[8];
                    interp_coef(cs, p, idx, coef);
                    double lo = FLT_MAX, hi = FLT_MIN;
                    for (int n = 0; n < 8; ++n) {
                        const double val = qin[at(cs, idx[n][0], idx[n][1], idx[n][2])];
                        lo = smin(lo, val);
                        hi = smax(hi, val);
                    }
                    r.lo = (float)lo;
                    r.hi = (float)hi;
                    r.within = (double)interp(fluid, cs, p) > limit;
                } else {
                    r.lo = r.hi = qin[c];
                    r.within = (double)fluid[c] > limit;
                }
                mm[c] = r;
            }
}

/* advect_cell (:234-274) */
static void advect_cell(float *q, const unsigned char *mask, float bg, const float *vel[3], int nx, int ny, int nz,
                        double dx, double dt, int maccormack, int trim, const float *fluid) {
    const long long n = (long long)nx * ny * nz;
    float *qin = (float *)malloc(sizeof(float) * n), *q0 = (float *)malloc(sizeof(float) * n);
    float *q1 = (float *)malloc(sizeof(float) * n), *full = (float *)malloc(sizeof(float) * 3 * n);
    minmax_t *mm = (minmax_t *)malloc(sizeof(minmax_t) * n);
    /* the reference reads inactive cells as the background */
    for (long long c = 0; c < n; ++c) qin[c] = (mask && !mask[c]) ? bg : q[c];
    cell_full(vel, nx, ny, nz, full);
    if (!maccormack) {
        semi_lagrangian_cell(qin, full, mask, bg, nx, ny, nz, dx, dt, q, NULL, fluid, trim);
    } else {
        semi_lagrangian_cell(qin, full, mask, bg, nx, ny, nz, dx, dt, q0, mm, fluid, trim);
        semi_lagrangian_cell(q0, full, mask, bg, nx, ny, nz, dx, -dt, q1, NULL, fluid, trim);
        for (long long c = 0; c < n; ++c) {
            if (mask && !mask[c]) {
                q[c] = bg;
            } else if (mm[c].within) {
                q[c] = q0[c];
            } else {
                const double lo = mm[c].lo, hi = mm[c].hi, x0 = q0[c];
                const double corr = 0.5 * (float)(qin[c] - q1[c]);
                if (x0 + corr < lo) q[c] = (float)lo;
                else if (x0 + corr > hi) q[c] = (float)hi;
                else q[c] = (float)(x0 + corr);
            }
        }
    }
    free(qin);
    free(q0);
    free(q1);
    free(full);
    free(mm);
}

/* macsmoke3::idle's advection (src/smoke/macsmoke3.cpp:270-281): the
 * scalar q (if not NULL; active where q_mask, all if NULL; background q_bg)
 * advected by u, v, w, then u, v, w by themselves. Arrays dense, x fastest:
 * u (nx+1)*ny*nz, v nx*(ny+1)*nz, w nx*ny*(nz+1), fluid and q nx*ny*nz. */
int oracle_advect3(int nx, int ny, int nz, double dx, double dt, int maccormack, int trim, float *u, float *v,
                   float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    if (nx < 2 || ny < 2 || nz < 2) return 1;
    float *vel[3] = {u, v, w};
    const float *cvel[3] = {u, v, w};
    if (q) advect_cell(q, q_mask, q_bg, cvel, nx, ny, nz, dx, dt, maccormack, trim, fluid);
    advect_u(vel, nx, ny, nz, dx, dt, maccormack, trim, fluid);
    return 0;
}

/* ------------------------------------------------------------------------
 * The 2D module, src/advection/macadvection2.cpp (WENO off): the same
 * passes as the 3D one on (nx, ny) grids --
 *   advect_vector :47-54, advect_u :133-165, advect_semiLagrangian_u :66-131
 *   advect_scalar :38-45, advect_cell :219-249, advect_semiLagrangian_cell :167-217
 * with bilinear interpolation (include/shiokaze/array/array_interpolator2.h:
 * 50-89) and the full vectors of include/shiokaze/array/macarray2.h:302-367.
 * Two differences of order from the 3D restatement, kept: the face full
 * vector sums its four faces with x outer, y inner (macarray2.h:359-360);
 * the interpolation weights are (i+1-x)(j+1-y), (x-i)(j+1-y), (i+1-x)(y-j),
 * (x-i)(y-j). Same scope: every velocity face active (src/smoke/
 * macsmoke2.cpp), the scalar's inactive cells reading its background. */

typedef struct {
    int w, h;
} shp2;

static shp2 face_shape2(int nx, int ny, int dim) {
    shp2 s = {nx + (dim == 0), ny + (dim == 1)};
    return s;
}

static long long at2(shp2 s, int i, int j) { return i + (long long)s.w * j; }

/* array_interpolator2::interpolate_coef (array_interpolator2.h:50-63) */
static void interp_coef2(shp2 s, const double p[2], int idx[4][2], double coef[4]) {
    const double x = smax(0.0, smin(s.w - 1., p[0]));
    const double y = smax(0.0, smin(s.h - 1., p[1]));
    const int i = (int)smin(x, s.w - 2.);
    const int j = (int)smin(y, s.h - 2.);
    for (int n = 0; n < 4; ++n) {
        idx[n][0] = i + (n & 1);
        idx[n][1] = j + ((n >> 1) & 1);
    }
    coef[0] = (i + 1 - x) * (j + 1 - y);
    coef[1] = (x - i) * (j + 1 - y);
    coef[2] = (i + 1 - x) * (y - j);
    coef[3] = (x - i) * (y - j);
}

/* array_interpolator2::interpolate<float> (:77-89, only_actives false) */
static float interp2(const float *a, shp2 s, const double p[2]) {
    int idx[4][2];
    double coef[4];
    interp_coef2(s, p, idx, coef);
    float value = 0.0f;
    for (int n = 0; n < 4; ++n)
        if (coef[n]) value = (float)((double)value + (double)a[at2(s, idx[n][0], idx[n][1])] * coef[n]);
    return value;
}

/* macarray2::convert_to_full onto faces (macarray2.h:347-367): full[dim][f*2 + c] */
static void face_full2(const float *comp[2], int nx, int ny, float *full[2]) {
    for (int dim = 0; dim < 2; ++dim) {
        const shp2 fs = face_shape2(nx, ny, dim);
        for (int j = 0; j < fs.h; ++j)
            for (int i = 0; i < fs.w; ++i) {
                double u[2] = {0.0, 0.0};
                for (int ud = 0; ud < 2; ++ud) {
                    if (ud == dim) {
                        u[ud] = comp[ud][at2(fs, i, j)];
                    } else {
                        const shp2 s = face_shape2(nx, ny, ud);
                        const int pi[2] = {i - (dim == 0), j - (dim == 1)};
                        for (int ii = 0; ii < 2; ++ii)
                            for (int jj = 0; jj < 2; ++jj) {
                                int q0 = pi[0] + ii, q1 = pi[1] + jj;
                                /* shape2::clamp */
                                if (q0 < 0) q0 = 0;
                                if (q0 > s.w - 1) q0 = s.w - 1;
                                if (q1 < 0) q1 = 0;
                                if (q1 > s.h - 1) q1 = s.h - 1;
                                u[ud] += comp[ud][at2(s, q0, q1)];
                            }
                        u[ud] /= 4.0;
                    }
                }
                float *o = full[dim] + 2 * at2(fs, i, j);
                o[0] = (float)u[0];
                o[1] = (float)u[1];
            }
    }
}

/* advect_semiLagrangian_u (:66-87), the trace in float as vec2r does */
static void semi_lagrangian_u2(const float *vin[2], int nx, int ny, double dx, double dt, float *out[2],
                               float *full[2]) {
    face_full2(vin, nx, ny, full);
    for (int dim = 0; dim < 2; ++dim) {
        const shp2 fs = face_shape2(nx, ny, dim);
        for (int j = 0; j < fs.h; ++j)
            for (int i = 0; i < fs.w; ++i) {
                const long long f = at2(fs, i, j);
                const float *u = full[dim] + 2 * f;
                if (u[0] || u[1]) {
                    const int ip[2] = {i, j};
                    double p[2];
                    for (int c = 0; c < 2; ++c) {
                        const float t = (float)(u[c] * dt);
                        const float t2 = (float)(t / dx);
                        p[c] = (double)ip[c] - (double)t2;
                    }
                    out[dim][f] = interp2(vin[dim], fs, p);
                } else {
                    out[dim][f] = vin[dim][f];
                }
            }
    }
}

/* the forward pass's min/max and narrow-band flag per face (:89-129) */
static void minmax_u2(const float *vin[2], float *full[2], const float *fluid, int nx, int ny, double dx, double dt,
                      int trim, minmax_t *mm[2]) {
    const shp2 cs = {nx, ny};
    const double limit = -dx * (double)trim;
    for (int dim = 0; dim < 2; ++dim) {
        const shp2 fs = face_shape2(nx, ny, dim);
        for (int j = 0; j < fs.h; ++j)
            for (int i = 0; i < fs.w; ++i) {
                const long long f = at2(fs, i, j);
                const float *uf = full[dim] + 2 * f;
                const double u[2] = {uf[0], uf[1]};
                const int ip[2] = {i, j};
                minmax_t r;
                double fp[2];
                if (u[0] || u[1]) {
                    double p[2];
                    for (int c = 0; c < 2; ++c) {
                        const double disp = u[c] * dt / dx;
                        p[c] = (double)ip[c] - disp;
                        fp[c] = (ip[c] + 0.5 * (dim != c)) - disp;
                    }
                    int idx[4][2];
                    double coef[4];
                    interp_coef2(fs, p, idx, coef);
                    double lo = DBL_MAX, hi = DBL_MIN;
                    for (int n = 0; n < 4; ++n) {
                        const double val = vin[dim][at2(fs, idx[n][0], idx[n][1])];
                        lo = smin(lo, val);
                        hi = smax(hi, val);
                    }
                    r.lo = (float)lo;
                    r.hi = (float)hi;
                } else {
                    for (int c = 0; c < 2; ++c) fp[c] = ip[c] + 0.5 * (dim != c);
                    r.lo = r.hi = vin[dim][f];
                }
                const double cp[2] = {fp[0] - 0.5, fp[1] - 0.5};
                r.within = (double)interp2(fluid, cs, cp) > limit;
                mm[dim][f] = r;
            }
    }
}

static void advect_u2(float *vel[2], int nx, int ny, double dx, double dt, int maccormack, int trim,
                      const float *fluid) {
    long long nf[2];
    float *vin[2], *v0[2], *v1[2], *full[2];
    minmax_t *mm[2];
    for (int d = 0; d < 2; ++d) {
        const shp2 fs = face_shape2(nx, ny, d);
        nf[d] = (long long)fs.w * fs.h;
        vin[d] = (float *)malloc(sizeof(float) * nf[d]);
        memcpy(vin[d], vel[d], sizeof(float) * nf[d]);
        v0[d] = (float *)malloc(sizeof(float) * nf[d]);
        v1[d] = (float *)malloc(sizeof(float) * nf[d]);
        full[d] = (float *)malloc(sizeof(float) * 2 * nf[d]);
        mm[d] = (minmax_t *)malloc(sizeof(minmax_t) * nf[d]);
    }
    const float *cvin[2] = {vin[0], vin[1]};
    if (!maccormack) {
        semi_lagrangian_u2(cvin, nx, ny, dx, dt, vel, full);
    } else {
        semi_lagrangian_u2(cvin, nx, ny, dx, dt, v0, full);
        minmax_u2(cvin, full, fluid, nx, ny, dx, dt, trim, mm);
        const float *cv0[2] = {v0[0], v0[1]};
        semi_lagrangian_u2(cv0, nx, ny, dx, -dt, v1, full);
        for (int d = 0; d < 2; ++d)
            for (long long f = 0; f < nf[d]; ++f) {
                if (mm[d][f].within) {
                    vel[d][f] = v0[d][f];
                } else {
                    const double lo = mm[d][f].lo, hi = mm[d][f].hi, x0 = v0[d][f];
                    const double corr = 0.5 * (float)(vin[d][f] - v1[d][f]);
                    if (x0 + corr < lo) vel[d][f] = (float)lo;
                    else if (x0 + corr > hi) vel[d][f] = (float)hi;
                    else vel[d][f] = (float)(x0 + corr);
                }
            }
    }
    for (int d = 0; d < 2; ++d) {
        free(vin[d]);
        free(v0[d]);
        free(v1[d]);
        free(full[d]);
        free(mm[d]);
    }
}

/* macarray2::convert_to_full onto cells (macarray2.h:302-340): full[c*2 + dim] */
static void cell_full2(const float *comp[2], int nx, int ny, float *full) {
    const shp2 cs = {nx, ny};
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            float *o = full + 2 * at2(cs, i, j);
            for (int dim = 0; dim < 2; ++dim) {
                const shp2 fs = face_shape2(nx, ny, dim);
                double value = 0.0;
                value += comp[dim][at2(fs, i, j)];
                value += comp[dim][at2(fs, i + (dim == 0), j + (dim == 1))];
                o[dim] = (float)(0.5 * value);
            }
        }
}

/* advect_semiLagrangian_cell (:167-217) */
static void semi_lagrangian_cell2(const float *qin, const float *full, const unsigned char *mask, float bg, int nx,
                                  int ny, double dx, double dt, float *out, minmax_t *mm, const float *fluid,
                                  int trim) {
    const shp2 cs = {nx, ny};
    const double limit = -dx * (double)trim;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const long long c = at2(cs, i, j);
            if (mask && !mask[c]) {
                out[c] = bg;
                continue;
            }
            const float *uf = full + 2 * c;
            const double u[2] = {uf[0], uf[1]};
            const int ip[2] = {i, j};
            const int moving = u[0] || u[1];
            double p[2];
            if (moving)
                for (int d = 0; d < 2; ++d) p[d] = (double)ip[d] - u[d] * dt / dx;
            out[c] = moving ? interp2(qin, cs, p) : qin[c];
            if (!mm) continue;
            minmax_t r;
            if (moving) {
                int idx[4][2];
                double coef[4];
                interp_coef2(cs, p, idx, coef);
                double lo = FLT_MAX, hi = FLT_MIN;
                for (int n = 0; n < 4; ++n) {
                    const double val = qin[at2(cs, idx[n][0], idx[n][1])];
                    lo = smin(lo, val);
                    hi = smax(hi, val);
                }
                r.lo = (float)lo;
                r.hi = (float)hi;
                r.within = (double)interp2(fluid, cs, p) > limit;
            } else {
                r.lo = r.hi = qin[c];
                r.within = (double)fluid[c] > limit;
            }
            mm[c] = r;
        }
}

static void advect_cell2(float *q, const unsigned char *mask, float bg, const float *vel[2], int nx, int ny,
                         double dx, double dt, int maccormack, int trim, const float *fluid) {
    const long long n = (long long)nx * ny;
    float *qin = (float *)malloc(sizeof(float) * n), *q0 = (float *)malloc(sizeof(float) * n);
    float *q1 = (float *)malloc(sizeof(float) * n), *full = (float *)malloc(sizeof(float) * 2 * n);
    minmax_t *mm = (minmax_t *)malloc(sizeof(minmax_t) * n);
    for (long long c = 0; c < n; ++c) qin[c] = (mask && !mask[c]) ? bg : q[c];
    cell_full2(vel, nx, ny, full);
    if (!maccormack) {
        semi_lagrangian_cell2(qin, full, mask, bg, nx, ny, dx, dt, q, NULL, fluid, trim);
    } else {
        semi_lagrangian_cell2(qin, full, mask, bg, nx, ny, dx, dt, q0, mm, fluid, trim);
        semi_lagrangian_cell2(q0, full, mask, bg, nx, ny, dx, -dt, q1, NULL, fluid, trim);
        for (long long c = 0; c < n; ++c) {
            if (mask && !mask[c]) {
                q[c] = bg;
            } else if (mm[c].within) {
                q[c] = q0[c];
            } else {
                const double lo = mm[c].lo, hi = mm[c].hi, x0 = q0[c];
                const double corr = 0.5 * (float)(qin[c] - q1[c]);
                if (x0 + corr < lo) q[c] = (float)lo;
                else if (x0 + corr > hi) q[c] = (float)hi;
                else q[c] = (float)(x0 + corr);
            }
        }
    }
    free(qin);
    free(q0);
    free(q1);
    free(full);
    free(mm);
}

/* macsmoke2's advection step: the scalar q (if not NULL) by u, v, then u, v
 * by themselves. u (nx+1)*ny, v nx*(ny+1), fluid and q nx*ny, x fastest. */
int oracle_advect2(int nx, int ny, double dx, double dt, int maccormack, int trim, float *u, float *v,
                   const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    if (nx < 2 || ny < 2) return 1;
    float *vel[2] = {u, v};
    const float *cvel[2] = {u, v};
    if (q) advect_cell2(q, q_mask, q_bg, cvel, nx, ny, dx, dt, maccormack, trim, fluid);
    advect_u2(vel, nx, ny, dx, dt, maccormack, trim, fluid);
    return 0;
}

/* ------------------------------------------------------------------------
 * macutility3::constrain_velocity (src/utility/macutility3.cpp:61-86): the
 * velocity's normal component into the solid removed at faces inside it,
 * and outflow through the domain's walls set to 0. */

/* array_derivative3::derivative (include/shiokaze/array/array_derivative3.h:
 * 51-95, 107-116): the trilinear gradient in index space, every corner
 * included, accumulated in float with double products */
static void derivative(const float *a, shp3 s, const double p[3], float out[3]) {
    const double x = smax(0.0, smin(s.w - 1., p[0]));
    const double y = smax(0.0, smin(s.h - 1., p[1]));
    const double z = smax(0.0, smin(s.d - 1., p[2]));
    const int i = (int)smin(x, s.w - 2.);
    const int j = (int)smin(y, s.h - 2.);
    const int k = (int)smin(z, s.d - 2.);
    double c[3][8];
    c[0][0] = -(k + 1 - z) * (j + 1 - y);
    c[0][1] = (k + 1 - z) * (j + 1 - y);
    c[0][2] = -(k + 1 - z) * (y - j);
    c[0][3] = (k + 1 - z) * (y - j);
    c[0][4] = -(z - k) * (j + 1 - y);
    c[0][5] = (z - k) * (j + 1 - y);
    c[0][6] = -(z - k) * (y - j);
    c[0][7] = (z - k) * (y - j);
    c[1][0] = -(k + 1 - z) * (i + 1 - x);
    c[1][1] = -(k + 1 - z) * (x - i);
    c[1][2] = (k + 1 - z) * (i + 1 - x);
    c[1][3] = (k + 1 - z) * (x - i);
    c[1][4] = -(z - k) * (i + 1 - x);
    c[1][5] = -(z - k) * (x - i);
    c[1][6] = (z - k) * (i + 1 - x);
    c[1][7] = (z - k) * (x - i);
    c[2][0] = -(i + 1 - x) * (j + 1 - y);
    c[2][1] = -(x - i) * (j + 1 - y);
    c[2][2] = -(i + 1 - x) * (y - j);
    c[2][3] = -(x - i) * (y - j);
    c[2][4] = (i + 1 - x) * (j + 1 - y);
    c[2][5] = (x - i) * (j + 1 - y);
    c[2][6] = (i + 1 - x) * (y - j);
    c[2][7] = (x - i) * (y - j);
    for (int d = 0; d < 3; ++d) {
        float r = 0.0f;
        for (int n = 0; n < 8; ++n)
            r = (float)((double)r + c[d][n] * (double)a[at(s, i + (n & 1), j + ((n >> 1) & 1), k + ((n >> 2) & 1))]);
        out[d] = r;
    }
}

/* u, v, w dense (operator() values: inactive faces hold the background),
 * updated on the faces whose mask is nonzero (every face if a mask is NULL).
 * solid is nodal (nx+1)(ny+1)(nz+1). The reference tests
 * levelset_exist(solid) (array_utility3.h:112-122) over the array's active
 * values; here over every value. It runs its face loop three times (the
 * `for( int dim : DIMS3 )` around parallel_actives, :68); so does this. */
int oracle_constrain_velocity3(int nx, int ny, int nz, double dx, const float *solid, float *u, float *v, float *w,
                               const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    if (nx < 2 || ny < 2 || nz < 2) return 1;
    const shp3 ns = {nx + 1, ny + 1, nz + 1};
    const long long nn = (long long)ns.w * ns.h * ns.d;
    int exists = 0;
    for (long long n = 0; n < nn && !exists; ++n) exists = solid[n] < 0.0;
    if (!exists) return 0;
    float *comp[3] = {u, v, w}, *save[3];
    const unsigned char *mask[3] = {mu, mv, mw};
    for (int d = 0; d < 3; ++d) {
        const shp3 fs = face_shape(nx, ny, nz, d);
        const long long nf = (long long)fs.w * fs.h * fs.d;
        save[d] = (float *)malloc(sizeof(float) * nf);
        memcpy(save[d], comp[d], sizeof(float) * nf);
    }
    const int shape[3] = {nx, ny, nz};
    for (int rep = 0; rep < 3; ++rep)
        for (int dim = 0; dim < 3; ++dim) {
            const shp3 fs = face_shape(nx, ny, nz, dim);
            for (int k = 0; k < fs.d; ++k)
                for (int j = 0; j < fs.h; ++j)
                    for (int i = 0; i < fs.w; ++i) {
                        const long long f = at(fs, i, j, k);
                        if (mask[dim] && !mask[dim][f]) continue;
                        const int ip[3] = {i, j, k};
                        double p[3];
                        for (int c = 0; c < 3; ++c) p[c] = ip[c] + 0.5 * (dim != c);
                        float val = comp[dim][f];
                        if ((double)interp(solid, ns, p) < 0.0) {
                            float dr[3];
                            derivative(solid, ns, p, dr);
                            double nrm[3];
                            for (int c = 0; c < 3; ++c) nrm[c] = (double)dr[c] / dx;
                            double n2 = 0.0;
                            for (int c = 0; c < 3; ++c) n2 += nrm[c] * nrm[c];
                            if (n2) {
                                /* macarray_interpolator3::interpolate (macarray_interpolator3.h:49-56) */
                                double uu[3];
                                for (int c = 0; c < 3; ++c) {
                                    double pos[3];
                                    for (int e = 0; e < 3; ++e) pos[e] = p[e] - 0.5 * (c != e);
                                    uu[c] = interp(save[c], face_shape(nx, ny, nz, c), pos);
                                }
                                double dot = 0.0;
                                for (int c = 0; c < 3; ++c) dot += uu[c] * nrm[c];
                                if (dot < 0.0) val = (float)(uu[dim] - nrm[dim] * dot);
                            }
                        }
                        if (ip[dim] == 0 && val < 0.0) val = 0.0f;
                        if (ip[dim] == shape[dim] && val > 0.0) val = 0.0f;
                        comp[dim][f] = val;
                    }
        }
    for (int d = 0; d < 3; ++d) free(save[d]);
    return 0;
}

/* ------------------------------------------------------------------------
 * array_extrapolator3::extrapolate (include/shiokaze/array/
 * array_extrapolator3.h:36-73) on one dense array with an active mask, as
 * array3::dilate runs it (array3.h:1661-1668, src/array/dilate3.h:43-95):
 * `count` times, every inactive in-bounds 6-neighbour of an active cell
 * becomes active with the float mean of its active neighbours (summed in
 * the order +x, -x, +y, -y, -z, +z), all values of one round computed from
 * the state before it. Returns the number of cells activated. */
long long oracle_extrapolate3(int w, int h, int d, float *a, unsigned char *active, int count) {
    const shp3 s = {w, h, d};
    const long long n = (long long)w * h * d;
    unsigned char *cand = (unsigned char *)malloc((size_t)n);
    float *val = (float *)malloc(sizeof(float) * (size_t)n);
    static const int q[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, -1}, {0, 0, 1}};
    long long total = 0;
    for (int it = 0; it < count; ++it) {
        memset(cand, 0, (size_t)n);
        for (int k = 0; k < d; ++k)
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    const long long c = at(s, i, j, k);
                    if (active[c]) continue;
                    float sum = 0.0f;
                    int weight = 0;
                    for (int m = 0; m < 6; ++m) {
                        const int qi = i + q[m][0], qj = j + q[m][1], qk = k + q[m][2];
                        if (qi < 0 || qj < 0 || qk < 0 || qi >= w || qj >= h || qk >= d) continue;
                        const long long e = at(s, qi, qj, qk);
                        if (active[e]) {
                            sum += a[e];
                            ++weight;
                        }
                    }
                    if (weight) {
                        cand[c] = 1;
                        val[c] = sum / weight;
                    }
                }
        long long added = 0;
        for (long long c = 0; c < n; ++c)
            if (cand[c]) {
                active[c] = 1;
                a[c] = val[c];
                ++added;
            }
        total += added;
    }
    free(cand);
    free(val);
    return total;
}
