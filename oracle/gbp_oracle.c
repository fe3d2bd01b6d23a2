/*
 * gbp_oracle.c -- CPU restatement of the reference's pressure projection on
 * dense grids. TEST INFRASTRUCTURE: the oracle. Only tests/, the smoke check
 * and bench.py's CPU-baseline leg load it (as liboracle.so via ctypes), and
 * only to check or time against; the shipped GPU library never calls it.
 *
 * It restates, for dense arrays (x fastest), what
 *   src/projection/macpressuresolver3.cpp:50-272 (3D) and
 *   src/projection/macpressuresolver2.cpp:48-238 (2D)
 * do, with the helpers they call:
 *   face fractions   src/utility/macutility3.cpp:94-194, macutility2.cpp:89-154,
 *                    include/shiokaze/utility/utility.h:162-214
 *   labelling        macpressuresolver3.cpp:121-156 (tile-major numbering of
 *                    the 16^3 tiled array, src/array/tiledarray3.cpp:314-330,
 *                    :491, :820; 16^2 tiles in 2D, tiledarray2.cpp:773)
 *   assembly         macpressuresolver3.cpp:163-199 (rows with columns sorted,
 *                    src/math/RCMatrix.cpp:249-272)
 *   volume correction / warm start  macpressuresolver3.cpp:204-242
 *   CG               src/linsolver/pcg.cpp:45-73 ->
 *                    local/include/pcgsolver/pcg_solver.h:246-295 (the
 *                    preconditioner returns its input, :379-384, so this is
 *                    plain CG with the infinity-norm stopping rule)
 *   velocity update  macpressuresolver3.cpp:252-268, macpressuresolver2.cpp:221-237
 *
 * Arithmetic follows the reference's expression order and types (Real=float
 * storage, double arithmetic; dot products summed in unknown order) so that
 * on a machine without fused multiply-add contraction it reproduces the
 * reference bit for bit. Sparse-array semantics (narrow band, flood fill) are
 * the caller's job: inputs are the dense values the reference would read
 * through operator().
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared gbp_oracle.c -o liboracle.so -lm
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define TILE 16

typedef struct {
    double residual;        /* Residual (pcg.cpp:76 default 1e-4) */
    int max_iterations;     /* MaxIterations (pcg.cpp:77 default 30000) */
    int warm_start;         /* WarmStart (macpressuresolver3.cpp:304) */
    double eps_fluid;       /* EpsFluid (macutility3.cpp:424) */
    double eps_solid;       /* EpsSolid (macutility3.cpp:425) */
    int second_order_fluid; /* SecondOrderAccurateFluid */
    int second_order_solid; /* SecondOrderAccurateSolid */
    double gain;            /* Gain (volume correction) */
    double surface_tension; /* project()'s surface_tension argument (macpressuresolver3.cpp:85-115) */
} oracle_params;

typedef struct {
    int iterations;
    int converged;
    double reresid;         /* |r|_inf / |b|_inf as pcg_solver.h returns it */
    long long unknowns;
    double b_inf;           /* |b|_inf of the system handed to CG */
} oracle_stats;

typedef struct {
    int dim, nx, ny, nz;
    double dx;
    double current_volume, target_volume, y_prev;
    double *prev;           /* warm-start pressure by unknown index */
    long long prev_n;
    int have_prev;
} oracle_ctx;

/* ---- helpers from include/shiokaze/utility/utility.h ------------------- */

/* utility::fraction (utility.h:162-170) */
static double fraction(double phi0, double phi1) {
    if (phi0 * phi1 >= 0.0) {
        if (phi0 < 0.0 || phi1 < 0.0) return 1.0;
        return 0.0;
    } else {
        const double eps = DBL_MIN;
        double mn = phi0 < phi1 ? phi0 : phi1;
        double d = fabs(phi1 - phi0);
        return -mn / (d > eps ? d : eps);
    }
}

/* utility::get_area (utility.h:179-214): area of {phi<0} in the unit square
 * whose corner values are q[i][j]; marching-squares polygon, shoelace sum. */
static double get_area(const double q[2][2]) {
    static const int quads[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    double v[4], p[8][2];
    int pnum = 0;
    for (int n = 0; n < 4; ++n) v[n] = q[quads[n][0]][quads[n][1]];
    for (int n = 0; n < 4; ++n) {
        if (v[n] < 0.0) {
            p[pnum][0] = quads[n][0];
            p[pnum][1] = quads[n][1];
            pnum++;
        }
        if (v[n] * v[(n + 1) % 4] < 0) {
            double y0 = v[n], y1 = v[(n + 1) % 4];
            if (y0 - y1) {
                double a = y0 / (y0 - y1);
                int p0x = quads[n][0], p0y = quads[n][1];
                int p1x = quads[(n + 1) % 4][0], p1y = quads[(n + 1) % 4][1];
                p[pnum][0] = (1.0 - a) * p0x + a * p1x;
                p[pnum][1] = (1.0 - a) * p0y + a * p1y;
                pnum++;
            }
        }
    }
    double sum = 0.0;
    for (int m = 0; m < pnum; m++) sum += p[m][0] * p[(m + 1) % pnum][1] - p[m][1] * p[(m + 1) % pnum][0];
    return 0.5 * sum;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ---- context ------------------------------------------------------------ */

oracle_ctx *oracle_create(int dim, int nx, int ny, int nz, double dx) {
    oracle_ctx *c = (oracle_ctx *)calloc(1, sizeof(oracle_ctx));
    c->dim = dim;
    c->nx = nx;
    c->ny = ny;
    c->nz = dim == 3 ? nz : 1;
    c->dx = dx;
    return c;
}

void oracle_destroy(oracle_ctx *c) {
    if (!c) return;
    free(c->prev);
    free(c);
}

/* macproject3_interface::set_target_volume (macpressuresolver3.cpp:45-48) */
void oracle_set_target_volume(oracle_ctx *c, double current_volume, double target_volume) {
    c->current_volume = current_volume;
    c->target_volume = target_volume;
}

/* ---- face fractions ------------------------------------------------------ */

/* Area fraction of face (i,j,k) normal to dim, 3D (macutility3.cpp:117-143). */
static float area3(const oracle_ctx *c, const float *solid, int dim, int i, int j, int k, const oracle_params *prm) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const size_t sx = (size_t)nx + 1, sxy = sx * ((size_t)ny + 1);
    int pi[3] = {i, j, k};
    int sh[3] = {nx, ny, nz};
#define S(a, b, cc) ((double)solid[(size_t)(a) + sx * (size_t)(b) + sxy * (size_t)(cc)])
    double area;
    if (pi[dim] == 0 || pi[dim] == sh[dim]) area = 0.0;
    else {
        double q[2][2];
        if (dim == 0) {
            q[0][0] = S(i, j, k); q[1][0] = S(i, j + 1, k); q[1][1] = S(i, j + 1, k + 1); q[0][1] = S(i, j, k + 1);
        } else if (dim == 1) {
            q[0][0] = S(i, j, k); q[1][0] = S(i + 1, j, k); q[1][1] = S(i + 1, j, k + 1); q[0][1] = S(i, j, k + 1);
        } else {
            q[0][0] = S(i, j, k); q[1][0] = S(i + 1, j, k); q[1][1] = S(i + 1, j + 1, k); q[0][1] = S(i, j + 1, k);
        }
        area = 1.0 - get_area(q);
    }
#undef S
    if (area && area < prm->eps_solid) area = prm->eps_solid;
    float a = (float)area;
    if (!prm->second_order_solid && a) a = 1.0f; /* macpressuresolver3.cpp:76-80 */
    return a;
}

/* Fluid fraction of face (i,j,k) normal to dim, 3D (macutility3.cpp:166-194). */
static float rho3(const oracle_ctx *c, const float *fluid, int fluid_exists, int dim, int i, int j, int k,
                  const oracle_params *prm) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    float r;
    if (!fluid_exists) r = 1.0f; /* levelset_exist(fluid) false: rhos.clear(1.0) */
    else {
        int a0 = clampi(i, 0, nx - 1), a1 = clampi(j, 0, ny - 1), a2 = clampi(k, 0, nz - 1);
        int b0 = clampi(i - (dim == 0), 0, nx - 1), b1 = clampi(j - (dim == 1), 0, ny - 1),
            b2 = clampi(k - (dim == 2), 0, nz - 1);
        double f0 = fluid[(size_t)a0 + (size_t)nx * ((size_t)a1 + (size_t)ny * a2)];
        double f1 = fluid[(size_t)b0 + (size_t)nx * ((size_t)b1 + (size_t)ny * b2)];
        double rho = fraction(f0, f1);
        if (rho && rho < prm->eps_fluid) rho = prm->eps_fluid;
        r = (float)rho;
    }
    if (!prm->second_order_fluid && r) r = 1.0f; /* macpressuresolver3.cpp:70-74 */
    return r;
}

/* 2D counterparts (macutility2.cpp:89-154): the face's two nodes. */
static float area2(const oracle_ctx *c, const float *solid, int dim, int i, int j, const oracle_params *prm) {
    const int nx = c->nx, ny = c->ny;
    const size_t sx = (size_t)nx + 1;
    int pi[2] = {i, j};
    int sh[2] = {nx, ny};
    double area;
    if (pi[dim] == 0 || pi[dim] == sh[dim]) area = 0.0;
    else {
        double s0 = solid[(size_t)i + sx * (size_t)j];
        double s1 = dim == 0 ? solid[(size_t)i + sx * (size_t)(j + 1)] : solid[(size_t)(i + 1) + sx * (size_t)j];
        area = 1.0 - fraction(s0, s1);
    }
    if (area && area < prm->eps_solid) area = prm->eps_solid;
    float a = (float)area;
    if (!prm->second_order_solid && a) a = 1.0f;
    return a;
}

static float rho2(const oracle_ctx *c, const float *fluid, int fluid_exists, int dim, int i, int j,
                  const oracle_params *prm) {
    const int nx = c->nx, ny = c->ny;
    float r;
    if (!fluid_exists) r = 1.0f;
    else {
        int a0 = clampi(i, 0, nx - 1), a1 = clampi(j, 0, ny - 1);
        int b0 = clampi(i - (dim == 0), 0, nx - 1), b1 = clampi(j - (dim == 1), 0, ny - 1);
        double rho = fraction(fluid[(size_t)a0 + (size_t)nx * a1], fluid[(size_t)b0 + (size_t)nx * b1]);
        if (rho && rho < prm->eps_fluid) rho = prm->eps_fluid;
        r = (float)rho;
    }
    if (!prm->second_order_fluid && r) r = 1.0f;
    return r;
}

/* Curvature of a cell for the surface-tension term (macpressuresolver3.cpp:
 * 93-101, macpressuresolver2.cpp:79-88): the level set at the clamped
 * neighbours summed in float (-x, +x, -y, +y[, -z, +z]), minus 6 (4) times the
 * cell's value in double, over dx^2, stored as float. */
static float st_curvature(const oracle_ctx *c, const float *fluid, int i, int j, int k) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
#define ST_F(a, b, q)                                                                              \
    fluid[(size_t)((a) < 0 ? 0 : (a) >= nx ? nx - 1 : (a)) +                                       \
          (size_t)nx * ((size_t)((b) < 0 ? 0 : (b) >= ny ? ny - 1 : (b)) +                         \
                        (size_t)ny * (size_t)((q) < 0 ? 0 : (q) >= nz ? nz - 1 : (q)))]
    float s = ST_F(i - 1, j, k) + ST_F(i + 1, j, k);
    s = s + ST_F(i, j - 1, k);
    s = s + ST_F(i, j + 1, k);
    double value;
    if (c->dim == 3) {
        s = s + ST_F(i, j, k - 1);
        s = s + ST_F(i, j, k + 1);
        value = ((double)s - 6.0 * (double)ST_F(i, j, k)) / (c->dx * c->dx);
    } else {
        value = ((double)s - 4.0 * (double)ST_F(i, j, k)) / (c->dx * c->dx);
    }
#undef ST_F
    return (float)value;
}

/* Surface tension (macpressuresolver3.cpp:103-113, macpressuresolver2.cpp:
 * 90-103), in place on the face velocities: every face with 0 < rho < 1 gets
 * -sgn dt/(dx rho) kappa (theta c+ + (1-theta) c-) added, the increment
 * rounded to float and added in float (array3.h:987-994). */
static void apply_surface_tension(const oracle_ctx *c, const float *fluid, float *const R[3], float *vel[3],
                                  double dt, double kappa) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, dim = c->dim;
    for (int d = 0; d < dim; ++d) {
        const int fx = nx + (d == 0), fy = ny + (d == 1), fz = dim == 3 ? nz + (d == 2) : 1;
        for (int k = 0; k < fz; ++k)
            for (int j = 0; j < fy; ++j)
                for (int i = 0; i < fx; ++i) {
                    const size_t f = (size_t)i + (size_t)fx * ((size_t)j + (size_t)fy * (size_t)k);
                    const double rho = R[d][f];
                    if (!(rho && rho < 1.0)) continue;
                    const int a0 = i >= nx ? nx - 1 : i, a1 = j >= ny ? ny - 1 : j, a2 = k >= nz ? nz - 1 : k;
                    int b0 = i - (d == 0), b1 = j - (d == 1), b2 = k - (d == 2);
                    b0 = b0 < 0 ? 0 : b0 >= nx ? nx - 1 : b0;
                    b1 = b1 < 0 ? 0 : b1 >= ny ? ny - 1 : b1;
                    b2 = b2 < 0 ? 0 : b2 >= nz ? nz - 1 : b2;
                    const float fa = fluid[(size_t)a0 + (size_t)nx * ((size_t)a1 + (size_t)ny * (size_t)a2)];
                    const double sgn = fa < 0.0 ? -1.0 : 1.0;
                    const double theta = sgn < 0 ? 1.0 - rho : rho;
                    const double face_c = theta * (double)st_curvature(c, fluid, a0, a1, a2) +
                                          (1.0 - theta) * (double)st_curvature(c, fluid, b0, b1, b2);
                    const float inc = (float)(-sgn * dt / (c->dx * rho) * kappa * face_c);
                    vel[d][f] = vel[d][f] + inc;
                }
    }
}

/* Face fraction arrays for every face: areas[d], rhos[d] sized as the face
 * grid of dimension d. */
void oracle_face_fractions(const oracle_ctx *c, const float *solid, const float *fluid, const oracle_params *prm,
                           float *ax, float *ay, float *az, float *rx, float *ry, float *rz) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const size_t ncell = (size_t)nx * ny * nz;
    int fluid_exists = 0;
    for (size_t n = 0; n < ncell; ++n)
        if (fluid[n] < 0.0f) { fluid_exists = 1; break; }
    float *A[3] = {ax, ay, az}, *R[3] = {rx, ry, rz};
    for (int d = 0; d < c->dim; ++d) {
        int fx = nx + (d == 0), fy = ny + (d == 1), fz = c->dim == 3 ? nz + (d == 2) : 1;
        for (int k = 0; k < fz; ++k)
            for (int j = 0; j < fy; ++j)
                for (int i = 0; i < fx; ++i) {
                    size_t n = (size_t)i + (size_t)fx * ((size_t)j + (size_t)fy * k);
                    if (c->dim == 3) {
                        A[d][n] = area3(c, solid, d, i, j, k, prm);
                        R[d][n] = rho3(c, fluid, fluid_exists, d, i, j, k, prm);
                    } else {
                        A[d][n] = area2(c, solid, d, i, j, prm);
                        R[d][n] = rho2(c, fluid, fluid_exists, d, i, j, prm);
                    }
                }
    }
}

/* ---- projection ------------------------------------------------------------ */

typedef struct {
    long long n;
    long long *rowstart;
    long long *col;
    double *val;
} csr;

static void csr_free(csr *m) {
    free(m->rowstart);
    free(m->col);
    free(m->val);
}

/* Insert (col,val) into a row kept sorted by column (RCMatrix.cpp:249-272;
 * each off-diagonal is added once and the diagonal once, so no merging). */
static void row_insert(long long *cols, double *vals, int *cnt, long long col, double v) {
    if (!v) return;
    int k = *cnt;
    while (k > 0 && cols[k - 1] > col) {
        cols[k] = cols[k - 1];
        vals[k] = vals[k - 1];
        --k;
    }
    cols[k] = col;
    vals[k] = v;
    (*cnt)++;
}

/* ---- worker threads for the element-wise loops of CG ----------------------- *
 * The matrix-vector product (one row per index, each row summed in its own
 * order), the vector updates and the maximum norm give the same bits however
 * their index range is split, so they run on oracle_set_threads(n) threads;
 * the dot products stay serial, in index order, as the reference sums them
 * (cblas_ddot). Results are therefore bit-identical for every thread count. */
#include <pthread.h>

typedef void (*range_fn)(void *arg, long long lo, long long hi, int t);
static struct {
    int n;                      /* threads including the caller */
    pthread_t th[64];
    pthread_barrier_t start, done;
    range_fn fn;
    void *arg;
    long long count;
    int quit;
} g_pool = {1};
static double g_part[64];       /* per-thread partial maxima */

static void pool_run_part(int t) {
    const long long n = g_pool.count, per = (n + g_pool.n - 1) / g_pool.n;
    const long long lo = per * t < n ? per * t : n, hi = lo + per < n ? lo + per : n;
    g_pool.fn(g_pool.arg, lo, hi, t);
}

static void *pool_main(void *p) {
    const int t = (int)(long long)p;
    for (;;) {
        pthread_barrier_wait(&g_pool.start);
        if (g_pool.quit) return NULL;
        pool_run_part(t);
        pthread_barrier_wait(&g_pool.done);
    }
}

/* Number of threads for the element-wise loops of CG (1 = all serial). */
void oracle_set_threads(int n) {
    if (n < 1) n = 1;
    if (n > 64) n = 64;
    if (g_pool.n > 1) {
        g_pool.quit = 1;
        pthread_barrier_wait(&g_pool.start);
        for (int t = 1; t < g_pool.n; ++t) pthread_join(g_pool.th[t], NULL);
        pthread_barrier_destroy(&g_pool.start);
        pthread_barrier_destroy(&g_pool.done);
        g_pool.quit = 0;
    }
    g_pool.n = n;
    if (n > 1) {
        pthread_barrier_init(&g_pool.start, NULL, (unsigned)n);
        pthread_barrier_init(&g_pool.done, NULL, (unsigned)n);
        for (int t = 1; t < n; ++t) pthread_create(&g_pool.th[t], NULL, pool_main, (void *)(long long)t);
    }
}

static void pool_for(long long count, range_fn fn, void *arg) {
    g_pool.fn = fn;
    g_pool.arg = arg;
    g_pool.count = count;
    if (g_pool.n == 1 || count < 65536) {
        for (int t = 0; t < g_pool.n; ++t) g_part[t] = 0.0;
        fn(arg, 0, count, 0);
        return;
    }
    pthread_barrier_wait(&g_pool.start);
    pool_run_part(0);
    pthread_barrier_wait(&g_pool.done);
}

typedef struct {
    const csr *A;
    double *x, *r, *s, *z;
    double alpha, beta;
} cg_args;

static void spmv_range(void *p, long long lo, long long hi, int t) {
    cg_args *a = (cg_args *)p;
    (void)t;
    for (long long i = lo; i < hi; ++i) {
        double acc = 0;
        for (long long e = a->A->rowstart[i]; e < a->A->rowstart[i + 1]; ++e) acc += a->A->val[e] * a->s[a->A->col[e]];
        a->z[i] = acc;
    }
}

/* x += alpha s; r += (-alpha) z; per-thread max |r| */
static void update_range(void *p, long long lo, long long hi, int t) {
    cg_args *a = (cg_args *)p;
    double m = 0.0;
    for (long long i = lo; i < hi; ++i) a->x[i] += a->alpha * a->s[i];
    for (long long i = lo; i < hi; ++i) {
        a->r[i] += (-a->alpha) * a->z[i];
        if (fabs(a->r[i]) > m) m = fabs(a->r[i]);
    }
    g_part[t] = m;
}

/* z = r + beta s */
static void direction_range(void *p, long long lo, long long hi, int t) {
    cg_args *a = (cg_args *)p;
    (void)t;
    for (long long i = lo; i < hi; ++i) {
        a->z[i] = a->r[i];
        a->z[i] += a->beta * a->s[i];
    }
}

/* PCGSolver<double>::solve with the identity preconditioner
 * (pcg_solver.h:246-295, :379-384). x is zeroed first. */
static void cg_solve(const csr *A, const double *b, double *x, const oracle_params *prm, oracle_stats *st) {
    const long long n = A->n;
    double *r = (double *)malloc(sizeof(double) * (n ? n : 1));
    double *s = (double *)malloc(sizeof(double) * (n ? n : 1));
    double *z = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (long long i = 0; i < n; ++i) { x[i] = 0.0; r[i] = b[i]; }
    double tolf = prm->residual < 1e-30 ? 1e-30 : prm->residual;
    /* abs_max: fabs(x[idamax]) -- first index of the largest |x| */
    double res = 0.0;
    for (long long i = 0; i < n; ++i) if (fabs(r[i]) > res) res = fabs(r[i]);
    double res0 = res;
    st->b_inf = res0;
    st->iterations = 0;
    st->converged = 1;
    st->reresid = res;
    if (res == 0.0 || n == 0) { free(r); free(s); free(z); return; }
    double tol = tolf * res;
    for (long long i = 0; i < n; ++i) z[i] = r[i];
    double rho = 0.0;
    for (long long i = 0; i < n; ++i) rho += z[i] * r[i];
    if (rho == 0.0 || rho != rho) { st->converged = 0; free(r); free(s); free(z); return; }
    for (long long i = 0; i < n; ++i) s[i] = z[i];
    int it;
    cg_args ca = {A, x, r, s, z, 0.0, 0.0};
    for (it = 0; it < prm->max_iterations; ++it) {
        ca.s = s;
        ca.z = z;
        pool_for(n, spmv_range, &ca);
        double sz = 0.0;
        for (long long i = 0; i < n; ++i) sz += s[i] * z[i];
        double alpha = rho / sz;
        ca.alpha = alpha;
        pool_for(n, update_range, &ca);
        res = 0.0;
        for (int t = 0; t < g_pool.n; ++t) if (g_part[t] > res) res = g_part[t];
        if (res <= tol) {
            st->iterations = it + 1;
            st->reresid = res / res0;
            st->converged = 1;
            free(r); free(s); free(z);
            return;
        }
        double rho_new = 0.0;
        for (long long i = 0; i < n; ++i) rho_new += r[i] * r[i];
        double beta = rho_new / rho;
        ca.beta = beta;
        pool_for(n, direction_range, &ca);
        double *t = s; s = z; z = t; /* s = beta*s + z */
        rho = rho_new;
    }
    st->iterations = it;
    st->reresid = res / res0;
    st->converged = 0;
    free(r); free(s); free(z);
}

/* Numbers the unknowns in the reference's serial tile-major order. A cell is
 * an unknown iff fluid<0 and some in-bounds neighbour has fluid<0 across a
 * face with area>0 and rho>0 (mark_body, macpressuresolver3.cpp:123-147).
 * index[cell] = number or -1. Returns the count. */
static long long label_cells(const oracle_ctx *c, const float *fluid, float *const A[3], float *const R[3],
                             long long *index) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, dim = c->dim;
    const size_t ncell = (size_t)nx * ny * nz;
    for (size_t n = 0; n < ncell; ++n) index[n] = -1;
    long long count = 0;
    int bx = (nx + TILE - 1) / TILE, by = (ny + TILE - 1) / TILE, bz = dim == 3 ? (nz + TILE - 1) / TILE : 1;
    for (int tk = 0; tk < bz; ++tk)
        for (int tj = 0; tj < by; ++tj)
            for (int ti = 0; ti < bx; ++ti) {
                int oi = ti * TILE, oj = tj * TILE, ok = tk * TILE;
                int Zx = nx - oi < TILE ? nx - oi : TILE, Zy = ny - oj < TILE ? ny - oj : TILE;
                int Zz = dim == 3 ? (nz - ok < TILE ? nz - ok : TILE) : 1;
                for (int kk = 0; kk < Zz; ++kk)
                    for (int jj = 0; jj < Zy; ++jj)
                        for (int ii = 0; ii < Zx; ++ii) {
                            int i = oi + ii, j = oj + jj, k = ok + kk;
                            size_t cn = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                            if (!(fluid[cn] < 0.0f)) continue;
                            int inside = 0;
                            for (int nq = 0; nq < 2 * dim && !inside; ++nq) {
                                int d = nq / 2, plus = (nq % 2) == 0;
                                int q[3] = {i, j, k};
                                q[d] += plus ? 1 : -1;
                                int sh[3] = {nx, ny, nz};
                                if (q[d] < 0 || q[d] >= sh[d]) continue;
                                size_t qn = (size_t)q[0] + (size_t)nx * ((size_t)q[1] + (size_t)ny * q[2]);
                                if (!(fluid[qn] < 0.0f)) continue;
                                int f[3] = {i, j, k};
                                if (plus) f[d] += 1;
                                int fx = nx + (d == 0), fy = ny + (d == 1);
                                size_t fn = (size_t)f[0] + (size_t)fx * ((size_t)f[1] + (size_t)fy * f[2]);
                                if (A[d][fn] && R[d][fn]) inside = 1;
                            }
                            if (inside) index[cn] = count++;
                        }
            }
    return count;
}

/* One projection, in place on the face velocities.
 * Dense layouts, x fastest: solid nodal (nx+1)(ny+1)(nz+1) [(nx+1)(ny+1) in
 * 2D], fluid nx*ny*nz, u (nx+1)*ny*nz, v nx*(ny+1)*nz, w nx*ny*(nz+1)
 * (w unused in 2D). pressure: cells (float, 0 off the unknowns).
 * index_out (optional): unknown number per cell or -1.
 * Returns 0. */
/* oracle_project plus, when on_u is not NULL, the faces the reference's
 * velocity update leaves active (1) or deactivates with set_off (0):
 * macpressuresolver3.cpp:252-267 and macpressuresolver2.cpp:221-236. */
int oracle_project_active(oracle_ctx *c, double dt, const float *solid, const float *fluid, float *u, float *v,
                          float *w, const oracle_params *prm, float *pressure, long long *index_out, oracle_stats *st,
                          unsigned char *on_u, unsigned char *on_v, unsigned char *on_w);

int oracle_project(oracle_ctx *c, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                   const oracle_params *prm, float *pressure, long long *index_out, oracle_stats *st) {
    return oracle_project_active(c, dt, solid, fluid, u, v, w, prm, pressure, index_out, st, NULL, NULL, NULL);
}

int oracle_project_active(oracle_ctx *c, double dt, const float *solid, const float *fluid, float *u, float *v,
                          float *w, const oracle_params *prm, float *pressure, long long *index_out, oracle_stats *st,
                          unsigned char *on_u, unsigned char *on_v, unsigned char *on_w) {
    unsigned char *on[3] = {on_u, on_v, on_w};
    const int nx = c->nx, ny = c->ny, nz = c->nz, dim = c->dim;
    const double dx = c->dx;
    const size_t ncell = (size_t)nx * ny * nz;
    size_t nf[3];
    for (int d = 0; d < 3; ++d)
        nf[d] = (d < dim) ? (size_t)(nx + (d == 0)) * (ny + (d == 1)) * (dim == 3 ? nz + (d == 2) : 1) : 1;
    float *A[3], *R[3];
    for (int d = 0; d < 3; ++d) {
        A[d] = (float *)calloc(nf[d], sizeof(float));
        R[d] = (float *)calloc(nf[d], sizeof(float));
    }
    oracle_face_fractions(c, solid, fluid, prm, A[0], A[1], A[2], R[0], R[1], R[2]);
    if (prm->surface_tension != 0.0) {
        float *vel_st[3] = {u, v, w};
        apply_surface_tension(c, fluid, R, vel_st, dt, prm->surface_tension);
    }
    int fluid_exists = 0;
    for (size_t n = 0; n < ncell; ++n)
        if (fluid[n] < 0.0f) { fluid_exists = 1; break; }
    (void)fluid_exists;

    long long *index = (long long *)malloc(sizeof(long long) * ncell);
    long long nunk = label_cells(c, fluid, A, R, index);
    st->unknowns = nunk;

    /* assembly (macpressuresolver3.cpp:163-199 / macpressuresolver2.cpp:148-179) */
    csr M;
    M.n = nunk;
    M.rowstart = (long long *)malloc(sizeof(long long) * (size_t)(nunk + 1));
    M.col = (long long *)malloc(sizeof(long long) * (size_t)(nunk ? nunk : 1) * 7);
    M.val = (double *)malloc(sizeof(double) * (size_t)(nunk ? nunk : 1) * 7);
    double *b = (double *)calloc((size_t)(nunk ? nunk : 1), sizeof(double));
    float *vel[3] = {u, v, w};
    /* rows are filled in unknown order so the CSR is contiguous */
    long long *cell_of = (long long *)malloc(sizeof(long long) * (size_t)(nunk ? nunk : 1));
    for (size_t cn = 0; cn < ncell; ++cn)
        if (index[cn] >= 0) cell_of[index[cn]] = (long long)cn;
    long long nnz = 0;
    for (long long row = 0; row < nunk; ++row) {
        size_t cn = (size_t)cell_of[row];
        int i = (int)(cn % nx), j = (int)((cn / nx) % ny), k = (int)(cn / ((size_t)nx * ny));
        M.rowstart[row] = nnz;
        long long cols[7];
        double vals[7];
        int cnt = 0;
        double rhs = 0.0;
        double diagonal = 0.0;
        for (int nq = 0; nq < 2 * dim; ++nq) {
            int d = nq / 2, plus = (nq % 2) == 0;
            int sgn = plus ? 1 : -1;
            int q[3] = {i, j, k};
            q[d] += sgn;
            int sh[3] = {nx, ny, nz};
            if (q[d] < 0 || q[d] >= sh[d]) continue;
            int f[3] = {i, j, k};
            if (plus) f[d] += 1;
            int fx = nx + (d == 0), fy = ny + (d == 1);
            size_t fn = (size_t)f[0] + (size_t)fx * ((size_t)f[1] + (size_t)fy * f[2]);
            double area = A[d][fn];
            if (dim == 3) {
                if (area) {
                    double rho = R[d][fn];
                    if (rho) {
                        double value = dt * area / (dx * dx * rho);
                        size_t qn = (size_t)q[0] + (size_t)nx * ((size_t)q[1] + (size_t)ny * q[2]);
                        if (fluid[qn] < 0.0f) row_insert(cols, vals, &cnt, index[qn], -value);
                        diagonal += value;
                    }
                    rhs += -sgn * area * (double)vel[d][fn] / dx;
                }
            } else {
                if (area) {
                    double rho = R[d][fn];
                    if (rho) {
                        double value = dt * area / (dx * dx * rho);
                        size_t qn = (size_t)q[0] + (size_t)nx * (size_t)q[1];
                        if (fluid[qn] < 0.0f) row_insert(cols, vals, &cnt, index[qn], -value);
                        diagonal += value;
                    }
                }
                rhs += -sgn * area * (double)vel[d][fn] / dx;
            }
        }
        row_insert(cols, vals, &cnt, row, diagonal);
        for (int e = 0; e < cnt; ++e) {
            M.col[nnz] = cols[e];
            M.val[nnz] = vals[e];
            nnz++;
        }
        b[row] = rhs;
    }
    M.rowstart[nunk] = nnz;

    /* volume correction (macpressuresolver3.cpp:204-217) */
    if (prm->gain && c->target_volume) {
        double xv = (c->current_volume - c->target_volume) / c->target_volume;
        double y = c->y_prev + xv * dt;
        c->y_prev = y;
        double kp = prm->gain * 2.3 / (25.0 * 0.01);
        double ki = kp * kp / 16.0;
        double rhs_correct = -(kp * xv + ki * y) / (xv + 1.0);
        for (long long r = 0; r < nunk; ++r) b[r] += rhs_correct;
    }

    /* warm start (macpressuresolver3.cpp:221-230): b -= A * prev */
    if (prm->warm_start) {
        if (!c->have_prev) {
            c->prev = (double *)calloc((size_t)(nunk ? nunk : 1), sizeof(double));
            c->prev_n = nunk;
            c->have_prev = 1;
        } else if (c->prev_n != nunk) {
            double *np = (double *)calloc((size_t)(nunk ? nunk : 1), sizeof(double));
            long long keep = c->prev_n < nunk ? c->prev_n : nunk;
            memcpy(np, c->prev, sizeof(double) * (size_t)keep);
            free(c->prev);
            c->prev = np;
            c->prev_n = nunk;
        }
        for (long long r = 0; r < nunk; ++r) {
            double sum = 0.0;
            for (long long e = M.rowstart[r]; e < M.rowstart[r + 1]; ++e) sum += c->prev[M.col[e]] * M.val[e];
            b[r] -= sum;
        }
    }

    double *x = (double *)calloc((size_t)(nunk ? nunk : 1), sizeof(double));
    cg_solve(&M, b, x, prm, st);

    if (prm->warm_start) {
        for (long long r = 0; r < nunk; ++r) x[r] += c->prev[r];
        memcpy(c->prev, x, sizeof(double) * (size_t)nunk);
    }

    /* scatter to the float pressure array (macpressuresolver3.cpp:245-248) */
    for (size_t cn = 0; cn < ncell; ++cn) pressure[cn] = index[cn] >= 0 ? (float)x[index[cn]] : 0.0f;

    /* velocity update (macpressuresolver3.cpp:252-268 / macpressuresolver2.cpp:221-237) */
    for (int d = 0; d < dim; ++d) {
        int fx = nx + (d == 0), fy = ny + (d == 1), fz = dim == 3 ? nz + (d == 2) : 1;
        int sh[3] = {nx, ny, nz};
        for (int k = 0; k < fz; ++k)
            for (int j = 0; j < fy; ++j)
                for (int i = 0; i < fx; ++i) {
                    size_t fn = (size_t)i + (size_t)fx * ((size_t)j + (size_t)fy * k);
                    int pi[3] = {i, j, k};
                    float rho = R[d][fn];
                    float *uu = &vel[d][fn];
                    if (on[0]) {
                        int keep = A[d][fn] && rho;
                        if (!keep && pi[d] == 0) {
                            size_t cn = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                            keep = fluid[cn] < 0.0f && (dim == 3 || *uu < 0.0f);
                        } else if (!keep && pi[d] == sh[d]) {
                            int m[3] = {i, j, k};
                            m[d] -= 1;
                            size_t cn = (size_t)m[0] + (size_t)nx * ((size_t)m[1] + (size_t)ny * m[2]);
                            keep = fluid[cn] < 0.0f && (dim == 3 || *uu > 0.0f);
                        }
                        on[d][fn] = (unsigned char)keep;
                    }
                    if (A[d][fn] && rho) {
                        if (pi[d] == 0 || pi[d] == sh[d]) *uu = 0.0f;
                        else {
                            size_t c0 = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                            int m[3] = {i, j, k};
                            m[d] -= 1;
                            size_t c1 = (size_t)m[0] + (size_t)nx * ((size_t)m[1] + (size_t)ny * m[2]);
                            float dp = pressure[c0] - pressure[c1];
                            double val = dt * (double)dp / ((double)rho * dx);
                            *uu -= (float)val;
                        }
                    } else {
                        /* boundary faces next to fluid are set to 0, the rest are
                         * deactivated, which reads back as the background 0 */
                        *uu = 0.0f;
                    }
                }
    }

    if (index_out) memcpy(index_out, index, sizeof(long long) * ncell);
    free(x);
    free(b);
    free(cell_of);
    csr_free(&M);
    free(index);
    for (int d = 0; d < 3; ++d) {
        free(A[d]);
        free(R[d]);
    }
    return 0;
}

/* Matrix-free pieces used by the tests to check the GPU's operator and
 * right-hand side without going through CG. diag/cpx/cpy/cpz/b are dense per
 * cell (0 off the unknowns); cp? is the coupling weight of the cell's +d face
 * (the negated off-diagonal, 0 unless both cells are unknowns). */
int oracle_assemble(oracle_ctx *c, double dt, const float *solid, const float *fluid, const float *u, const float *v,
                    const float *w, const oracle_params *prm, double *diag, double *cpx, double *cpy, double *cpz,
                    double *b, long long *index_out) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, dim = c->dim;
    const double dx = c->dx;
    const size_t ncell = (size_t)nx * ny * nz;
    size_t nf[3];
    for (int d = 0; d < 3; ++d)
        nf[d] = (d < dim) ? (size_t)(nx + (d == 0)) * (ny + (d == 1)) * (dim == 3 ? nz + (d == 2) : 1) : 1;
    float *A[3], *R[3];
    for (int d = 0; d < 3; ++d) {
        A[d] = (float *)calloc(nf[d], sizeof(float));
        R[d] = (float *)calloc(nf[d], sizeof(float));
    }
    oracle_face_fractions(c, solid, fluid, prm, A[0], A[1], A[2], R[0], R[1], R[2]);
    long long *index = index_out ? index_out : (long long *)malloc(sizeof(long long) * ncell);
    label_cells(c, fluid, A, R, index);
    const float *vel[3] = {u, v, w};
    float *vel_st[3] = {NULL, NULL, NULL};
    if (prm->surface_tension != 0.0) {
        for (int d = 0; d < dim; ++d) {
            vel_st[d] = (float *)malloc(nf[d] * sizeof(float));
            memcpy(vel_st[d], vel[d], nf[d] * sizeof(float));
        }
        apply_surface_tension(c, fluid, R, vel_st, dt, prm->surface_tension);
        for (int d = 0; d < dim; ++d) vel[d] = vel_st[d];
    }
    double *cp[3] = {cpx, cpy, cpz};
    for (size_t cn = 0; cn < ncell; ++cn) {
        diag[cn] = 0.0;
        b[cn] = 0.0;
        for (int d = 0; d < dim; ++d) cp[d][cn] = 0.0;
        if (index[cn] < 0) continue;
        int i = (int)(cn % nx), j = (int)((cn / nx) % ny), k = (int)(cn / ((size_t)nx * ny));
        double rhs = 0.0, diagonal = 0.0;
        for (int nq = 0; nq < 2 * dim; ++nq) {
            int d = nq / 2, plus = (nq % 2) == 0;
            int sgn = plus ? 1 : -1;
            int q[3] = {i, j, k};
            q[d] += sgn;
            int sh[3] = {nx, ny, nz};
            if (q[d] < 0 || q[d] >= sh[d]) continue;
            int f[3] = {i, j, k};
            if (plus) f[d] += 1;
            int fx = nx + (d == 0), fy = ny + (d == 1);
            size_t fn = (size_t)f[0] + (size_t)fx * ((size_t)f[1] + (size_t)fy * f[2]);
            double area = A[d][fn];
            if (area) {
                double rho = R[d][fn];
                if (rho) {
                    double value = dt * area / (dx * dx * rho);
                    size_t qn = (size_t)q[0] + (size_t)nx * ((size_t)q[1] + (size_t)ny * q[2]);
                    if (plus && fluid[qn] < 0.0f) cp[d][cn] = value;
                    diagonal += value;
                }
                rhs += -sgn * area * (double)vel[d][fn] / dx;
            }
        }
        diag[cn] = diagonal;
        b[cn] = rhs;
    }
    if (!index_out) free(index);
    for (int d = 0; d < 3; ++d) {
        free(A[d]);
        free(R[d]);
        free(vel_st[d]);
    }
    return 0;
}
