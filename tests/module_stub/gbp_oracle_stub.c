/*
 * gbp_oracle_stub.c -- TEST INFRASTRUCTURE: a stand-in for libgbp's
 * advection entry points (2D and 3D) that runs the oracle (oracle/advect_oracle.c, in
 * liboracle.so) on the CPU, and the same for the solid constraint of the
 * velocity, its extrapolation, and the projection (oracle/gbp_oracle.c: scenes, volume
 * correction, warm start, gbp_project / gbp_project_active with the active
 * sets, gbp_project_bricks on the expanded bricks). tests/test_oracle.py links the gbadvection3, gbutility3 and
 * gbprojection2/3 plugin modules against it to check the modules' boundary
 * (dense copies of the reference's tiled arrays, the active masks, the
 * write-back over active faces and cells, the faces turned off, the
 * pressure's active cells) against the reference's own modules without a
 * GPU. The shipped modules link the real libgbp.so.
 */
#include <stdlib.h>
#include <string.h>

#include "gbp.h"

int oracle_constrain_velocity3(int nx, int ny, int nz, double dx, const float *solid, float *u, float *v, float *w,
                               const unsigned char *mu, const unsigned char *mv, const unsigned char *mw);
int oracle_advect3(int nx, int ny, int nz, double dx, double dt, int maccormack, int trim, float *u, float *v,
                   float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg);

struct gbp_ctx {
    int device;
};

int gbp_create(int device, gbp_ctx **out) {
    *out = (gbp_ctx *)malloc(sizeof(gbp_ctx));
    (*out)->device = device;
    return GBP_OK;
}

void gbp_destroy(gbp_ctx *ctx) { free(ctx); }

const char *gbp_strerror(int status) { return status ? "oracle stub: bad argument" : "ok"; }

void gbp_advect_params_default(gbp_advect_params *p) {
    p->maccormack = 1;
    p->trim_narrowband = 1;
    p->advect_velocity = 1;
}

int gbp_advect3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, double dt, const gbp_advect_params *p, float *u,
                float *v, float *w, const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    (void)ctx;
    if (p->advect_velocity)
        return oracle_advect3(nx, ny, nz, dx, dt, p->maccormack, p->trim_narrowband, u, v, w, fluid, q, q_mask, q_bg);
    /* the scalar alone: the oracle also advects the velocity, so give it copies */
    const size_t n[3] = {(size_t)(nx + 1) * ny * nz, (size_t)nx * (ny + 1) * nz, (size_t)nx * ny * (nz + 1)};
    float *c[3];
    const float *src[3] = {u, v, w};
    for (int d = 0; d < 3; ++d) {
        c[d] = (float *)malloc(sizeof(float) * n[d]);
        memcpy(c[d], src[d], sizeof(float) * n[d]);
    }
    int rc = oracle_advect3(nx, ny, nz, dx, dt, p->maccormack, p->trim_narrowband, c[0], c[1], c[2], fluid, q, q_mask,
                            q_bg);
    for (int d = 0; d < 3; ++d) free(c[d]);
    return rc;
}

int oracle_advect2(int nx, int ny, double dx, double dt, int maccormack, int trim, float *u, float *v,
                   const float *fluid, float *q, const unsigned char *q_mask, float q_bg);

int gbp_advect2(gbp_ctx *ctx, int nx, int ny, double dx, double dt, const gbp_advect_params *p, float *u, float *v,
                const float *fluid, float *q, const unsigned char *q_mask, float q_bg) {
    (void)ctx;
    if (p->advect_velocity)
        return oracle_advect2(nx, ny, dx, dt, p->maccormack, p->trim_narrowband, u, v, fluid, q, q_mask, q_bg);
    const size_t n[2] = {(size_t)(nx + 1) * ny, (size_t)nx * (ny + 1)};
    float *c[2];
    const float *src[2] = {u, v};
    for (int d = 0; d < 2; ++d) {
        c[d] = (float *)malloc(sizeof(float) * n[d]);
        memcpy(c[d], src[d], sizeof(float) * n[d]);
    }
    int rc = oracle_advect2(nx, ny, dx, dt, p->maccormack, p->trim_narrowband, c[0], c[1], fluid, q, q_mask, q_bg);
    for (int d = 0; d < 2; ++d) free(c[d]);
    return rc;
}

int gbp_constrain_velocity3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid, float *u, float *v,
                            float *w, const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    (void)ctx;
    return oracle_constrain_velocity3(nx, ny, nz, dx, solid, u, v, w, mu, mv, mw);
}

long long oracle_extrapolate3(int w, int h, int d, float *a, unsigned char *active, int count);

int gbp_extrapolate3(gbp_ctx *ctx, int w, int h, int d, float *a, unsigned char *active, int count,
                     long long *activated) {
    (void)ctx;
    long long n = oracle_extrapolate3(w, h, d, a, active, count);
    if (activated) *activated = n;
    return GBP_OK;
}

int gbp_extrapolate_constrain_velocity3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid,
                                        float *u, float *v, float *w, unsigned char *mu, unsigned char *mv,
                                        unsigned char *mw, int width) {
    (void)ctx;
    float *c[3] = {u, v, w};
    unsigned char *m[3] = {mu, mv, mw};
    if (mu)
        for (int d = 0; d < 3; ++d) oracle_extrapolate3(nx + (d == 0), ny + (d == 1), nz + (d == 2), c[d], m[d], width);
    return oracle_constrain_velocity3(nx, ny, nz, dx, solid, u, v, w, mu, mv, mw);
}


/* ---- projection, backed by oracle/gbp_oracle.c ---------------------------- */

typedef struct {
    double residual;
    int max_iterations;
    int warm_start;
    double eps_fluid;
    double eps_solid;
    int second_order_fluid;
    int second_order_solid;
    double gain;
    double surface_tension;
} oracle_params;

typedef struct {
    int iterations;
    int converged;
    double reresid;
    long long unknowns;
    double b_inf;
} oracle_stats;

typedef struct oracle_ctx oracle_ctx;
oracle_ctx *oracle_create(int dim, int nx, int ny, int nz, double dx);
void oracle_destroy(oracle_ctx *c);
void oracle_set_target_volume(oracle_ctx *c, double current_volume, double target_volume);
int oracle_project_active(oracle_ctx *c, double dt, const float *solid, const float *fluid, float *u, float *v,
                          float *w, const oracle_params *prm, float *pressure, long long *index_out, oracle_stats *st,
                          unsigned char *on_u, unsigned char *on_v, unsigned char *on_w);

struct gbp_scene {
    oracle_ctx *oc;
    int dim, nx, ny, nz;
};

void gbp_params_default(gbp_params *p) {
    memset(p, 0, sizeof(*p));
    p->residual = 1e-4;
    p->max_iterations = 30000;
    p->eps_fluid = 1e-2;
    p->eps_solid = 1e-2;
    p->second_order_fluid = 1;
    p->second_order_solid = 1;
    p->gain = 1.0;
    p->mg_smooth = 1;
    p->mg_coarsest = 4;
    p->inner_tolerance = 1e-3;
    p->iterations_per_sync = 16;
    p->tile_classes = 1;
}

int gbp_scene_create(gbp_ctx *ctx, int dim, int nx, int ny, int nz, double dx, gbp_scene **out) {
    (void)ctx;
    gbp_scene *s = (gbp_scene *)malloc(sizeof(gbp_scene));
    s->dim = dim;
    s->nx = nx;
    s->ny = ny;
    s->nz = dim == 3 ? nz : 1;
    s->oc = oracle_create(dim, nx, ny, s->nz, dx);
    *out = s;
    return GBP_OK;
}

void gbp_scene_destroy(gbp_scene *s) {
    if (!s) return;
    oracle_destroy(s->oc);
    free(s);
}

int gbp_scene_set_target_volume(gbp_scene *s, double current_volume, double target_volume) {
    oracle_set_target_volume(s->oc, current_volume, target_volume);
    return GBP_OK;
}

int gbp_project_active(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                       const gbp_params *params, float *pressure, gbp_stats *stats, unsigned char *unknown,
                       unsigned char *u_active, unsigned char *v_active, unsigned char *w_active) {
    gbp_params p;
    gbp_params_default(&p);
    if (params) p = *params;
    oracle_params op = {p.residual, p.max_iterations, p.warm_start, p.eps_fluid, p.eps_solid,
                        p.second_order_fluid, p.second_order_solid, p.gain, p.surface_tension};
    const size_t ncell = (size_t)s->nx * s->ny * s->nz;
    long long *index = unknown ? (long long *)malloc(sizeof(long long) * ncell) : NULL;
    oracle_stats st;
    memset(&st, 0, sizeof(st));
    oracle_project_active(s->oc, dt, solid, fluid, u, v, s->dim == 3 ? w : NULL, &op, pressure, index, &st,
                          u_active, v_active, s->dim == 3 ? w_active : NULL);
    if (unknown)
        for (size_t n = 0; n < ncell; ++n) unknown[n] = index[n] >= 0 ? 1 : 0;
    free(index);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = st.iterations;
        stats->outer_iterations = 1;
        stats->converged = st.converged;
        stats->reresid = st.reresid;
        stats->unknowns = st.unknowns;
    }
    return st.converged ? GBP_OK : GBP_ERR_NOT_CONVERGED;
}

int gbp_project(gbp_scene *s, double dt, const float *solid, const float *fluid, float *u, float *v, float *w,
                const gbp_params *params, float *pressure, gbp_stats *stats) {
    return gbp_project_active(s, dt, solid, fluid, u, v, w, params, pressure, stats, NULL, NULL, NULL, NULL);
}

/* gbp_project_bricks / gbp_bricks_expand on the CPU: the bricks expanded
 * to dense arrays (the rule of include/gbp.h), gbp_project_active above on
 * them, and the listed output bricks gathered back. */
static void stub_expand(int nx, int ny, int nz, const gbp_bricks *in, float *dense) {
    const int nbx = (nx + 7) / 8, nby = (ny + 7) / 8;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int sl = in->slot[(i >> 3) + (size_t)nbx * ((j >> 3) + (size_t)nby * (k >> 3))];
                float val = in->background;
                if (sl >= 0) val = in->values[(size_t)sl * GBP_BRICK_CELLS + (i & 7) + 8 * ((j & 7) + 8 * (k & 7))];
                else if (sl == GBP_BRICK_FILL) val = in->fill;
                dense[i + (size_t)nx * (j + (size_t)ny * k)] = val;
            }
}

static void stub_gather(int nx, int ny, int nz, const float *dense, const unsigned char *flags, gbp_bricks_out *o) {
    const int nbx = (nx + 7) / 8, nby = (ny + 7) / 8, nbz = (nz + 7) / 8;
    for (int bz = 0; bz < nbz; ++bz)
        for (int by = 0; by < nby; ++by)
            for (int bx = 0; bx < nbx; ++bx) {
                const int sl = o->slot[bx + (size_t)nbx * (by + (size_t)nby * bz)];
                if (sl < 0) continue;
                for (int c = 0; c < GBP_BRICK_CELLS; ++c) {
                    const int i = 8 * bx + (c & 7), j = 8 * by + ((c >> 3) & 7), k = 8 * bz + (c >> 6);
                    const size_t n = (size_t)sl * GBP_BRICK_CELLS + c;
                    const int in = i < nx && j < ny && k < nz;
                    const size_t d = i + (size_t)nx * (j + (size_t)ny * k);
                    o->values[n] = in ? dense[d] : 0.0f;
                    if (o->active) o->active[n] = in ? flags[d] : 0;
                }
            }
}

int gbp_bricks_expand(gbp_ctx *ctx, int nx, int ny, int nz, const gbp_bricks *in, float *dense, void *stream) {
    (void)ctx;
    (void)stream;
    stub_expand(nx, ny, nz, in, dense);
    return GBP_OK;
}

int gbp_project_bricks(gbp_scene *s, double dt, const gbp_bricks *solid, const gbp_bricks *fluid, const gbp_bricks *u,
                       const gbp_bricks *v, const gbp_bricks *w, const gbp_params *params, gbp_bricks_out *pressure,
                       gbp_bricks_out *u_out, gbp_bricks_out *v_out, gbp_bricks_out *w_out, gbp_stats *stats) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const int ext[5][3] = {{nx + 1, ny + 1, nz + 1}, {nx, ny, nz}, {nx + 1, ny, nz}, {nx, ny + 1, nz}, {nx, ny, nz + 1}};
    const gbp_bricks *in[5] = {solid, fluid, u, v, w};
    float *dense[5];
    unsigned char *flags[4];
    for (int a = 0; a < 5; ++a) {
        dense[a] = (float *)malloc(sizeof(float) * (size_t)ext[a][0] * ext[a][1] * ext[a][2]);
        stub_expand(ext[a][0], ext[a][1], ext[a][2], in[a], dense[a]);
    }
    for (int o = 0; o < 4; ++o) flags[o] = (unsigned char *)malloc((size_t)ext[o + 1][0] * ext[o + 1][1] * ext[o + 1][2]);
    float *p = (float *)malloc(sizeof(float) * (size_t)nx * ny * nz);
    const int rc = gbp_project_active(s, dt, dense[0], dense[1], dense[2], dense[3], dense[4], params, p, stats,
                                      flags[0], flags[1], flags[2], flags[3]);
    gbp_bricks_out *outs[4] = {pressure, u_out, v_out, w_out};
    const float *src[4] = {p, dense[2], dense[3], dense[4]};
    for (int o = 0; o < 4; ++o)
        if (outs[o]) stub_gather(ext[o + 1][0], ext[o + 1][1], ext[o + 1][2], src[o], flags[o], outs[o]);
    for (int a = 0; a < 5; ++a) free(dense[a]);
    for (int o = 0; o < 4; ++o) free(flags[o]);
    free(p);
    return rc;
}
