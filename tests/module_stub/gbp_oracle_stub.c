/*
 * gbp_oracle_stub.c -- TEST INFRASTRUCTURE: a stand-in for libgbp's
 * advection entry points that runs the oracle (oracle/advect_oracle.c, in
 * liboracle.so) on the CPU, and the same for the solid constraint of the
 * velocity. tests/test_oracle.py links the gbadvection3 and gbutility3
 * plugin modules against it to check the modules' boundary (dense copies
 * of the reference's tiled arrays, the active masks, the write-back over
 * active faces and cells) against the reference's own macadvection3 and
 * macutility3 without a GPU.
 * The shipped module links the real libgbp.so.
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

int gbp_constrain_velocity3(gbp_ctx *ctx, int nx, int ny, int nz, double dx, const float *solid, float *u, float *v,
                            float *w, const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    (void)ctx;
    return oracle_constrain_velocity3(nx, ny, nz, dx, solid, u, v, w, mu, mv, mw);
}
