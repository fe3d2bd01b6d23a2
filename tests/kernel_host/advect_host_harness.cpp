// advect_host_harness.cpp -- TEST INFRASTRUCTURE: the per-element code of
// the advection and solid-constraint kernels (shiokaze_gb300/csrc/
// advect_core.cuh, the same source the CUDA kernels call), compiled for the
// host with g++ -ffp-contract=off and run element by element in the
// kernels' launch order. tests/test_kernel_host.py compares it with the
// reference's fixtures and the oracle bit for bit, so every CPU test run
// checks the kernels' arithmetic and indexing. The kernels are data-parallel
// with no dependence between elements of one launch (forward passes write
// scratch only; backward passes read the step's input only at their own
// element), so the sequential order gives the parallel result. Not part of
// the library.
#include <algorithm>
#include <cmath>
#include <vector>

#include "advect_core.cuh"
using namespace gba;
extern "C" int host_advect3(int nx, int ny, int nz, double dx, double dt, int mac, int trim, float *u, float *v,
                           float *w, const float *fluid, float *q, const unsigned char *mask, float bg) {
    Dims g{};
    g.nx = nx; g.ny = ny; g.nz = nz; g.dx = dx;
    int e = 0;
    const double m = std::frexp(dx, &e);
    const double inv = 1.0 / dx;
    g.pow2 = (m == 0.5 && std::isfinite(inv) && (double)(float)inv == inv) ? 1 : 0;
    g.inv_dx = inv; g.inv_dx_f = (float)inv; g.limit = -dx * (double)trim;
    long long cells = (long long)nx * ny * nz;
    long long nf0 = (long long)(nx + 1) * ny * nz, nf1 = (long long)nx * (ny + 1) * nz, nf2 = (long long)nx * ny * (nz + 1);
    std::vector<float> v0(nf0 + nf1 + nf2), q0(cells);
    std::vector<MinMax> vmm(nf0 + nf1 + nf2), qmm(cells);
    StepArgs s{};
    s.g = g; s.dt = dt; s.u = u; s.v = v; s.w = w; s.fluid = fluid; s.q = q; s.mask = mask; s.bg = bg;
    s.v0 = v0.data(); s.vmm = vmm.data(); s.off1 = nf0; s.off2 = nf0 + nf1; s.q0 = q0.data(); s.qmm = qmm.data();
    long long nfmax = std::max(nf0, std::max(nf1, nf2));
    if (q) {
        if (mac) {
            for (long long c = 0; c < cells; ++c) cell_forward<true>(s, (unsigned)c);
            for (long long c = 0; c < cells; ++c) cell_backward(s, (unsigned)c);
        } else {
            for (long long c = 0; c < cells; ++c) cell_forward<false>(s, (unsigned)c);
            for (long long c = 0; c < cells; ++c) q[c] = q0[c];
        }
    }
    if (mac) {
        for (int d = 0; d < 3; ++d) for (long long f = 0; f < nfmax; ++f) face_forward<true>(s, d, (unsigned)f);
        for (int d = 0; d < 3; ++d) for (long long f = 0; f < nfmax; ++f) face_backward(s, d, (unsigned)f);
    } else {
        for (int d = 0; d < 3; ++d) for (long long f = 0; f < nfmax; ++f) face_forward<false>(s, d, (unsigned)f);
        for (long long f = 0; f < nf0; ++f) u[f] = v0[f];
        for (long long f = 0; f < nf1; ++f) v[f] = v0[nf0 + f];
        for (long long f = 0; f < nf2; ++f) w[f] = v0[nf0 + nf1 + f];
    }
    return 0;
}

extern "C" int host_constrain3(int nx, int ny, int nz, double dx, const float *solid, float *u, float *v, float *w,
                              const unsigned char *mu, const unsigned char *mv, const unsigned char *mw) {
    long long nf0 = (long long)(nx + 1) * ny * nz, nf1 = (long long)nx * (ny + 1) * nz, nf2 = (long long)nx * ny * (nz + 1);
    std::vector<float> save(nf0 + nf1 + nf2);
    std::copy(u, u + nf0, save.begin()); std::copy(v, v + nf1, save.begin() + nf0); std::copy(w, w + nf2, save.begin() + nf0 + nf1);
    long long nodes = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    int exists = 0;
    for (long long i = 0; i < nodes; ++i) exists |= solid[i] < 0.0f;
    ConstrainArgs c{};
    Dims g{}; g.nx = nx; g.ny = ny; g.nz = nz; g.dx = dx;
    c.g = g; c.solid = solid; c.save = save.data(); c.off1 = nf0; c.off2 = nf0 + nf1; c.u = u; c.v = v; c.w = w;
    c.mu = mu; c.mv = mv; c.mw = mw; c.exists = &exists;
    long long nfmax = std::max(nf0, std::max(nf1, nf2));
    for (int d = 0; d < 3; ++d) for (long long f = 0; f < nfmax; ++f) constrain_face(c, d, (unsigned)f);
    return 0;
}

// The 2D passes (face_forward2 ... cell_backward2) in the kernels' order.
extern "C" int host_advect2(int nx, int ny, double dx, double dt, int mac, int trim, float *u, float *v,
                           const float *fluid, float *q, const unsigned char *mask, float bg) {
    Dims g{};
    g.nx = nx; g.ny = ny; g.nz = 1; g.dx = dx;
    int e = 0;
    const double m = std::frexp(dx, &e);
    const double inv = 1.0 / dx;
    g.pow2 = (m == 0.5 && std::isfinite(inv) && (double)(float)inv == inv) ? 1 : 0;
    g.inv_dx = inv; g.inv_dx_f = (float)inv; g.limit = -dx * (double)trim;
    long long cells = (long long)nx * ny;
    long long nf0 = (long long)(nx + 1) * ny, nf1 = (long long)nx * (ny + 1);
    std::vector<float> v0(nf0 + nf1), q0(cells);
    std::vector<MinMax> vmm(nf0 + nf1), qmm(cells);
    StepArgs s{};
    s.g = g; s.dt = dt; s.u = u; s.v = v; s.w = nullptr; s.fluid = fluid; s.q = q; s.mask = mask; s.bg = bg;
    s.v0 = v0.data(); s.vmm = vmm.data(); s.off1 = nf0; s.off2 = 0; s.q0 = q0.data(); s.qmm = qmm.data();
    long long nfmax = std::max(nf0, nf1);
    if (q) {
        if (mac) {
            for (long long c = 0; c < cells; ++c) cell_forward2<true>(s, (unsigned)c);
            for (long long c = 0; c < cells; ++c) cell_backward2(s, (unsigned)c);
        } else {
            for (long long c = 0; c < cells; ++c) cell_forward2<false>(s, (unsigned)c);
            for (long long c = 0; c < cells; ++c) q[c] = q0[c];
        }
    }
    if (mac) {
        for (int d = 0; d < 2; ++d) for (long long f = 0; f < nfmax; ++f) face_forward2<true>(s, d, (unsigned)f);
        for (int d = 0; d < 2; ++d) for (long long f = 0; f < nfmax; ++f) face_backward2(s, d, (unsigned)f);
    } else {
        for (int d = 0; d < 2; ++d) for (long long f = 0; f < nfmax; ++f) face_forward2<false>(s, d, (unsigned)f);
        for (long long f = 0; f < nf0; ++f) u[f] = v0[f];
        for (long long f = 0; f < nf1; ++f) v[f] = v0[nf0 + f];
    }
    return 0;
}
