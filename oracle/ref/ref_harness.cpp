/*
 * ref_harness.cpp -- drives the reference's own pressure projection
 * (src/projection/macpressuresolver{2,3}.cpp, loaded through its module loader
 * src/core/module.cpp:103-172 by the name "macpressuresolver{2,3}") on dense
 * inputs, for the oracle.
 *
 * TEST INFRASTRUCTURE. This file is compiled against the reference's headers
 * by oracle/ref/Makefile into oracle/_ref/libref_harness.so. Only tests and
 * fixture generation load it. The shipped library never does.
 *
 * Dense -> sparse conversion follows the reference's scene setup
 * (src/utility/macutility3.cpp:317-358, assign_initial_variables): a level set
 * value is stored only where |v| < band, then the array is marked as a level
 * set of half-width `band` and flood filled, so inactive cells read +band
 * outside and -band inside. A "constant" level set (mode 1) is an array with
 * background value v[0] and no active cells, as the smoke scene builds its
 * fluid (src/smoke/macsmoke3.cpp:106). Velocity faces are all activated.
 *
 * After project() the harness reads pressure and velocity back through
 * operator(), which applies background/fill semantics, and reports which
 * pressure cells are active (the reference sets pressure only at unknowns,
 * macpressuresolver3.cpp:245-248) and which velocity faces stay active (its
 * velocity update deactivates closed faces, :252-267).
 */
#include <shiokaze/array/array2.h>
#include <shiokaze/array/array3.h>
#include <shiokaze/array/macarray2.h>
#include <shiokaze/array/macarray3.h>
#include <shiokaze/core/configuration.h>
#include <shiokaze/core/configurable.h>
#include <shiokaze/projection/macproject2_interface.h>
#include <shiokaze/advection/macadvection2_interface.h>
#include <shiokaze/advection/macadvection3_interface.h>
#include <shiokaze/utility/macutility3_interface.h>
#include <shiokaze/array/array_extrapolator3.h>

#include "gbarray_adapter.h"
#include <shiokaze/projection/macproject3_interface.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fcntl.h>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <unistd.h>

SHKZ_USING_NAMESPACE

namespace {

struct harness {
    int dim = 3;
    int nx = 0, ny = 0, nz = 1;
    double dx = 0.0;
    configuration *config = nullptr;
    std::unique_ptr<macproject3_driver> proj3;
    std::unique_ptr<macproject2_driver> proj2;
    shape3 shape3_;
    shape2 shape2_;
};

std::map<std::string, std::string> parse_kv(const char *kv) {
    std::map<std::string, std::string> out;
    if (!kv) return out;
    std::istringstream ss(kv);
    std::string tok;
    while (ss >> tok) {
        auto pos = tok.find('=');
        if (pos != std::string::npos) out[tok.substr(0, pos)] = tok.substr(pos + 1);
    }
    return out;
}

// Runs fn with stdout sent to log_path (appended), so the reference's console
// output (iteration count, residual, phase timings) can be parsed afterwards.
template <class F> void with_stdout_to(const char *log_path, F fn) {
    if (!log_path || !*log_path) { fn(); return; }
    fflush(stdout);
    int saved = dup(1);
    int fd = open(log_path, O_WRONLY | O_CREAT | O_APPEND, 0644);
    if (fd >= 0) { dup2(fd, 1); close(fd); }
    fn();
    fflush(stdout);
    if (saved >= 0) { dup2(saved, 1); close(saved); }
}

void fill_levelset3(array3<Real> &a, const shape3 &s, const float *v, int mode, float band) {
    if (mode == 1) {
        a.initialize(s, v[0]);
        return;
    }
    a.initialize(s, 0.0);
    for (int k = 0; k < (int)s.d; ++k)
        for (int j = 0; j < (int)s.h; ++j)
            for (int i = 0; i < (int)s.w; ++i) {
                float x = v[i + (size_t)s.w * (j + (size_t)s.h * k)];
                if (std::abs(x) < band) a.set(i, j, k, x);
            }
    a.set_as_levelset(band);
    a.flood_fill();
}

void fill_levelset2(array2<Real> &a, const shape2 &s, const float *v, int mode, float band) {
    if (mode == 1) {
        a.initialize(s, v[0]);
        return;
    }
    a.initialize(s, 0.0);
    for (int j = 0; j < (int)s.h; ++j)
        for (int i = 0; i < (int)s.w; ++i) {
            float x = v[i + (size_t)s.w * j];
            if (std::abs(x) < band) a.set(i, j, x);
        }
    a.set_as_levelset(band);
    a.flood_fill();
}

bool g_config_ready = false;

// The reference's arrays configure themselves from the global configuration,
// and every configuration lookup needs a group on the stack
// (src/core/configuration.cpp:298-301), as src/ui/ui.cpp:631 pushes.
configuration &install_global_config(const char *kv) {
    configuration &config = configurable::set_global_configuration(configuration(parse_kv(kv)));
    config.push_group("Harness", "Harness");
    g_config_ready = true;
    return config;
}

}  // namespace

extern "C" {

/* Creates a reference projector. dim is 2 or 3 (nz ignored for 2).
 * kv: whitespace-separated Key=Value settings of the reference's
 * configuration (Residual, MaxIterations, WarmStart, EpsFluid, EpsSolid,
 * SecondOrderAccurateFluid, SecondOrderAccurateSolid, Threads, ...). */
void *ref_create(int dim, int nx, int ny, int nz, double dx, const char *kv, const char *log_path) {
    auto *h = new harness();
    h->dim = dim;
    h->nx = nx;
    h->ny = ny;
    h->nz = (dim == 3) ? nz : 1;
    h->dx = dx;
    h->config = &install_global_config(kv);
    with_stdout_to(log_path, [&]() {
        if (dim == 3) {
            h->shape3_ = shape3(nx, ny, nz);
            h->proj3.reset(new macproject3_driver("macpressuresolver3"));
            (*h->proj3).set_environment("shape", &h->shape3_);
            (*h->proj3).set_environment("dx", &h->dx);
            h->proj3->setup_now(*h->config);
        } else {
            h->shape2_ = shape2(nx, ny);
            h->proj2.reset(new macproject2_driver("macpressuresolver2"));
            (*h->proj2).set_environment("shape", &h->shape2_);
            (*h->proj2).set_environment("dx", &h->dx);
            h->proj2->setup_now(*h->config);
        }
    });
    return h;
}

void ref_destroy(void *hp) { delete static_cast<harness *>(hp); }

/* macproject{2,3}_interface::set_target_volume (macpressuresolver3.cpp:45-48):
 * the volumes the next project() corrects towards (macpressuresolver3.cpp:
 * 204-217). */
void ref_set_target_volume(void *hp, double current_volume, double target_volume) {
    auto *h = static_cast<harness *>(hp);
    if (h->dim == 3) (*h->proj3)->set_target_volume(current_volume, target_volume);
    else (*h->proj2)->set_target_volume(current_volume, target_volume);
}

/* One projection. Arrays are dense, x fastest:
 *   solid: nodal (nx+1)(ny+1)(nz+1), fluid: cells nx*ny*nz,
 *   u: (nx+1)*ny*nz, v: nx*(ny+1)*nz, w: nx*ny*(nz+1)   (in/out),
 *   pressure: cells (out), active: cells, 1 where pressure is active (out),
 *   on_u, on_v, on_w: per face, 1 where the velocity face is still active
 *   after project() (out, each may be NULL).
 * solid_mode/fluid_mode: 0 = narrow-band level set of half-width band,
 * 1 = constant array (value = first element).
 * surface_tension: project()'s own argument (0 = none).
 * Returns wall-clock milliseconds of project(). */
double ref_project(void *hp, double dt, const float *solid, int solid_mode, float solid_band,
                   const float *fluid, int fluid_mode, float fluid_band, float *u, float *v, float *w,
                   double surface_tension, float *pressure, unsigned char *active, unsigned char *on_u,
                   unsigned char *on_v, unsigned char *on_w, const char *log_path) {
    unsigned char *on[3] = {on_u, on_v, on_w};
    auto *h = static_cast<harness *>(hp);
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    double ms = 0.0;
    if (h->dim == 3) {
        const shape3 s = h->shape3_;
        array3<Real> solid_a, fluid_a;
        fill_levelset3(solid_a, s.nodal(), solid, solid_mode, solid_band);
        fill_levelset3(fluid_a, s, fluid, fluid_mode, fluid_band);
        macarray3<Real> vel(s);
        vel.activate_all();
        float *comp[3] = {u, v, w};
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i)
                        vel[d].set(i, j, k, comp[d][i + (size_t)fs.w * (j + (size_t)fs.h * k)]);
        }
        with_stdout_to(log_path, [&]() {
            auto t0 = std::chrono::steady_clock::now();
            (*h->proj3)->project(dt, vel, solid_a, fluid_a, surface_tension);
            auto t1 = std::chrono::steady_clock::now();
            ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        });
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const size_t n = i + (size_t)fs.w * (j + (size_t)fs.h * k);
                        comp[d][n] = vel[d](i, j, k);
                        if (on[d]) on[d][n] = vel[d].active(i, j, k) ? 1 : 0;
                    }
        }
        const array3<Real> &p = *(*h->proj3)->get_pressure();
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    size_t n = i + (size_t)nx * (j + (size_t)ny * k);
                    pressure[n] = p(i, j, k);
                    active[n] = p.active(i, j, k) ? 1 : 0;
                }
    } else {
        const shape2 s = h->shape2_;
        array2<Real> solid_a, fluid_a;
        fill_levelset2(solid_a, s.nodal(), solid, solid_mode, solid_band);
        fill_levelset2(fluid_a, s, fluid, fluid_mode, fluid_band);
        macarray2<Real> vel(s);
        vel.activate_all();
        float *comp[2] = {u, v};
        for (int d = 0; d < 2; ++d) {
            const shape2 fs = s.face(d);
            for (int j = 0; j < (int)fs.h; ++j)
                for (int i = 0; i < (int)fs.w; ++i)
                    vel[d].set(i, j, comp[d][i + (size_t)fs.w * j]);
        }
        with_stdout_to(log_path, [&]() {
            auto t0 = std::chrono::steady_clock::now();
            (*h->proj2)->project(dt, vel, solid_a, fluid_a, surface_tension);
            auto t1 = std::chrono::steady_clock::now();
            ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        });
        for (int d = 0; d < 2; ++d) {
            const shape2 fs = s.face(d);
            for (int j = 0; j < (int)fs.h; ++j)
                for (int i = 0; i < (int)fs.w; ++i) {
                    const size_t n = i + (size_t)fs.w * j;
                    comp[d][n] = vel[d](i, j);
                    if (on[d]) on[d][n] = vel[d].active(i, j) ? 1 : 0;
                }
        }
        const array2<Real> &p = *(*h->proj2)->get_pressure();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t n = i + (size_t)nx * j;
                pressure[n] = p(i, j);
                active[n] = p.active(i, j) ? 1 : 0;
            }
    }
    return ms;
}

/* Reads a level set back through the reference's sparse array semantics
 * (operator()), to check that the dense input survives the sparse round trip.
 * shape is the array's own shape (nodal for solid). */
void ref_levelset_roundtrip(int dim, int sx, int sy, int sz, const float *in, int mode, float band, float *out) {
    if (!g_config_ready) install_global_config("");
    if (dim == 3) {
        array3<Real> a;
        shape3 s(sx, sy, sz);
        fill_levelset3(a, s, in, mode, band);
        for (int k = 0; k < sz; ++k)
            for (int j = 0; j < sy; ++j)
                for (int i = 0; i < sx; ++i) out[i + (size_t)sx * (j + (size_t)sy * k)] = a(i, j, k);
    } else {
        array2<Real> a;
        shape2 s(sx, sy);
        fill_levelset2(a, s, in, mode, band);
        for (int j = 0; j < sy; ++j)
            for (int i = 0; i < sx; ++i) out[i + (size_t)sx * j] = a(i, j);
    }
}

/* The plugin modules' dense copy (shiokaze_gb300/module/gbarray_adapter.h)
 * against a read of every cell through operator(), on an array built from
 * `in` by fill_levelset{2,3} (mode 0 narrow band + flood fill, mode 1
 * constant) or, mode 2, as a velocity component: background `band`, cells
 * with |v| < band active, no fill. Writes both copies and their times
 * (best of `reps`). */
void ref_densify_compare(int dim, int sx, int sy, int sz, const float *in, int mode, float band, int reps,
                         float *out_adapter, float *out_lookup, double *ms_adapter, double *ms_lookup) {
    if (!g_config_ready) install_global_config("");
    using clock = std::chrono::steady_clock;
    auto best = [&](auto &&fn) {
        double b = 1e300;
        for (int r = 0; r < (reps > 0 ? reps : 1); ++r) {
            const auto t0 = clock::now();
            fn();
            b = std::min(b, std::chrono::duration<double, std::milli>(clock::now() - t0).count());
        }
        return b;
    };
    if (dim == 3) {
        array3<Real> a;
        shape3 s(sx, sy, sz);
        if (mode == 2) {
            a.initialize(s, band);
            for (int k = 0; k < sz; ++k)
                for (int j = 0; j < sy; ++j)
                    for (int i = 0; i < sx; ++i) {
                        const float x = in[i + (size_t)sx * (j + (size_t)sy * k)];
                        if (std::abs(x) < band) a.set(i, j, k, x);
                    }
        } else {
            fill_levelset3(a, s, in, mode, band);
        }
        *ms_adapter = best([&] { gbarray::densify_passes(a, out_adapter); });
        *ms_lookup = best([&] {
            for (int k = 0; k < sz; ++k)
                for (int j = 0; j < sy; ++j)
                    for (int i = 0; i < sx; ++i) out_lookup[i + (size_t)sx * (j + (size_t)sy * k)] = a(i, j, k);
        });
    } else {
        array2<Real> a;
        shape2 s(sx, sy);
        if (mode == 2) {
            a.initialize(s, band);
            for (int j = 0; j < sy; ++j)
                for (int i = 0; i < sx; ++i) {
                    const float x = in[i + (size_t)sx * j];
                    if (std::abs(x) < band) a.set(i, j, x);
                }
        } else {
            fill_levelset2(a, s, in, mode, band);
        }
        *ms_adapter = best([&] { gbarray::densify_passes(a, out_adapter); });
        *ms_lookup = best([&] {
            for (int j = 0; j < sy; ++j)
                for (int i = 0; i < sx; ++i) out_lookup[i + (size_t)sx * j] = a(i, j);
        });
    }
}

/* The plugin modules' bricks (gbarray_adapter.h to_bricks) of a 3D array
 * built as in ref_densify_compare: the bricks expanded by the rule of
 * include/gbp.h (gbp_bricks) into out_expanded, every cell read through
 * operator() into out_lookup, the brick counts (listed, fill, background)
 * into counts, and the bricks themselves (slot per brick, listed values,
 * background and fill) for the GPU's expansion test. values_out holds up to
 * one brick per brick of the array. */
void ref_bricks_compare(int sx, int sy, int sz, const float *in, int mode, float band, float *out_expanded,
                        float *out_lookup, long long *counts, int *slot_out, float *values_out, float *bg_fill) {
    if (!g_config_ready) install_global_config("");
    array3<Real> a;
    shape3 s(sx, sy, sz);
    if (mode == 2) {
        a.initialize(s, band);
        for (int k = 0; k < sz; ++k)
            for (int j = 0; j < sy; ++j)
                for (int i = 0; i < sx; ++i) {
                    const float x = in[i + (size_t)sx * (j + (size_t)sy * k)];
                    if (std::abs(x) < band) a.set(i, j, k, x);
                }
    } else {
        fill_levelset3(a, s, in, mode, band);
    }
    gbarray::Bricks b;
    gbarray::to_bricks(a, b);
    counts[0] = counts[1] = counts[2] = 0;
    for (int sl : b.slot) counts[sl >= 0 ? 0 : sl == GBP_BRICK_FILL ? 1 : 2] += 1;
    for (int k = 0; k < sz; ++k)
        for (int j = 0; j < sy; ++j)
            for (int i = 0; i < sx; ++i) {
                const int sl = b.slot[b.brick(i, j, k)];
                const size_t n = i + (size_t)sx * (j + (size_t)sy * k);
                out_expanded[n] = sl >= 0 ? b.values[(size_t)sl * GBP_BRICK_CELLS + gbarray::Bricks::offset(i, j, k)]
                                          : sl == GBP_BRICK_FILL ? b.fill : b.background;
                out_lookup[n] = a(i, j, k);
            }
    std::copy(b.slot.begin(), b.slot.end(), slot_out);
    std::copy(b.values.begin(), b.values.end(), values_out);
    bg_fill[0] = b.background;
    bg_fill[1] = b.fill;
}

/* The reference's macadvection3 (src/advection/macadvection3.cpp), loaded
 * by name, on dense 3D arrays, in macsmoke3::idle's order
 * (src/smoke/macsmoke3.cpp:270-281): the scalar (if q is given) advected by
 * the velocity, then the velocity by itself. kv: the module's keys
 * (MacCormack, WENO, TrimNarrowBand). u, v, w: every face active (the smoke
 * scene's velocity, macsmoke3.cpp:115), in/out. fluid: level set built as
 * in ref_project. q: cells, in/out, background q_bg; the cells with
 * q_mask[c] != 0 are active (all if q_mask is NULL). Outputs are read
 * through operator(). Returns wall-clock milliseconds of the two calls. */
double ref_advect3(int nx, int ny, int nz, double dx, double dt, const char *kv, float *u, float *v, float *w,
                   const float *fluid, int fluid_mode, float fluid_band, float *q, const unsigned char *q_mask,
                   float q_bg, const char *log_path) {
    configuration &config = install_global_config(kv);
    shape3 s(nx, ny, nz);
    double dxv = dx, ms = 0.0;
    with_stdout_to(log_path, [&]() {
        macadvection3_driver adv("macadvection3");
        adv.set_environment("shape", &s);
        adv.set_environment("dx", &dxv);
        adv.setup_now(config);
        array3<Real> fluid_a;
        fill_levelset3(fluid_a, s, fluid, fluid_mode, fluid_band);
        // the advected velocity and macsmoke3's copy of it (the second
        // argument, which advect_vector does not read)
        macarray3<Real> vel(s), save(s);
        vel.activate_all();
        save.activate_all();
        float *comp[3] = {u, v, w};
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const float x = comp[d][i + (size_t)fs.w * (j + (size_t)fs.h * k)];
                        vel[d].set(i, j, k, x);
                        save[d].set(i, j, k, x);
                    }
        }
        array3<Real> qa;
        if (q) {
            qa.initialize(s, q_bg);
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const size_t n = i + (size_t)nx * (j + (size_t)ny * k);
                        if (!q_mask || q_mask[n]) qa.set(i, j, k, q[n]);
                    }
        }
        auto t0 = std::chrono::steady_clock::now();
        if (q) adv->advect_scalar(qa, vel, fluid_a, dt, "density");
        adv->advect_vector(vel, save, fluid_a, dt, "velocity");
        ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i)
                        comp[d][i + (size_t)fs.w * (j + (size_t)fs.h * k)] = vel[d](i, j, k);
        }
        if (q)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) q[i + (size_t)nx * (j + (size_t)ny * k)] = qa(i, j, k);
    });
    return ms;
}

/* The reference's macadvection2 (src/advection/macadvection2.cpp) on dense
 * 2D arrays, in macsmoke2's order (src/smoke/macsmoke2.cpp:244-254): the
 * scalar (if q is given) by the velocity, then the velocity by itself. As
 * ref_advect3 otherwise: u, v every face active, in/out; fluid built as in
 * ref_project; q background q_bg, active where q_mask (all if NULL). */
double ref_advect2(int nx, int ny, double dx, double dt, const char *kv, float *u, float *v, const float *fluid,
                   int fluid_mode, float fluid_band, float *q, const unsigned char *q_mask, float q_bg,
                   const char *log_path) {
    configuration &config = install_global_config(kv);
    shape2 s(nx, ny);
    double dxv = dx, ms = 0.0;
    with_stdout_to(log_path, [&]() {
        macadvection2_driver adv("macadvection2");
        adv.set_environment("shape", &s);
        adv.set_environment("dx", &dxv);
        adv.setup_now(config);
        array2<Real> fluid_a;
        fill_levelset2(fluid_a, s, fluid, fluid_mode, fluid_band);
        macarray2<Real> vel(s), save(s);
        vel.activate_all();
        save.activate_all();
        float *comp[2] = {u, v};
        for (int d = 0; d < 2; ++d) {
            const shape2 fs = s.face(d);
            for (int j = 0; j < (int)fs.h; ++j)
                for (int i = 0; i < (int)fs.w; ++i) {
                    const float x = comp[d][i + (size_t)fs.w * j];
                    vel[d].set(i, j, x);
                    save[d].set(i, j, x);
                }
        }
        array2<Real> qa;
        if (q) {
            qa.initialize(s, q_bg);
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t n = i + (size_t)nx * j;
                    if (!q_mask || q_mask[n]) qa.set(i, j, q[n]);
                }
        }
        auto t0 = std::chrono::steady_clock::now();
        if (q) adv->advect_scalar(qa, vel, fluid_a, dt);
        adv->advect_vector(vel, save, fluid_a, dt);
        ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        for (int d = 0; d < 2; ++d) {
            const shape2 fs = s.face(d);
            for (int j = 0; j < (int)fs.h; ++j)
                for (int i = 0; i < (int)fs.w; ++i) comp[d][i + (size_t)fs.w * j] = vel[d](i, j);
        }
        if (q)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) q[i + (size_t)nx * j] = qa(i, j);
    });
    return ms;
}

/* Loads, configures and initializes the 2D advection module the
 * configuration names (Advection=<name>, default macadvection2); returns 1. */
int ref_advect2_load(int nx, int ny, double dx, const char *kv, const char *log_path) {
    configuration &config = install_global_config(kv);
    shape2 s(nx, ny);
    double dxv = dx;
    with_stdout_to(log_path, [&]() {
        macadvection2_driver adv("macadvection2");
        adv.set_environment("shape", &s);
        adv.set_environment("dx", &dxv);
        adv.setup_now(config);
    });
    return 1;
}

/* Loads, configures and initializes the advection module the
 * configuration names (Advection=<name>, default macadvection3) through the
 * reference's loader, without calling it; returns 1. For checking that a
 * replacement module loads in place of macadvection3. */
int ref_advect_load(int nx, int ny, int nz, double dx, const char *kv, const char *log_path) {
    configuration &config = install_global_config(kv);
    shape3 s(nx, ny, nz);
    double dxv = dx;
    with_stdout_to(log_path, [&]() {
        macadvection3_driver adv("macadvection3");
        adv.set_environment("shape", &s);
        adv.set_environment("dx", &dxv);
        adv.setup_now(config);
    });
    return 1;
}

/* The reference's macutility3::constrain_velocity
 * (src/utility/macutility3.cpp:61-86), loaded by name, on dense 3D arrays:
 * solid is the nodal level set (built as in ref_project from solid_mode /
 * solid_band), u, v, w the face velocities (in/out), active where the
 * component's mask is nonzero (every face if the mask is NULL; inactive
 * faces read 0, the velocity's background). Outputs are read through
 * operator(). Returns 1. */
int ref_constrain3(int nx, int ny, int nz, double dx, const char *kv, const float *solid, int solid_mode,
                   float solid_band, float *u, float *v, float *w, const unsigned char *mu, const unsigned char *mv,
                   const unsigned char *mw, const char *log_path) {
    configuration &config = install_global_config(kv);
    shape3 s(nx, ny, nz);
    double dxv = dx;
    with_stdout_to(log_path, [&]() {
        macutility3_driver util("macutility3");
        util.set_environment("shape", &s);
        util.set_environment("dx", &dxv);
        util.setup_now(config);
        array3<Real> solid_a;
        fill_levelset3(solid_a, s.nodal(), solid, solid_mode, solid_band);
        macarray3<Real> vel(s);
        float *comp[3] = {u, v, w};
        const unsigned char *mask[3] = {mu, mv, mw};
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const size_t n = i + (size_t)fs.w * (j + (size_t)fs.h * k);
                        if (!mask[d] || mask[d][n]) vel[d].set(i, j, k, comp[d][n]);
                    }
        }
        util->constrain_velocity(solid_a, vel);
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i)
                        comp[d][i + (size_t)fs.w * (j + (size_t)fs.h * k)] = vel[d](i, j, k);
        }
    });
    return 1;
}

/* macutility3::extrapolate_and_constrain_velocity (src/utility/
 * macutility3.cpp:88-92) through the module loader (kv may select another
 * MacUtility module): the velocity holds comp values on the faces marked in
 * mu/mv/mw (in/out: the active sets after the call); the solid as in
 * ref_constrain3. Values read back through operator(). */
int ref_extrapolate_constrain3(int nx, int ny, int nz, double dx, const char *kv, const float *solid, int solid_mode,
                               float solid_band, float *u, float *v, float *w, unsigned char *mu, unsigned char *mv,
                               unsigned char *mw, int width, const char *log_path) {
    configuration &config = install_global_config(kv);
    shape3 s(nx, ny, nz);
    double dxv = dx;
    with_stdout_to(log_path, [&]() {
        macutility3_driver util("macutility3");
        util.set_environment("shape", &s);
        util.set_environment("dx", &dxv);
        util.setup_now(config);
        array3<Real> solid_a;
        fill_levelset3(solid_a, s.nodal(), solid, solid_mode, solid_band);
        macarray3<Real> vel(s);
        float *comp[3] = {u, v, w};
        unsigned char *mask[3] = {mu, mv, mw};
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const size_t n = i + (size_t)fs.w * (j + (size_t)fs.h * k);
                        if (mask[d][n]) vel[d].set(i, j, k, comp[d][n]);
                    }
        }
        util->extrapolate_and_constrain_velocity(solid_a, vel, width);
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = s.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const size_t n = i + (size_t)fs.w * (j + (size_t)fs.h * k);
                        comp[d][n] = vel[d](i, j, k);
                        mask[d][n] = vel[d].active(i, j, k) ? 1 : 0;
                    }
        }
    });
    return 1;
}

/* The reference's array_extrapolator3::extrapolate on a dense 3D array of
 * shape w x h x d: active where active[c] != 0 (values elsewhere ignored;
 * the array's background is 0), `count` rounds. On return, a holds the
 * values read through operator() and active the active set. Returns the
 * number of cells the reference reports as extrapolated. */
long long ref_extrapolate3(int w, int h, int d, float *a, unsigned char *active, int count) {
    install_global_config("");
    long long added = 0;
    with_stdout_to("/dev/null", [&]() {
        shape3 s(w, h, d);
        array3<Real> arr(s, 0.0);
        for (int k = 0; k < d; ++k)
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    const size_t n = i + (size_t)w * (j + (size_t)h * k);
                    if (active[n]) arr.set(i, j, k, a[n]);
                }
        added = (long long)array_extrapolator3::extrapolate<Real>(arr, count);
        for (int k = 0; k < d; ++k)
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    const size_t n = i + (size_t)w * (j + (size_t)h * k);
                    a[n] = arr(i, j, k);
                    active[n] = arr.active(i, j, k) ? 1 : 0;
                }
    });
    return added;
}

}  // extern "C"
