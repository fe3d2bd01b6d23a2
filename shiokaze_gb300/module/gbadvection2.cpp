// gbadvection2.cpp -- Shiokaze plugin module "gbadvection2": 2D MAC
// advection on the GPU behind macadvection2_interface
// (include/shiokaze/advection/macadvection2_interface.h:38-85), a drop-in for
// "macadvection2" (src/advection/macadvection2.cpp) with bilinear
// interpolation. Selected with Advection=gbadvection2; compiled against the
// reference's headers and linked to libgbp.so.
//
// As gbadvection3: its callers are the 2D smoke solvers (src/smoke/
// macsmoke2.cpp:244-254), whose velocity has every face active
// (macsmoke2.cpp:106) and whose density has no filled cells. The module
// copies the reference's tiled arrays to dense arrays with operator()'s
// values (gbarray_adapter.h), calls gbp_advect2 and writes the result back
// over the active faces and cells, as the reference's parallel_actives loops
// do (macadvection2.cpp:74-87, :177-189). A velocity with inactive faces, a
// scalar with filled cells, or WENO=Yes is refused with a message and exit.
#include <shiokaze/advection/macadvection2_interface.h>
#include <shiokaze/array/array2.h>
#include <shiokaze/array/macarray2.h>
#include <shiokaze/core/console.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbarray_adapter.h"
#include "gbp.h"

SHKZ_USING_NAMESPACE

class gbadvection2 : public macadvection2_interface {
protected:
    LONG_NAME("GB300 MAC Advection 2D")
    ARGUMENT_NAME("GBAdvection")

    virtual void advect_scalar(array2<Real> &scalar, const macarray2<Real> &velocity, const array2<Real> &fluid,
                               double dt) override {
        const int nx = m_shape.w, ny = m_shape.h;
        std::vector<float> vel[2], f, q((size_t)nx * ny);
        densify_velocity(velocity, vel);
        densify_fluid(fluid, f);
        expect(scalar.shape() == m_shape, "scalar array has another shape");
        size_t filled = 0;
        scalar.const_parallel_inside([&](int, int, const auto &) { __atomic_add_fetch(&filled, 1, __ATOMIC_RELAXED); });
        expect(filled == 0, "scalar arrays with filled cells are not supported");
        gbarray::densify(scalar, q.data());
        std::vector<unsigned char> mask(q.size(), 0);
        scalar.const_parallel_actives([&](int i, int j, const auto &) { mask[i + (size_t)nx * j] = 1; });
        gbp_advect_params p = m_params;
        p.advect_velocity = 0;
        run(p, dt, vel, f, q.data(), mask.data(), scalar.get_background_value(), "scalar");
        scalar.parallel_actives([&](int i, int j, auto &it, int) { it.set(q[i + (size_t)nx * j]); });
    }

    // The reference traces u by its own full velocity; `velocity` is not read
    // (macadvection2.cpp:66-76 uses v_in only).
    virtual void advect_vector(macarray2<Real> &u, const macarray2<Real> &, const array2<Real> &fluid,
                               double dt) override {
        const int nx = m_shape.w;
        std::vector<float> vel[2], f;
        densify_velocity(u, vel);
        densify_fluid(fluid, f);
        run(m_params, dt, vel, f, nullptr, nullptr, 0.0f, "velocity");
        u.parallel_actives([&](int dim, int i, int j, auto &it, int) {
            const int fx = nx + (dim == 0);
            it.set(vel[dim][i + (size_t)fx * j]);
        });
    }

    virtual void configure(configuration &config) override {
        gbp_advect_params_default(&m_params);
        bool maccormack = m_params.maccormack != 0, weno = false;
        unsigned trim = (unsigned)m_params.trim_narrowband;
        config.get_bool("MacCormack", maccormack, "Whether to use MacCormack method");
        config.get_bool("WENO", weno, "Whether to use WENO interpolation for advection");
        config.get_unsigned("TrimNarrowBand", trim, "Narrow band count to turn to semi-Lagrangian advection");
        config.get_integer("Device", m_device, "CUDA device");
        expect(!weno, "WENO interpolation is not available (bilinear only)");
        m_params.maccormack = maccormack;
        m_params.trim_narrowband = (int)trim;
    }
    virtual void initialize(const shape2 &shape, double dx) override {
        m_shape = shape;
        m_dx = dx;
    }

public:
    virtual ~gbadvection2() {
        if (m_ctx) gbp_destroy(m_ctx);
    }

private:
    void run(const gbp_advect_params &p, double dt, std::vector<float> vel[2], std::vector<float> &f, float *q,
             const unsigned char *mask, float bg, const char *what) {
        if (!m_ctx) check(gbp_create(m_device, &m_ctx), "gbp_create");
        check(gbp_advect2(m_ctx, m_shape.w, m_shape.h, m_dx, dt, &p, vel[0].data(), vel[1].data(), f.data(), q, mask,
                          bg),
              "gbp_advect2");
        console::dump("gbadvection2: advected %s (%s)\n", what, p.maccormack ? "MacCormack" : "semi-Lagrangian");
    }

    void densify_velocity(const macarray2<Real> &velocity, std::vector<float> vel[2]) {
        for (int d = 0; d < 2; ++d) {
            const shape2 fs = m_shape.face(d);
            expect(velocity[d].shape() == fs, "velocity array has another shape");
            expect(velocity[d].count() == fs.count(), "every velocity face must be active");
            vel[d].resize(fs.count());
            gbarray::densify(velocity[d], vel[d].data());
        }
    }

    void densify_fluid(const array2<Real> &fluid, std::vector<float> &f) {
        expect(fluid.shape() == m_shape, "fluid array has another shape");
        f.resize(m_shape.count());
        gbarray::densify(fluid, f.data());
    }

    static void expect(bool ok, const char *what) {
        if (!ok) {
            std::fprintf(stderr, "gbadvection2: %s\n", what);
            std::exit(-1);
        }
    }

    static void check(int rc, const char *what) {
        if (rc != GBP_OK) {
            std::fprintf(stderr, "gbadvection2: %s failed: %s\n", what, gbp_strerror(rc));
            std::exit(-1);
        }
    }

    gbp_advect_params m_params;
    int m_device{0};
    gbp_ctx *m_ctx{nullptr};
    shape2 m_shape;
    double m_dx{0.0};
};

extern "C" module *create_instance() { return new gbadvection2(); }
extern "C" const char *license() { return "MIT"; }
