// gbprojection2.cpp -- Shiokaze plugin module "gbprojection2": the GB300
// pressure projection behind macproject2_interface
// (include/shiokaze/projection/macproject2_interface.h), a drop-in for
// "macpressuresolver2" (src/projection/macpressuresolver2.cpp). Selected with
// Projection=gbprojection2. Dense copy with operator()'s values
// (gbarray_adapter.h), gbp_project_active, and the reference's output state
// as in gbprojection3.cpp: the projected velocity on the active faces, the
// faces its velocity update deactivates turned off (closed faces other than
// walls next to fluid with outgoing flow, macpressuresolver2.cpp:233-235),
// the pressure set on every unknown (:215-218).
#include <shiokaze/array/array2.h>
#include <shiokaze/array/macarray2.h>
#include <shiokaze/core/console.h>
#include <shiokaze/projection/macproject2_interface.h>

#include <vector>

#include "gbarray_adapter.h"
#include "gbprojection_common.h"

SHKZ_USING_NAMESPACE

class gbprojection2 : public macproject2_interface {
protected:
    LONG_NAME("GB300 Pressure Projection 2D")
    ARGUMENT_NAME("GBProjection")

    virtual void set_target_volume(double current_volume, double target_volume) override {
        if (m_scene) gbprojection::check(gbp_scene_set_target_volume(m_scene, current_volume, target_volume), "set_target_volume");
        m_current_volume = current_volume;
        m_target_volume = target_volume;
    }

    virtual void project(double dt, macarray2<Real> &velocity, const array2<Real> &solid, const array2<Real> &fluid,
                         double surface_tension, const std::vector<signed_rigidbody2_interface *> *) override {
        const int nx = m_shape.w, ny = m_shape.h;
        m_params.surface_tension = surface_tension;
        std::vector<float> s((size_t)(nx + 1) * (ny + 1)), f((size_t)nx * ny), p(f.size());
        expect_shape(solid.shape(), nx + 1, ny + 1, "solid");
        expect_shape(fluid.shape(), nx, ny, "fluid");
        gbarray::densify(solid, s.data());
        gbarray::densify(fluid, f.data());
        std::vector<float> vel[2];
        for (int d = 0; d < 2; ++d) {
            const int fx = nx + (d == 0), fy = ny + (d == 1);
            expect_shape(velocity[d].shape(), fx, fy, "velocity");
            vel[d].resize((size_t)fx * fy);
            gbarray::densify(velocity[d], vel[d].data());
        }
        if (!m_scene) {
            gbprojection::check(gbp_create(m_device, &m_ctx), "gbp_create");
            gbprojection::check(gbp_scene_create(m_ctx, 2, nx, ny, 1, m_dx, &m_scene), "gbp_scene_create");
            if (m_target_volume) gbp_scene_set_target_volume(m_scene, m_current_volume, m_target_volume);
        }
        gbp_stats st;
        std::vector<unsigned char> unknown(f.size()), on[2];
        for (int d = 0; d < 2; ++d) on[d].resize(vel[d].size());
        int rc = gbp_project_active(m_scene, dt, s.data(), f.data(), vel[0].data(), vel[1].data(), nullptr,
                                    &m_params, p.data(), &st, unknown.data(), on[0].data(), on[1].data(), nullptr);
        gbprojection::check(rc, "gbp_project_active");
        m_pressure.clear();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t n = i + (size_t)nx * j;
                if (unknown[n]) m_pressure.set(i, j, p[n]);
            }
        velocity.parallel_actives([&](int dim, int i, int j, auto &it, int tn) {
            const int fx = nx + (dim == 0);
            const size_t n = i + (size_t)fx * j;
            if (on[dim][n]) it.set(vel[dim][n]);
            else it.set_off();
        });
    }

    static void expect_shape(const shape2 &s, int w, int h, const char *what) {
        if ((int)s.w != w || (int)s.h != h) {
            std::fprintf(stderr, "gbprojection2: %s array is %ux%u, expected %dx%d\n", what, s.w, s.h, w, h);
            std::exit(-1);
        }
    }

    virtual void configure(configuration &config) override {
        gbp_params_default(&m_params);
        gbprojection::configure_params(config, m_params, m_device);
    }
    virtual void initialize(const shape2 &shape, double dx) override {
        m_shape = shape;
        m_dx = dx;
    }
    virtual void post_initialize() override { m_pressure.initialize(m_shape); }
    virtual const array2<Real> *get_pressure() const override { return &m_pressure; }

public:
    virtual ~gbprojection2() {
        if (m_scene) gbp_scene_destroy(m_scene);
        if (m_ctx) gbp_destroy(m_ctx);
    }

private:
    gbp_params m_params;
    int m_device{0};
    gbp_ctx *m_ctx{nullptr};
    gbp_scene *m_scene{nullptr};
    shape2 m_shape;
    double m_dx{0.0};
    double m_current_volume{0.0}, m_target_volume{0.0};
    array2<Real> m_pressure{this};
};

extern "C" module *create_instance() { return new gbprojection2(); }
extern "C" const char *license() { return "MIT"; }
