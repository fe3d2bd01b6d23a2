// gbprojection3.cpp -- Shiokaze plugin module "gbprojection3": the GB300
// pressure projection behind macproject3_interface
// (include/shiokaze/projection/macproject3_interface.h:38-99), a drop-in
// for "macpressuresolver3" (src/projection/macpressuresolver3.cpp). Selected
// with Projection=gbprojection3; compiled against the reference's headers
// and linked to libgbp.so.
//
// The reference's arrays are sparse (tiled, narrow band); project() copies
// them to dense arrays with exactly operator()'s values (background, fill
// and active values; gbarray_adapter.h, one pass over the filled and active
// cells instead of one lookup per cell) and calls gbp_project_active. The
// output state is the reference's: the projected velocity is written to the
// faces that were active, as its velocity update iterates actives
// (macpressuresolver3.cpp:252), and the faces it deactivates there (closed
// faces that are not walls next to fluid, :264-266) are turned off with
// set_off; the pressure is set on every unknown, a pressure of 0 included
// (:245-248), and the other cells are left inactive.
#include <shiokaze/array/array3.h>
#include <shiokaze/array/macarray3.h>
#include <shiokaze/core/console.h>
#include <shiokaze/projection/macproject3_interface.h>

#include <vector>

#include "gbarray_adapter.h"
#include "gbprojection_common.h"

SHKZ_USING_NAMESPACE

class gbprojection3 : public macproject3_interface {
protected:
    LONG_NAME("GB300 Pressure Projection 3D")
    ARGUMENT_NAME("GBProjection")

    virtual void set_target_volume(double current_volume, double target_volume) override {
        if (m_scene) gbprojection::check(gbp_scene_set_target_volume(m_scene, current_volume, target_volume), "set_target_volume");
        m_current_volume = current_volume;
        m_target_volume = target_volume;
    }

    virtual void project(double dt, macarray3<Real> &velocity, const array3<Real> &solid, const array3<Real> &fluid,
                         double surface_tension, const std::vector<signed_rigidbody3_interface *> *) override {
        const int nx = m_shape.w, ny = m_shape.h, nz = m_shape.d;
        m_params.surface_tension = surface_tension;
        std::vector<float> s((size_t)(nx + 1) * (ny + 1) * (nz + 1)), f((size_t)nx * ny * nz), p(f.size());
        expect_shape(solid.shape(), nx + 1, ny + 1, nz + 1, "solid");
        expect_shape(fluid.shape(), nx, ny, nz, "fluid");
        gbarray::densify(solid, s.data());
        gbarray::densify(fluid, f.data());
        std::vector<float> vel[3];
        for (int d = 0; d < 3; ++d) {
            const int fx = nx + (d == 0), fy = ny + (d == 1), fz = nz + (d == 2);
            expect_shape(velocity[d].shape(), fx, fy, fz, "velocity");
            vel[d].resize((size_t)fx * fy * fz);
            gbarray::densify(velocity[d], vel[d].data());
        }
        if (!m_scene) {
            gbprojection::check(gbp_create(m_device, &m_ctx), "gbp_create");
            gbprojection::check(gbp_scene_create(m_ctx, 3, nx, ny, nz, m_dx, &m_scene), "gbp_scene_create");
            if (m_target_volume) gbp_scene_set_target_volume(m_scene, m_current_volume, m_target_volume);
        }
        gbp_stats st;
        std::vector<unsigned char> unknown(f.size()), on[3];
        for (int d = 0; d < 3; ++d) on[d].resize(vel[d].size());
        int rc = gbp_project_active(m_scene, dt, s.data(), f.data(), vel[0].data(), vel[1].data(), vel[2].data(),
                                    &m_params, p.data(), &st, unknown.data(), on[0].data(), on[1].data(),
                                    on[2].data());
        gbprojection::check(rc, "gbp_project_active");
        console::dump("gbprojection3: %d iterations, Reresid=%e, %.3f ms\n", st.iterations, st.reresid, st.ms_total);
        console::write(get_argument_name() + "_number_projection_iteration", st.iterations);
        m_pressure.clear();
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t n = i + (size_t)nx * (j + (size_t)ny * k);
                    if (unknown[n]) m_pressure.set(i, j, k, p[n]);
                }
        velocity.parallel_actives([&](int dim, int i, int j, int k, auto &it, int tn) {
            const int fx = nx + (dim == 0), fy = ny + (dim == 1);
            const size_t n = i + (size_t)fx * (j + (size_t)fy * k);
            if (on[dim][n]) it.set(vel[dim][n]);
            else it.set_off();
        });
    }

    // the reference indexes these arrays by the simulation's shape and
    // exits on a mismatch in its debug builds (array3.h bound checks)
    static void expect_shape(const shape3 &s, int w, int h, int d, const char *what) {
        if ((int)s.w != w || (int)s.h != h || (int)s.d != d) {
            std::fprintf(stderr, "gbprojection3: %s array is %ux%ux%u, expected %dx%dx%d\n", what, s.w, s.h, s.d, w, h, d);
            std::exit(-1);
        }
    }

    virtual void configure(configuration &config) override {
        gbp_params_default(&m_params);
        gbprojection::configure_params(config, m_params, m_device);
    }
    virtual void initialize(const shape3 &shape, double dx) override {
        m_shape = shape;
        m_dx = dx;
    }
    virtual void post_initialize() override { m_pressure.initialize(m_shape); }
    virtual const array3<Real> *get_pressure() const override { return &m_pressure; }

public:
    virtual ~gbprojection3() {
        if (m_scene) gbp_scene_destroy(m_scene);
        if (m_ctx) gbp_destroy(m_ctx);
    }

private:
    gbp_params m_params;
    int m_device{0};
    gbp_ctx *m_ctx{nullptr};
    gbp_scene *m_scene{nullptr};
    shape3 m_shape;
    double m_dx{0.0};
    double m_current_volume{0.0}, m_target_volume{0.0};
    array3<Real> m_pressure{this};
};

extern "C" module *create_instance() { return new gbprojection3(); }
extern "C" const char *license() { return "MIT"; }
