// gbutility3.cpp -- Shiokaze plugin module "gbutility3": the MAC utility
// module (macutility3_interface, include/shiokaze/utility/
// macutility3_interface.h:36-226) with the solid constraint of the velocity
// on the GPU. Selected with MacUtility=gbutility3 in place of "macutility3"
// (src/utility/macutility3.cpp); compiled against the reference's headers
// and linked to libgbp.so.
//
// constrain_velocity (macutility3.cpp:61-86) runs gbp_constrain_velocity3:
// the module copies the solid and the velocity to dense arrays with
// operator()'s values (gbarray_adapter.h), marks the active faces, and writes
// the result back over them, as the reference's parallel_actives loop does.
// extrapolate_and_constrain_velocity (:88-92) runs
// gbp_extrapolate_constrain_velocity3: the velocity grown over its inactive
// faces (array_extrapolator3, as the tiled array's dilate runs it), then
// constrained over the grown active sets; the faces it activates are set
// in the reference's arrays. Every
// other member is forwarded to the reference's macutility3, loaded by the
// same loader under this module's own key (GBUtilityBase), so the results
// of the whole interface are the reference's.
#include <shiokaze/array/array_utility3.h>
#include <shiokaze/core/console.h>
#include <shiokaze/utility/macutility3_interface.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbarray_adapter.h"
#include "gbp.h"

SHKZ_USING_NAMESPACE

class gbutility3 : public macutility3_interface {
protected:
    LONG_NAME("GB300 MAC Utility 3D")
    ARGUMENT_NAME("GBUtility")

    virtual void constrain_velocity(const array3<Real> &solid, macarray3<Real> &velocity) const override {
        // levelset_exist (array_utility3.h:112-122) on the solid's active
        // values, as the reference decides whether to do anything
        if (!array_utility3::levelset_exist(solid)) return;
        const int nx = m_shape.w, ny = m_shape.h, nz = m_shape.d;
        expect(solid.shape() == m_shape.nodal(), "solid array is not nodal");
        std::vector<float> s(m_shape.nodal().count()), vel[3];
        std::vector<unsigned char> mask[3];
        gbarray::densify(solid, s.data());
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = m_shape.face(d);
            expect(velocity[d].shape() == fs, "velocity array has another shape");
            vel[d].resize(fs.count());
            gbarray::densify(velocity[d], vel[d].data());
            mask[d].assign(fs.count(), 0);
            unsigned char *m = mask[d].data();
            velocity[d].const_parallel_actives([&](int i, int j, int k, const auto &) {
                m[i + (size_t)fs.w * (j + (size_t)fs.h * k)] = 1;
            });
        }
        if (!m_ctx) check(gbp_create(m_device, &m_ctx), "gbp_create");
        check(gbp_constrain_velocity3(m_ctx, nx, ny, nz, m_dx, s.data(), vel[0].data(), vel[1].data(), vel[2].data(),
                                      mask[0].data(), mask[1].data(), mask[2].data()),
              "gbp_constrain_velocity3");
        velocity.parallel_actives([&](int dim, int i, int j, int k, auto &it, int) {
            const int fx = nx + (dim == 0), fy = ny + (dim == 1);
            it.set(vel[dim][i + (size_t)fx * (j + (size_t)fy * k)]);
        });
    }
    virtual void extrapolate_and_constrain_velocity(const array3<Real> &solid, macarray3<Real> &velocity,
                                                    int extrapolate_width) const override {
        // macarray_extrapolator3::extrapolate (each component grown over its
        // inactive faces, macarray_extrapolator3.h:44-48), then the
        // constraint over the grown active sets (macutility3.cpp:88-92),
        // both on the GPU in one call; without a solid level set
        // (levelset_exist on its active values) only the extrapolation
        const int nx = m_shape.w, ny = m_shape.h, nz = m_shape.d;
        const bool constrain = array_utility3::levelset_exist(solid);
        std::vector<float> vel[3];
        std::vector<unsigned char> mask[3], was[3];
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = m_shape.face(d);
            expect(velocity[d].shape() == fs, "velocity array has another shape");
            vel[d].resize(fs.count());
            gbarray::densify(velocity[d], vel[d].data());
            mask[d].assign(fs.count(), 0);
            unsigned char *m = mask[d].data();
            velocity[d].const_parallel_actives([&](int i, int j, int k, const auto &) {
                m[i + (size_t)fs.w * (j + (size_t)fs.h * k)] = 1;
            });
            was[d] = mask[d];
        }
        if (!m_ctx) check(gbp_create(m_device, &m_ctx), "gbp_create");
        if (constrain) {
            expect(solid.shape() == m_shape.nodal(), "solid array is not nodal");
            std::vector<float> s(m_shape.nodal().count());
            gbarray::densify(solid, s.data());
            check(gbp_extrapolate_constrain_velocity3(m_ctx, nx, ny, nz, m_dx, s.data(), vel[0].data(), vel[1].data(),
                                                      vel[2].data(), mask[0].data(), mask[1].data(), mask[2].data(),
                                                      extrapolate_width),
                  "gbp_extrapolate_constrain_velocity3");
        } else {
            for (int d = 0; d < 3; ++d)
                check(gbp_extrapolate3(m_ctx, nx + (d == 0), ny + (d == 1), nz + (d == 2), vel[d].data(),
                                       mask[d].data(), extrapolate_width, nullptr),
                      "gbp_extrapolate3");
        }
        // the faces active before take their new values; the faces the
        // extrapolation activated are set (which activates them)
        velocity.parallel_actives([&](int dim, int i, int j, int k, auto &it, int) {
            const int fx = nx + (dim == 0), fy = ny + (dim == 1);
            it.set(vel[dim][i + (size_t)fx * (j + (size_t)fy * k)]);
        });
        for (int d = 0; d < 3; ++d) {
            const shape3 fs = m_shape.face(d);
            for (int k = 0; k < (int)fs.d; ++k)
                for (int j = 0; j < (int)fs.h; ++j)
                    for (int i = 0; i < (int)fs.w; ++i) {
                        const size_t n = i + (size_t)fs.w * (j + (size_t)fs.h * k);
                        if (mask[d][n] && !was[d][n]) velocity[d].set(i, j, k, vel[d][n]);
                    }
        }
    }

    // the rest of the interface: the reference's own module
    virtual double compute_max_u(const macarray3<Real> &velocity) const override {
        return m_base->compute_max_u(velocity);
    }
    virtual void compute_area_fraction(const array3<Real> &solid, macarray3<Real> &areas) const override {
        m_base->compute_area_fraction(solid, areas);
    }
    virtual void compute_fluid_fraction(const array3<Real> &fluid, macarray3<Real> &rhos) const override {
        m_base->compute_fluid_fraction(fluid, rhos);
    }
    virtual void compute_face_density(const array3<Real> &solid, const array3<Real> &fluid,
                                      macarray3<Real> &density) const override {
        m_base->compute_face_density(solid, fluid, density);
    }
    virtual double get_kinetic_energy(const array3<Real> &solid, const array3<Real> &fluid,
                                      const macarray3<Real> &velocity) const override {
        return m_base->get_kinetic_energy(solid, fluid, velocity);
    }
    virtual double get_gravitational_potential_energy(const array3<Real> &solid, const array3<Real> &fluid,
                                                      vec3d gravity) const override {
        return m_base->get_gravitational_potential_energy(solid, fluid, gravity);
    }
    virtual double get_surfacetension_potential_energy(const array3<Real> &solid, const array3<Real> &fluid,
                                                       double tension_coeff) const override {
        return m_base->get_surfacetension_potential_energy(solid, fluid, tension_coeff);
    }
    virtual double get_total_energy(const array3<Real> &solid, const array3<Real> &fluid,
                                    const macarray3<Real> &velocity, vec3d gravity,
                                    double tension_coeff) const override {
        return m_base->get_total_energy(solid, fluid, velocity, gravity, tension_coeff);
    }
    virtual std::tuple<double, double, double> get_all_kinds_of_energy(const array3<Real> &solid,
                                                                       const array3<Real> &fluid,
                                                                       const macarray3<Real> &velocity,
                                                                       vec3d gravity,
                                                                       double tension_coeff) const override {
        return m_base->get_all_kinds_of_energy(solid, fluid, velocity, gravity, tension_coeff);
    }
    virtual void get_velocity_jacobian(const vec3d &p, const macarray3<Real> &velocity,
                                       vec3r jacobian[DIM3]) const override {
        m_base->get_velocity_jacobian(p, velocity, jacobian);
    }
    virtual void assign_initial_variables(const dylibloader &dylib, macarray3<Real> &velocity, array3<Real> *solid,
                                          array3<Real> *fluid, array3<Real> *density) const override {
        m_base->assign_initial_variables(dylib, velocity, solid, fluid, density);
    }
    virtual void add_force(vec3d p, vec3d f, macarray3<Real> &external_force) const override {
        m_base->add_force(p, f, external_force);
    }

    virtual void configure(configuration &config) override {
        config.get_integer("Device", m_device, "CUDA device");
    }
    virtual void initialize(const shape3 &shape, double dx) override {
        m_shape = shape;
        m_dx = dx;
    }

public:
    virtual ~gbutility3() {
        if (m_ctx) gbp_destroy(m_ctx);
    }

private:
    static void expect(bool ok, const char *what) {
        if (!ok) {
            std::fprintf(stderr, "gbutility3: %s\n", what);
            std::exit(-1);
        }
    }
    static void check(int rc, const char *what) {
        if (rc != GBP_OK) {
            std::fprintf(stderr, "gbutility3: %s failed: %s\n", what, gbp_strerror(rc));
            std::exit(-1);
        }
    }

    // the reference's module, under this module's own key so that
    // MacUtility=gbutility3 does not select this module again
    macutility3_driver m_base{this, "GBUtilityBase:macutility3"};
    int m_device{0};
    mutable gbp_ctx *m_ctx{nullptr};
    shape3 m_shape;
    double m_dx{0.0};
};

extern "C" module *create_instance() { return new gbutility3(); }
extern "C" const char *license() { return "MIT"; }
