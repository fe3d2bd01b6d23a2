// gbprojection3.cpp -- Shiokaze plugin module "gbprojection3": the GB300
// pressure projection behind macproject3_interface
// (include/shiokaze/projection/macproject3_interface.h:38-99), a drop-in
// for "macpressuresolver3" (src/projection/macpressuresolver3.cpp). Selected
// with Projection=gbprojection3; compiled against the reference's headers
// and linked to libgbp.so.
//
// The reference's arrays are sparse (tiled, narrow band); project() cuts
// them into bricks of 8^3 cells with exactly operator()'s values
// (background, fill and active values; gbarray_adapter.h, passes over the
// filled and active cells only) and calls gbp_project_bricks, which ships
// the listed bricks, expands them on the GPU and returns the listed output
// bricks. The output state is the reference's: the projected velocity is written to the
// faces that were active, as its velocity update iterates actives
// (macpressuresolver3.cpp:252), and the faces it deactivates there (closed
// faces that are not walls next to fluid, :264-266) are turned off with
// set_off; the pressure is set on every unknown, a pressure of 0 included
// (:245-248), and the other cells are left inactive.
#include <shiokaze/array/array3.h>
#include <shiokaze/array/macarray3.h>
#include <shiokaze/core/console.h>
#include <shiokaze/projection/macproject3_interface.h>

#include <algorithm>
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
        expect_shape(solid.shape(), nx + 1, ny + 1, nz + 1, "solid");
        expect_shape(fluid.shape(), nx, ny, nz, "fluid");
        // the inputs as bricks (only the listed ones travel; the GPU expands
        // them); the brick buffers are members, kept from call to call
        gbarray::Bricks &bs = m_bs, &bf = m_bf, *bv = m_bv;
        gbarray::to_bricks(solid, bs);
        gbarray::to_bricks(fluid, bf);
        for (int d = 0; d < 3; ++d) {
            expect_shape(velocity[d].shape(), nx + (d == 0), ny + (d == 1), nz + (d == 2), "velocity");
            gbarray::to_bricks(velocity[d], bv[d]);
        }
        // outputs: the velocity where it has active faces (its listed
        // bricks); the pressure where a cell can be fluid (a listed brick of
        // the fluid level set, or a filled or background one whose value is
        // negative)
        gbarray::BricksOut &po = m_po, *vo = m_vo;
        po.nbx = bf.nbx;
        po.nby = bf.nby;
        po.slot.assign(bf.slot.size(), -1);
        long long pc = 0;
        for (size_t b = 0; b < bf.slot.size(); ++b) {
            const int sl = bf.slot[b];
            if (sl >= 0 || (sl == GBP_BRICK_FILL && bf.fill < 0.0f) || (sl == GBP_BRICK_BACKGROUND && bf.background < 0.0f))
                po.slot[b] = (int)pc++;
        }
        po.resize(pc);
        for (int d = 0; d < 3; ++d) {
            vo[d].nbx = bv[d].nbx;
            vo[d].nby = bv[d].nby;
            vo[d].slot.resize(bv[d].slot.size());
            for (size_t b = 0; b < bv[d].slot.size(); ++b) vo[d].slot[b] = bv[d].slot[b] >= 0 ? bv[d].slot[b] : -1;
            vo[d].resize(bv[d].count());
        }
        if (!m_scene) {
            gbprojection::check(gbp_create(m_device, &m_ctx), "gbp_create");
            gbprojection::check(gbp_scene_create(m_ctx, 3, nx, ny, nz, m_dx, &m_scene), "gbp_scene_create");
            if (m_target_volume) gbp_scene_set_target_volume(m_scene, m_current_volume, m_target_volume);
        }
        gbp_stats st;
        const gbp_bricks in_s = bs.view(), in_f = bf.view(), in_u = bv[0].view(), in_v = bv[1].view(),
                         in_w = bv[2].view();
        gbp_bricks_out out_p = po.view(), out_u = vo[0].view(), out_v = vo[1].view(), out_w = vo[2].view();
        int rc = gbp_project_bricks(m_scene, dt, &in_s, &in_f, &in_u, &in_v, &in_w, &m_params, &out_p, &out_u, &out_v,
                                    &out_w, &st);
        gbprojection::check(rc, "gbp_project_bricks");
        console::dump("gbprojection3: %d iterations, Reresid=%e, %.3f ms\n", st.iterations, st.reresid, st.ms_total);
        console::write(get_argument_name() + "_number_projection_iteration", st.iterations);
        m_pressure.clear();
        for (int bz = 0; bz < bf.nbz; ++bz)
            for (int by = 0; by < bf.nby; ++by)
                for (int bx = 0; bx < bf.nbx; ++bx) {
                    const int sl = po.slot[(size_t)bx + (size_t)bf.nbx * (by + (size_t)bf.nby * bz)];
                    if (sl < 0) continue;
                    for (int k = 8 * bz; k < std::min(8 * bz + 8, nz); ++k)
                        for (int j = 8 * by; j < std::min(8 * by + 8, ny); ++j)
                            for (int i = 8 * bx; i < std::min(8 * bx + 8, nx); ++i) {
                                const size_t n = po.index(i, j, k);
                                if (po.active[n]) m_pressure.set(i, j, k, po.values[n]);
                            }
                }
        velocity.parallel_actives([&](int dim, int i, int j, int k, auto &it, int tn) {
            const size_t n = vo[dim].index(i, j, k);
            if (vo[dim].active[n]) it.set(vo[dim].values[n]);
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
    gbarray::Bricks m_bs, m_bf, m_bv[3];
    gbarray::BricksOut m_po, m_vo[3];
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
