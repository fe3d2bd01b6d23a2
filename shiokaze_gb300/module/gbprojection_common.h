// gbprojection_common.h -- configuration shared by the Shiokaze plugin
// modules gbprojection2 / gbprojection3 (the drop-in replacements for
// macpressuresolver2 / macpressuresolver3).
//
// Keys read from the reference's configuration, with its defaults:
//   Residual, MaxIterations (src/linsolver/pcg.cpp:39-44),
//   SecondOrderAccurateFluid, SecondOrderAccurateSolid, Gain, WarmStart
//   (src/projection/macpressuresolver3.cpp:274-280),
//   EpsFluid, EpsSolid (src/utility/macutility3.cpp:407-411),
// plus this module's own: Solver (cg | mgpcg), Precision (fp64 | mixed),
// MGSmooth, MGCoarsest, InnerTolerance, Device.
#pragma once

#include <shiokaze/core/configuration.h>

#include <cstdio>
#include <cstdlib>
#include <string>

#include "gbp.h"

namespace gbprojection {

inline void configure_params(shiokaze_v1::configuration &config, gbp_params &p, int &device) {
    double residual = p.residual;
    unsigned max_iter = (unsigned)p.max_iterations;
    bool warm = p.warm_start != 0, so_fluid = p.second_order_fluid != 0, so_solid = p.second_order_solid != 0;
    config.get_double("Residual", residual, "Tolerable residual");
    config.get_unsigned("MaxIterations", max_iter, "Maximal iteration count");
    config.get_bool("SecondOrderAccurateFluid", so_fluid, "Whether to enforce second order accuracy");
    config.get_bool("SecondOrderAccurateSolid", so_solid, "Whether to enforce second order accuracy for solid surfaces");
    config.get_double("Gain", p.gain, "Rate for volume correction");
    config.get_bool("WarmStart", warm, "Start from the solution of previous pressure");
    config.get_double("EpsFluid", p.eps_fluid, "Minimal bound for fluid fraction");
    config.get_double("EpsSolid", p.eps_solid, "Minimal bound for solid fraction");
    std::string solver = p.solver == GBP_SOLVER_MGPCG ? "mgpcg" : "cg";
    std::string precision = p.precision == GBP_PRECISION_MIXED ? "mixed" : "fp64";
    config.get_string("Solver", solver, "Linear solver on the GPU: cg (the reference's) or mgpcg");
    config.get_string("Precision", precision, "fp64 or mixed (FP32 inner solve, FP64 refinement)");
    config.get_integer("MGSmooth", p.mg_smooth, "Red-black sweeps per multigrid level");
    config.get_integer("MGCoarsest", p.mg_coarsest, "Coarsest multigrid edge");
    config.get_double("InnerTolerance", p.inner_tolerance, "Relative residual of each mixed-precision inner solve");
    config.get_integer("IterationsPerSync", p.iterations_per_sync, "CG iterations between host convergence checks");
    bool staging = p.tma_staging != 0, classes = p.tile_classes != 0;
    config.get_bool("TMAStaging", staging, "Stage the FP32 fine-level stencils in shared memory by TMA");
    config.get_bool("TileClasses", classes, "Use per-tile coupling classes in the multigrid kernels");
    p.tma_staging = staging;
    p.tile_classes = classes;
    config.get_integer("Device", device, "CUDA device");
    p.residual = residual;
    p.max_iterations = (int)max_iter;
    p.warm_start = warm;
    p.second_order_fluid = so_fluid;
    p.second_order_solid = so_solid;
    p.solver = solver == "mgpcg" ? GBP_SOLVER_MGPCG : GBP_SOLVER_CG;
    p.precision = precision == "mixed" ? GBP_PRECISION_MIXED : GBP_PRECISION_FP64;
}

// The reference has no error returns and exits on unrecoverable errors
// (src/core/module.cpp:112-115); a failed CUDA call does the same here.
inline void check(int rc, const char *what) {
    if (rc != GBP_OK && rc != GBP_ERR_NOT_CONVERGED) {
        std::fprintf(stderr, "gbprojection: %s failed: %s\n", what, gbp_strerror(rc));
        std::exit(-1);
    }
}

}  // namespace gbprojection
