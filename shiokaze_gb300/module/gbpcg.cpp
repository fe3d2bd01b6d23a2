// gbpcg.cpp -- Shiokaze plugin module "gbpcg": the reference's LinSolver
// "pcg" (src/linsolver/pcg.cpp:29-84) on the GPU, behind
// RCMatrix_solver_interface (include/shiokaze/linsolver/RCMatrix_solver.h:
// 37-95). Selected with LinSolver=gbpcg wherever the reference creates an
// RCMatrix_solver_driver (e.g. macpressuresolver3, macstreamfuncsolver3);
// compiled against the reference's headers and linked to libgbp.so.
//
// solve() reads the matrix row by row through const_for_each (as pcg.cpp
// builds its SparseMatrix), converts b, and calls gbp_csr_cg: plain FP64 CG
// from x = 0 with the reference solver's stopping rule and iteration count.
// The keys are pcg.cpp's: Residual, MaxIterations, and ModifiedIC /
// MinDiagRatio, which the reference reads but whose factorisation its
// preconditioner then discards (pcg_solver.h:379-384); they are accepted
// and have no effect here either. Device selects the CUDA device.
#include <shiokaze/core/console.h>
#include <shiokaze/linsolver/RCMatrix_solver.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbp.h"

SHKZ_USING_NAMESPACE

template <class N, class T> class gbpcg_solver : public RCMatrix_solver_interface<N, T> {
protected:
    LONG_NAME("GB300 Conjugate Gradient Solver")
    ARGUMENT_NAME("GBPCG")

    virtual void configure(configuration &config) override {
        config.get_double("Residual", m_residual, "Tolerable residual");
        config.get_double("ModifiedIC", m_mic, "Modified incomplete cholesky (no effect, as in pcg)");
        config.get_double("MinDiagRatio", m_min_diag, "Minimal diagonal ratio (no effect, as in pcg)");
        config.get_unsigned("MaxIterations", m_max_iterations, "Maximal iteration count");
        config.get_integer("Device", m_device, "CUDA device");
    }

    virtual typename RCMatrix_solver_interface<N, T>::Result solve(const RCMatrix_interface<N, T> *A,
                                                                   const RCMatrix_vector_interface<N, T> *b,
                                                                   RCMatrix_vector_interface<N, T> *x) const override {
        const N n = A->rows();
        std::vector<long long> rowstart((size_t)n + 1, 0), cols;
        std::vector<double> vals;
        for (N row = 0; row < n; ++row) {
            A->const_for_each(row, [&](N column, T value) {
                cols.push_back((long long)column);
                vals.push_back((double)value);
            });
            rowstart[(size_t)row + 1] = (long long)cols.size();
        }
        std::vector<T> rhs;
        b->convert_to(rhs);
        std::vector<double> bd(rhs.begin(), rhs.end()), xd((size_t)n, 0.0);
        if (!m_ctx && gbp_create(m_device, &m_ctx) != GBP_OK) {
            std::fprintf(stderr, "gbpcg: gbp_create failed: %s\n", gbp_strerror(GBP_ERR_NO_DEVICE));
            std::exit(-1);
        }
        gbp_csr_stats st;
        const int rc = gbp_csr_cg(m_ctx, (long long)n, rowstart.data(), cols.data(), vals.data(), bd.data(),
                                  xd.data(), m_residual, (int)m_max_iterations, &st);
        if (rc != GBP_OK && rc != GBP_ERR_NOT_CONVERGED && rc != GBP_ERR_NAN) {
            // the reference has no error returns and exits on unrecoverable
            // errors (src/core/module.cpp:112-115)
            std::fprintf(stderr, "gbpcg: gbp_csr_cg failed: %s\n", gbp_strerror(rc));
            std::exit(-1);
        }
        std::vector<T> result(xd.begin(), xd.end());
        x->convert_from(result);
        return {(N)st.iterations, (T)st.reresid};
    }

public:
    virtual ~gbpcg_solver() {
        if (m_ctx) gbp_destroy(m_ctx);
    }

private:
    double m_residual{1e-4};
    unsigned m_max_iterations{30000};
    double m_mic{0.97};
    double m_min_diag{0.25};
    int m_device{0};
    mutable gbp_ctx *m_ctx{nullptr};
};

extern "C" module *create_instance() { return new gbpcg_solver<INDEX_TYPE, FLOAT_TYPE>(); }
extern "C" const char *license() { return "MIT"; }
