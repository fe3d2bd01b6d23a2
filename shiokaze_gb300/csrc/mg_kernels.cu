// mg_kernels.cu -- multigrid-preconditioned CG (MGPCG) on the matrix-free
// operator, in FP64 or with an FP32 inner solve inside FP64 iterative
// refinement.
//
// Multigrid (published method: geometric multigrid as a CG preconditioner,
// McAdams, Sifakis and Teran 2010, here with the Galerkin coarse operator of
// piecewise-constant 2x2x2 aggregation, which keeps the ghost-fluid Dirichlet
// and cut-cell Neumann weights without special cases):
//   coarse operator  A_{l+1} = P^T A_l P, P = injection from the parent:
//                    coupling of two coarse cells = sum of the 4 fine
//                    couplings across their shared face; diagonal = sum of
//                    the children's diagonals minus twice their internal
//                    couplings. Computed in FP64.
//   V-cycle          pre-smooth red then black Gauss-Seidel (from x = 0),
//                    residual restricted by summing the 8 children,
//                    recurse, add `alpha` times the injected correction,
//                    post-smooth black then red (the adjoint order), so the
//                    preconditioner is symmetric; a fixed number of
//                    symmetric sweep pairs on the coarsest level.
//   CG               z = M r, rho = z.r, p = z + beta p, q = A p,
//                    alpha = rho / p.q, x += alpha p, r -= alpha q, with the
//                    reference's stopping rule |r|_inf <= Residual |r0|_inf.
//
// Vectors and operator arrays of a level are in T (double or float); dot
// products and norms are accumulated in FP64. Cells with inv == 0 (no
// unknown) keep x = 0.
//
// Algorithmic DRAM bytes per fine cell, with s = sizeof(T):
//   presmooth        read b, inv, cx, cy, cz; write x                 6 s
//   sweep (1 colour) read x, b, inv, cx, cy, cz (half the cells
//                    written); counted as a full pass                 7 s
//   restrict         read x, b, diag, cx, cy, cz; write b_c / 8      6 s + s/8
//   post_black       read x, x_c / 8, b, inv, cx, cy, cz; write half x  7 s
//   direction        read z, p; write p                               3 s
//   spmv             read p, diag, cx, cy, cz; write q                6 s
//   update           read x, p, r, q; write x, r                      6 s
#include "gbp_internal.cuh"
#include "gbp_kernels.h"
#include "gbp_mg.h"

namespace gbp {
namespace {

// Gate: 0 = run unless the solve is done; 1 = also skip once the inner
// solve of the mixed path has stopped; 2 = run only when the inner solve
// has stopped and the solve is not done (outer refinement step).
__device__ __forceinline__ bool gated(const Scalars *sc, int gate) {
    const volatile Scalars *v = sc;
    if (v->done) return true;
    if (gate == 1) return v->inner_done != 0;
    if (gate == 2) return v->inner_done == 0;
    return false;
}

template <class F> __device__ __forceinline__ void for_each_cell(const Grid &g, F f) {
    const int tx = threadIdx.x & (TILE_X - 1), ty = threadIdx.x / TILE_X;
    for (long long t = blockIdx.x; t < g.ntiles; t += gridDim.x) {
        int i0, j0, k0;
        tile_origin(g, t, i0, j0, k0);
        const int i = i0 + tx, j = j0 + ty;
        if (i >= g.nx || j >= g.ny) continue;
        const int kend = min(k0 + g.tz, g.nz);
        for (int k = k0; k < kend; ++k) f(i, j, k, cell_index(g, i, j, k));
    }
}

// sum_n c_n x_n over the in-bounds neighbours of cell c, x read through X.
template <class T, class X>
__device__ __forceinline__ T neighbour_sum(const MgLevel<T> &L, int i, int j, int k, long long c, X xat) {
    const Grid &g = L.g;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    T s = T(0);
    if (i > 0) s += L.cx[c - 1] * xat(c - 1, i - 1, j, k);
    if (i + 1 < g.nx) s += L.cx[c] * xat(c + 1, i + 1, j, k);
    if (j > 0) s += L.cy[c - sy] * xat(c - sy, i, j - 1, k);
    if (j + 1 < g.ny) s += L.cy[c] * xat(c + sy, i, j + 1, k);
    if (g.dim == 3) {
        if (k > 0) s += L.cz[c - sz] * xat(c - sz, i, j, k - 1);
        if (k + 1 < g.nz) s += L.cz[c] * xat(c + sz, i, j, k + 1);
    }
    return s;
}

// ---- operator setup -----------------------------------------------------------

// Level 0 in T from the FP64 assembly, and the inverse diagonal.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_fine_setup_kernel(Grid g, Operator<double> A, T *diag, T *inv,
                                                                      T *cx, T *cy, T *cz, bool copy) {
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        const double d = A.diag[c];
        inv[c] = d > 0.0 ? T(1.0 / d) : T(0);
        if (copy) {
            diag[c] = T(d);
            cx[c] = T(A.cx[c]);
            cy[c] = T(A.cy[c]);
            if (g.dim == 3) cz[c] = T(A.cz[c]);
        }
    });
}

// Galerkin coarse operator of 2x2x2 aggregation, one thread per coarse cell.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_coarsen_kernel(MgLevel<T> F, MgLevel<T> C, T *cdiag, T *cinv,
                                                                   T *ccx, T *ccy, T *ccz) {
    const Grid &fg = F.g;
    for_each_cell(C.g, [&](int I, int J, int K, long long cc) {
        double d = 0.0, ex = 0.0, ey = 0.0, ez = 0.0;
        const int kmax = fg.dim == 3 ? 2 : 1;
        for (int c2 = 0; c2 < kmax; ++c2)
            for (int b2 = 0; b2 < 2; ++b2)
                for (int a2 = 0; a2 < 2; ++a2) {
                    const int i = 2 * I + a2, j = 2 * J + b2, k = 2 * K + c2;
                    if (i >= fg.nx || j >= fg.ny || k >= fg.nz) continue;
                    const long long f = cell_index(fg, i, j, k);
                    d += (double)F.diag[f];
                    const double wx = F.cx[f], wy = F.cy[f];
                    if (a2 == 0) d -= 2.0 * wx; else ex += wx;
                    if (b2 == 0) d -= 2.0 * wy; else ey += wy;
                    if (fg.dim == 3) {
                        const double wz = F.cz[f];
                        if (c2 == 0) d -= 2.0 * wz; else ez += wz;
                    }
                }
        // a coupling to a neighbour outside the grid is 0 on the fine level too
        if (2 * I + 1 >= fg.nx) ex = 0.0;
        if (2 * J + 1 >= fg.ny) ey = 0.0;
        if (fg.dim == 3 && 2 * K + 1 >= fg.nz) ez = 0.0;
        // an aggregate whose indicator has (numerically) no energy is
        // dropped from the coarse problem: it is a floating Neumann pocket
        const bool active = d > 1e-12 * (ex + ey + ez + 1e-300);
        cdiag[cc] = T(active ? d : 0.0);
        cinv[cc] = active ? T(1.0 / d) : T(0);
        ccx[cc] = T(ex);
        ccy[cc] = T(ey);
        if (fg.dim == 3) ccz[cc] = T(ez);
    });
}

// ---- V-cycle --------------------------------------------------------------------
//
// The smoothing kernels of the global-memory levels run in a pair layout:
// a tile is 64 (x) by 8 (y) by TZ cells, each thread owning the two
// x-adjacent cells (i, i+1) of a row, one red and one black. A one-colour
// pass then keeps every lane busy and each thread has two independent cells
// in flight. The operator, b and the other colour's x are read through the
// read-only path (a colour pass never reads what it writes).

template <class F> __device__ __forceinline__ void for_each_pair(const Grid &g, F f) {
    const int px = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int ntx2 = (g.nx + 63) >> 6;
    const long long ntiles2 = (long long)ntx2 * g.nty * g.ntz;
    for (long long t = blockIdx.x; t < ntiles2; t += gridDim.x) {
        const long long tx = t % ntx2, r = t / ntx2;
        const int i = (int)tx * 64 + 2 * px;
        const int j = (int)(r % g.nty) * TILE_Y + ty;
        const int k0 = (int)(r / g.nty) * g.tz;
        if (i >= g.nx || j >= g.ny) continue;
        const int kend = min(k0 + g.tz, g.nz);
        const bool second = i + 1 < g.nx;
        for (int k = k0; k < kend; ++k) f(i, j, k, cell_index(g, i, j, k), second);
    }
}

// sum_n c_n x_n with the couplings read through the read-only path
template <class T, class X>
__device__ __forceinline__ T nsum_ro(const MgLevel<T> &L, int i, int j, int k, long long c, X xat) {
    const Grid &g = L.g;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    T s = T(0);
    if (i > 0) s += __ldg(L.cx + c - 1) * xat(c - 1, i - 1, j, k);
    if (i + 1 < g.nx) s += __ldg(L.cx + c) * xat(c + 1, i + 1, j, k);
    if (j > 0) s += __ldg(L.cy + c - sy) * xat(c - sy, i, j - 1, k);
    if (j + 1 < g.ny) s += __ldg(L.cy + c) * xat(c + sy, i, j + 1, k);
    if (g.dim == 3) {
        if (k > 0) s += __ldg(L.cz + c - sz) * xat(c - sz, i, j, k - 1);
        if (k + 1 < g.nz) s += __ldg(L.cz + c) * xat(c + sz, i, j, k + 1);
    }
    return s;
}

// Red (i+j+k even) then black Gauss-Seidel from x = 0 in one pass: red
// cells get b inv, black cells use their red neighbours' b inv.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_presmooth_kernel(MgLevel<T> L, const Scalars *sc, int gate) {
    if (gated(sc, gate)) return;
    auto red_value = [&](long long n, int, int, int) { return __ldg(L.b + n) * __ldg(L.inv + n); };
    for_each_pair(L.g, [&](int i, int j, int k, long long c, bool second) {
        const bool a_red = ((i + j + k) & 1) == 0;
        for (int h = 0; h < (second ? 2 : 1); ++h) {
            const long long cc = c + h;
            const bool red = (h == 0) == a_red;
            T xv;
            if (red) xv = __ldg(L.b + cc) * __ldg(L.inv + cc);
            else xv = (__ldg(L.b + cc) + nsum_ro(L, i + h, j, k, cc, red_value)) * __ldg(L.inv + cc);
            L.x[cc] = xv;
        }
    });
}

// One colour of Gauss-Seidel: x_c = (b_c + sum c_n x_n) inv_c.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_sweep_kernel(MgLevel<T> L, int color, const Scalars *sc,
                                                                 int gate) {
    if (gated(sc, gate)) return;
    auto xval = [&](long long n, int, int, int) { return __ldg(L.x + n); };
    for_each_pair(L.g, [&](int i, int j, int k, long long c, bool second) {
        const int h = ((i + j + k) & 1) == color ? 0 : 1;
        if (h == 1 && !second) return;
        const long long cc = c + h;
        L.x[cc] = (__ldg(L.b + cc) + nsum_ro(L, i + h, j, k, cc, xval)) * __ldg(L.inv + cc);
    });
}

// Residual b - A x of level L summed over each coarse cell's children.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_restrict_kernel(MgLevel<T> L, MgLevel<T> C, const Scalars *sc,
                                                                    int gate) {
    if (gated(sc, gate)) return;
    const Grid &fg = L.g;
    auto xval = [&](long long n, int, int, int) { return __ldg(L.x + n); };
    for_each_cell(C.g, [&](int I, int J, int K, long long cc) {
        T sum = T(0);
        const int kmax = fg.dim == 3 ? 2 : 1;
        for (int c2 = 0; c2 < kmax; ++c2)
            for (int b2 = 0; b2 < 2; ++b2)
                for (int a2 = 0; a2 < 2; ++a2) {
                    const int i = 2 * I + a2, j = 2 * J + b2, k = 2 * K + c2;
                    if (i >= fg.nx || j >= fg.ny || k >= fg.nz) continue;
                    const long long f = cell_index(fg, i, j, k);
                    const T s = nsum_ro(L, i, j, k, f, xval);
                    sum += __ldg(L.b + f) - (__ldg(L.diag + f) * __ldg(L.x + f) - s);
                }
        C.b[cc] = sum;
    });
}

// Black Gauss-Seidel on x + alpha P x_c: the red neighbours are read with
// their parent's correction added on the fly; the correction of the red
// cells themselves is never stored, since the red pass that follows
// recomputes them from the new black values.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_post_black_kernel(MgLevel<T> L, MgLevel<T> C, T alpha,
                                                                      const Scalars *sc, int gate) {
    if (gated(sc, gate)) return;
    const Grid &cg = C.g;
    const bool d3 = L.g.dim == 3;
    auto corrected = [&](long long n, int ni, int nj, int nk) {
        return __ldg(L.x + n) + alpha * __ldg(C.x + cell_index(cg, ni >> 1, nj >> 1, d3 ? (nk >> 1) : 0));
    };
    for_each_pair(L.g, [&](int i, int j, int k, long long c, bool second) {
        const int h = ((i + j + k) & 1) == 1 ? 0 : 1;
        if (h == 1 && !second) return;
        const long long cc = c + h;
        L.x[cc] = (__ldg(L.b + cc) + nsum_ro(L, i + h, j, k, cc, corrected)) * __ldg(L.inv + cc);
    });
}

// Last red pass of the fine level, fused with the preconditioned dot
// rho' = z . r (z = x, r = b on the fine level) over every cell; the last
// block sets beta = rho'/rho (0 when a new direction starts).
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_red_dot_kernel(MgLevel<T> L, Scalars *sc, Partials *pt,
                                                                   int gate, int do_red) {
    if (gated(sc, gate)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    double dot = 0.0;
    auto xval = [&](long long n, int, int, int) { return __ldg(L.x + n); };
    for_each_pair(L.g, [&](int i, int j, int k, long long c, bool second) {
        const int hr = ((i + j + k) & 1) == 0 ? 0 : 1;  // red cell of the pair
        for (int h = 0; h < (second ? 2 : 1); ++h) {
            const long long cc = c + h;
            const T bv = __ldg(L.b + cc);
            T xv;
            if (do_red && h == hr) {
                xv = (bv + nsum_ro(L, i + h, j, k, cc, xval)) * __ldg(L.inv + cc);
                L.x[cc] = xv;
            } else {
                xv = L.x[cc];
            }
            dot = fma((double)xv, (double)bv, dot);
        }
    });
    const double bs = block_sum(dot, sh);
    if (threadIdx.x == 0) pt->a[blockIdx.x] = bs;
    if (last_block(&sc->counter[4])) {
        const double rho_new = reduce_partials_sum(pt->a, gridDim.x, sh);
        if (threadIdx.x == 0) {
            if (sc->first) {
                sc->beta = 0.0;
                sc->first = 0;
            } else {
                sc->beta = rho_new / sc->rho;
            }
            sc->rho = rho_new;
            if (rho_new != rho_new) {
                sc->done = 1;
                sc->status = 3;
            }
            sc->counter[4] = 0;
        }
    }
}

// Coarsest level: `pairs` symmetric sweep pairs (red, black, black, red)
// from x = 0 in FP64, one block, the level held in shared memory.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_coarsest_kernel(MgLevel<T> L, int pairs, const Scalars *sc,
                                                                    int gate) {
    if (gated(sc, gate)) return;
    __shared__ double sb[MG_COARSEST_MAX], sinv[MG_COARSEST_MAX], scx[MG_COARSEST_MAX], scy[MG_COARSEST_MAX],
        scz[MG_COARSEST_MAX], sx[MG_COARSEST_MAX];
    const Grid &g = L.g;
    const int n = (int)g.ncell;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        sb[c] = L.b[c];
        sinv[c] = L.inv[c];
        scx[c] = L.cx[c];
        scy[c] = L.cy[c];
        scz[c] = g.dim == 3 ? (double)L.cz[c] : 0.0;
        sx[c] = 0.0;
    }
    __syncthreads();
    const int sy = g.nx, sz = g.nx * g.ny;
    auto relax = [&](int color) {
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            const int i = c % g.nx, j = (c / g.nx) % g.ny, k = c / sz;
            if (((i + j + k) & 1) != color) continue;
            double s = 0.0;
            if (i > 0) s += scx[c - 1] * sx[c - 1];
            if (i + 1 < g.nx) s += scx[c] * sx[c + 1];
            if (j > 0) s += scy[c - sy] * sx[c - sy];
            if (j + 1 < g.ny) s += scy[c] * sx[c + sy];
            if (k > 0) s += scz[c - sz] * sx[c - sz];
            if (k + 1 < g.nz) s += scz[c] * sx[c + sz];
            sx[c] = (sb[c] + s) * sinv[c];
        }
        __syncthreads();
    };
    for (int p = 0; p < pairs; ++p) {
        relax(0);
        relax(1);
        relax(1);
        relax(0);
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) L.x[c] = T(sx[c]);
}


// ---- coarse tail: the small levels in one block ---------------------------------

template <class T> struct TailArgs {
    int nt;  // tail levels (tail-relative index 0 = the finest of them)
    MgLevel<T> lv[MG_MAX_LEVELS];
    MgSettings ms;
};

template <class T> struct SLevel {
    int nx, ny, nz, dim, n;
    T *b, *x, *inv, *diag, *cx, *cy, *cz;
};

template <class T, class X>
__device__ __forceinline__ T snb(const SLevel<T> &L, int i, int j, int k, int c, X xat) {
    const int sy = L.nx, sz = L.nx * L.ny;
    T s = T(0);
    if (i > 0) s += L.cx[c - 1] * xat(c - 1);
    if (i + 1 < L.nx) s += L.cx[c] * xat(c + 1);
    if (j > 0) s += L.cy[c - sy] * xat(c - sy);
    if (j + 1 < L.ny) s += L.cy[c] * xat(c + sy);
    if (L.dim == 3) {
        if (k > 0) s += L.cz[c - sz] * xat(c - sz);
        if (k + 1 < L.nz) s += L.cz[c] * xat(c + sz);
    }
    return s;
}

template <class T, class F> __device__ __forceinline__ void s_for_each(const SLevel<T> &L, F f) {
    for (int c = threadIdx.x; c < L.n; c += blockDim.x) {
        const int i = c % L.nx, t = c / L.nx, j = t % L.ny, k = t / L.ny;
        f(i, j, k, c);
    }
    __syncthreads();
}

// The V-cycle below (and including) the tail's finest level, from shared
// memory, with the same smoother, transfers and coarsest solve as the
// global-memory kernels. Input: b of the finest tail level (global);
// output: its x (global).
template <class T>
__global__ void __launch_bounds__(MG_TAIL_THREADS) mg_tail_kernel(TailArgs<T> A, const Scalars *sc, int gate) {
    if (gated(sc, gate)) return;
    extern __shared__ __align__(16) unsigned char tail_smem[];
    SLevel<T> S[MG_MAX_LEVELS];
    size_t off = 0;
    T *base = reinterpret_cast<T *>(tail_smem);
    for (int l = 0; l < A.nt; ++l) {
        const Grid &g = A.lv[l].g;
        SLevel<T> &L = S[l];
        L.nx = g.nx;
        L.ny = g.ny;
        L.nz = g.nz;
        L.dim = g.dim;
        L.n = (int)g.ncell;
        T **arr[7] = {&L.b, &L.x, &L.inv, &L.diag, &L.cx, &L.cy, &L.cz};
        for (int a = 0; a < 7; ++a) {
            *arr[a] = base + off;
            off += (size_t)L.n;
        }
    }
    // FP64 iterate of the coarsest level after the T arrays
    size_t off_bytes = off * sizeof(T);
    off_bytes = (off_bytes + 15) / 16 * 16;
    double *xc = reinterpret_cast<double *>(tail_smem + off_bytes);

    for (int l = 0; l < A.nt; ++l) {
        const MgLevel<T> &G = A.lv[l];
        SLevel<T> &L = S[l];
        for (int c = threadIdx.x; c < L.n; c += blockDim.x) {
            L.inv[c] = G.inv[c];
            L.diag[c] = G.diag[c];
            L.cx[c] = G.cx[c];
            L.cy[c] = G.cy[c];
            L.cz[c] = L.dim == 3 ? G.cz[c] : T(0);
            if (l == 0) L.b[c] = G.b[c];
        }
    }
    __syncthreads();
    const int smooth = A.ms.smooth;
    const T alpha = T(A.ms.alpha);
    // descend
    for (int l = 0; l + 1 < A.nt; ++l) {
        const SLevel<T> &L = S[l];
        s_for_each(L, [&](int i, int j, int k, int c) {
            const T inv = L.inv[c];
            if (((i + j + k) & 1) == 0) {
                L.x[c] = L.b[c] * inv;
            } else {
                const T s = snb(L, i, j, k, c, [&](int n) { return L.b[n] * L.inv[n]; });
                L.x[c] = (L.b[c] + s) * inv;
            }
        });
        for (int sw = 1; sw < smooth; ++sw)
            for (int color = 0; color < 2; ++color)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != color) return;
                    L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int n) { return L.x[n]; })) * L.inv[c];
                });
        const SLevel<T> &C = S[l + 1];
        s_for_each(C, [&](int I, int J, int K, int cc) {
            T sum = T(0);
            const int kmax = L.dim == 3 ? 2 : 1;
            for (int c2 = 0; c2 < kmax; ++c2)
                for (int b2 = 0; b2 < 2; ++b2)
                    for (int a2 = 0; a2 < 2; ++a2) {
                        const int i = 2 * I + a2, j = 2 * J + b2, k = 2 * K + c2;
                        if (i >= L.nx || j >= L.ny || k >= L.nz) continue;
                        const int f = i + L.nx * (j + L.ny * k);
                        const T s = snb(L, i, j, k, f, [&](int n) { return L.x[n]; });
                        sum += L.b[f] - (L.diag[f] * L.x[f] - s);
                    }
            C.b[cc] = sum;
        });
    }
    // coarsest level: symmetric sweep pairs in FP64
    {
        const SLevel<T> &L = S[A.nt - 1];
        for (int c = threadIdx.x; c < L.n; c += blockDim.x) xc[c] = 0.0;
        __syncthreads();
        for (int p = 0; p < A.ms.coarsest_pairs; ++p) {
            const int order[4] = {0, 1, 1, 0};
            for (int q = 0; q < 4; ++q)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != order[q]) return;
                    const int sy = L.nx, sz = L.nx * L.ny;
                    double s = 0.0;
                    if (i > 0) s += (double)L.cx[c - 1] * xc[c - 1];
                    if (i + 1 < L.nx) s += (double)L.cx[c] * xc[c + 1];
                    if (j > 0) s += (double)L.cy[c - sy] * xc[c - sy];
                    if (j + 1 < L.ny) s += (double)L.cy[c] * xc[c + sy];
                    if (L.dim == 3) {
                        if (k > 0) s += (double)L.cz[c - sz] * xc[c - sz];
                        if (k + 1 < L.nz) s += (double)L.cz[c] * xc[c + sz];
                    }
                    xc[c] = ((double)L.b[c] + s) * (double)L.inv[c];
                });
        }
        for (int c = threadIdx.x; c < L.n; c += blockDim.x) L.x[c] = T(xc[c]);
        __syncthreads();
    }
    // ascend
    for (int l = A.nt - 2; l >= 0; --l) {
        const SLevel<T> &L = S[l];
        const SLevel<T> &C = S[l + 1];
        s_for_each(L, [&](int i, int j, int k, int c) {
            if (((i + j + k) & 1) != 1) return;
            const T s = snb(L, i, j, k, c, [&](int n) {
                const int ni = n % L.nx, t = n / L.nx, nj = t % L.ny, nk = t / L.ny;
                return L.x[n] + alpha * C.x[(ni >> 1) + C.nx * ((nj >> 1) + C.ny * (L.dim == 3 ? (nk >> 1) : 0))];
            });
            L.x[c] = (L.b[c] + s) * L.inv[c];
        });
        for (int sw = 1; sw < smooth; ++sw)
            for (int color = 0; color < 2; ++color)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != color) return;
                    L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int n) { return L.x[n]; })) * L.inv[c];
                });
        s_for_each(L, [&](int i, int j, int k, int c) {
            if (((i + j + k) & 1) != 0) return;
            L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int n) { return L.x[n]; })) * L.inv[c];
        });
    }
    const SLevel<T> &L0 = S[0];
    for (int c = threadIdx.x; c < L0.n; c += blockDim.x) A.lv[0].x[c] = L0.x[c];
}

// ---- CG on T vectors ------------------------------------------------------------

// p = z + beta p
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) pcg_direction_kernel(Grid g, const T *__restrict__ z, T *p,
                                                                      const Scalars *sc, int gate) {
    if (gated(sc, gate)) return;
    const T beta = T(sc->beta);
    if (beta == T(0)) {
        for_each_cell(g, [&](int, int, int, long long c) { p[c] = z[c]; });
    } else {
        for_each_cell(g, [&](int, int, int, long long c) { p[c] = z[c] + beta * p[c]; });
    }
}

// q = A p, p.q in FP64; the last block sets alpha = rho / p.q.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) pcg_spmv_kernel(MgLevel<T> L, const T *__restrict__ p, T *q,
                                                                 Scalars *sc, Partials *pt, int gate) {
    if (gated(sc, gate)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    double dot = 0.0;
    for_each_cell(L.g, [&](int i, int j, int k, long long c) {
        const T s = neighbour_sum(L, i, j, k, c, [&](long long n, int, int, int) { return p[n]; });
        const T qv = L.diag[c] * p[c] - s;
        q[c] = qv;
        dot = fma((double)p[c], (double)qv, dot);
    });
    const double bs = block_sum(dot, sh);
    if (threadIdx.x == 0) pt->a[blockIdx.x] = bs;
    if (last_block(&sc->counter[5])) {
        const double pq = reduce_partials_sum(pt->a, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->pap = pq;
            sc->alpha = sc->rho / pq;
            sc->counter[5] = 0;
        }
    }
}

// x += alpha p (x = alpha p on the first update of an inner solve),
// r -= alpha q, |r|_inf in FP64. mode 0: the solve's own stopping rule
// (|r|_inf <= tol sets done); mode 1: inner solve of the mixed path
// (|r|_inf <= inner_tol or the inner cap sets inner_done).
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) pcg_update_kernel(Grid g, T *x, T *r, const T *__restrict__ p,
                                                                   const T *__restrict__ q, Scalars *sc,
                                                                   Partials *pt, int mode, int gate) {
    if (gated(sc, gate)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    const T alpha = T(sc->alpha);
    const bool overwrite = sc->first_update != 0;
    double mx = 0.0;
    for_each_cell(g, [&](int, int, int, long long c) {
        x[c] = overwrite ? alpha * p[c] : x[c] + alpha * p[c];
        const T rv = r[c] - alpha * q[c];
        r[c] = rv;
        mx = fmax(mx, fabs((double)rv));
    });
    const double bm = block_max(mx, sh);
    if (threadIdx.x == 0) pt->b[blockIdx.x] = bm;
    if (last_block(&sc->counter[6])) {
        const double res = reduce_partials_max(pt->b, gridDim.x, sh);
        if (threadIdx.x == 0) {
            sc->first_update = 0;
            sc->iter += 1;
            const bool bad = res != res || sc->alpha != sc->alpha;
            if (mode == 0) {
                sc->res = res;
                if (bad) {
                    sc->done = 1;
                    sc->status = 3;
                } else if (res <= sc->tol) {
                    sc->done = 1;
                    sc->status = 1;
                } else if (sc->iter >= sc->max_iter) {
                    sc->done = 1;
                    sc->status = 2;
                }
            } else {
                sc->inner_iter += 1;
                if (bad) {
                    sc->done = 1;
                    sc->status = 3;
                } else if (res <= sc->inner_tol || sc->inner_iter >= sc->inner_max || sc->iter >= sc->max_iter) {
                    sc->inner_done = 1;
                }
            }
            sc->counter[6] = 0;
        }
    }
}

// ---- mixed precision: FP64 refinement --------------------------------------------

// x64 += d (the inner solve's FP32 correction); gated on inner_done.
__global__ void __launch_bounds__(BLOCK_THREADS, 6) refine_accumulate_kernel(Grid g, double *x, const float *d,
                                                                          const Scalars *sc) {
    if (gated(sc, 2)) return;
    for_each_cell(g, [&](int, int, int, long long c) { x[c] += (double)d[c]; });
}

// r64 = b - A64 (prev + x64) with the FP64 operator, |r64|_inf; r_f = r64.
// The last block applies the stopping rule and, unless done, opens the
// next inner solve. Also serves as the initial residual (gate 0).
__global__ void __launch_bounds__(BLOCK_THREADS, 6) refine_residual_kernel(Grid g, Operator<double> A,
                                                                        const double *__restrict__ b,
                                                                        const double *__restrict__ prev,
                                                                        const double *__restrict__ x, double *r,
                                                                        float *rf, double *zero_x, Scalars *sc,
                                                                        Partials *pt, int initial, double residual,
                                                                        int max_iter, double inner_rel,
                                                                        int inner_max) {
    if (!initial && gated(sc, 2)) return;
    __shared__ double sh[BLOCK_THREADS / 32];
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    auto X = [&](long long c) {
        double v = x ? x[c] : 0.0;
        if (prev) v += prev[c];
        return v;
    };
    double mx = 0.0;
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        double acc = A.diag[c] * X(c);
        if (i > 0) acc -= A.cx[c - 1] * X(c - 1);
        if (i + 1 < g.nx) acc -= A.cx[c] * X(c + 1);
        if (j > 0) acc -= A.cy[c - sy] * X(c - sy);
        if (j + 1 < g.ny) acc -= A.cy[c] * X(c + sy);
        if (g.dim == 3) {
            if (k > 0) acc -= A.cz[c - sz] * X(c - sz);
            if (k + 1 < g.nz) acc -= A.cz[c] * X(c + sz);
        }
        const double rv = b[c] - acc;
        r[c] = rv;
        if (rf) rf[c] = (float)rv;
        if (zero_x) zero_x[c] = 0.0;
        mx = fmax(mx, fabs(rv));
    });
    const double bm = block_max(mx, sh);
    if (threadIdx.x == 0) pt->c[blockIdx.x] = bm;
    if (last_block(&sc->counter[7])) {
        const double res = reduce_partials_max(pt->c, gridDim.x, sh);
        if (threadIdx.x == 0) {
            if (initial) {
                const double tolf = residual < 1e-30 ? 1e-30 : residual;
                sc->res0 = res;
                sc->tol = tolf * res;
                sc->iter = 0;
                sc->outer_iter = 0;
                sc->max_iter = max_iter;
                sc->inner_max = inner_max;
                sc->status = 0;
                sc->done = 0;
            } else {
                sc->outer_iter += 1;
            }
            sc->res = res;
            if (res != res) {
                sc->done = 1;
                sc->status = 3;
            } else if (res <= sc->tol) {
                sc->done = 1;
                sc->status = 1;
            } else if (sc->iter >= sc->max_iter) {
                sc->done = 1;
                sc->status = 2;
            } else {
                // open an inner solve on r_f = r64
                sc->inner_done = 0;
                sc->inner_iter = 0;
                sc->first = 1;
                sc->first_update = 1;
                sc->inner_res0 = res;
                sc->inner_tol = inner_rel * res;
            }
            sc->counter[7] = 0;
        }
    }
}

template <class T> int nblocks(const Grid &g, int grid_blocks) {
    long long b = g.ntiles < grid_blocks ? g.ntiles : grid_blocks;
    return b < 1 ? 1 : (int)b;
}

// blocks for the pair-layout kernels (64-wide tiles)
int pblocks(const Grid &g, int grid_blocks) {
    const long long t = (long long)((g.nx + 63) / 64) * g.nty * g.ntz;
    long long b = t < grid_blocks ? t : grid_blocks;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

template <class T>
cudaError_t mg_setup(const Grid &g0, Operator<double> A, const MgHierarchy<T> &H, int grid_blocks,
                     cudaStream_t stream) {
    const MgLevel<T> &L0 = H.levels[0];
    const bool copy = !H.fine_aliases_fp64;
    mg_fine_setup_kernel<T><<<nblocks<T>(g0, grid_blocks), BLOCK_THREADS, 0, stream>>>(
        g0, A, const_cast<T *>(L0.diag), const_cast<T *>(L0.inv), const_cast<T *>(L0.cx), const_cast<T *>(L0.cy),
        const_cast<T *>(L0.cz), copy);
    for (int l = 0; l + 1 < H.nlevels; ++l) {
        const MgLevel<T> &F = H.levels[l], &C = H.levels[l + 1];
        mg_coarsen_kernel<T><<<nblocks<T>(C.g, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            F, C, const_cast<T *>(C.diag), const_cast<T *>(C.inv), const_cast<T *>(C.cx), const_cast<T *>(C.cy),
            const_cast<T *>(C.cz));
    }
    return cudaGetLastError();
}

template <class T>
cudaError_t mg_vcycle(const MgHierarchy<T> &H, const MgSettings &ms, Scalars *sc, Partials *pt, int gate,
                      int grid_blocks, cudaStream_t stream, long long *launches) {
    const int L = H.nlevels;
    const bool has_tail = H.tail < L;
    const int G = has_tail ? H.tail : L - 1;  // first level solved by the bottom kernel
    long long n = 0;
    // descend through the global-memory levels
    for (int l = 0; l < G; ++l) {
        const MgLevel<T> &F = H.levels[l];
        const int nb = pblocks(F.g, grid_blocks);
        mg_presmooth_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, sc, gate);
        ++n;
        for (int s = 1; s < ms.smooth; ++s) {
            mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 0, sc, gate);
            mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 1, sc, gate);
            n += 2;
        }
        const MgLevel<T> &C = H.levels[l + 1];
        mg_restrict_kernel<T><<<nblocks<T>(C.g, grid_blocks), BLOCK_THREADS, 0, stream>>>(F, C, sc, gate);
        ++n;
    }
    // bottom: the shared-memory tail, or the coarsest level alone
    if (has_tail) {
        TailArgs<T> A;
        A.nt = L - G;
        for (int l = G; l < L; ++l) A.lv[l - G] = H.levels[l];
        A.ms = ms;
        mg_tail_kernel<T><<<1, MG_TAIL_THREADS, H.tail_smem, stream>>>(A, sc, gate);
    } else {
        mg_coarsest_kernel<T><<<1, BLOCK_THREADS, 0, stream>>>(H.levels[L - 1], ms.coarsest_pairs, sc, gate);
    }
    ++n;
    // ascend
    for (int l = G - 1; l >= 0; --l) {
        const MgLevel<T> &F = H.levels[l], &C = H.levels[l + 1];
        const int nb = pblocks(F.g, grid_blocks);
        mg_post_black_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, C, T(ms.alpha), sc, gate);
        ++n;
        for (int s = 1; s < ms.smooth; ++s) {
            mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 0, sc, gate);
            mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 1, sc, gate);
            n += 2;
        }
        if (l > 0) {
            mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 0, sc, gate);
        } else {
            mg_red_dot_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, sc, pt, gate, 1);
        }
        ++n;
    }
    if (G == 0) {
        // a single level: the coarsest solve is the whole preconditioner;
        // the dot comes from a pass that does not update
        mg_red_dot_kernel<T><<<pblocks(H.levels[0].g, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            H.levels[0], sc, pt, gate, 0);
        ++n;
    }
    *launches += n;
    return cudaGetLastError();
}

// Opt-in to the shared memory the tail kernel needs (once per process).
template <class T> cudaError_t mg_tail_enable(size_t bytes) {
    return cudaFuncSetAttribute(mg_tail_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
template cudaError_t mg_tail_enable<double>(size_t);
template cudaError_t mg_tail_enable<float>(size_t);

template <class T>
cudaError_t pcg_iteration(const MgHierarchy<T> &H, const MgSettings &ms, T *x, T *r, T *z, T *p, T *q, Scalars *sc,
                          Partials *pt, int mode, int grid_blocks, cudaStream_t stream, long long *launches) {
    const int gate = mode == 1 ? 1 : 0;
    cudaError_t e = mg_vcycle(H, ms, sc, pt, gate, grid_blocks, stream, launches);
    if (e != cudaSuccess) return e;
    const MgLevel<T> &L0 = H.levels[0];
    const int nb = nblocks<T>(L0.g, grid_blocks);
    pcg_direction_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0.g, z, p, sc, gate);
    pcg_spmv_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0, p, q, sc, pt, gate);
    pcg_update_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0.g, x, r, p, q, sc, pt, mode, gate);
    *launches += 3;
    return cudaGetLastError();
}

cudaError_t refine_residual(const Grid &g, Operator<double> A, const double *b, const double *prev, const double *x,
                            double *r, float *rf, double *zero_x, Scalars *sc, Partials *pt, bool initial,
                            double residual, int max_iter, double inner_rel, int inner_max, int grid_blocks,
                            cudaStream_t stream) {
    refine_residual_kernel<<<nblocks<double>(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(
        g, A, b, prev, x, r, rf, zero_x, sc, pt, initial ? 1 : 0, residual, max_iter, inner_rel, inner_max);
    return cudaGetLastError();
}

cudaError_t refine_accumulate(const Grid &g, double *x, const float *d, const Scalars *sc, int grid_blocks,
                              cudaStream_t stream) {
    refine_accumulate_kernel<<<nblocks<double>(g, grid_blocks), BLOCK_THREADS, 0, stream>>>(g, x, d, sc);
    return cudaGetLastError();
}

// benchmarking: one launch of a V-cycle kernel on level 0
template <class T>
cudaError_t mg_bench_launch(const MgHierarchy<T> &H, int which, Scalars *sc, Partials *pt, int grid_blocks,
                            cudaStream_t stream) {
    const MgLevel<T> &F = H.levels[0];
    const int nb = pblocks(F.g, grid_blocks);
    switch (which) {
    case 0: mg_presmooth_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, sc, 0); break;
    case 1: mg_sweep_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, 0, sc, 0); break;
    case 2:
        if (H.nlevels < 2) return cudaErrorInvalidValue;
        mg_restrict_kernel<T><<<nblocks<T>(H.levels[1].g, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            F, H.levels[1], sc, 0);
        break;
    case 3:
        if (H.nlevels < 2) return cudaErrorInvalidValue;
        mg_post_black_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, H.levels[1], T(1), sc, 0);
        break;
    case 4: mg_red_dot_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(F, sc, pt, 0, 1); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <class T>
cudaError_t pcg_bench_launch(const MgHierarchy<T> &H, int which, T *x, T *r, T *z, T *p, T *q, Scalars *sc,
                             Partials *pt, int grid_blocks, cudaStream_t stream) {
    const MgLevel<T> &L0 = H.levels[0];
    const int nb = nblocks<T>(L0.g, grid_blocks);
    switch (which) {
    case 0: pcg_direction_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0.g, z, p, sc, 0); break;
    case 1: pcg_spmv_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0, p, q, sc, pt, 0); break;
    case 2: pcg_update_kernel<T><<<nb, BLOCK_THREADS, 0, stream>>>(L0.g, x, r, p, q, sc, pt, 0, 0); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template cudaError_t pcg_bench_launch<double>(const MgHierarchy<double> &, int, double *, double *, double *,
                                              double *, double *, Scalars *, Partials *, int, cudaStream_t);
template cudaError_t pcg_bench_launch<float>(const MgHierarchy<float> &, int, float *, float *, float *, float *,
                                             float *, Scalars *, Partials *, int, cudaStream_t);
template cudaError_t mg_setup<double>(const Grid &, Operator<double>, const MgHierarchy<double> &, int, cudaStream_t);
template cudaError_t mg_setup<float>(const Grid &, Operator<double>, const MgHierarchy<float> &, int, cudaStream_t);
template cudaError_t pcg_iteration<double>(const MgHierarchy<double> &, const MgSettings &, double *, double *,
                                           double *, double *, double *, Scalars *, Partials *, int, int,
                                           cudaStream_t, long long *);
template cudaError_t pcg_iteration<float>(const MgHierarchy<float> &, const MgSettings &, float *, float *, float *,
                                          float *, float *, Scalars *, Partials *, int, int, cudaStream_t,
                                          long long *);
template cudaError_t mg_bench_launch<double>(const MgHierarchy<double> &, int, Scalars *, Partials *, int,
                                             cudaStream_t);
template cudaError_t mg_bench_launch<float>(const MgHierarchy<float> &, int, Scalars *, Partials *, int,
                                            cudaStream_t);

}  // namespace gbp
