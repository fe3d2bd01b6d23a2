// mg_kernels.cu -- multigrid hierarchy setup of one scene: the fine level in
// T with its inverse diagonal, and the Galerkin coarse operators. The
// iteration itself (V-cycle, CG, refinement) is in batch_kernels.cu.
//
// Multigrid (published method: geometric multigrid as a CG preconditioner,
// McAdams, Sifakis and Teran 2010, here with the Galerkin coarse operator of
// piecewise-constant 2x2x2 aggregation, which keeps the ghost-fluid Dirichlet
// and cut-cell Neumann weights without special cases):
//   coarse operator  A_{l+1} = P^T A_l P, P = injection from the parent:
//                    coupling of two coarse cells = sum of the 4 fine
//                    couplings across their shared face; diagonal = sum of
//                    the children's diagonals minus twice their internal
//                    couplings. Computed in FP64 for the FP64
//                    hierarchy, in float-float for the FP32 one.
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
#include <algorithm>

#include "gbp_convert.cuh"
#include "gbp_floatfloat.cuh"
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

// 1/d in the level's type: FP64 division for the FP64 hierarchy; for the
// FP32 one the correctly rounded FP32 reciprocal of the rounded diagonal
// (no FP64 division, whose pipe is scarce on this GPU; the preconditioner
// only needs a consistent value).
template <class T> __device__ __forceinline__ T recip(double d);
template <> __device__ __forceinline__ double recip<double>(double d) { return 1.0 / d; }
template <> __device__ __forceinline__ float recip<float>(double d) { return __frcp_rn(d2f_rn(d)); }

// FP64 to the level's type; to FP32 by integer instructions (gbp_convert.cuh)
template <class T> __device__ __forceinline__ T narrow(double v);
template <> __device__ __forceinline__ double narrow<double>(double v) { return v; }
template <> __device__ __forceinline__ float narrow<float>(double v) { return d2f_rn(v); }

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
                                                                      T *cx, T *cy, T *cz, bool copy, T *lo0, T *lo1,
                                                                      T *lo2, T *lo3) {
    for_each_cell(g, [&](int i, int j, int k, long long c) {
        const double d = A.diag[c];
        inv[c] = positive_bits(d) ? recip<T>(d) : T(0);
        if (copy) {
            const double v[4] = {d, A.cx[c], A.cy[c], g.dim == 3 ? A.cz[c] : 0.0};
            T *hi[4] = {diag, cx, cy, cz};
            T *lo[4] = {lo0, lo1, lo2, lo3};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q == 3 && g.dim != 3) break;
                const T h = narrow<T>(v[q]);
                hi[q][c] = h;
                if constexpr (sizeof(T) == 4)
                    if (lo0) lo[q][c] = split_lo(v[q], h);
            }
        }
    });
}

// Galerkin coarse operator of 2x2x2 aggregation, one thread per coarse cell.
// The FP32 hierarchy sums in float-float (its terms are floats and 2 w is
// exact) and rounds once to float: FP32 instructions only, where the FP64
// sums of every child took most of its setup time on this GPU's scarce
// FP64 pipe (about one FP64 operation per clock per SM). The FP64
// hierarchy sums in FP64.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) mg_coarsen_kernel(MgLevel<T> F, MgLevel<T> C, T *cdiag, T *cinv,
                                                                   T *ccx, T *ccy, T *ccz) {
    const Grid &fg = F.g;
    if constexpr (sizeof(T) == 4) {
        for_each_cell(C.g, [&](int I, int J, int K, long long cc) {
            FloatFloat d, ex, ey, ez;
            const int kmax = fg.dim == 3 ? 2 : 1;
            for (int c2 = 0; c2 < kmax; ++c2)
                for (int b2 = 0; b2 < 2; ++b2)
                    for (int a2 = 0; a2 < 2; ++a2) {
                        const int i = 2 * I + a2, j = 2 * J + b2, k = 2 * K + c2;
                        if (i >= fg.nx || j >= fg.ny || k >= fg.nz) continue;
                        const long long f = cell_index(fg, i, j, k);
                        d.add(F.diag[f]);
                        const float wx = F.cx[f], wy = F.cy[f];
                        if (a2 == 0) d.add(-2.0f * wx); else ex.add(wx);
                        if (b2 == 0) d.add(-2.0f * wy); else ey.add(wy);
                        if (fg.dim == 3) {
                            const float wz = F.cz[f];
                            if (c2 == 0) d.add(-2.0f * wz); else ez.add(wz);
                        }
                    }
            float vx = ex.value(), vy = ey.value(), vz = ez.value();
            if (2 * I + 1 >= fg.nx) vx = 0.0f;
            if (2 * J + 1 >= fg.ny) vy = 0.0f;
            if (fg.dim == 3 && 2 * K + 1 >= fg.nz) vz = 0.0f;
            // an aggregate whose indicator has (numerically) no energy is
            // dropped (a floating Neumann pocket); its float-float sum of
            // exactly cancelling terms is 0 or below 2^-40 of the couplings
            const float dv = d.value();
            const bool active = dv > 1e-9f * (vx + vy + vz) + 1e-37f;
            cdiag[cc] = T(active ? dv : 0.0f);
            cinv[cc] = active ? __frcp_rn(dv) : T(0);
            ccx[cc] = T(vx);
            ccy[cc] = T(vy);
            if (fg.dim == 3) ccz[cc] = T(vz);
        });
        return;
    }
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

// Tile classes of level L (TILE_MIXED / TILE_EMPTY / the common coupling).
// mode 0: box b is pair tile b of L.g (64 x 8 x tz cells); mode 1: box b
// holds the fine cells of cell tile b of the coarser grid gc (64 x 16 x
// 2 tz_c, a restriction item). A cell contributes its diagonal and the
// coupling of each face whose neighbour is inside the grid, the ones the
// stencils read. Values are compared through their bit patterns (integer
// min and max: no FP64 instruction, and "uniform" means bitwise equal).
template <class T> struct Bits;
template <> struct Bits<float> {
    using U = unsigned;
    static __device__ U of(float v) { return __float_as_uint(v); }
    static __device__ float value(U u) { return __uint_as_float(u); }
};
template <> struct Bits<double> {
    using U = unsigned long long;
    static __device__ U of(double v) { return (U)__double_as_longlong(v); }
    static __device__ double value(U u) { return __longlong_as_double((long long)u); }
};

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS) mg_classify_kernel(MgLevel<T> L, Grid gc, int mode, T *out,
                                                                    long long nbox) {
    using U = typename Bits<T>::U;
    __shared__ U slo[BLOCK_THREADS / 32], shi[BLOCK_THREADS / 32];
    __shared__ int sany[BLOCK_THREADS / 32];
    const Grid &g = L.g;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    // box extents: 64 x by x bz, by = 8 or 16 (log2 yb)
    const int yb = mode == 0 ? 3 : 4;
    const int bz = mode == 0 ? g.tz : (g.dim == 3 ? 2 * gc.tz : 1);
    const int nb = (64 << yb) * bz;
    for (long long b = blockIdx.x; b < nbox; b += gridDim.x) {
        int i0, j0, k0;
        if (mode == 0) {
            const long long ntx2 = (g.nx + 63) / 64;
            const long long r = b / ntx2;
            i0 = (int)(b - r * ntx2) * 64;
            j0 = (int)(r % g.nty) * TILE_Y;
            k0 = (int)(r / g.nty) * g.tz;
        } else {
            int I0, J0, K0;
            tile_origin(gc, b, I0, J0, K0);
            i0 = 2 * I0;
            j0 = 2 * J0;
            k0 = g.dim == 3 ? 2 * K0 : 0;
        }
        U lo = ~U(0), hi = 0;
        int any = 0;
        for (int q = threadIdx.x; q < nb; q += blockDim.x) {
            const int i = i0 + (q & 63), j = j0 + ((q >> 6) & ((1 << yb) - 1)), k = k0 + (q >> (6 + yb));
            if (i >= g.nx || j >= g.ny || k >= g.nz) continue;
            const long long c = cell_index(g, i, j, k);
            any |= (Bits<T>::of(L.diag[c]) << 1) != 0;  // diag != 0 (either sign of 0)
            auto see = [&](T v) {
                const U u = Bits<T>::of(v);
                lo = u < lo ? u : lo;
                hi = u > hi ? u : hi;
            };
            if (i > 0) see(L.cx[c - 1]);
            if (i + 1 < g.nx) see(L.cx[c]);
            if (j > 0) see(L.cy[c - sy]);
            if (j + 1 < g.ny) see(L.cy[c]);
            if (g.dim == 3) {
                if (k > 0) see(L.cz[c - sz]);
                if (k + 1 < g.nz) see(L.cz[c]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const U l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
            lo = l2 < lo ? l2 : lo;
            hi = h2 > hi ? h2 : hi;
            any |= __shfl_xor_sync(0xffffffffu, any, o);
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) {
            slo[wid] = lo;
            shi[wid] = hi;
            sany[wid] = any;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < BLOCK_THREADS / 32; ++w) {
                lo = slo[w] < lo ? slo[w] : lo;
                hi = shi[w] > hi ? shi[w] : hi;
                any |= sany[w];
            }
            // (lo > hi: no face in the box)
            T cls = T(TILE_MIXED);
            if (!any && lo == 0 && hi == 0) cls = T(TILE_EMPTY);
            else if (lo == hi) cls = Bits<T>::value(lo);
            // a common value that is not a coupling (negative, NaN) is no class
            if (!(cls >= T(0)) && cls != T(TILE_EMPTY)) cls = T(TILE_MIXED);
            out[b] = cls;
        }
        __syncthreads();
    }
}

// One read of a level for both classifications: mg_class_parts_kernel
// reduces each sub-box of 64 x 8 x gz cells (gz divides both box depths:
// the pair tiles' tz and the restriction boxes' 2 tz of the coarser grid)
// to the min and max coupling bit patterns and the any-unknown flag, with
// mg_classify_kernel's reads; mg_class_combine_kernel then forms each pair
// tile's and each restriction box's class from its sub-boxes. min, max and
// or are exact, so the classes equal those of the two-pass form.
template <class T> struct ClassPart {
    typename Bits<T>::U lo, hi;
    int any;
};

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS) mg_class_parts_kernel(MgLevel<T> L, int gz, ClassPart<T> *parts,
                                                                       int sxn, int syn, long long nsub) {
    using U = typename Bits<T>::U;
    __shared__ U slo[BLOCK_THREADS / 32], shi[BLOCK_THREADS / 32];
    __shared__ int sany[BLOCK_THREADS / 32];
    const Grid &g = L.g;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const int nb = 64 * 8 * gz;
    for (long long b = blockIdx.x; b < nsub; b += gridDim.x) {
        const long long r = b / sxn;
        const int i0 = (int)(b - r * sxn) * 64, j0 = (int)(r % syn) * 8, k0 = (int)(r / syn) * gz;
        U lo = ~U(0), hi = 0;
        int any = 0;
        for (int q = threadIdx.x; q < nb; q += blockDim.x) {
            const int i = i0 + (q & 63), j = j0 + ((q >> 6) & 7), k = k0 + (q >> 9);
            if (i >= g.nx || j >= g.ny || k >= g.nz) continue;
            const long long c = cell_index(g, i, j, k);
            any |= (Bits<T>::of(L.diag[c]) << 1) != 0;  // diag != 0 (either sign of 0)
            auto see = [&](T v) {
                const U u = Bits<T>::of(v);
                lo = u < lo ? u : lo;
                hi = u > hi ? u : hi;
            };
            if (i > 0) see(L.cx[c - 1]);
            if (i + 1 < g.nx) see(L.cx[c]);
            if (j > 0) see(L.cy[c - sy]);
            if (j + 1 < g.ny) see(L.cy[c]);
            if (g.dim == 3) {
                if (k > 0) see(L.cz[c - sz]);
                if (k + 1 < g.nz) see(L.cz[c]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const U l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
            lo = l2 < lo ? l2 : lo;
            hi = h2 > hi ? h2 : hi;
            any |= __shfl_xor_sync(0xffffffffu, any, o);
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) {
            slo[wid] = lo;
            shi[wid] = hi;
            sany[wid] = any;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < BLOCK_THREADS / 32; ++w) {
                lo = slo[w] < lo ? slo[w] : lo;
                hi = shi[w] > hi ? shi[w] : hi;
                any |= sany[w];
            }
            parts[b] = ClassPart<T>{lo, hi, any};
        }
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS) mg_class_combine_kernel(Grid g, Grid gc, int gz,
                                                                         const ClassPart<T> *parts, int sxn, int syn,
                                                                         int szn, T *tcp, long long np, T *tcr,
                                                                         long long nr) {
    using U = typename Bits<T>::U;
    const long long ntx2 = (g.nx + 63) / 64;
    const int bz1 = g.dim == 3 ? 2 * gc.tz : 1;
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < np + nr;
         b += (long long)gridDim.x * blockDim.x) {
        int sx, sy0, ny2, sz0, nz2;  // the box's sub-boxes: column sx, rows sy0.., planes sz0..
        if (b < np) {
            const long long r = b / ntx2;
            sx = (int)(b - r * ntx2);
            sy0 = (int)(r % g.nty);
            ny2 = 1;
            sz0 = (int)(r / g.nty) * (g.tz / gz);
            nz2 = g.tz / gz;
        } else {
            int I0, J0, K0;
            tile_origin(gc, b - np, I0, J0, K0);
            sx = (2 * I0) / 64;
            sy0 = (2 * J0) / 8;
            ny2 = 2;
            sz0 = (g.dim == 3 ? 2 * K0 : 0) / gz;
            nz2 = bz1 / gz;
        }
        U lo = ~U(0), hi = 0;
        int any = 0;
        for (int zz = sz0; zz < sz0 + nz2 && zz < szn; ++zz)
            for (int yy = sy0; yy < sy0 + ny2 && yy < syn; ++yy) {
                const ClassPart<T> q = parts[sx + (long long)sxn * (yy + (long long)syn * zz)];
                lo = q.lo < lo ? q.lo : lo;
                hi = q.hi > hi ? q.hi : hi;
                any |= q.any;
            }
        // mg_classify_kernel's rule
        T cls = T(TILE_MIXED);
        if (!any && lo == 0 && hi == 0) cls = T(TILE_EMPTY);
        else if (lo == hi) cls = Bits<T>::value(lo);
        if (!(cls >= T(0)) && cls != T(TILE_EMPTY)) cls = T(TILE_MIXED);
        if (b < np) tcp[b] = cls;
        else tcr[b - np] = cls;
    }
}

template <class T> int nblocks(const Grid &g, int grid_blocks) {
    long long b = g.ntiles < grid_blocks ? g.ntiles : grid_blocks;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

template <class T>
cudaError_t mg_setup(const Grid &g0, Operator<double> A, const MgHierarchy<T> &H, bool level0_done, int grid_blocks,
                     cudaStream_t stream) {
    const MgLevel<T> &L0 = H.levels[0];
    const bool copy = !H.fine_aliases_fp64;
    if (!level0_done)
        mg_fine_setup_kernel<T><<<nblocks<T>(g0, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            g0, A, const_cast<T *>(L0.diag), const_cast<T *>(L0.inv), const_cast<T *>(L0.cx), const_cast<T *>(L0.cy),
            const_cast<T *>(L0.cz), copy, H.lo[0], H.lo[1], H.lo[2], H.lo[3]);
    for (int l = 0; l + 1 < H.nlevels; ++l) {
        const MgLevel<T> &F = H.levels[l], &C = H.levels[l + 1];
        mg_coarsen_kernel<T><<<nblocks<T>(C.g, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            F, C, const_cast<T *>(C.diag), const_cast<T *>(C.inv), const_cast<T *>(C.cx), const_cast<T *>(C.cy),
            const_cast<T *>(C.cz));
    }
    // tile classes of the levels the global-memory kernels run: one read of
    // the level into sub-box partials (in the hierarchy's scratch), then the
    // classes from them; the two-pass form where there is no scratch
    for (int l = 0; l < H.tail && l + 1 < H.nlevels; ++l) {
        const MgLevel<T> &F = H.levels[l], &C = H.levels[l + 1];
        if (!F.tcp || !F.tcr) continue;
        const long long np = (long long)((F.g.nx + 63) / 64) * F.g.nty * F.g.ntz, nr = C.g.ntiles;
        const int bz1 = F.g.dim == 3 ? 2 * C.g.tz : 1;
        int gz = F.g.tz;
        for (int a = bz1; a;) {  // gcd(tz, bz1)
            const int t = gz % a;
            gz = a;
            a = t;
        }
        const int sxn = (F.g.nx + 63) / 64, syn = F.g.nty, szn = (F.g.nz + gz - 1) / gz;
        const long long nsub = (long long)sxn * syn * szn;
        if (H.class_parts && nsub * (long long)sizeof(ClassPart<T>) <= (long long)H.class_parts_bytes) {
            auto *parts = static_cast<ClassPart<T> *>(H.class_parts);
            mg_class_parts_kernel<T><<<(int)std::min<long long>(nsub, grid_blocks), BLOCK_THREADS, 0, stream>>>(
                F, gz, parts, sxn, syn, nsub);
            const long long nt = np + nr;
            mg_class_combine_kernel<T><<<(int)std::min<long long>((nt + BLOCK_THREADS - 1) / BLOCK_THREADS, grid_blocks),
                                         BLOCK_THREADS, 0, stream>>>(F.g, C.g, gz, parts, sxn, syn, szn, F.tcp, np,
                                                                     F.tcr, nr);
            continue;
        }
        mg_classify_kernel<T><<<(int)std::min<long long>(np, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            F, C.g, 0, F.tcp, np);
        mg_classify_kernel<T><<<(int)std::min<long long>(nr, grid_blocks), BLOCK_THREADS, 0, stream>>>(
            F, C.g, 1, F.tcr, nr);
    }
    return cudaGetLastError();
}

template cudaError_t mg_setup<double>(const Grid &, Operator<double>, const MgHierarchy<double> &, bool, int,
                                      cudaStream_t);
template cudaError_t mg_setup<float>(const Grid &, Operator<double>, const MgHierarchy<float> &, bool, int,
                                     cudaStream_t);

}  // namespace gbp
