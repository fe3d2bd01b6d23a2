// batch_kernels.cu -- the MGPCG iteration over a work list of (level, tile)
// items spanning every scene of a batch (see gbp_batch.h).
//
// The arithmetic is that of the single-level kernels it generalises: red
// (i+j+k even) / black Gauss-Seidel on pair tiles (each thread owns the two
// x-adjacent cells of a row, one of each colour), Galerkin restriction by
// summing the 8 children's residuals, post-smoothing black (reading the red
// neighbours with their parent's correction added) then red, a shared-memory
// tail per scene for the small levels, and CG with FP64 dot products.
// Algorithmic DRAM bytes per fine cell (s = sizeof(T)): presmooth 6 s,
// sweep 7 s, restrict 6 s + s/8, post_black 7 s + s/8, red_dot 7 s,
// direction 3 s, spmv 6 s, update 6 s, refine_accumulate 12 B (d f32 read,
// x64 read+write), refine_residual 8+32+8+8+4 = 60 B (x64, operator, b, r64
// write, r_f write).
#include "gbp_batch.h"

namespace gbp {
namespace {

constexpr int SITE_DOT = 4, SITE_SPMV = 5, SITE_UPDATE = 6, SITE_REFINE = 7;

__device__ __forceinline__ bool gated(const Scalars *sc, int gate) {
    const volatile Scalars *v = sc;
    if (v->done) return true;
    if (gate == 1) return v->inner_done != 0;
    if (gate == 2) return v->inner_done == 0;
    return false;
}

// Ticket of one item of a scene; true in every thread of the block whose
// item took the scene's last ticket (all threads must call it).
__device__ __forceinline__ bool item_last(unsigned int *counter, int count) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(counter, 1u) == (unsigned)(count - 1);
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

__device__ __forceinline__ double sum_range(const double *part, int begin, int count, double *sh) {
    double v = 0.0;
    for (int t = threadIdx.x; t < count; t += blockDim.x) v += __ldcg(part + begin + t);
    return block_sum(v, sh);
}

__device__ __forceinline__ double max_range(const double *part, int begin, int count, double *sh) {
    double v = 0.0;
    for (int t = threadIdx.x; t < count; t += blockDim.x) v = fmax(v, __ldcg(part + begin + t));
    return block_max(v, sh);
}

// cells (i, i+1) of the pair tile t: f(i, j, k, c, second)
template <class F> __device__ __forceinline__ void pair_tile1(const Grid &g, long long t, F f) {
    const int px = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int ntx2 = (g.nx + 63) >> 6;
    const long long tx = t % ntx2, r = t / ntx2;
    const int i = (int)tx * 64 + 2 * px;
    const int j = (int)(r % g.nty) * TILE_Y + ty;
    const int k0 = (int)(r / g.nty) * g.tz;
    if (i >= g.nx || j >= g.ny) return;
    const int kend = min(k0 + g.tz, g.nz);
    const bool second = i + 1 < g.nx;
    for (int k = k0; k < kend; ++k) f(i, j, k, cell_index(g, i, j, k), second);
}

// cells of the cell tile t: f(i, j, k, c)
template <class F> __device__ __forceinline__ void cell_tile1(const Grid &g, long long t, F f) {
    int i0, j0, k0;
    tile_origin(g, t, i0, j0, k0);
    const int i = i0 + (threadIdx.x & (TILE_X - 1)), j = j0 + threadIdx.x / TILE_X;
    if (i >= g.nx || j >= g.ny) return;
    const int kend = min(k0 + g.tz, g.nz);
    for (int k = k0; k < kend; ++k) f(i, j, k, cell_index(g, i, j, k));
}

// every tile of an item
template <class F> __device__ __forceinline__ void pair_tile(const Grid &g, const BItem &it, F f) {
    for (int t = 0; t < it.ntiles; ++t) pair_tile1(g, (long long)it.tile + t, f);
}
template <class F> __device__ __forceinline__ void cell_tile(const Grid &g, const BItem &it, F f) {
    for (int t = 0; t < it.ntiles; ++t) cell_tile1(g, (long long)it.tile + t, f);
}

template <class T, class X>
__device__ __forceinline__ T nsum(const BLevel<T> &L, int i, int j, int k, long long c, X xat) {
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


// The level and scene of the current item, held in shared memory and
// reloaded only when the item's level changes (each work list holds one
// level per scene, so once per scene per block). Kernels then read the
// descriptors from shared memory instead of chasing item -> level -> scene
// pointers in global memory for every item.
template <class T> struct ItemCtx {
    BLevel<T> L;
    BScene<T> S;
    int skip;
    double alpha, beta;
    int overwrite;
};

template <class T>
__device__ __forceinline__ void refresh(ItemCtx<T> &c, int &cur_ref, const BItem &it, const BLevel<T> *levels,
                                        const BScene<T> *scenes, int gate) {
    if (it.ref == cur_ref) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        c.L = levels[it.ref];
        c.S = scenes[c.L.scene];
        c.skip = gate < 0 ? 0 : gated(c.S.sc, gate);
        c.alpha = c.S.sc->alpha;
        c.beta = c.S.sc->beta;
        c.overwrite = c.S.sc->first_update;
    }
    __syncthreads();
    cur_ref = it.ref;
}

// Reduction over a work list with one partial per (block, scene): a block
// walks its items (sorted by scene), accumulates a scene's cells in
// `acc`, and flushes when the scene changes. The flush of block b for a
// scene whose items occupy list positions [begin, begin+count) goes to slot
// (b - begin) mod gridDim.x of that range; min(count, gridDim.x) blocks
// flush per scene, and the one taking the scene's last ticket combines the
// slots in slot order (deterministic for a given batch and grid).
template <class T, class Acc, class Body, class Finish>
__device__ __forceinline__ void reduce_items(const BSeg *__restrict__ segs, int nseg, int n, double *part,
                                             const BLevel<T> *levels, const BScene<T> *scenes, int gate,
                                             ItemCtx<T> &ctx, Body body, Finish finish) {
    __shared__ double sh[BLOCK_THREADS / 32];
    int cur = -1;
    BItem first{};
    Acc acc;
    acc.reset();
    auto flush = [&]() {
        const double v = acc.block(sh);
        const int B = gridDim.x;
        const int slot = (int)((((long long)blockIdx.x - first.begin) % B + B) % B);
        if (threadIdx.x == 0) part[first.begin + slot] = v;
        finish(first, min(first.count, B));
    };
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        if (it.ref != cur) {
            // one level per scene in a list: a new level is a new scene
            if (cur >= 0 && !ctx.skip) flush();
            refresh(ctx, cur, it, levels, scenes, gate);
            first = it;
            acc.reset();
        }
        if (!ctx.skip) body(it, acc);
    }
    if (cur >= 0 && !ctx.skip) flush();
}

struct SumAcc {
    double v;
    __device__ void reset() { v = 0.0; }
    __device__ double block(double *sh) { return block_sum(v, sh); }
};
struct MaxAcc {
    double v;
    __device__ void reset() { v = 0.0; }
    __device__ double block(double *sh) { return block_max(v, sh); }
};

// ---- smoothing and transfers on the global-memory levels --------------------------

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) presmooth_kernel(const BLevel<T> *__restrict__ levels,
                                                                     const BSeg *__restrict__ segs, int nseg, int n,
                                                                     const BScene<T> *__restrict__ scenes, int gate) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, gate);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        auto red_value = [&](long long m, int, int, int) { return __ldg(L.b + m) * __ldg(L.inv + m); };
        pair_tile(L.g, it, [&](int i, int j, int k, long long c, bool second) {
            const bool a_red = ((i + j + k) & 1) == 0;
            for (int h = 0; h < (second ? 2 : 1); ++h) {
                const long long cc = c + h;
                T xv;
                if ((h == 0) == a_red) xv = __ldg(L.b + cc) * __ldg(L.inv + cc);
                else xv = (__ldg(L.b + cc) + nsum(L, i + h, j, k, cc, red_value)) * __ldg(L.inv + cc);
                L.x[cc] = xv;
            }
        });
    }
}

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) sweep_kernel(const BLevel<T> *__restrict__ levels,
                                                                 const BSeg *__restrict__ segs, int nseg, int n,
                                                                 const BScene<T> *__restrict__ scenes, int gate,
                                                                 int color) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, gate);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        auto xval = [&](long long m, int, int, int) { return __ldg(L.x + m); };
        pair_tile(L.g, it, [&](int i, int j, int k, long long c, bool second) {
            const int h = ((i + j + k) & 1) == color ? 0 : 1;
            if (h == 1 && !second) return;
            const long long cc = c + h;
            L.x[cc] = (__ldg(L.b + cc) + nsum(L, i + h, j, k, cc, xval)) * __ldg(L.inv + cc);
        });
    }
}

// items are cell tiles of the coarse grid gc
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) restrict_kernel(const BLevel<T> *__restrict__ levels,
                                                                    const BSeg *__restrict__ segs, int nseg, int n,
                                                                    const BScene<T> *__restrict__ scenes, int gate) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, gate);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        const Grid &fg = L.g;
        auto xval = [&](long long m, int, int, int) { return __ldg(L.x + m); };
        cell_tile(L.gc, it, [&](int I, int J, int K, long long cc) {
            T sum = T(0);
            const int kmax = fg.dim == 3 ? 2 : 1;
            for (int c2 = 0; c2 < kmax; ++c2)
                for (int b2 = 0; b2 < 2; ++b2)
                    for (int a2 = 0; a2 < 2; ++a2) {
                        const int i = 2 * I + a2, j = 2 * J + b2, k = 2 * K + c2;
                        if (i >= fg.nx || j >= fg.ny || k >= fg.nz) continue;
                        const long long f = cell_index(fg, i, j, k);
                        const T s = nsum(L, i, j, k, f, xval);
                        sum += __ldg(L.b + f) - (__ldg(L.diag + f) * __ldg(L.x + f) - s);
                    }
            L.bc[cc] = sum;
        });
    }
}

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) post_black_kernel(const BLevel<T> *__restrict__ levels,
                                                                      const BSeg *__restrict__ segs, int nseg, int n,
                                                                      const BScene<T> *__restrict__ scenes, int gate,
                                                                      T alpha) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, gate);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        const Grid &cg = L.gc;
        const bool d3 = L.g.dim == 3;
        auto corrected = [&](long long m, int ni, int nj, int nk) {
            return __ldg(L.x + m) + alpha * __ldg(L.xc + cell_index(cg, ni >> 1, nj >> 1, d3 ? (nk >> 1) : 0));
        };
        pair_tile(L.g, it, [&](int i, int j, int k, long long c, bool second) {
            const int h = ((i + j + k) & 1) == 1 ? 0 : 1;
            if (h == 1 && !second) return;
            const long long cc = c + h;
            L.x[cc] = (__ldg(L.b + cc) + nsum(L, i + h, j, k, cc, corrected)) * __ldg(L.inv + cc);
        });
    }
}

// Last red pass of the fine level, with rho' = z . r (z = x, r = b there)
// per scene; the scene's last flush sets beta (0 for a new direction).
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) red_dot_kernel(const BLevel<T> *__restrict__ levels,
                                                                   const BSeg *__restrict__ segs, int nseg, int n,
                                                                   const BScene<T> *__restrict__ scenes, int gate,
                                                                   double *part, const int *__restrict__ scene_of) {
    __shared__ double shf[BLOCK_THREADS / 32];
    __shared__ ItemCtx<T> ctx;
    reduce_items<T, SumAcc>(
        segs, nseg, n, part, levels, scenes, gate, ctx,
        [&](const BItem &it, SumAcc &acc) {
            const BLevel<T> &L = ctx.L;
            auto xval = [&](long long m, int, int, int) { return __ldg(L.x + m); };
            pair_tile(L.g, it, [&](int i, int j, int k, long long c, bool second) {
                const int hr = ((i + j + k) & 1) == 0 ? 0 : 1;
                for (int h = 0; h < (second ? 2 : 1); ++h) {
                    const long long cc = c + h;
                    const T bv = __ldg(L.b + cc);
                    T xv;
                    if (h == hr) {
                        xv = (bv + nsum(L, i + h, j, k, cc, xval)) * __ldg(L.inv + cc);
                        L.x[cc] = xv;
                    } else {
                        xv = L.x[cc];
                    }
                    acc.v = fma((double)xv, (double)bv, acc.v);
                }
            });
        },
        [&](const BItem &it, int flushes) {
            Scalars *sc = ctx.S.sc;
            if (item_last(&sc->counter[SITE_DOT], flushes)) {
                const double rho_new = sum_range(part, it.begin, flushes, shf);
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
                    sc->counter[SITE_DOT] = 0;
                }
            }
        });
}

// ---- shared-memory tail, one block per scene -----------------------------------

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

// The V-cycle of the levels lv[0..nt) from shared memory: b of lv[0] in,
// x of lv[0] out, same smoother, transfers and coarsest solve (FP64
// symmetric sweep pairs) as the global levels.
template <class T>
__global__ void __launch_bounds__(MG_TAIL_THREADS) tail_kernel(const BTail<T> *__restrict__ tails,
                                                               const BScene<T> *__restrict__ scenes, int gate,
                                                               MgSettings ms) {
    const int s = blockIdx.x;
    const BTail<T> &A = tails[s];
    if (A.nt <= 0) return;
    if (gated(scenes[s].sc, gate)) return;
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
    const T alpha = T(ms.alpha);
    for (int l = 0; l + 1 < A.nt; ++l) {
        const SLevel<T> &L = S[l];
        s_for_each(L, [&](int i, int j, int k, int c) {
            const T inv = L.inv[c];
            if (((i + j + k) & 1) == 0) {
                L.x[c] = L.b[c] * inv;
            } else {
                L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int m) { return L.b[m] * L.inv[m]; })) * inv;
            }
        });
        for (int sw = 1; sw < ms.smooth; ++sw)
            for (int color = 0; color < 2; ++color)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != color) return;
                    L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int m) { return L.x[m]; })) * L.inv[c];
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
                        sum += L.b[f] - (L.diag[f] * L.x[f] - snb(L, i, j, k, f, [&](int m) { return L.x[m]; }));
                    }
            C.b[cc] = sum;
        });
    }
    {
        const SLevel<T> &L = S[A.nt - 1];
        for (int c = threadIdx.x; c < L.n; c += blockDim.x) xc[c] = 0.0;
        __syncthreads();
        for (int p = 0; p < ms.coarsest_pairs; ++p) {
            const int order[4] = {0, 1, 1, 0};
            for (int q = 0; q < 4; ++q)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != order[q]) return;
                    const int sy = L.nx, sz = L.nx * L.ny;
                    double acc = 0.0;
                    if (i > 0) acc += (double)L.cx[c - 1] * xc[c - 1];
                    if (i + 1 < L.nx) acc += (double)L.cx[c] * xc[c + 1];
                    if (j > 0) acc += (double)L.cy[c - sy] * xc[c - sy];
                    if (j + 1 < L.ny) acc += (double)L.cy[c] * xc[c + sy];
                    if (L.dim == 3) {
                        if (k > 0) acc += (double)L.cz[c - sz] * xc[c - sz];
                        if (k + 1 < L.nz) acc += (double)L.cz[c] * xc[c + sz];
                    }
                    xc[c] = ((double)L.b[c] + acc) * (double)L.inv[c];
                });
        }
        for (int c = threadIdx.x; c < L.n; c += blockDim.x) L.x[c] = T(xc[c]);
        __syncthreads();
    }
    for (int l = A.nt - 2; l >= 0; --l) {
        const SLevel<T> &L = S[l];
        const SLevel<T> &C = S[l + 1];
        s_for_each(L, [&](int i, int j, int k, int c) {
            if (((i + j + k) & 1) != 1) return;
            L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int m) {
                         const int mi = m % L.nx, t = m / L.nx, mj = t % L.ny, mk = t / L.ny;
                         return L.x[m] +
                                alpha * C.x[(mi >> 1) + C.nx * ((mj >> 1) + C.ny * (L.dim == 3 ? (mk >> 1) : 0))];
                     })) * L.inv[c];
        });
        for (int sw = 1; sw < ms.smooth; ++sw)
            for (int color = 0; color < 2; ++color)
                s_for_each(L, [&](int i, int j, int k, int c) {
                    if (((i + j + k) & 1) != color) return;
                    L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int m) { return L.x[m]; })) * L.inv[c];
                });
        s_for_each(L, [&](int i, int j, int k, int c) {
            if (((i + j + k) & 1) != 0) return;
            L.x[c] = (L.b[c] + snb(L, i, j, k, c, [&](int m) { return L.x[m]; })) * L.inv[c];
        });
    }
    const SLevel<T> &L0 = S[0];
    for (int c = threadIdx.x; c < L0.n; c += blockDim.x) A.lv[0].x[c] = L0.x[c];
}

// ---- CG on the fine level -----------------------------------------------------------

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) direction_kernel(const BLevel<T> *__restrict__ levels,
                                                                     const BSeg *__restrict__ segs, int nseg, int n,
                                                                     const BScene<T> *__restrict__ scenes, int gate) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, gate);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        const BScene<T> &S = ctx.S;
        const T beta = T(ctx.beta);
        if (beta == T(0)) cell_tile(L.g, it, [&](int, int, int, long long c) { S.p[c] = S.z[c]; });
        else cell_tile(L.g, it, [&](int, int, int, long long c) { S.p[c] = S.z[c] + beta * S.p[c]; });
    }
}

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) spmv_kernel(const BLevel<T> *__restrict__ levels,
                                                                const BSeg *__restrict__ segs, int nseg, int n,
                                                                const BScene<T> *__restrict__ scenes, int gate,
                                                                double *part, const int *__restrict__ scene_of) {
    __shared__ double shf[BLOCK_THREADS / 32];
    __shared__ ItemCtx<T> ctx;
    reduce_items<T, SumAcc>(
        segs, nseg, n, part, levels, scenes, gate, ctx,
        [&](const BItem &it, SumAcc &acc) {
            const BLevel<T> &L = ctx.L;
            const BScene<T> &S = ctx.S;
            auto pval = [&](long long m, int, int, int) { return __ldg(S.p + m); };
            cell_tile(L.g, it, [&](int i, int j, int k, long long c) {
                const T pc = __ldg(S.p + c);
                const T qv = __ldg(L.diag + c) * pc - nsum(L, i, j, k, c, pval);
                S.q[c] = qv;
                acc.v = fma((double)pc, (double)qv, acc.v);
            });
        },
        [&](const BItem &it, int flushes) {
            Scalars *sc = ctx.S.sc;
            if (item_last(&sc->counter[SITE_SPMV], flushes)) {
                const double pq = sum_range(part, it.begin, flushes, shf);
                if (threadIdx.x == 0) {
                    sc->pap = pq;
                    sc->alpha = sc->rho / pq;
                    sc->counter[SITE_SPMV] = 0;
                }
            }
        });
}

// x += alpha p (x = alpha p on the first update of a solve), r -= alpha q,
// |r|_inf. mode 0: the solve's stopping rule; mode 1: inner solve.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) update_kernel(const BLevel<T> *__restrict__ levels,
                                                                  const BSeg *__restrict__ segs, int nseg, int n,
                                                                  const BScene<T> *__restrict__ scenes, int gate,
                                                                  double *part, int mode, BatchCounters *cnt,
                                                                  const int *__restrict__ scene_of) {
    __shared__ double shf[BLOCK_THREADS / 32];
    __shared__ ItemCtx<T> ctx;
    reduce_items<T, MaxAcc>(
        segs, nseg, n, part, levels, scenes, gate, ctx,
        [&](const BItem &it, MaxAcc &acc) {
            const BLevel<T> &L = ctx.L;
            const BScene<T> &S = ctx.S;
            const T alpha = T(ctx.alpha);
            const bool overwrite = ctx.overwrite != 0;
            cell_tile(L.g, it, [&](int, int, int, long long c) {
                const T pc = S.p[c];
                S.x[c] = overwrite ? alpha * pc : S.x[c] + alpha * pc;
                const T rv = S.r[c] - alpha * S.q[c];
                S.r[c] = rv;
                acc.v = fmax(acc.v, fabs((double)rv));
            });
        },
        [&](const BItem &it, int flushes) {
            Scalars *sc = ctx.S.sc;
            if (item_last(&sc->counter[SITE_UPDATE], flushes)) {
                const double res = max_range(part, it.begin, flushes, shf);
                if (threadIdx.x == 0) {
                    sc->first_update = 0;
                    sc->iter += 1;
                    const bool bad = res != res || sc->alpha != sc->alpha;
                    int finished = 0;
                    if (mode == 0) {
                        sc->res = res;
                        if (bad) {
                            sc->status = 3;
                            finished = 1;
                        } else if (res <= sc->tol) {
                            sc->status = 1;
                            finished = 1;
                        } else if (sc->iter >= sc->max_iter) {
                            sc->status = 2;
                            finished = 1;
                        }
                    } else {
                        sc->inner_iter += 1;
                        if (bad) {
                            sc->status = 3;
                            finished = 1;
                        } else if (res <= sc->inner_tol || sc->inner_iter >= sc->inner_max ||
                                   sc->iter >= sc->max_iter) {
                            sc->inner_done = 1;
                        }
                    }
                    if (finished) {
                        sc->done = 1;
                        atomicSub(&cnt->remaining, 1);
                    }
                    sc->counter[SITE_UPDATE] = 0;
                }
            }
        });
}

// ---- mixed precision: FP64 refinement -------------------------------------------------

template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) refine_accumulate_kernel(const BLevel<T> *__restrict__ levels,
                                                                             const BSeg *__restrict__ segs, int nseg, int n,
                                                                             const BScene<T> *__restrict__ scenes) {
    __shared__ ItemCtx<T> ctx;
    int cur = -1;
    int sgc = 0;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const BItem it = item_at(segs, nseg, w, sgc);
        refresh(ctx, cur, it, levels, scenes, 2);
        if (ctx.skip) continue;
        const BLevel<T> &L = ctx.L;
        const BScene<T> &S = ctx.S;
        cell_tile(L.g, it, [&](int, int, int, long long c) { S.x64[c] += (double)S.x[c]; });
    }
}

// r64 = b - A64 (prev + x64) (x64 absent: initial), r_T = r64, |r64|_inf;
// the scene's last flush applies the stopping rule and opens the next inner
// solve. initial: sets the threshold, zeroes x64.
template <class T>
__global__ void __launch_bounds__(BLOCK_THREADS, 6) refine_residual_kernel(
    const BLevel<T> *__restrict__ levels, const BSeg *__restrict__ segs, int nseg, int n,
    const BScene<T> *__restrict__ scenes, double *part, int initial, double residual, int max_iter,
    double inner_rel, int inner_max, BatchCounters *cnt, const int *__restrict__ scene_of) {
    __shared__ double shf[BLOCK_THREADS / 32];
    __shared__ ItemCtx<T> ctx;
    reduce_items<T, MaxAcc>(
        segs, nseg, n, part, levels, scenes, initial ? -1 : 2, ctx,
        [&](const BItem &it, MaxAcc &acc) {
            const BLevel<T> &L = ctx.L;
            const BScene<T> &S = ctx.S;
            const Grid &g = L.g;
            const long long sy = g.nx, sz = (long long)g.nx * g.ny;
            const Operator<double> &A = S.A;
            auto X = [&](long long c) {
                double v = initial ? 0.0 : S.x64[c];
                if (S.prev) v += S.prev[c];
                return v;
            };
            cell_tile(g, it, [&](int i, int j, int k, long long c) {
                double a = A.diag[c] * X(c);
                if (i > 0) a -= A.cx[c - 1] * X(c - 1);
                if (i + 1 < g.nx) a -= A.cx[c] * X(c + 1);
                if (j > 0) a -= A.cy[c - sy] * X(c - sy);
                if (j + 1 < g.ny) a -= A.cy[c] * X(c + sy);
                if (g.dim == 3) {
                    if (k > 0) a -= A.cz[c - sz] * X(c - sz);
                    if (k + 1 < g.nz) a -= A.cz[c] * X(c + sz);
                }
                const double rv = S.b[c] - a;
                S.r64[c] = rv;
                S.r[c] = T(rv);
                acc.v = fmax(acc.v, fabs(rv));
            });
            if (initial) cell_tile(g, it, [&](int, int, int, long long c) { S.x64[c] = 0.0; });
        },
        [&](const BItem &it, int flushes) {
            Scalars *sc = ctx.S.sc;
            if (item_last(&sc->counter[SITE_REFINE], flushes)) {
                const double res = max_range(part, it.begin, flushes, shf);
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
                    int finished = 1;
                    if (res != res) {
                        sc->status = 3;
                    } else if (res <= sc->tol) {
                        sc->status = 1;
                    } else if (sc->iter >= sc->max_iter) {
                        sc->status = 2;
                    } else {
                        finished = 0;
                        sc->inner_done = 0;
                        sc->inner_iter = 0;
                        sc->first = 1;
                        sc->first_update = 1;
                        sc->inner_res0 = res;
                        sc->inner_tol = inner_rel * res;
                    }
                    if (finished) {
                        sc->done = 1;
                        atomicSub(&cnt->remaining, 1);
                    }
                    sc->counter[SITE_REFINE] = 0;
                }
            }
        });
}

}  // namespace

template <class T>
cudaError_t b_presmooth(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                        const BScene<T> *scenes) {
    presmooth_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_sweep(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                    int color) {
    sweep_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate, color);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_restrict(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                       const BScene<T> *scenes) {
    restrict_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_post_black(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                         const BScene<T> *scenes, T alpha) {
    post_black_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate, alpha);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_red_dot(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                      double *part) {
    red_dot_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate, part, L.scene_of);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_tail(const BLaunch &L, const BTail<T> *tails, int nscenes, const BScene<T> *scenes, MgSettings ms,
                   size_t smem) {
    tail_kernel<T><<<nscenes, MG_TAIL_THREADS, smem, L.stream>>>(tails, scenes, L.gate, ms);
    return cudaGetLastError();
}
template <class T> cudaError_t b_tail_enable(size_t bytes) {
    return cudaFuncSetAttribute(tail_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
template <class T>
cudaError_t b_direction(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                        const BScene<T> *scenes) {
    direction_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_spmv(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                   double *part) {
    spmv_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate, part, L.scene_of);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_update(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                     double *part, int mode, BatchCounters *cnt) {
    update_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes, L.gate, part, mode, cnt,
                                                               L.scene_of);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_refine_accumulate(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                                const BScene<T> *scenes) {
    refine_accumulate_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(levels, segs, nseg, n, scenes);
    return cudaGetLastError();
}
template <class T>
cudaError_t b_refine_residual(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                              const BScene<T> *scenes, double *part, int initial, double residual, int max_iter,
                              double inner_rel, int inner_max, BatchCounters *cnt) {
    refine_residual_kernel<T><<<L.blocks, BLOCK_THREADS, 0, L.stream>>>(
        levels, segs, nseg, n, scenes, part, initial, residual, max_iter, inner_rel, inner_max, cnt, L.scene_of);
    return cudaGetLastError();
}

#define GBP_BATCH_INSTANTIATE(T)                                                                                   \
    template cudaError_t b_presmooth<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *); \
    template cudaError_t b_sweep<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *, int); \
    template cudaError_t b_restrict<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *);  \
    template cudaError_t b_post_black<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *, \
                                         T);                                                                       \
    template cudaError_t b_red_dot<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *,    \
                                      double *);                                                                   \
    template cudaError_t b_tail<T>(const BLaunch &, const BTail<T> *, int, const BScene<T> *, MgSettings, size_t);  \
    template cudaError_t b_tail_enable<T>(size_t);                                                                 \
    template cudaError_t b_direction<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *); \
    template cudaError_t b_spmv<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *,       \
                                   double *);                                                                      \
    template cudaError_t b_update<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int, const BScene<T> *,     \
                                     double *, int, BatchCounters *);                                              \
    template cudaError_t b_refine_accumulate<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int,           \
                                                const BScene<T> *);                                                \
    template cudaError_t b_refine_residual<T>(const BLaunch &, const BLevel<T> *, const BSeg *, int, int,             \
                                              const BScene<T> *, double *, int, double, int, double, int,          \
                                              BatchCounters *);

GBP_BATCH_INSTANTIATE(double)
GBP_BATCH_INSTANTIATE(float)

}  // namespace gbp
