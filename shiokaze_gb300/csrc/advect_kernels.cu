// advect_kernels.cu -- MacCormack / semi-Lagrangian advection of a cell
// scalar and of the MAC velocity on dense device grids (see advect.h and
// advect_core.cuh). Compiled with --fmad=false: every result equals the
// reference's scalar C++ bit for bit.
//
// A MacCormack step is four launches: scalar forward (forward value and the
// limiter's record per cell), scalar backward (+ the limited correction,
// written in place), velocity forward, velocity backward (in place). The
// backward kernels read the step's input only at their own face or cell, so
// writing the result over it is safe; the forward kernels read neighbours
// and write scratch. One semi-Lagrangian pass is the forward kernel and a
// copy back.
//
// One thread per face (blockIdx.y = component) or cell. Algorithmic DRAM
// bytes per face of a MacCormack velocity step: forward reads u (4; the
// neighbours come from cache) and writes the forward value and the limiter
// record (4 + 8), backward reads them and the input (16) and writes the
// result (4): 32 B. Cell scalar: the same 32 B plus the fluid level set read
// twice (8) and, on the cell passes, the 3 velocity components' two faces
// (counted once, 12). The arithmetic is the reference's: trilinear weights
// and sums in FP64 on every trace (three per face, two per cell), which on
// this GPU's FP64 pipe, not DRAM, bounds the kernels.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "advect.h"
#include "advect_core.cuh"

namespace gbp {
namespace {

using gba::Dims;
using gba::StepArgs;

constexpr int ADV_THREADS = 256;

// one thread per face, blockIdx.y = component
template <bool MAC>
__global__ void __launch_bounds__(ADV_THREADS) adv_face_forward(StepArgs a) {
    gba::face_forward<MAC>(a, (int)blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(ADV_THREADS) adv_face_backward(StepArgs a) {
    gba::face_backward(a, (int)blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

// one thread per cell
template <bool MAC>
__global__ void __launch_bounds__(ADV_THREADS) adv_cell_forward(StepArgs a) {
    gba::cell_forward<MAC>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(ADV_THREADS) adv_cell_backward(StepArgs a) {
    gba::cell_backward(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// the 2D passes: one thread per face (blockIdx.y = component) or cell
template <bool MAC>
__global__ void __launch_bounds__(ADV_THREADS) adv2_face_forward(StepArgs a) {
    gba::face_forward2<MAC>(a, (int)blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(ADV_THREADS) adv2_face_backward(StepArgs a) {
    gba::face_backward2(a, (int)blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

template <bool MAC>
__global__ void __launch_bounds__(ADV_THREADS) adv2_cell_forward(StepArgs a) {
    gba::cell_forward2<MAC>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(ADV_THREADS) adv2_cell_backward(StepArgs a) {
    gba::cell_backward2(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// levelset_exist (include/shiokaze/array/array_utility3.h:112-122): any
// negative value of the solid sets the flag
__global__ void __launch_bounds__(ADV_THREADS) cst_any_negative(const float *__restrict__ solid, long long n,
                                                               int *flag) {
    bool neg = false;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        neg |= solid[i] < 0.0f;
    if (__syncthreads_or(neg) && threadIdx.x == 0) *flag = 1;
}

// one thread per face, blockIdx.y = component
__global__ void __launch_bounds__(ADV_THREADS) cst_face(gba::ConstrainArgs a) {
    gba::constrain_face(a, (int)blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

Dims make_dims(int nx, int ny, int nz, double dx, int trim_narrowband) {
    Dims g{};
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.dx = dx;
    int e = 0;
    const double m = std::frexp(dx, &e);
    const double inv = 1.0 / dx;
    g.pow2 = (m == 0.5 && std::isfinite(inv) && (double)(float)inv == inv) ? 1 : 0;
    g.inv_dx = inv;
    g.inv_dx_f = (float)inv;
    g.limit = -dx * (double)trim_narrowband;
    return g;
}

unsigned blocks_for(long long n) { return (unsigned)((n + ADV_THREADS - 1) / ADV_THREADS); }

}  // namespace

cudaError_t advect_reserve(AdvectWork &w, long long faces, long long cells) {
    if (faces > w.face_cap) {
        cudaFree(w.v0);
        cudaFree(w.vmm);
        w.v0 = nullptr;
        w.vmm = nullptr;
        w.face_cap = 0;
        cudaError_t e = cudaMalloc(&w.v0, sizeof(float) * (size_t)faces);
        if (e == cudaSuccess) e = cudaMalloc(&w.vmm, sizeof(gba::MinMax) * (size_t)faces);
        if (e != cudaSuccess) return e;
        w.face_cap = faces;
    }
    if (cells > w.cell_cap) {
        cudaFree(w.q0);
        cudaFree(w.qmm);
        w.q0 = nullptr;
        w.qmm = nullptr;
        w.cell_cap = 0;
        cudaError_t e = cudaMalloc(&w.q0, sizeof(float) * (size_t)cells);
        if (e == cudaSuccess) e = cudaMalloc(&w.qmm, sizeof(gba::MinMax) * (size_t)cells);
        if (e != cudaSuccess) return e;
        w.cell_cap = cells;
    }
    return cudaSuccess;
}

void advect_release(AdvectWork &w) {
    cudaFree(w.ext_a);
    cudaFree(w.ext_m);
    cudaFree(w.ext_count);
    cudaFree(w.flag);
    cudaFree(w.v0);
    cudaFree(w.vmm);
    cudaFree(w.q0);
    cudaFree(w.qmm);
    w = AdvectWork{};
}

cudaError_t advect_run(AdvectWork &w, const AdvectArgs &a, cudaStream_t st, long long *launches) {
    const long long cells = (long long)a.nx * a.ny * a.nz;
    const long long nf0 = (long long)(a.nx + 1) * a.ny * a.nz, nf1 = (long long)a.nx * (a.ny + 1) * a.nz,
                    nf2 = (long long)a.nx * a.ny * (a.nz + 1);
    long long nfmax = nf0 > nf1 ? nf0 : nf1;
    if (nf2 > nfmax) nfmax = nf2;
    cudaError_t e = advect_reserve(w, a.velocity ? nf0 + nf1 + nf2 : 0, a.q ? cells : 0);
    if (e != cudaSuccess) return e;
    StepArgs s{};
    s.g = make_dims(a.nx, a.ny, a.nz, a.dx, a.trim_narrowband);
    s.dt = a.dt;
    s.u = a.u;
    s.v = a.v;
    s.w = a.w;
    s.fluid = a.fluid;
    s.q = a.q;
    s.mask = a.q_mask;
    s.bg = a.q_bg;
    s.v0 = w.v0;
    s.vmm = w.vmm;
    s.off1 = nf0;
    s.off2 = nf0 + nf1;
    s.q0 = w.q0;
    s.qmm = w.qmm;
    if (a.q) {
        if (a.maccormack) {
            adv_cell_forward<true><<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            adv_cell_backward<<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            *launches += 2;
        } else {
            adv_cell_forward<false><<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            *launches += 1;
            e = cudaMemcpyAsync(a.q, w.q0, sizeof(float) * (size_t)cells, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
    }
    if (!a.velocity) return cudaGetLastError();
    const dim3 fgrid(blocks_for(nfmax), 3);
    if (a.maccormack) {
        adv_face_forward<true><<<fgrid, ADV_THREADS, 0, st>>>(s);
        adv_face_backward<<<fgrid, ADV_THREADS, 0, st>>>(s);
        *launches += 2;
    } else {
        adv_face_forward<false><<<fgrid, ADV_THREADS, 0, st>>>(s);
        *launches += 1;
        float *dst[3] = {a.u, a.v, a.w};
        const long long n[3] = {nf0, nf1, nf2}, o[3] = {0, s.off1, s.off2};
        for (int d = 0; d < 3; ++d) {
            e = cudaMemcpyAsync(dst[d], w.v0 + o[d], sizeof(float) * (size_t)n[d], cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaGetLastError();
}

cudaError_t advect_run2(AdvectWork &w, const AdvectArgs &a, cudaStream_t st, long long *launches) {
    const long long cells = (long long)a.nx * a.ny;
    const long long nf0 = (long long)(a.nx + 1) * a.ny, nf1 = (long long)a.nx * (a.ny + 1);
    const long long nfmax = nf0 > nf1 ? nf0 : nf1;
    cudaError_t e = advect_reserve(w, a.velocity ? nf0 + nf1 : 0, a.q ? cells : 0);
    if (e != cudaSuccess) return e;
    StepArgs s{};
    s.g = make_dims(a.nx, a.ny, 1, a.dx, a.trim_narrowband);
    s.dt = a.dt;
    s.u = a.u;
    s.v = a.v;
    s.w = nullptr;
    s.fluid = a.fluid;
    s.q = a.q;
    s.mask = a.q_mask;
    s.bg = a.q_bg;
    s.v0 = w.v0;
    s.vmm = w.vmm;
    s.off1 = nf0;
    s.off2 = 0;
    s.q0 = w.q0;
    s.qmm = w.qmm;
    if (a.q) {
        if (a.maccormack) {
            adv2_cell_forward<true><<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            adv2_cell_backward<<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            *launches += 2;
        } else {
            adv2_cell_forward<false><<<blocks_for(cells), ADV_THREADS, 0, st>>>(s);
            *launches += 1;
            e = cudaMemcpyAsync(a.q, w.q0, sizeof(float) * (size_t)cells, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
    }
    if (!a.velocity) return cudaGetLastError();
    const dim3 fgrid(blocks_for(nfmax), 2);
    if (a.maccormack) {
        adv2_face_forward<true><<<fgrid, ADV_THREADS, 0, st>>>(s);
        adv2_face_backward<<<fgrid, ADV_THREADS, 0, st>>>(s);
        *launches += 2;
    } else {
        adv2_face_forward<false><<<fgrid, ADV_THREADS, 0, st>>>(s);
        *launches += 1;
        e = cudaMemcpyAsync(a.u, w.v0, sizeof(float) * (size_t)nf0, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(a.v, w.v0 + nf0, sizeof(float) * (size_t)nf1, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// One dilation round of the extrapolation (see extrapolate_run), one thread
// per cell: an active cell keeps its value; an inactive one with active
// neighbours takes sum / weight, the float sum in the reference's neighbour
// order (array_extrapolator3.h:50-60) divided by the count; the rest keep
// their value and stay inactive. Activations are counted per warp.
__global__ void __launch_bounds__(256) ext_round(int W, int H, int D, const float *__restrict__ ain,
                                                 const unsigned char *__restrict__ min, float *__restrict__ aout,
                                                 unsigned char *__restrict__ mout, unsigned long long *added) {
    const long long n = (long long)W * H * D, sy = W, sz = (long long)W * H;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long c = base + threadIdx.x;
        bool newly = false;
        if (c < n) {
            unsigned char act = min[c];
            float val = ain[c];
            if (!act) {
                const int i = (int)(c % W), j = (int)((c / W) % H), k = (int)(c / sz);
                float sum = 0.0f;
                int weight = 0;
                auto see = [&](bool in, long long e) {
                    if (in && min[e]) {
                        sum += ain[e];
                        ++weight;
                    }
                };
                see(i + 1 < W, c + 1);
                see(i > 0, c - 1);
                see(j + 1 < H, c + sy);
                see(j > 0, c - sy);
                see(k > 0, c - sz);
                see(k + 1 < D, c + sz);
                if (weight) {
                    val = sum / (float)weight;
                    act = 1;
                    newly = true;
                }
            }
            aout[c] = val;
            mout[c] = act;
        }
        const unsigned b = __ballot_sync(0xffffffffu, newly);
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(added, (unsigned long long)__popc(b));
    }
}

cudaError_t extrapolate_run(AdvectWork &w, int W, int H, int D, float *a, unsigned char *m, int count,
                            cudaStream_t st, long long *launches, unsigned long long *activated_host) {
    const long long n = (long long)W * H * D;
    if (n > w.ext_cap) {
        cudaFree(w.ext_a);
        cudaFree(w.ext_m);
        w.ext_a = nullptr;
        w.ext_m = nullptr;
        w.ext_cap = 0;
        cudaError_t e = cudaMalloc(&w.ext_a, sizeof(float) * (size_t)n);
        if (e == cudaSuccess) e = cudaMalloc(&w.ext_m, (size_t)n);
        if (e != cudaSuccess) return e;
        w.ext_cap = n;
    }
    if (!w.ext_count) {
        cudaError_t e = cudaMalloc(&w.ext_count, sizeof(unsigned long long));
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemsetAsync(w.ext_count, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    float *ab[2] = {a, w.ext_a};
    unsigned char *mb[2] = {m, w.ext_m};
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 8);
    int cur = 0;
    for (int r = 0; r < count; ++r) {
        ext_round<<<blocks, 256, 0, st>>>(W, H, D, ab[cur], mb[cur], ab[cur ^ 1], mb[cur ^ 1], w.ext_count);
        *launches += 1;
        cur ^= 1;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (cur) {  // an odd count ended in the second buffers
        if ((e = cudaMemcpyAsync(a, w.ext_a, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(m, w.ext_m, (size_t)n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    }
    if (activated_host)
        e = cudaMemcpyAsync(activated_host, w.ext_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    return e;
}

cudaError_t constrain_run(AdvectWork &w, const ConstrainArgs &a, cudaStream_t st, long long *launches) {
    const long long nf0 = (long long)(a.nx + 1) * a.ny * a.nz, nf1 = (long long)a.nx * (a.ny + 1) * a.nz,
                    nf2 = (long long)a.nx * a.ny * (a.nz + 1);
    long long nfmax = nf0 > nf1 ? nf0 : nf1;
    if (nf2 > nfmax) nfmax = nf2;
    cudaError_t e = advect_reserve(w, nf0 + nf1 + nf2, 0);
    if (e == cudaSuccess && !w.flag) e = cudaMalloc(&w.flag, sizeof(int));
    if (e != cudaSuccess) return e;
    // the saved velocity the constraint interpolates (macutility3.cpp:63-64)
    float *src[3] = {a.u, a.v, a.w};
    const long long n[3] = {nf0, nf1, nf2}, o[3] = {0, nf0, nf0 + nf1};
    for (int d = 0; d < 3; ++d) {
        e = cudaMemcpyAsync(w.v0 + o[d], src[d], sizeof(float) * (size_t)n[d], cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    e = cudaMemsetAsync(w.flag, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const long long nodes = (long long)(a.nx + 1) * (a.ny + 1) * (a.nz + 1);
    long long nb = (nodes + ADV_THREADS - 1) / ADV_THREADS;
    if (nb > 4096) nb = 4096;
    cst_any_negative<<<(unsigned)nb, ADV_THREADS, 0, st>>>(a.solid, nodes, w.flag);
    gba::ConstrainArgs c{};
    c.g = make_dims(a.nx, a.ny, a.nz, a.dx, 0);
    c.solid = a.solid;
    c.save = w.v0;
    c.off1 = nf0;
    c.off2 = nf0 + nf1;
    c.u = a.u;
    c.v = a.v;
    c.w = a.w;
    c.mu = a.mu;
    c.mv = a.mv;
    c.mw = a.mw;
    c.exists = w.flag;
    cst_face<<<dim3(blocks_for(nfmax), 3), ADV_THREADS, 0, st>>>(c);
    *launches += 2;
    return cudaGetLastError();
}

}  // namespace gbp
