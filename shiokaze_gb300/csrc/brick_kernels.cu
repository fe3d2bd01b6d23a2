// brick_kernels.cu -- sparse arrays in bricks of 8^3 cells, expanded to and
// gathered from the dense arrays the projection runs on (include/gbp.h,
// gbp_bricks). The reference's tiled arrays (src/array/tiledarray3.cpp)
// travel as their listed bricks only.
//
// Algorithmic DRAM bytes: expand writes 4 B per dense cell and reads 4 B per
// listed cell (plus a slot per brick); gather reads 4 (+1) B and writes 4
// (+1) B per listed output cell.
#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "brick_kernels.h"

namespace gbp {
namespace {

constexpr int kBrick = 8;

// One block per row (j, k) of the dense array, threads along x.
__global__ void __launch_bounds__(256) brick_expand_kernel(int nx, int ny, int nz, int nbx, int nby, float background,
                                                           float fill, const int *__restrict__ slot,
                                                           const float *__restrict__ values, float *__restrict__ dense) {
    const long long rows = (long long)ny * nz;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int k = (int)(r / ny), j = (int)(r - (long long)k * ny);
        const long long brow = (long long)nbx * ((j >> 3) + (long long)nby * (k >> 3));
        const int inner = 8 * ((j & 7) + 8 * (k & 7));
        float *out = dense + r * nx;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const int s = __ldg(slot + brow + (i >> 3));
            float val = background;
            if (s >= 0) val = __ldg(values + (long long)s * (kBrick * kBrick * kBrick) + inner + (i & 7));
            else if (s == -2) val = fill;
            out[i] = val;
        }
    }
}

// One thread per cell of the listed output bricks (zero beyond the extent).
__global__ void __launch_bounds__(256) brick_gather_kernel(int nx, int ny, int nz, int nbx, int nby,
                                                           const long long *__restrict__ brick_of,
                                                           long long count, const float *__restrict__ dense,
                                                           const unsigned char *__restrict__ flags,
                                                           float *__restrict__ out, unsigned char *__restrict__ out_flags) {
    const long long total = count * (kBrick * kBrick * kBrick);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long b = __ldg(brick_of + (t >> 9));
        const int cell = (int)(t & 511);
        const long long bz = b / ((long long)nbx * nby), rem = b - bz * nbx * nby;
        const int by = (int)(rem / nbx), bx = (int)(rem - (long long)by * nbx);
        const int i = bx * 8 + (cell & 7), j = by * 8 + ((cell >> 3) & 7), k = (int)bz * 8 + (cell >> 6);
        float val = 0.0f;
        unsigned char fl = 0;
        if (i < nx && j < ny && k < nz) {
            const long long c = i + (long long)nx * (j + (long long)ny * k);
            val = __ldg(dense + c);
            if (flags) fl = __ldg(flags + c);
        }
        out[t] = val;
        if (out_flags) out_flags[t] = fl;
    }
}

}  // namespace

cudaError_t launch_brick_expand(int nx, int ny, int nz, float background, float fill, const int *slot,
                                const float *values, float *dense, int grid_blocks, cudaStream_t stream) {
    const long long rows = (long long)ny * nz;
    const int blocks = (int)(rows < 8LL * grid_blocks ? rows : 8LL * grid_blocks);
    if (blocks < 1) return cudaSuccess;
    brick_expand_kernel<<<blocks, 256, 0, stream>>>(nx, ny, nz, (nx + 7) / 8, (ny + 7) / 8, background, fill, slot,
                                                    values, dense);
    return cudaGetLastError();
}

cudaError_t launch_brick_gather(int nx, int ny, int nz, const long long *brick_of, long long count, const float *dense,
                                const unsigned char *flags, float *out, unsigned char *out_flags, int grid_blocks,
                                cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    const long long need = (count * 512 + 255) / 256;
    const int blocks = (int)(need < 4LL * grid_blocks ? need : 4LL * grid_blocks);
    brick_gather_kernel<<<blocks, 256, 0, stream>>>(nx, ny, nz, (nx + 7) / 8, (ny + 7) / 8, brick_of, count, dense,
                                                    flags, out, out_flags);
    return cudaGetLastError();
}

}  // namespace gbp
