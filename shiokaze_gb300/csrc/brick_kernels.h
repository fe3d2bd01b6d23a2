// brick_kernels.h -- launch functions of brick_kernels.cu (sparse arrays in
// bricks of 8^3 cells, include/gbp.h gbp_bricks).
#pragma once

#include <cuda_runtime.h>

namespace gbp {

// dense (nx*ny*nz, x fastest) <- the bricks' cell values (slot per brick,
// values per listed brick; see gbp_bricks).
cudaError_t launch_brick_expand(int nx, int ny, int nz, float background, float fill, const int *slot,
                                const float *values, float *dense, int grid_blocks, cudaStream_t stream);
// out[s * 512 + cell] <- dense at brick brick_of[s] (and out_flags from
// flags when both are given); 0 beyond the extent.
cudaError_t launch_brick_gather(int nx, int ny, int nz, const long long *brick_of, long long count, const float *dense,
                                const unsigned char *flags, float *out, unsigned char *out_flags, int grid_blocks,
                                cudaStream_t stream);

}  // namespace gbp
