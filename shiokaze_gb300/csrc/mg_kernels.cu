// mg_kernels.cu -- multigrid preconditioner kernels (filled in next).
#include "gbp_internal.cuh"
