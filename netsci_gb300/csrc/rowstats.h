// Row mean / standard deviation on the device (rowstats.cu).
#pragma once
#include <cuda_runtime.h>

namespace nsg {
// u[row] = mean of row; when sigma is non-null also the population standard
// deviation. a is row-major m x n on the device; u, sigma hold m floats.
void row_stats(const float* a, float* u, float* sigma, int m, int n, cudaStream_t st);
}  // namespace nsg
