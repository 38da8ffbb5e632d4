// Host entry points of the Hedetniemi APSP kernels (apsp.cu).
#pragma once

#include <cuda_runtime.h>

namespace nsg {

// H <- shortest path lengths (device n x n); returns the min-plus products
// run (Jacobi steps, or squarings when repeated squaring applies, see
// apsp.cu). Blocks on s.
int apsp_lengths(const float* A, float* H, int n, int max_path_length, cudaStream_t s);
// Product schedule for later solves: -1 automatic (squaring where it is
// exact), 0 Jacobi steps only, 1 squaring wherever the fixed point is asked
// for on a symmetric, zero-diagonal, non-negative A (float weights then
// within rounding of the reference's association).
void apsp_set_method(int method);
// H and paths (device, n*L*n ints) as netcalc/src/hedetniemi_gpu.cu:148-235.
// Blocks on s.
void apsp_paths(const float* A, float* H, int* paths, int n, int L, float tolerance,
                cudaStream_t s);
// mode 0: 1/r, mode 1: -ln r; asynchronous.
void corr_to_adjacency(const float* C, float* A, int n, int mode, cudaStream_t s);

}  // namespace nsg
