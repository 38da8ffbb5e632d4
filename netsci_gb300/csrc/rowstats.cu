// Row mean and population standard deviation of a row-major m x n float
// matrix (netcalc/src/math_utils_gpu.cu:22-198, math_utils.cpp:6-36).
//
// Summation order, which fixes every bit of the result: thread slot t of
// 1024 adds a[row][t], a[row][t + 1024], ... sequentially in float from 0,
// then the 1024 partial sums are folded pairwise, p[t] += p[t + s] for
// s = 512, 256, ..., 1; mean = p[0] / (float)n. The deviation pass sums
// (a - mean)^2 the same way and takes sqrt(p[0] / (float)n). All roundings
// are IEEE round-to-nearest (__fadd_rn etc., so the compiler cannot contract
// them into fused multiply-adds).
//
// One 1024-thread CTA per row (grid-stride over rows): the 1024 slots are
// the threads, loads a[row][t + 1024 i] are coalesced, the fold runs in
// shared memory down to 64 values and in warp shuffles below. A pass reads
// the row once from HBM (the deviation pass's second read hits L2 for rows
// up to tens of MB).
#include <cuda_runtime.h>

#include "errors.h"
#include "rowstats.h"

namespace nsg {
namespace {

constexpr int kSlots = 1024;

// Pairwise fold of the 1024 per-thread values; the result is valid in thread 0.
__device__ __forceinline__ float fold_1024(float v, float* s) {
    const int t = threadIdx.x;
    s[t] = v;
    __syncthreads();
#pragma unroll
    for (int w = 512; w >= 64; w >>= 1) {
        if (t < w) s[t] = __fadd_rn(s[t], s[t + w]);
        __syncthreads();
    }
    float r = 0.f;
    if (t < 32) {
        r = __fadd_rn(s[t], s[t + 32]);
#pragma unroll
        for (int w = 16; w >= 1; w >>= 1) r = __fadd_rn(r, __shfl_down_sync(0xffffffffu, r, w));
    }
    __syncthreads();  // s is reused by the next fold
    return r;
}

__global__ void __launch_bounds__(kSlots) row_stats_kernel(const float* __restrict__ a,
                                                          float* __restrict__ u,
                                                          float* __restrict__ sigma, int m, int n) {
    __shared__ float s[kSlots];
    __shared__ float s_mean;
    const int t = threadIdx.x;
    const float fn = static_cast<float>(n);
    for (int row = blockIdx.x; row < m; row += gridDim.x) {
        const float* r = a + static_cast<size_t>(row) * n;
        float acc = 0.f;
        for (int j = t; j < n; j += kSlots) acc = __fadd_rn(acc, __ldg(r + j));
        const float total = fold_1024(acc, s);
        if (t == 0) {
            const float mu = __fdiv_rn(total, fn);
            u[row] = mu;
            s_mean = mu;
        }
        if (!sigma) continue;
        __syncthreads();
        const float mu = s_mean;
        float sq = 0.f;
        for (int j = t; j < n; j += kSlots) {
            const float dv = __fsub_rn(__ldg(r + j), mu);
            sq = __fadd_rn(sq, __fmul_rn(dv, dv));
        }
        const float tot2 = fold_1024(sq, s);
        if (t == 0) sigma[row] = __fsqrt_rn(__fdiv_rn(tot2, fn));
    }
}

}  // namespace

void row_stats(const float* a, float* u, float* sigma, int m, int n, cudaStream_t st) {
    if (m < 0 || n < 0) invalid("row statistics need m >= 0 and n >= 0");
    if (m == 0) return;
    if (n == 0) invalid("row statistics need n >= 1");
    int dev = 0, sms = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    NSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = m < 2 * sms ? m : 2 * sms;
    row_stats_kernel<<<grid, kSlots, 0, st>>>(a, u, sigma, m, n);
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
