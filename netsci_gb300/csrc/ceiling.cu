// Issue-rate ceilings of the cell-grid kernels' inner loops, measured on the
// device the library runs on (nsg_measure_issue_ceiling).
//
// The search and count kernels are bound by CUDA-core instruction issue. A
// nominal peak of one operation per lane per clock (SMs x 128 x clock)
// misjudges them both ways: packed f32x2 subtractions and three-input max
// do two operations per instruction, while shared-memory broadcasts, the
// admission test and the loop add instructions that are no operation of the
// estimator. These kernels run the very loops of the two kernels
// (gridk::pass1_chunk and gridk::count_chunk) on one staged tile per warp,
// with the same CTA shape and occupancy, but with no memory traffic, no
// range setup and, in the search, a bound that no frame passes (no list
// update ever runs). Their operation rate is what the two kernels could
// reach if nothing but their distance arithmetic cost time: the ceiling that
// the kernels' own rates are divided by.
#include <algorithm>
#include <limits>
#include <vector>

#include "engine.h"
#include "ksg_grid.cuh"

namespace nsg {
namespace {

constexpr int kMixFrames = 64;  // the search scans 64-frame halves of its tile

template <int D, int KL>
__global__ void __launch_bounds__(32 * kGridWarps, 4)
    mix_search_kernel(const float* __restrict__ src, int reps, float bound, unsigned long long* sink) {
    __shared__ __align__(16) float s_tile[kGridWarps][2 * D * kGridChunk];
    __shared__ int s_jt[kGridWarps][kGridChunk];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    float* tile = s_tile[wid];
    int* jt = s_jt[wid];
    for (int f = lane; f < kGridChunk; f += 32) {
#pragma unroll
        for (int c = 0; c < 2 * D; ++c) tile[c * kGridChunk + f] = __ldg(src + c * kGridChunk + f);
        jt[f] = f;
    }
    __syncwarp();
    float qa[D], qb[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        qa[c] = __ldg(src + c * kGridChunk + lane);
        qb[c] = __ldg(src + (D + c) * kGridChunk + 2 * lane + 1);
    }
    float bd[KL];
    int bj[KL];
#pragma unroll
    for (int s = 0; s < KL; ++s) {
        bd[s] = bound;
        bj[s] = -1;
    }
    bool self_seen = false, tied = false;
    for (int r = 0; r < reps; ++r) {
        const int h = (r & 1) * kMixFrames;
        gridk::pass1_chunk<D, KL, false>(tile + h, jt + h, kMixFrames, qa, qb, bd, bj, self_seen, tied, nullptr,
                                         nullptr);
    }
    if (self_seen || tied || bj[0] != -1) atomicAdd(sink, 1ull);
}

template <int D>
__global__ void __launch_bounds__(32 * kGridWarps, 4)
    mix_count_kernel(const float* __restrict__ src, int reps, float eps, unsigned long long* sink) {
    __shared__ __align__(16) float s_tile[kGridWarps][D * kGridChunk];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    float* tile = s_tile[wid];
    for (int f = lane; f < kGridChunk; f += 32) {
#pragma unroll
        for (int c = 0; c < D; ++c) tile[c * kGridChunk + f] = __ldg(src + c * kGridChunk + f);
    }
    __syncwarp();
    float q[D];
#pragma unroll
    for (int c = 0; c < D; ++c) q[c] = __ldg(src + c * kGridChunk + (lane >> 1));
    float e[kCountGroup];
    int cnt[kCountGroup];
#pragma unroll
    for (int p = 0; p < kCountGroup; ++p) {
        e[p] = eps * (1.0f + 0.25f * p);
        cnt[p] = 0;
    }
    const int half = lane & 1;
    for (int r = 0; r < reps; ++r) gridk::count_chunk<D>(tile, kGridChunk, half, q, e, cnt);
    int total = 0;
#pragma unroll
    for (int p = 0; p < kCountGroup; ++p) total += cnt[p];
    atomicAdd(sink, static_cast<unsigned long long>(total));
}

template <typename K>
float timed_ms(K kernel, int grid, const float* src, int reps, float arg, unsigned long long* sink) {
    cudaEvent_t e0, e1;
    NSG_CUDA(cudaEventCreate(&e0));
    NSG_CUDA(cudaEventCreate(&e1));
    kernel<<<grid, 32 * kGridWarps>>>(src, reps / 4 + 1, arg, sink);  // warm-up
    NSG_CUDA(cudaGetLastError());
    NSG_CUDA(cudaEventRecord(e0));
    kernel<<<grid, 32 * kGridWarps>>>(src, reps, arg, sink);
    NSG_CUDA(cudaGetLastError());
    NSG_CUDA(cudaEventRecord(e1));
    NSG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    NSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

template <int D>
void measure(double* search_gops, double* count_gops) {
    constexpr int KL = 6;  // k = 6: the search kernel instance KMAX = 8
    // one wave of CTAs at the real kernels' occupancy
    const int sms = sm_count();
    const int grid_s = sms * grid_search_ctas_per_sm(D, KL + 2);
    const int grid_c = sms * grid_count_ctas_per_sm(D);
    // frames: a smooth pseudo-random pattern, distinct per plane
    std::vector<float> h(2 * D * kGridChunk);
    for (size_t i = 0; i < h.size(); ++i) h[i] = static_cast<float>((i * 2654435761u) % 1000u) * 0.01f;
    DeviceBuffer src(h.size() * sizeof(float));
    DeviceBuffer sink(sizeof(unsigned long long));
    NSG_CUDA(cudaMemcpy(src.get(), h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    NSG_CUDA(cudaMemset(sink.get(), 0, sizeof(unsigned long long)));
    const float neg_inf = -std::numeric_limits<float>::infinity();
    const int reps_s = 4000, reps_c = 2000;
    const float ms_s = timed_ms(mix_search_kernel<D, KL>, grid_s, src.as<float>(), reps_s, neg_inf,
                                sink.as<unsigned long long>());
    const float ms_c = timed_ms(mix_count_kernel<D>, grid_c, src.as<float>(), reps_c, 5.0f,
                                sink.as<unsigned long long>());
    // search: per query-frame evaluation 4d operations (2d subtractions,
    // 2d-1 maxima, one comparison); counts: per query-frame distance 2d-1
    // operations, plus one comparison per pair of the group
    const double lanes_s = static_cast<double>(grid_s) * 32 * kGridWarps;
    const double ops_s = lanes_s * kMixFrames * reps_s * 4.0 * D;
    const double lanes_c = static_cast<double>(grid_c) * 32 * kGridWarps;
    const double dists = lanes_c * (kGridChunk / 2) * reps_c;
    const double ops_c = dists * (2.0 * D - 1.0) + dists * kCountGroup;
    *search_gops = ops_s / (ms_s * 1e-3) / 1e9;
    *count_gops = ops_c / (ms_c * 1e-3) / 1e9;
}

}  // namespace

void measure_issue_ceiling(int d, double* search_gops, double* count_gops) {
    switch (d) {
        case 1: measure<1>(search_gops, count_gops); break;
        case 2: measure<2>(search_gops, count_gops); break;
        case 3: measure<3>(search_gops, count_gops); break;
        default: invalid("d must be 1, 2 or 3");
    }
}

}  // namespace nsg
