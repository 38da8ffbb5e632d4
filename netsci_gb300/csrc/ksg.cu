// KSG finalize kernel and kernel-registry lookups.
#include <cmath>

#include "common.cuh"
#include "ksg.cuh"
#include "ksg_registry.cuh"

namespace nsg {
namespace {

// One warp per pair: the float sum of the pair's per-sample psi terms in
// sample order, then the KSG formula and the generalized-correlation
// transform, with the reference's operation order and precisions:
//   netcalc/src/mutual_information_gpu.cu:1065-1074 (sum, divide, formula)
//   netcalc/src/generalized_correlation_gpu.cpp:16-31 (transform in double)
// The sum is sequential on purpose: it reproduces the reference's float
// rounding sequence exactly, about m dependent adds per pair. The warp copies
// the row into shared memory a chunk at a time with coalesced loads, and
// lane 0 adds the chunk from there, so the chain of adds waits on shared
// memory rather than on a global load per term.
constexpr int kFinalWarps = 8;
constexpr int kFinalChunk = 1024;

__global__ void __launch_bounds__(kFinalWarps * 32) ksg_final_kernel(KsgFinalArgs A) {
    __shared__ __align__(16) float s_row[kFinalWarps][kFinalChunk];
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * kFinalWarps + (threadIdx.x >> 5);
    if (p >= A.npairs) return;
    float* row = s_row[threadIdx.x >> 5];
    const KsgPairDesc P = A.pairs[p];
    const int m = P.m;
    const float* __restrict__ s = A.psum + P.scratch;
    float avg = 0.f;
    for (int base = 0; base < m; base += kFinalChunk) {
        const int n = min(kFinalChunk, m - base);
        __syncwarp();
        for (int q = lane; q < n; q += 32) row[q] = __ldg(s + base + q);
        __syncwarp();
        if (lane == 0) {
            const int n4 = n & ~3;
            for (int q = 0; q < n4; q += 4) {
                const float4 v = *reinterpret_cast<const float4*>(row + q);
                avg = __fadd_rn(avg, v.x);
                avg = __fadd_rn(avg, v.y);
                avg = __fadd_rn(avg, v.z);
                avg = __fadd_rn(avg, v.w);
            }
            for (int q = n4; q < n; ++q) avg = __fadd_rn(avg, row[q]);
        }
    }
    if (lane != 0) return;
    avg = __fdiv_rn(avg, static_cast<float>(m));
    const float inv_k = __double2float_rn(__ddiv_rn(1.0, static_cast<double>(static_cast<float>(A.k))));
    const float mi = __fsub_rn(__fsub_rn(__fadd_rn(__ldg(A.psi + m), __ldg(A.psi + A.k)), inv_k), avg);
    if (A.mi) A.mi[P.out] = mi;
    if (A.gc || A.w) {
        float gc = 0.f;
        if (static_cast<double>(mi) > 0.0) {
            const double scale = -(2.0 / static_cast<double>(static_cast<float>(A.d)));
            const float e = __double2float_rn(exp(scale * static_cast<double>(mi)));
            gc = __double2float_rn(sqrt(1.0 - static_cast<double>(e)));
        }
        if (A.gc) A.gc[P.out] = gc;
        if (A.w) {
            A.w[P.out] = gc > 0.f ? __double2float_rn(-log(static_cast<double>(gc)))
                                  : __int_as_float(0x7f800000);
        }
    }
}

}  // namespace

// Smallest instantiated list length holding the sample itself and its k+1
// nearest neighbours.
int ksg_kmax_for(int k) {
    if (k < 1) return 0;
    for (int kmax : {6, 8, 16, 32, 64}) {
        if (k + 2 <= kmax) return kmax;
    }
    return 0;
}

static const KsgKernelEntry* entries_for(int d, int* count) {
    switch (d) {
        case 1: return ksg_entries_d1(count);
        case 2: return ksg_entries_d2(count);
        case 3: return ksg_entries_d3(count);
        default: *count = 0; return nullptr;
    }
}

const KsgKernelEntry* ksg_find_entry(int d, int kmax, int threads, int r, int frames,
                                     int variant, int tma) {
    int n = 0;
    const KsgKernelEntry* e = entries_for(d, &n);
    for (int i = 0; i < n; ++i) {
        if (e[i].kmax == kmax && e[i].threads == threads && e[i].r == r &&
            e[i].frames == frames && (variant < 0 || e[i].variant == variant) &&
            (tma < 0 || e[i].tma == tma)) {
            return &e[i];
        }
    }
    return nullptr;
}

int ksg_list_entries(int d, int kmax, const KsgKernelEntry** out, int cap) {
    int n = 0, c = 0;
    const KsgKernelEntry* e = entries_for(d, &n);
    for (int i = 0; i < n; ++i) {
        if (e[i].kmax == kmax) {
            if (c < cap) out[c] = &e[i];
            ++c;
        }
    }
    return c;
}

KsgShape ksg_default_shape(int d, int kmax) {
    (void)d;
    if (kmax >= 64) return {64, 1, 512};
    if (kmax >= 16) return {128, 1, 1024};
    return {256, 1, 1024};
}

bool ksg_shape_supported(int d, int kmax, const KsgShape& s) {
    return ksg_find_entry(d, kmax, s.threads, s.r, s.frames, -1) != nullptr;
}

int ksg_ctas_per_sm(int d, int kmax, const KsgShape& s) {
    const KsgKernelEntry* e = ksg_find_entry(d, kmax, s.threads, s.r, s.frames, -1);
    return e ? e->ctas_per_sm() : 0;
}

void ksg_launch_counts(const KsgCountArgs& a, int d, int kmax, const KsgShape& s, int grid,
                       cudaStream_t st) {
    const KsgKernelEntry* e = ksg_find_entry(d, kmax, s.threads, s.r, s.frames, -1);
    if (!e) fail(NSG_ERR_UNSUPPORTED, "no KSG kernel instantiated for this shape");
    e->launch(a, grid, st);
    NSG_CUDA(cudaGetLastError());
}

void ksg_launch_final(const KsgFinalArgs& a, cudaStream_t st) {
    if (a.npairs <= 0) return;
    const int grid = (a.npairs + kFinalWarps - 1) / kFinalWarps;
    ksg_final_kernel<<<grid, kFinalWarps * 32, 0, st>>>(a);
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
