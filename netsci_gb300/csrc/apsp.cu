// Hedetniemi all-pairs shortest paths on the GPU.
//
// One step computes, for every (i, j),
//     Hn[i][j] = min_k fl(A[j][k] + H[k][i])
// the update of netcalc/src/hedetniemi_gpu.cu:28-45, as a Jacobi step from H
// into a second buffer (the reference updates H in place). Every entry is a
// minimum of single roundings, so the result does not depend on the order k
// is visited in and matches the CPU restatement bit for bit.
//
// Kernel shape: a 128 x 64 output tile per CTA of 256 threads, 8 x 4 outputs
// per thread (about 80 registers, three CTAs per SM), k in slabs of 16
// staged in shared memory as interleaved pairs
// (k, k+1), so one packed add (add.rn.f32x2) forms two candidate sums and one
// three-input min folds both into the running minimum: two instructions per
// two (i, j, k) terms. The work is FADD/FMNMX issue-bound on CUDA cores; a
// min-plus product has no tensor-core form.
//
// Convergence: step t writes changed[t] = 1 when any entry differs from H;
// step t+1 returns at once when changed[t] == 0 (H is then a fixed point and
// both buffers hold it).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "apsp.h"
#include "common.cuh"

namespace nsg {
namespace {

constexpr int kTileI = 128;  // output rows i per CTA
constexpr int kTileJ = 64;   // output columns j per CTA
constexpr int kSlab = 16;    // k values per stage (8 pairs)
constexpr int kThreads = 256;
constexpr int kHLoads = (kSlab * kTileI) / kThreads;  // elements per thread per slab
constexpr int kALoads = (kSlab * kTileJ) / kThreads;

__global__ void __launch_bounds__(kThreads, 2)
hedetniemi_step_kernel(const float* __restrict__ A, const float* __restrict__ H,
                       float* __restrict__ Hn, int n, int* changed, int step) {
    if (step > 0 && changed[step - 1] == 0) return;  // fixed point reached earlier
    __shared__ __align__(16) float2 Hs[kSlab / 2][kTileI];  // (H[k][i], H[k+1][i])
    __shared__ __align__(16) float2 As[kSlab / 2][kTileJ];  // (A[j][k], A[j][k+1])
    const float inf = __int_as_float(0x7f800000);
    const int tid = threadIdx.x;
    // Rows i = i0 + 32w + 2tx + {0,1} for w = 0..3: the lanes of a warp read
    // consecutive 16-byte pairs of Hs (no bank replays). Columns
    // j = j0 + 32w + 2ty + {0,1} for w = 0..1: two addresses per warp.
    const int tx = tid & 15;
    const int ty = tid >> 4;
    const int i0 = blockIdx.y * kTileI;
    const int j0 = blockIdx.x * kTileJ;

    float acc[8][4];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = inf;

    for (int k0 = 0; k0 < n; k0 += kSlab) {
        __syncthreads();
#pragma unroll
        for (int e = 0; e < kHLoads; ++e) {
            const int idx = e * kThreads + tid;
            const int kk = idx / kTileI;
            const int ii = idx - kk * kTileI;
            const int k = k0 + kk, i = i0 + ii;
            reinterpret_cast<float*>(&Hs[kk >> 1][ii])[kk & 1] =
                (k < n && i < n) ? __ldg(H + (size_t)k * n + i) : inf;
        }
#pragma unroll
        for (int e = 0; e < kALoads; ++e) {
            const int idx = e * kThreads + tid;
            const int jj = idx / kSlab;
            const int kk = idx - jj * kSlab;
            const int k = k0 + kk, j = j0 + jj;
            reinterpret_cast<float*>(&As[kk >> 1][jj])[kk & 1] =
                (k < n && j < n) ? __ldg(A + (size_t)j * n + k) : inf;
        }
        __syncthreads();
#pragma unroll
        for (int kp = 0; kp < kSlab / 2; ++kp) {
            float2 h[8], a[4];
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                h[2 * w] = Hs[kp][32 * w + 2 * tx];
                h[2 * w + 1] = Hs[kp][32 * w + 2 * tx + 1];
            }
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                a[2 * w] = As[kp][32 * w + 2 * ty];
                a[2 * w + 1] = As[kp][32 * w + 2 * ty + 1];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float2 s = nsg_add2(a[v], h[u]);
                    acc[u][v] = nsg_min3(acc[u][v], s.x, s.y);
                }
        }
    }

    bool diff = false;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int i = i0 + 32 * (u >> 1) + 2 * tx + (u & 1);
        if (i >= n) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = j0 + 32 * (v >> 1) + 2 * ty + (v & 1);
            if (j >= n) continue;
            const size_t o = (size_t)i * n + j;
            if (__float_as_int(acc[u][v]) != __float_as_int(__ldg(H + o))) diff = true;
            Hn[o] = acc[u][v];
        }
    }
    if (__syncthreads_or(diff) && tid == 0) changed[step] = 1;
}

// Back-walk of netcalc/src/hedetniemi_gpu.cu:70-107 over snapshots Hi[p]
// (H before step p). Diagonal cells hold i.
__global__ void hedetniemi_walk_kernel(const float* __restrict__ H, const float* __restrict__ Hi,
                                       const float* __restrict__ A, int* __restrict__ paths,
                                       float tolerance, int n, int L) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    int* cell = paths + (size_t)i * L * n + (size_t)j * L;
    if (i == j) {
        for (int p = 0; p < L; ++p) cell[p] = i;
        return;
    }
    float len = H[(size_t)i * n + j];
    int k = j;
    for (int p = L - 1; p >= 0; --p) {
        const float* hp = Hi + (size_t)p * n * n + (size_t)i * n;
        for (int q = 0; q < n; ++q) {
            if (q == j) continue;
            const float a = A[(size_t)q * n + k];
            if (__fsub_rn(__fadd_rn(hp[q], a), len) < tolerance) {
                len = __fsub_rn(len, a);
                k = q;
                break;
            }
        }
        cell[p] = k;
    }
}

// mode 0: 1/r adjacency (netcalc/src/hedetniemi_gpu.cu:10-26);
// mode 1: -ln(r) adjacency, evaluated in double and rounded to float.
__global__ void corr_to_adj_kernel(const float* __restrict__ C, float* __restrict__ A, int n,
                                   int mode) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * n) return;
    const int i = static_cast<int>(idx / n), j = static_cast<int>(idx % n);
    const float c = C[idx];
    const float inf = __int_as_float(0x7f800000);
    float v;
    if (i == j) {
        v = 0.f;
    } else if (mode == 0) {
        v = (c == 0.f) ? inf : __fdiv_rn(1.f, c);
    } else {
        v = (c > 0.f) ? __double2float_rn(-log(static_cast<double>(c))) : inf;
    }
    A[idx] = v;
}

void launch_step(const float* A, const float* H, float* Hn, int n, int* changed, int step,
                 cudaStream_t s) {
    dim3 grid((n + kTileJ - 1) / kTileJ, (n + kTileI - 1) / kTileI);
    hedetniemi_step_kernel<<<grid, kThreads, 0, s>>>(A, H, Hn, n, changed, step);
    NSG_CUDA(cudaGetLastError());
}

// Workspace allocated and freed in the order of the solver's stream, so a
// solve does not wait for kernels on other streams.
struct DevMem {
    void* p = nullptr;
    cudaStream_t s;
    DevMem(size_t bytes, cudaStream_t st) : s(st) {
        NSG_CUDA(cudaMallocAsync(&p, bytes > 0 ? bytes : 1, st));
    }
    ~DevMem() { if (p) cudaFreeAsync(p, s); }
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
};

}  // namespace

int apsp_lengths(const float* A, float* H, int n, int max_path_length, cudaStream_t s) {
    if (n < 0 || max_path_length < 0) invalid("negative size or path length");
    const size_t nn = (size_t)n * n;
    NSG_CUDA(cudaMemcpyAsync(H, A, nn * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (max_path_length == 0 || n == 0) return 0;
    DevMem tmp(nn * sizeof(float), s);
    DevMem changed(sizeof(int) * max_path_length, s);
    NSG_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int) * max_path_length, s));
    float* buf[2] = {H, static_cast<float*>(tmp.p)};
    int* ch = static_cast<int*>(changed.p);
    // Launch in chunks; read the last step's flag between chunks so long runs
    // stop shortly after the fixed point instead of queueing empty steps.
    const int chunk = 8;
    int t = 0;
    int last_flag = 1;
    while (t < max_path_length && last_flag) {
        const int end = std::min(max_path_length, t + chunk);
        for (; t < end; ++t) launch_step(A, buf[t & 1], buf[(t + 1) & 1], n, ch, t, s);
        NSG_CUDA(cudaMemcpyAsync(&last_flag, ch + (t - 1), sizeof(int), cudaMemcpyDeviceToHost, s));
        NSG_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<int> flags(t);
    NSG_CUDA(cudaMemcpyAsync(flags.data(), ch, sizeof(int) * t, cudaMemcpyDeviceToHost, s));
    NSG_CUDA(cudaStreamSynchronize(s));
    int steps = t;
    for (int q = 0; q < t; ++q) {
        if (flags[q] == 0) {
            steps = q + 1;
            break;
        }
    }
    // Result lives in buf[t & 1]; when converged both buffers hold it.
    if (buf[t & 1] != H) {
        NSG_CUDA(cudaMemcpyAsync(H, buf[t & 1], nn * sizeof(float), cudaMemcpyDeviceToDevice, s));
        NSG_CUDA(cudaStreamSynchronize(s));
    }
    return steps;
}

void apsp_paths(const float* A, float* H, int* paths, int n, int L, float tolerance,
                cudaStream_t s) {
    if (n < 0 || L < 1) invalid("paths need n >= 0 and maxPathLength >= 1");
    const size_t nn = (size_t)n * n;
    NSG_CUDA(cudaMemsetAsync(paths, 0xff, sizeof(int) * nn * L, s));  // -1
    if (n == 0) return;
    DevMem tmp(nn * sizeof(float), s);
    DevMem snaps(nn * L * sizeof(float), s);
    DevMem changed(sizeof(int) * L, s);
    NSG_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int) * L, s));
    NSG_CUDA(cudaMemcpyAsync(H, A, nn * sizeof(float), cudaMemcpyDeviceToDevice, s));
    float* buf[2] = {H, static_cast<float*>(tmp.p)};
    float* Hi = static_cast<float*>(snaps.p);
    for (int p = 0; p < L; ++p) {
        NSG_CUDA(cudaMemcpyAsync(Hi + nn * p, buf[p & 1], nn * sizeof(float),
                                 cudaMemcpyDeviceToDevice, s));
        launch_step(A, buf[p & 1], buf[(p + 1) & 1], n, static_cast<int*>(changed.p), p, s);
    }
    if (buf[L & 1] != H) {
        NSG_CUDA(cudaMemcpyAsync(H, buf[L & 1], nn * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    dim3 block(32, 8);
    dim3 grid((n + 31) / 32, (n + 7) / 8);
    hedetniemi_walk_kernel<<<grid, block, 0, s>>>(H, Hi, A, paths, tolerance, n, L);
    NSG_CUDA(cudaGetLastError());
    NSG_CUDA(cudaStreamSynchronize(s));
}

void corr_to_adjacency(const float* C, float* A, int n, int mode, cudaStream_t s) {
    if (n <= 0) return;
    const size_t nn = (size_t)n * n;
    const int threads = 256;
    corr_to_adj_kernel<<<static_cast<unsigned>((nn + threads - 1) / threads), threads, 0, s>>>(
        C, A, n, mode);
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
