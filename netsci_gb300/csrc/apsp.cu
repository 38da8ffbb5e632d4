// Hedetniemi all-pairs shortest paths on the GPU.
//
// One step computes, for every (i, j),
//     Hn[i][j] = min_k fl(A[j][k] + H[k][i])
// the update of netcalc/src/hedetniemi_gpu.cu:28-45, as a Jacobi step from H
// into a second buffer (the reference updates H in place). Every entry is a
// minimum of single roundings, so the result does not depend on the order k
// is visited in and matches the CPU restatement bit for bit.
//
// The iterate is kept transposed, X = H^T, so both operands of a step are
// contiguous along k:
//     Xn[j][i] = Hn[i][j] = min_k fl(X[i][k] + A[j][k]).
// X and a copy of A live in P x P buffers (P = n rounded up to 128, +inf
// outside n x n, so padded k contribute nothing and no load needs a bound
// check); the result is transposed back into H once at the end.
//
// Kernel shape: a 64 x 64 output tile per CTA of 256 threads, 4 x 4 outputs
// per thread (four CTAs per SM, 64 registers; 128 x 64 tiles at 8 x 4 per
// thread and two CTAs per SM took 12% longer). k runs in slabs of 32 (16
// took 6% longer: twice the barriers): both operand tiles (64 rows of 32
// floats each) are copied into shared memory with 16-byte cp.async into two
// buffers, so the next slab loads while this one is reduced. Rows are padded
// to 36 floats, which keeps the 16-byte reads of a quarter-warp on distinct
// banks. Each thread reads four consecutive k of a
// row at once; one packed add (add.rn.f32x2) forms the sums for (k, k+1) and
// one three-input min folds both into the running minimum: two instructions
// per two (i, j, k) terms. The work is FADD/FMNMX issue-bound on CUDA cores;
// a min-plus product has no tensor-core form.
//
// Convergence: step t writes changed[t] = 1 when any entry differs from the
// previous iterate; step t+1 returns at once when changed[t] == 0 (the
// iterate is then a fixed point and both buffers hold it).
//
// Repeated squaring. When the path length is unbounded (maxPathLength >=
// n-1) and A is symmetric with a zero diagonal and no negative weight, the
// iteration's fixed point is the all-pairs shortest-path matrix A*, and
// H <- H (x) H reaches it in ceil(log2(hop diameter)) products instead of
// one step per hop (H_t = A^(2^t); once a product changes nothing, every
// higher power is equal). The same step kernel does the product with the
// iterate as both operands. A squared entry sums two partial paths, where a
// Jacobi step adds one edge to a path, so on float weights the roundings can
// differ from the reference's in the last bits. On integer-valued weights
// whose path sums stay below 2^24 every sum is exact in float, and squaring
// gives the reference's fixed point bit for bit; the automatic mode squares
// only then (analyze_kernel checks A on the device) and runs Jacobi steps
// otherwise.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "apsp.h"
#include "common.cuh"

namespace nsg {
namespace {

constexpr int kTileI = 64;  // output rows i per CTA (rows of X)
constexpr int kTileJ = 64;   // output columns j per CTA (rows of A)
constexpr int kSlab = 32;    // k values per stage
constexpr int kRow = 36;     // shared-memory row stride (floats)
constexpr int kThreads = 256;
constexpr int kPad = 128;    // P is a multiple of this (and of kTileJ, kSlab)

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void __launch_bounds__(kThreads, 4)
hedetniemi_step_kernel(const float* __restrict__ X, const float* __restrict__ Ap,
                       float* __restrict__ Xn, int n, int P, int* changed, int step) {
    if (step > 0 && changed[step - 1] == 0) return;  // fixed point reached earlier
    __shared__ __align__(16) float Xs[2][kTileI][kRow];
    __shared__ __align__(16) float As[2][kTileJ][kRow];
    const float inf = __int_as_float(0x7f800000);
    const int tid = threadIdx.x;
    // rows i = i0 + tx + 16u (u < 4), columns j = j0 + ty + 16v (v < 4)
    const int tx = tid & 15;
    const int ty = tid >> 4;
    const int i0 = blockIdx.y * kTileI;
    const int j0 = blockIdx.x * kTileJ;
    const float* xg = X + (size_t)i0 * P;
    const float* ag = Ap + (size_t)j0 * P;
    // 64 + 64 rows of eight 16-byte chunks: four chunks per thread
    auto load_slab = [&](int buf, int k0) {
#pragma unroll
        constexpr int kChunks = kSlab / 4;  // 16-byte chunks per row
        static_assert((kChunks * (kTileI + kTileJ)) % kThreads == 0, "whole chunks per thread");
        for (int e = 0; e < (kChunks * (kTileI + kTileJ)) / kThreads; ++e) {
            const int c = tid + kThreads * e;
            if (c < kChunks * kTileI) {
                const int r = c / kChunks, q = c % kChunks;
                cp_async16(&Xs[buf][r][4 * q], xg + (size_t)r * P + k0 + 4 * q);
            } else {
                const int c2 = c - kChunks * kTileI;
                const int r = c2 / kChunks, q = c2 % kChunks;
                cp_async16(&As[buf][r][4 * q], ag + (size_t)r * P + k0 + 4 * q);
            }
        }
        cp_async_commit();
    };

    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = inf;

    const int nslab = P / kSlab;
    load_slab(0, 0);
    for (int sl = 0; sl < nslab; ++sl) {
        if (sl + 1 < nslab) {
            load_slab((sl + 1) & 1, (sl + 1) * kSlab);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int b = sl & 1;
#pragma unroll
        for (int kq = 0; kq < kSlab / 4; ++kq) {
            float4 x[4], a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = *reinterpret_cast<const float4*>(&Xs[b][tx + 16 * u][4 * kq]);
#pragma unroll
            for (int v = 0; v < 4; ++v) a[v] = *reinterpret_cast<const float4*>(&As[b][ty + 16 * v][4 * kq]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float2 s0 = nsg_add2(make_float2(x[u].x, x[u].y), make_float2(a[v].x, a[v].y));
                    const float2 s1 = nsg_add2(make_float2(x[u].z, x[u].w), make_float2(a[v].z, a[v].w));
                    acc[u][v] = nsg_min3(acc[u][v], s0.x, s0.y);
                    acc[u][v] = nsg_min3(acc[u][v], s1.x, s1.y);
                }
        }
        __syncthreads();  // the buffer is refilled two slabs on
    }

    bool diff = false;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = i0 + tx + 16 * u;
        if (i >= n) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = j0 + ty + 16 * v;
            if (j >= n) continue;
            const size_t o = (size_t)j * P + i;
            if (__float_as_int(acc[u][v]) != __float_as_int(__ldg(X + o))) diff = true;
            Xn[o] = acc[u][v];
        }
    }
    if (__syncthreads_or(diff) && tid == 0) changed[step] = 1;
}

// Properties of A that decide whether repeated squaring applies:
// flags bit 0 asymmetric, bit 1 non-zero diagonal, bit 2 a negative weight or
// NaN, bit 3 a finite weight that is not an integer; *wmax = the largest
// finite weight (as non-negative float bits, so integer max orders them).
__global__ void analyze_kernel(const float* __restrict__ A, int n, int* flags, int* wmax) {
    int f = 0, w = 0;
    const size_t nn = (size_t)n * n;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = static_cast<int>(idx / n), j = static_cast<int>(idx % n);
        const float a = __ldg(A + idx);
        if (__float_as_int(a) != __float_as_int(__ldg(A + (size_t)j * n + i))) f |= 1;
        if (i == j && a != 0.f) f |= 2;
        if (!(a >= 0.f)) f |= 4;
        if (a >= 0.f && a < __int_as_float(0x7f800000)) {
            if (a != rintf(a)) f |= 8;
            w = max(w, __float_as_int(a));
        }
    }
    f = __reduce_or_sync(0xffffffffu, f);
    w = __reduce_max_sync(0xffffffffu, w);
    if ((threadIdx.x & 31) == 0) {
        if (f) atomicOr(flags, f);
        atomicMax(wmax, w);
    }
}

// dst (P x P) = src (n x n, stride n) or its transpose, +inf outside n x n.
__global__ void pad_copy_kernel(const float* __restrict__ src, float* __restrict__ dst, int n, int P,
                                int transpose) {
    __shared__ float t[32][33];
    const float inf = __int_as_float(0x7f800000);
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // dst tile: rows by.., columns bx..
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int sr = transpose ? bx + yy : by + yy;
        const int sc = transpose ? by + threadIdx.x : bx + threadIdx.x;
        t[yy][threadIdx.x] = (sr < n && sc < n) ? __ldg(src + (size_t)sr * n + sc) : inf;
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int r = by + yy, c = bx + threadIdx.x;
        dst[(size_t)r * P + c] = transpose ? t[threadIdx.x][yy] : t[yy][threadIdx.x];
    }
}

// H (n x n) = the n x n corner of X (stride P), transposed.
__global__ void unpad_transpose_kernel(const float* __restrict__ X, float* __restrict__ H, int n, int P) {
    __shared__ float t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // H tile: rows by.., columns bx..
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y)
        t[yy][threadIdx.x] = __ldg(X + (size_t)(bx + yy) * P + by + threadIdx.x);
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int r = by + yy, c = bx + threadIdx.x;
        if (r < n && c < n) H[(size_t)r * n + c] = t[threadIdx.x][yy];
    }
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

void launch_step(const float* Ap, const float* X, float* Xn, int n, int P, int* changed, int step,
                 cudaStream_t s) {
    dim3 grid(P / kTileJ, P / kTileI);
    hedetniemi_step_kernel<<<grid, kThreads, 0, s>>>(X, Ap, Xn, n, P, changed, step);
    NSG_CUDA(cudaGetLastError());
}

void launch_pad(const float* src, float* dst, int n, int P, bool transpose, cudaStream_t s) {
    pad_copy_kernel<<<dim3(P / 32, P / 32), dim3(32, 8), 0, s>>>(src, dst, n, P, transpose ? 1 : 0);
    NSG_CUDA(cudaGetLastError());
}

void launch_unpad(const float* X, float* H, int n, int P, cudaStream_t s) {
    unpad_transpose_kernel<<<dim3((n + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, s>>>(X, H, n, P);
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

// Padded copy of A and the two transposed iterates X = H^T, both starting at A^T.
struct Iterates {
    int P;
    DevMem mem;
    float* Ap;
    float* X[2];
    Iterates(const float* A, int n, cudaStream_t s)
        : P((n + kPad - 1) / kPad * kPad), mem(sizeof(float) * 3 * (size_t)P * P, s) {
        const size_t pp = (size_t)P * P;
        Ap = static_cast<float*>(mem.p);
        X[0] = Ap + pp;
        X[1] = Ap + 2 * pp;
        launch_pad(A, Ap, n, P, false, s);
        launch_pad(A, X[0], n, P, true, s);
        launch_pad(A, X[1], n, P, true, s);
    }
};

std::atomic<int> g_method{-1};

// Whether repeated squaring gives this solve's result (see the file comment):
// 0 no, 1 exactly (integer weights), 2 within rounding (requested on float
// weights).
int use_squaring(const float* A, int n, int max_path_length, cudaStream_t s) {
    const int method = g_method.load();
    if (method == 0 || n < 2 || max_path_length < n - 1) return 0;
    DevMem info(2 * sizeof(int), s);
    int* d = static_cast<int*>(info.p);
    NSG_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(int), s));
    const size_t nn = (size_t)n * n;
    const int blocks = static_cast<int>(std::min<size_t>((nn + 255) / 256, 4096));
    analyze_kernel<<<blocks, 256, 0, s>>>(A, n, d, d + 1);
    NSG_CUDA(cudaGetLastError());
    int h[2] = {0, 0};
    NSG_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
    NSG_CUDA(cudaStreamSynchronize(s));
    if (h[0] & 7) return 0;                // asymmetric, diagonal, negative or NaN
    float wmax;
    std::memcpy(&wmax, &h[1], sizeof(float));
    // integer weights with every path sum (at most n-1 edges) exact in float
    if (!(h[0] & 8) && static_cast<double>(wmax) * (n - 1) < 16777216.0) return 1;
    return method == 1 ? 2 : 0;            // squaring requested on any weights
}

}  // namespace

void apsp_set_method(int method) {
    if (method < -1 || method > 1) invalid("method must be -1, 0 or 1");
    g_method.store(method);
}

int apsp_lengths(const float* A, float* H, int n, int max_path_length, cudaStream_t s) {
    if (n < 0 || max_path_length < 0) invalid("negative size or path length");
    const size_t nn = (size_t)n * n;
    if (max_path_length == 0 || n == 0) {
        NSG_CUDA(cudaMemcpyAsync(H, A, nn * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return 0;
    }
    if (const int sq = use_squaring(A, n, max_path_length, s)) {
        // A symmetric: X = A^T = A; each product X <- X (x) X
        Iterates it(A, n, s);
        int log2n = 0;
        while ((1 << log2n) < n) ++log2n;
        // Exact sums: powers up to 2^t >= n - 1, then the product that changes
        // nothing. Rounded sums: once every shortest path is covered, a product
        // can still lower an entry by an ulp through another split of a path's
        // sum; those descents are bounded and short, and products that find
        // nothing to change return at once.
        const int cap = sq == 1 ? log2n + 2 : log2n + 64;
        DevMem changed(sizeof(int) * cap, s);
        NSG_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int) * cap, s));
        int* ch = static_cast<int*>(changed.p);
        for (int t = 0; t < cap; ++t) launch_step(it.X[t & 1], it.X[t & 1], it.X[(t + 1) & 1], n, it.P, ch, t, s);
        std::vector<int> flags(cap);
        NSG_CUDA(cudaMemcpyAsync(flags.data(), ch, sizeof(int) * cap, cudaMemcpyDeviceToHost, s));
        NSG_CUDA(cudaStreamSynchronize(s));
        int products = cap;
        for (int q = 0; q < cap; ++q) {
            if (flags[q] == 0) {
                products = q + 1;
                break;
            }
        }
        if (products == cap && flags[cap - 1]) fail(NSG_ERR_CUDA, "shortest-path squaring did not converge");
        launch_unpad(it.X[cap & 1], H, n, it.P, s);
        NSG_CUDA(cudaStreamSynchronize(s));
        return products;
    }
    Iterates it(A, n, s);
    DevMem changed(sizeof(int) * max_path_length, s);
    NSG_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int) * max_path_length, s));
    int* ch = static_cast<int*>(changed.p);
    // Launch in chunks; read the last step's flag between chunks so long runs
    // stop shortly after the fixed point instead of queueing empty steps.
    const int chunk = 8;
    int t = 0;
    int last_flag = 1;
    while (t < max_path_length && last_flag) {
        const int end = std::min(max_path_length, t + chunk);
        for (; t < end; ++t) launch_step(it.Ap, it.X[t & 1], it.X[(t + 1) & 1], n, it.P, ch, t, s);
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
    // The result lives in X[t & 1]; when converged both buffers hold it.
    launch_unpad(it.X[t & 1], H, n, it.P, s);
    NSG_CUDA(cudaStreamSynchronize(s));
    return steps;
}

void apsp_paths(const float* A, float* H, int* paths, int n, int L, float tolerance,
                cudaStream_t s) {
    if (n < 0 || L < 1) invalid("paths need n >= 0 and maxPathLength >= 1");
    const size_t nn = (size_t)n * n;
    NSG_CUDA(cudaMemsetAsync(paths, 0xff, sizeof(int) * nn * L, s));  // -1
    if (n == 0) return;
    Iterates it(A, n, s);
    DevMem snaps(nn * L * sizeof(float), s);
    DevMem changed(sizeof(int) * L, s);
    NSG_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int) * L, s));
    float* Hi = static_cast<float*>(snaps.p);
    for (int p = 0; p < L; ++p) {
        launch_unpad(it.X[p & 1], Hi + nn * p, n, it.P, s);  // H before step p
        launch_step(it.Ap, it.X[p & 1], it.X[(p + 1) & 1], n, it.P, static_cast<int*>(changed.p), p, s);
    }
    launch_unpad(it.X[L & 1], H, n, it.P, s);
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
