// Cell-grid KSG: grid construction kernels, the instantiations of the grid
// pass-1 / count kernels and their launchers (ksg_grid.cuh has the search).
#include <cuda_runtime.h>

#include <algorithm>

#include "errors.h"
#include "ksg_grid.cuh"
#include "ksg_grid.h"

namespace nsg {
namespace {

constexpr int kPrepThreads = 1024;
constexpr int kSample = 2048;       // frames sampled per coordinate for the quantiles

// In-place ascending bitonic sort of n = kSample floats in shared memory.
__device__ void bitonic_sort(float* v) {
    for (int size = 2; size <= kSample; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (int t = threadIdx.x; t < kSample / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const float a = v[lo], b = v[hi];
                if ((a > b) == asc) {
                    v[lo] = b;
                    v[hi] = a;
                }
            }
        }
    }
    __syncthreads();
}

// Number of edges <= x among e[0..n) (sorted ascending): the bin of x.
__device__ __forceinline__ int bin_of(const float* e, int n, float x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Exclusive scan of cnt[0..n) (n <= 1024) into out[0..n], out[n] = total.
__device__ void block_scan(const int* cnt, int* out, int n) {
    __shared__ int s_warp[32];
    const int t = threadIdx.x;
    const int v = t < n ? cnt[t] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((t & 31) >= o) x += y;
    }
    if ((t & 31) == 31) s_warp[t >> 5] = x;
    __syncthreads();
    if (t < 32) {
        int w = t < (blockDim.x >> 5) ? s_warp[t] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (t >= o) w += y;
        }
        s_warp[t] = w;
    }
    __syncthreads();
    const int incl = x + ((t >> 5) ? s_warp[(t >> 5) - 1] : 0);
    if (t < n) out[t] = incl - v;
    if (t == n - 1) out[n] = incl;
    __syncthreads();
}

// Query order of a grid's cells (the layout is described in ksg_grid.h):
// cnt[c] holds the frames of row-major cell c. The Z-order codes of a
// Gp x Gp square (Gp = G rounded up to a power of two, at most 32) are
// ranked, skipping cells outside G x G, and the counts accumulated in that
// order. tmp1, tmp2: shared scratch of 1024 and 1025 ints.
__device__ void build_query_order(const int* cnt, int G, int* start, int* tmp1, int* tmp2) {
    int* qstart = start + grid_qoff(G);
    unsigned short* qcell = reinterpret_cast<unsigned short*>(qstart + grid_qoff(G));
    int Gp = 1;
    while (Gp < G) Gp <<= 1;
    const int ncode = Gp * Gp;
    const int t = threadIdx.x;
    int row = 0, col = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        row |= ((t >> (2 * b + 1)) & 1) << b;
        col |= ((t >> (2 * b)) & 1) << b;
    }
    const bool valid = t < ncode && row < G && col < G;
    if (t < ncode) tmp1[t] = valid ? 1 : 0;
    __syncthreads();
    block_scan(tmp1, tmp2, ncode);
    const int rank = t < ncode ? tmp2[t] : 0;
    __syncthreads();
    if (valid) {
        qcell[rank] = static_cast<unsigned short>(row * G + col);
        tmp1[rank] = cnt[row * G + col];
    }
    __syncthreads();
    block_scan(tmp1, tmp2, G * G);
    for (int c = t; c <= G * G; c += blockDim.x) qstart[c] = tmp2[c];
}

// One CTA per node: axes, quantile edges, cells, counting sort by cell.
template <int D>
__global__ void __launch_bounds__(kPrepThreads) grid_node_kernel(GridNode* nodes) {
    __shared__ float s_val[D][kSample];
    __shared__ float s_e1[kGridMaxG], s_e2[kGridMaxG];
    __shared__ int s_cnt[kGridMaxG * kGridMaxG];
    __shared__ int s_start[kGridMaxG * kGridMaxG + 1];
    __shared__ int s_tmp1[kGridMaxG * kGridMaxG], s_tmp2[kGridMaxG * kGridMaxG + 1];
    __shared__ int s_axis[2];
    GridNode nd = nodes[blockIdx.x];
    const int m = nd.m, G = nd.G, t = threadIdx.x;
    const int S = kSample;
    for (int s = t; s < S; s += blockDim.x) {
        const int j = static_cast<int>((static_cast<long long>(s) * m) / S);
#pragma unroll
        for (int c = 0; c < D; ++c) s_val[c][s] = __ldg(nd.x + static_cast<long long>(c) * nd.ld + j);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) bitonic_sort(s_val[c]);
    if (t == 0) {
        // widest and second-widest coordinates by their 10-90% spread
        float w[D];
#pragma unroll
        for (int c = 0; c < D; ++c) w[c] = s_val[c][(S * 9) / 10] - s_val[c][S / 10];
        int c1 = 0;
        for (int c = 1; c < D; ++c)
            if (w[c] > w[c1]) c1 = c;
        int c2 = -1;
        for (int c = 0; c < D; ++c)
            if (c != c1 && (c2 < 0 || w[c] > w[c2])) c2 = c;
        s_axis[0] = c1;
        s_axis[1] = c2;
    }
    __syncthreads();
    const int c1 = s_axis[0], c2 = s_axis[1];
    if (t < kGridMaxG) {
        const float inf = __int_as_float(0x7f800000);
        s_e1[t] = t < G - 1 ? s_val[c1][((t + 1) * S) / G] : inf;
        s_e2[t] = (c2 >= 0 && t < G - 1) ? s_val[c2][((t + 1) * S) / G] : inf;
        nd.e1[t] = s_e1[t];
        nd.e2[t] = s_e2[t];
    }
    if (t == 0) {
        nodes[blockIdx.x].c1 = c1;
        nodes[blockIdx.x].c2 = c2;
    }
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    const float* x1 = nd.x + static_cast<long long>(c1) * nd.ld;
    const float* x2 = c2 >= 0 ? nd.x + static_cast<long long>(c2) * nd.ld : nullptr;
    for (int j = t; j < m; j += blockDim.x) {
        const int b1 = bin_of(s_e1, G - 1, __ldg(x1 + j));
        const int b2 = x2 ? bin_of(s_e2, G - 1, __ldg(x2 + j)) : 0;
        const int cell = b1 * G + b2;
        nd.cell[j] = static_cast<unsigned short>(cell);
        atomicAdd(&s_cnt[cell], 1);
    }
    __syncthreads();
    block_scan(s_cnt, s_start, G * G);
    for (int c = t; c <= G * G; c += blockDim.x) nd.start[c] = s_start[c];
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) {
        const int cell = nd.cell[j];
        const int pos = s_start[cell] + atomicAdd(&s_cnt[cell], 1);
        nd.perm[pos] = j;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            nd.sx[static_cast<long long>(c) * m + pos] = __ldg(nd.x + static_cast<long long>(c) * nd.ld + j);
        }
    }
    __syncthreads();
    build_query_order(s_cnt, G, nd.start, s_tmp1, s_tmp2);
}

// One CTA per node, after grid_node_kernel: the scale estimate of every
// frame (GridNode::est), from the frames of the 3 x 3 cells around its own.
// Consecutive threads take consecutive positions, mostly of one cell, so
// they read the same neighbour frames.
template <int D>
__global__ void __launch_bounds__(kPrepThreads) grid_node_est_kernel(const GridNode* nodes) {
    const GridNode nd = nodes[blockIdx.x];
    const int m = nd.m, G = nd.G;
    const long long st = m;
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) {
        const int j = __ldg(nd.perm + pos);
        const int c = __ldg(nd.cell + j);
        const int row = c / G, col = c - (c / G) * G;
        float q[D];
#pragma unroll
        for (int cc = 0; cc < D; ++cc) q[cc] = __ldg(nd.sx + cc * st + pos);
        float bd[kEstRank];
        int bj[kEstRank];
#pragma unroll
        for (int s = 0; s < kEstRank; ++s) {
            bd[s] = __int_as_float(0x7f800000);
            bj[s] = -1;
        }
        const int c0 = max(col - 1, 0), c1 = min(col + 1, G - 1);
        for (int r = max(row - 1, 0); r <= min(row + 1, G - 1); ++r) {
            const int lo = __ldg(nd.start + r * G + c0), hi = __ldg(nd.start + r * G + c1 + 1);
            for (int f = lo; f < hi; ++f) {
                float dm = 0.f;
#pragma unroll
                for (int cc = 0; cc < D; ++cc) dm = fmaxf(dm, fabsf(q[cc] - __ldg(nd.sx + cc * st + f)));
                if (f != pos && dm < bd[kEstRank - 1]) ksgk::list_insert<kEstRank>(bd, bj, dm, f);
            }
        }
        nd.est[j] = bd[kEstRank - 1];
    }
}

// One CTA per pair of the batch: cells over (bin of a on its c1, bin of b on
// its c1), counting sort, both nodes' coordinates copied in that order.
template <int D>
__global__ void __launch_bounds__(kPrepThreads) grid_pair_kernel(const KsgPairDesc* pairs,
                                                                GridPair* gps,
                                                                const GridNode* nodes) {
    __shared__ int s_cnt[kGridMaxG * kGridMaxG];
    __shared__ int s_start[kGridMaxG * kGridMaxG + 1];
    __shared__ int s_tmp1[kGridMaxG * kGridMaxG], s_tmp2[kGridMaxG * kGridMaxG + 1];
    const KsgPairDesc P = pairs[blockIdx.x];
    const GridPair gp = gps[blockIdx.x];
    const GridNode na = nodes[gp.a], nb = nodes[gp.b];
    const int m = P.m, G = na.G, t = threadIdx.x;
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) {
        const int cell = (na.cell[j] / G) * G + nb.cell[j] / G;
        atomicAdd(&s_cnt[cell], 1);
    }
    __syncthreads();
    block_scan(s_cnt, s_start, G * G);
    for (int c = t; c <= G * G; c += blockDim.x) gp.start[c] = s_start[c];
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) {
        const int cell = (na.cell[j] / G) * G + nb.cell[j] / G;
        const int pos = s_start[cell] + atomicAdd(&s_cnt[cell], 1);
        gp.perm[pos] = j;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            gp.sx[static_cast<long long>(c) * m + pos] = __ldg(P.xa + static_cast<long long>(c) * P.ld + j);
            gp.sx[static_cast<long long>(D + c) * m + pos] =
                __ldg(P.xb + static_cast<long long>(c) * P.ld + j);
        }
    }
    __syncthreads();
    build_query_order(s_cnt, G, gp.start, s_tmp1, s_tmp2);
}

// The same pair grid, written plane by plane through shared memory: each
// frame's position is computed once, then every output plane (the original
// indices and the 2d coordinates) is scattered into a shared-memory buffer
// and written out with coalesced stores, instead of scattering 2d + 1 values
// per frame across global memory. Dynamic shared memory: 8 * mpad bytes
// (positions, then the plane buffer) with mpad >= m.
template <int D>
__global__ void __launch_bounds__(kPrepThreads) grid_pair_staged_kernel(const KsgPairDesc* pairs,
                                                                       GridPair* gps,
                                                                       const GridNode* nodes, int mpad) {
    extern __shared__ int s_dyn[];
    __shared__ int s_cnt[kGridMaxG * kGridMaxG];
    __shared__ int s_start[kGridMaxG * kGridMaxG + 1];
    __shared__ int s_tmp1[kGridMaxG * kGridMaxG], s_tmp2[kGridMaxG * kGridMaxG + 1];
    int* s_pos = s_dyn;
    int* s_buf = s_dyn + mpad;
    const KsgPairDesc P = pairs[blockIdx.x];
    const GridPair gp = gps[blockIdx.x];
    const GridNode na = nodes[gp.a], nb = nodes[gp.b];
    const int m = P.m, G = na.G, t = threadIdx.x;
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) {
        const int cell = (na.cell[j] / G) * G + nb.cell[j] / G;
        s_pos[j] = cell;
        atomicAdd(&s_cnt[cell], 1);
    }
    __syncthreads();
    block_scan(s_cnt, s_start, G * G);
    for (int c = t; c <= G * G; c += blockDim.x) gp.start[c] = s_start[c];
    for (int c = t; c < G * G; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) {
        const int cell = s_pos[j];
        s_pos[j] = s_start[cell] + atomicAdd(&s_cnt[cell], 1);
    }
    __syncthreads();
    for (int j = t; j < m; j += blockDim.x) s_buf[s_pos[j]] = j;
    __syncthreads();
    for (int q = t; q < m; q += blockDim.x) gp.perm[q] = s_buf[q];
    float* fbuf = reinterpret_cast<float*>(s_buf);
#pragma unroll 1
    for (int c = 0; c < 2 * D; ++c) {
        const float* src = c < D ? P.xa + static_cast<long long>(c) * P.ld : P.xb + static_cast<long long>(c - D) * P.ld;
        __syncthreads();
        for (int j = t; j < m; j += blockDim.x) fbuf[s_pos[j]] = __ldg(src + j);
        __syncthreads();
        float* dst = gp.sx + static_cast<long long>(c) * m;
        for (int q = t; q < m; q += blockDim.x) dst[q] = fbuf[q];
    }
    __syncthreads();
    build_query_order(s_cnt, G, gp.start, s_tmp1, s_tmp2);
}

// psi[n_x] + psi[n_y] per sample from the raw counts (self included), as
// write_outputs does in the exhaustive kernel.
__global__ void grid_combine_kernel(const KsgPairDesc* pairs, const int* cnt_a, const int* cnt_b,
                                    const float* psi, float* psum, int* nx_out, int* ny_out) {
    const KsgPairDesc P = pairs[blockIdx.x];
    for (int i = threadIdx.x; i < P.m; i += blockDim.x) {
        const long long o = P.scratch + i;
        const int nx = min(max(cnt_a[o] - 1, 0), P.m);
        const int ny = min(max(cnt_b[o] - 1, 0), P.m);
        psum[o] = __fadd_rn(__ldg(psi + nx), __ldg(psi + ny));
        if (nx_out) nx_out[o] = nx;
        if (ny_out) ny_out[o] = ny;
    }
}

// Query orders (see kOrderBits and kOrderBlock). A warp's queries then have
// boxes of nearly the same cells, so the union of their boxes is smaller
// than in a grid's Z order of cells. Any order gives the same results;
// these only shorten the scans.
constexpr int kOrderThreads = 256;
constexpr int kOrderKeyBits = 4 * kOrderBits;          // Z code of the four box corners
constexpr int kOrderBins = 1 << (kOrderKeyBits - 4);   // counting-sort bins: the top bits
constexpr int kOrderSortMax = 32;
// Counts orders sort their bins on the low key bits up to this m (keys and
// bins: 8 bytes per query of shared memory).
constexpr int kOrderSortLowMaxM = 20480;
static_assert(2 * kOrderSortLowMaxM <= kOrderMaxM, "the attribute covers both arrays");
static_assert(kOrderBins % kOrderThreads == 0, "bins split evenly over the CTA");

// Coarse cell (cell >> 1: kOrderBits bits) of x on an axis whose edges give
// the thresholds t[L - 1] = e[2L - 1], L = 1..15, padded with +inf where the
// grid has fewer cells and ended by a NaN (never <= x): the number of
// thresholds <= x, by four branch-free steps over the 16 sorted entries.
static_assert(kOrderBits == 4 && kGridMaxG <= 32, "coarse cells are cell pairs of a grid of <= 32 cells");
__device__ __forceinline__ unsigned coarse_cell(const float* t, float x) {
    unsigned b = t[7] <= x ? 8u : 0u;
    b += t[b + 3] <= x ? 4u : 0u;
    b += t[b + 1] <= x ? 2u : 0u;
    b += t[b] <= x ? 1u : 0u;
    return b;
}

// Bits of v < 16 spread to positions 0, 4, 8, 12.
__device__ __forceinline__ unsigned spread4(unsigned v) {
    return (v & 1u) | (v & 2u) << 3 | (v & 4u) << 6 | (v & 8u) << 9;
}

// Z code of the box [x - h, x + h] x [y - h, y + h] in coarse cells: bit b
// of corner q (low row, low column, high row, high column) at bit 4b + q.
__device__ __forceinline__ unsigned box_key(const float* t1, const float* t2, float x, float y, float h) {
    return spread4(coarse_cell(t1, x - h)) | spread4(coarse_cell(t2, y - h)) << 1 |
           spread4(coarse_cell(t1, x + h)) << 2 | spread4(coarse_cell(t2, y + h)) << 3;
}

// Writes out[rank] = pos for every position pos < m of a grid, ranks in
// ascending order of the 16-bit keys s_key[pos]: a counting sort on the top
// twelve bits (shared-memory atomics). With s_tmp (m more words of shared
// memory; m <= 65536) each bin of at most kOrderSortMax positions, most
// bins, is then sorted on the low four bits by one thread in shared memory;
// larger bins, where many queries share one box, keep the atomics' order,
// so the work stays O(m). Without s_tmp the low bits are ignored. Called by
// the whole CTA after it has written s_key.
__device__ void write_key_order(const unsigned* s_key, int m, int* out, unsigned* s_tmp) {
    __shared__ int s_bin[kOrderBins];
    __shared__ int s_part[kOrderThreads];
    for (int b = threadIdx.x; b < kOrderBins; b += blockDim.x) s_bin[b] = 0;
    __syncthreads();
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) atomicAdd(&s_bin[s_key[pos] >> 4], 1);
    __syncthreads();
    // exclusive prefix over the bins: kPer bins per thread
    constexpr int kPer = kOrderBins / kOrderThreads;
    int acc = 0;
    for (int q = 0; q < kPer; ++q) acc += s_bin[threadIdx.x * kPer + q];
    s_part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < kOrderThreads; ++t) {
            const int v = s_part[t];
            s_part[t] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = s_part[threadIdx.x];
    for (int q = 0; q < kPer; ++q) {
        const int b = threadIdx.x * kPer + q;
        const int v = s_bin[b];
        s_bin[b] = run;
        run += v;
    }
    __syncthreads();
    if (!s_tmp) {
        for (int pos = threadIdx.x; pos < m; pos += blockDim.x) out[atomicAdd(&s_bin[s_key[pos] >> 4], 1)] = pos;
        return;
    }
    // entries (low key bits << 16 | pos): their order is the order wanted
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) {
        const unsigned key = s_key[pos];
        s_tmp[atomicAdd(&s_bin[key >> 4], 1)] = (key & 15u) << 16 | static_cast<unsigned>(pos);
    }
    __syncthreads();
    // s_bin[b] is now the end of bin b
    for (int b = threadIdx.x; b < kOrderBins; b += blockDim.x) {
        const int lo = b == 0 ? 0 : s_bin[b - 1], hi = s_bin[b];
        if (hi - lo > kOrderSortMax) continue;
        for (int r = lo + 1; r < hi; ++r) {
            const unsigned v = s_tmp[r];
            int t = r;
            while (t > lo && s_tmp[t - 1] > v) {
                s_tmp[t] = s_tmp[t - 1];
                --t;
            }
            s_tmp[t] = v;
        }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < m; r += blockDim.x) out[r] = static_cast<int>(s_tmp[r] & 0xffffu);
}

// Count order of one count group per CTA: boxes of the largest eps of the
// group's pairs on the node grid. Dynamic shared memory: corder_ld keys,
// then, with `sort_low`, corder_ld words for write_key_order's bins.
__global__ void __launch_bounds__(kOrderThreads) grid_count_order_kernel(GridArgs A, int sort_low) {
    extern __shared__ unsigned s_key[];
    __shared__ float s_t[2][16];
    const CountGroup grp = A.groups[blockIdx.x];
    const GridNode nd = A.nodes[grp.node];
    const float* eps = grp.side ? A.eps_b : A.eps_a;
    const int m = nd.m;
    if (threadIdx.x < 32) {
        const int L = threadIdx.x & 15;
        const float* e = threadIdx.x < 16 ? nd.e1 : nd.e2;
        s_t[threadIdx.x >> 4][L] = L < 15 ? e[2 * L + 1] : __int_as_float(0x7fc00000);
    }
    __syncthreads();
    long long o[kCountGroup];
#pragma unroll
    for (int p = 0; p < kCountGroup; ++p) o[p] = A.pairs[grp.pairs[p]].scratch;  // unused slots repeat pairs[0]
    // the grid's coordinates in storage order (coalesced)
    const float* x1 = nd.sx + static_cast<long long>(nd.c1) * m;
    const float* x2 = nd.c2 >= 0 ? nd.sx + static_cast<long long>(nd.c2) * m : nullptr;
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) {
        const int j = __ldg(nd.perm + pos);
        float e = __ldg(eps + o[0] + j);
#pragma unroll
        for (int p = 1; p < kCountGroup; ++p) e = fmaxf(e, __ldg(eps + o[p] + j));
        s_key[pos] = box_key(s_t[0], s_t[1], __ldg(x1 + pos), x2 ? __ldg(x2 + pos) : 0.f, e);
    }
    __syncthreads();
    write_key_order(s_key, m, A.corder + static_cast<long long>(blockIdx.x) * A.corder_ld,
                    sort_low ? s_key + A.corder_ld : nullptr);
}

// Search order: cells in kOrderBlock x kOrderBlock blocks, blocks in Z
// order, and within a block the queries by size class. Box Z codes of the
// estimates, which serve the counts, made the search slower (197 against
// 175 ms per 8192-pair batch at m = 10000): a warp's queries then spread
// over more cells than its seed rectangle allows, and its lists fill later.
constexpr int kOrderBlocks = (kGridMaxG + kOrderBlock - 1) / kOrderBlock;  // per axis
constexpr int kOrderClasses = 64;
static_assert(kOrderBlocks * kOrderBlocks * kOrderClasses == kOrderBins, "one counting-sort bin per class");

__device__ __forceinline__ unsigned block_zcode(int bx, int by) {
    unsigned z = 0;
#pragma unroll
    for (int b = 0; b < 3; ++b) z |= ((bx >> b) & 1u) << (2 * b + 1) | ((by >> b) & 1u) << (2 * b);
    return z;
}

// Size class of a box size e >= 0: its quarter octave (the float's exponent
// and top two mantissa bits; +inf and NaN land in the top class).
__device__ __forceinline__ unsigned size_bits(float e) {
    return isnan(e) ? 0xffffffffu : __float_as_uint(fmaxf(e, 0.f)) >> 21;
}

// Search order of one pair per CTA: the size class of the geometric mean of
// the two nodes' scale estimates, which follows the k-th joint distance
// closely enough to group queries with similar boxes (rank correlation 0.89
// with it, against 0.86 for the larger estimate, in a CPU model of the
// protein trajectories); the smallest class present becomes class 0. Dynamic
// shared memory: m keys.
__global__ void __launch_bounds__(kOrderThreads) grid_pair_order_kernel(const KsgPairDesc* pairs,
                                                                       const GridPair* gps,
                                                                       const GridNode* nodes) {
    extern __shared__ unsigned s_key[];
    __shared__ unsigned s_lo;
    const GridPair gp = gps[blockIdx.x];
    const GridNode na = nodes[gp.a], nb = nodes[gp.b];
    const int m = pairs[blockIdx.x].m, G = na.G;
    if (threadIdx.x == 0) s_lo = 0xffffffffu;
    __syncthreads();
    unsigned lo = 0xffffffffu;
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) {
        const int j = __ldg(gp.perm + pos);
        s_key[pos] = size_bits(sqrtf(__ldg(na.est + j) * __ldg(nb.est + j)));
        lo = min(lo, s_key[pos]);
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    if ((threadIdx.x & 31) == 0) atomicMin(&s_lo, lo);
    __syncthreads();
    lo = s_lo;
    for (int pos = threadIdx.x; pos < m; pos += blockDim.x) {
        const int j = __ldg(gp.perm + pos);
        const int row = __ldg(na.cell + j) / G, col = __ldg(nb.cell + j) / G;
        const unsigned d = s_key[pos] - lo;
        const unsigned cls = d < static_cast<unsigned>(kOrderClasses) ? d : kOrderClasses - 1;
        s_key[pos] = (block_zcode(row / kOrderBlock, col / kOrderBlock) * kOrderClasses + cls) << 4;
    }
    __syncthreads();
    write_key_order(s_key, m, gp.qpos, nullptr);
}

// One CTA per row.
__global__ void grid_gather_kernel(const GatherRow* rows, int d, int* fault) {
    const GatherRow g = rows[blockIdx.x];
    const float inf = __int_as_float(0x7f800000);
    for (int s = threadIdx.x; s < g.ld_out; s += blockDim.x) {
        int f = 0;
        if (s < g.m) {
            f = __ldg(g.fmap + s);
            if (f < 0 || f >= g.ld) {
                atomicOr(fault, FAULT_BAD_INDEX);
                f = 0;
            }
        }
        for (int c = 0; c < d; ++c) {
            g.out[static_cast<long long>(c) * g.ld_out + s] =
                s < g.m ? __ldg(g.x + static_cast<long long>(c) * g.ld + f) : inf;
        }
    }
}

template <int D>
void launch_pass1(const GridArgs& a, int kmax, int grid, cudaStream_t st) {
    const dim3 b(32 * kGridWarps);
    switch (kmax) {
        case 6: ksg_grid_pass1_kernel<D, 6, false><<<grid, b, 0, st>>>(a); break;
        case 8: ksg_grid_pass1_kernel<D, 8, false><<<grid, b, 0, st>>>(a); break;
        case 16: ksg_grid_pass1_kernel<D, 16, false><<<grid, b, 0, st>>>(a); break;
        case 32: ksg_grid_pass1_kernel<D, 32, false><<<grid, b, 0, st>>>(a); break;
        case 64: ksg_grid_pass1_kernel<D, 64, false><<<grid, b, 0, st>>>(a); break;
        default: fail(NSG_ERR_UNSUPPORTED, "no grid kernel for this k");
    }
}

}  // namespace

void append_count_groups(const GridPair* gps, int npairs, std::vector<CountGroup>& out) {
    for (int side = 0; side < 2; ++side) {
        // pairs by node, in first-appearance order of the nodes
        std::vector<std::pair<int, int>> keyed(npairs);
        for (int p = 0; p < npairs; ++p) keyed[p] = {side ? gps[p].b : gps[p].a, p};
        std::stable_sort(keyed.begin(), keyed.end(),
                         [](const std::pair<int, int>& x, const std::pair<int, int>& y) { return x.first < y.first; });
        for (size_t s = 0; s < keyed.size();) {
            CountGroup g{};
            g.node = keyed[s].first;
            g.side = side;
            while (s < keyed.size() && keyed[s].first == g.node && g.npairs < kCountGroup) {
                g.pairs[g.npairs++] = keyed[s].second;
                ++s;
            }
            for (int q = g.npairs; q < kCountGroup; ++q) g.pairs[q] = g.pairs[0];
            out.push_back(g);
        }
    }
}

int grid_cells_per_axis(int m) {
    int g = 1;
    while ((g + 1) * (g + 1) * 10 <= m && g < kGridMaxG) ++g;
    return g;
}

void grid_launch_nodes(GridNode* nodes, int nnodes, int d, bool est, cudaStream_t st) {
    if (nnodes <= 0) return;
    switch (d) {
        case 1:
            grid_node_kernel<1><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            if (est) grid_node_est_kernel<1><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            break;
        case 2:
            grid_node_kernel<2><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            if (est) grid_node_est_kernel<2><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            break;
        case 3:
            grid_node_kernel<3><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            if (est) grid_node_est_kernel<3><<<nnodes, kPrepThreads, 0, st>>>(nodes);
            break;
        default: invalid("d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

bool grid_orders_pay(long long search_warps, int sms) {
    return search_warps >= static_cast<long long>(kOrderMinWaves) * 32 * sms;
}

size_t grid_node_bytes(int m, int d) {
    auto a16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    const size_t mm = static_cast<size_t>(m);
    return a16(2 * kGridMaxG * sizeof(float)) + grid_index_bytes(grid_cells_per_axis(m)) +
           a16(mm * sizeof(unsigned short)) + a16(mm * sizeof(int)) + a16(mm * sizeof(float)) +
           a16(static_cast<size_t>(d) * mm * sizeof(float));
}

GridNode grid_node_at(unsigned char* base, const float* x, int ld, int m) {
    auto a16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    const size_t mm = static_cast<size_t>(m);
    GridNode n{};
    n.x = x;
    n.ld = ld;
    n.m = m;
    n.G = grid_cells_per_axis(m);
    n.e1 = reinterpret_cast<float*>(base);
    n.e2 = n.e1 + kGridMaxG;
    base += a16(2 * kGridMaxG * sizeof(float));
    n.start = reinterpret_cast<int*>(base);
    base += grid_index_bytes(n.G);
    n.cell = reinterpret_cast<unsigned short*>(base);
    base += a16(mm * sizeof(unsigned short));
    n.perm = reinterpret_cast<int*>(base);
    base += a16(mm * sizeof(int));
    n.est = reinterpret_cast<float*>(base);
    base += a16(mm * sizeof(float));
    n.sx = reinterpret_cast<float*>(base);
    return n;
}

size_t grid_pair_place(GridPair& g, size_t off, int m, int d) {
    auto a16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    const size_t mm = static_cast<size_t>(m);
    g.start = reinterpret_cast<int*>(off);
    off += grid_index_bytes(grid_cells_per_axis(m));
    g.perm = reinterpret_cast<int*>(off);
    off += a16(mm * sizeof(int));
    g.qpos = reinterpret_cast<int*>(off);
    off += a16(mm * sizeof(int));
    g.sx = reinterpret_cast<float*>(off);
    off += a16(static_cast<size_t>(2 * d) * mm * sizeof(float));
    return off;
}

void grid_pair_rebase(GridPair& g, const void* base) {
    const uintptr_t b = reinterpret_cast<uintptr_t>(base);
    g.start = reinterpret_cast<int*>(b + reinterpret_cast<uintptr_t>(g.start));
    g.perm = reinterpret_cast<int*>(b + reinterpret_cast<uintptr_t>(g.perm));
    g.qpos = reinterpret_cast<int*>(b + reinterpret_cast<uintptr_t>(g.qpos));
    g.sx = reinterpret_cast<float*>(b + reinterpret_cast<uintptr_t>(g.sx));
}

namespace {

// Largest dynamic shared memory the staged pair-grid kernel asks for.
constexpr size_t kPairStagedSmem = size_t(160) << 10;

template <int D>
void launch_pairs(const KsgPairDesc* pairs, GridPair* gps, const GridNode* nodes, int npairs, int max_m,
                  cudaStream_t st) {
    const int mpad = (max_m + 3) & ~3;
    const size_t smem = sizeof(int) * 2 * static_cast<size_t>(mpad);
    if (smem <= kPairStagedSmem) {
        // set on every launch: the attribute belongs to the current device
        NSG_CUDA(cudaFuncSetAttribute(grid_pair_staged_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(kPairStagedSmem)));
        grid_pair_staged_kernel<D><<<npairs, kPrepThreads, smem, st>>>(pairs, gps, nodes, mpad);
    } else {
        grid_pair_kernel<D><<<npairs, kPrepThreads, 0, st>>>(pairs, gps, nodes);
    }
}

}  // namespace

int grid_launch_pairs(const KsgPairDesc* pairs, GridPair* gps, const GridNode* nodes, int npairs,
                      int max_m, int d, bool order, cudaStream_t st) {
    if (npairs <= 0) return 0;
    switch (d) {
        case 1: launch_pairs<1>(pairs, gps, nodes, npairs, max_m, st); break;
        case 2: launch_pairs<2>(pairs, gps, nodes, npairs, max_m, st); break;
        case 3: launch_pairs<3>(pairs, gps, nodes, npairs, max_m, st); break;
        default: invalid("d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
    if (!order || max_m > kOrderMaxM) return 0;
    // set on every launch: the attribute belongs to the current device
    NSG_CUDA(cudaFuncSetAttribute(grid_pair_order_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sizeof(unsigned) * kOrderMaxM)));
    grid_pair_order_kernel<<<npairs, kOrderThreads, sizeof(unsigned) * static_cast<size_t>(max_m), st>>>(
        pairs, gps, nodes);
    NSG_CUDA(cudaGetLastError());
    return 1;
}

void grid_launch_search(const GridArgs& a, int d, int kmax, int grid, bool tie_record, cudaStream_t st) {
    if (tie_record) {
        grid_launch_search_rec(a, d, kmax, grid, st);
        return;
    }
    switch (d) {
        case 1: launch_pass1<1>(a, kmax, grid, st); break;
        case 2: launch_pass1<2>(a, kmax, grid, st); break;
        case 3: launch_pass1<3>(a, kmax, grid, st); break;
        default: invalid("d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

GridArgs grid_launch_count_order(const GridArgs& a, cudaStream_t st) {
    GridArgs c = a;
    if (c.corder && c.corder_ld <= kOrderMaxM && c.ngroups > 0) {
        // keys, and up to kOrderSortLowMaxM the bins' second copy
        const int sort_low = c.corder_ld <= kOrderSortLowMaxM ? 1 : 0;
        const size_t smem = sizeof(unsigned) * static_cast<size_t>(c.corder_ld) * (1 + sort_low);
        // set on every launch: the attribute belongs to the current device
        NSG_CUDA(cudaFuncSetAttribute(grid_count_order_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(sizeof(unsigned) * kOrderMaxM)));
        grid_count_order_kernel<<<c.ngroups, kOrderThreads, smem, st>>>(c, sort_low);
        NSG_CUDA(cudaGetLastError());
    } else {
        c.corder = nullptr;
    }
    return c;
}

void grid_launch_count_kernel(const GridArgs& c, int d, int grid, cudaStream_t st) {
    const dim3 b(32 * kGridWarps);
    switch (d) {
        case 1: ksg_grid_count_kernel<1><<<grid, b, 0, st>>>(c); break;
        case 2: ksg_grid_count_kernel<2><<<grid, b, 0, st>>>(c); break;
        case 3: ksg_grid_count_kernel<3><<<grid, b, 0, st>>>(c); break;
        default: invalid("d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

void grid_launch_counts(const GridArgs& a, int d, int grid, cudaStream_t st) {
    grid_launch_count_kernel(grid_launch_count_order(a, st), d, grid, st);
}

void grid_launch_combine(const KsgPairDesc* pairs, int npairs, const int* cnt_a, const int* cnt_b,
                         const float* psi, float* psum, int* nx, int* ny, cudaStream_t st) {
    if (npairs <= 0) return;
    grid_combine_kernel<<<npairs, 256, 0, st>>>(pairs, cnt_a, cnt_b, psi, psum, nx, ny);
    NSG_CUDA(cudaGetLastError());
}

void grid_launch_gather(const GatherRow* rows, int nrows, int d, int* fault, cudaStream_t st) {
    if (nrows <= 0) return;
    grid_gather_kernel<<<nrows, 256, 0, st>>>(rows, d, fault);
    NSG_CUDA(cudaGetLastError());
}

int grid_search_ctas_per_sm(int d, int kmax) {
    int n = 0;
    const int b = 32 * kGridWarps;
    cudaError_t e = cudaSuccess;
#define NSG_OCC(D_, K_) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ksg_grid_pass1_kernel<D_, K_, false>, b, 0)
    switch (d * 100 + kmax) {
        case 106: NSG_OCC(1, 6); break;
        case 108: NSG_OCC(1, 8); break;
        case 116: NSG_OCC(1, 16); break;
        case 132: NSG_OCC(1, 32); break;
        case 164: NSG_OCC(1, 64); break;
        case 206: NSG_OCC(2, 6); break;
        case 208: NSG_OCC(2, 8); break;
        case 216: NSG_OCC(2, 16); break;
        case 232: NSG_OCC(2, 32); break;
        case 264: NSG_OCC(2, 64); break;
        case 306: NSG_OCC(3, 6); break;
        case 308: NSG_OCC(3, 8); break;
        case 316: NSG_OCC(3, 16); break;
        case 332: NSG_OCC(3, 32); break;
        case 364: NSG_OCC(3, 64); break;
        default: return 1;
    }
#undef NSG_OCC
    cuda_check(e, "occupancy query");
    return n > 0 ? n : 1;
}

int grid_count_ctas_per_sm(int d) {
    int n = 0;
    const int b = 32 * kGridWarps;
    cudaError_t e = cudaSuccess;
    switch (d) {
        case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ksg_grid_count_kernel<1>, b, 0); break;
        case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ksg_grid_count_kernel<2>, b, 0); break;
        case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ksg_grid_count_kernel<3>, b, 0); break;
        default: return 1;
    }
    cuda_check(e, "occupancy query");
    return n > 0 ? n : 1;
}

}  // namespace nsg
