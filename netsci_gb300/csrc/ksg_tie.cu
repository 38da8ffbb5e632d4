// Tie resolution for the KSG count kernel.
//
// A sample whose k-th and (k+1)-th nearest joint distances are equal (and
// non-zero) has a neighbour set that the reference CPU path picks by the
// order its std::sort leaves equal distances in
// (netcalc/src/mutual_information_cpu.cpp:48-77). The search kernels append
// such samples to a list, unless every frame at the tied distance has the same
// marginal pair (then any order gives the same eps); this kernel takes the list
// one warp at a time:
//
//   1. the warp writes the sample's full joint-distance row (the reference's
//      arithmetic) and the identity index array into its scratch rows;
//   2. the warp replays the reference sort's order on the prefix that holds
//      the neighbours (the steps sort_prefix.h restates, partitions found 32
//      elements at a time with ballots);
//   3. the lanes holding sorted positions 1..k compute eps_a / eps_b, a warp
//      max-reduction combines them;
//   4. the marginal counts are recounted over all frames with warp ballots
//      and population counts, and the sample's psi term is rewritten.
//
// Runs between the count kernel and the finalize kernel, with a fixed grid
// that walks the tie list through an atomic counter (an empty list costs one
// launch that returns at once).
#include "common.cuh"
#include "engine.h"
#include "ksg.cuh"
#include "sort_prefix.h"

namespace nsg {
namespace {

constexpr int kWarpsPerCta = 8;
constexpr int kCtasPerSm = 6;  // latency-bound: 48 warps per SM (40 registers) replays about 6% faster than 32
constexpr int kStack = 64;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int tie_frame(const int* __restrict__ fmap, int s, int ld, int* fault) {
    if (!fmap) return s;
    const int f = __ldg(fmap + s);
    if (f < 0 || f >= ld) {
        atomicOr(fault, FAULT_BAD_INDEX);
        return 0;
    }
    return f;
}

template <int D>
__device__ __forceinline__ float tie_marginal(const float (&q)[D], const float* __restrict__ x,
                                              int ld, int src) {
    float v = fabsf(q[0] - __ldg(x + src));
#pragma unroll
    for (int c = 1; c < D; ++c) v = fmaxf(v, fabsf(q[c] - __ldg(x + (size_t)c * ld + src)));
    return v;
}

// sort_prefix_like_reference (sort_prefix.h) run by a whole warp: the same
// segments, pivots and swaps, with each unguarded partition found 32
// positions at a time. The partition of [first+1, last) around pk swaps the
// t-th element from the left that is not below pk (a left stopper) with the
// t-th element from the right that is not above pk (a right stopper, the
// scan may reach the pivot itself at `first`) while the former lies left of
// the latter; the elements between them are untouched until then, so the
// stoppers can be read from the array as it was. The cut is the first left
// stopper past the last swap, or that swap's right position if it comes
// first. The pairs found by one round of ballots touch distinct positions,
// so lane t swaps the round's t-th pair, all at once. Lane 0 holds the
// segment stack; all lanes load and vote. A segment whose depth budget runs
// out is heapsorted by lane 0 (heap_sort_like_reference). Same result as the
// serial routine, element for element.
__device__ bool sort_prefix_warp(const float* key, int* idx, int n, int T, SortSegment* stack,
                                 int cap, int lane) {
    if (n <= 1) return true;
    constexpr int kThreshold = 16;
    int top = 0;
    if (lane == 0) stack[0] = {0, n, 2 * floor_log2(n)};
    top = 1;
    int prefix_end = 0;
    while (top > 0) {
        --top;
        SortSegment sg{};
        if (lane == 0) sg = stack[top];
        int first = __shfl_sync(kFull, sg.first, 0);
        int last = __shfl_sync(kFull, sg.last, 0);
        int depth = __shfl_sync(kFull, sg.depth, 0);
        while (last - first > kThreshold) {
            if (depth == 0) {
                if (lane == 0) heap_sort_like_reference(key, idx + first, last - first);
                __syncwarp();
                break;
            }
            --depth;
            // median of three moved to `first` (lane 0)
            if (lane == 0) {
                const int a = first + 1, b = first + (last - first) / 2, c = last - 1;
                const float ka = key[idx[a]], kb = key[idx[b]], kc = key[idx[c]];
                int pick;
                if (ka < kb) {
                    if (kb < kc) pick = b;
                    else if (ka < kc) pick = c;
                    else pick = a;
                } else if (ka < kc) {
                    pick = a;
                } else if (kb < kc) {
                    pick = c;
                } else {
                    pick = b;
                }
                const int t = idx[first];
                idx[first] = idx[pick];
                idx[pick] = t;
            }
            __syncwarp();
            const float pk = key[idx[first]];
            // left stoppers from first+1 up, right stoppers from last-1 down
            int lbase = first + 1, rbase = last - 1;  // next chunk starts
            int lchunk = 0, rchunk = 0;               // current chunk starts
            unsigned lmask = 0, rmask = 0;
            bool lend = false, rend = false;
            int prev_r = -1;                          // right position of the last swap
            int cut;
            for (;;) {
                while (lmask == 0 && !lend) {
                    if (lbase >= last) {
                        lend = true;
                        break;
                    }
                    const int p = lbase + lane;
                    const bool st = p < last && !(key[idx[p]] < pk);
                    lmask = __ballot_sync(kFull, st);
                    lchunk = lbase;
                    lbase += 32;
                }
                while (rmask == 0 && !rend) {
                    if (rbase < first) {
                        rend = true;
                        break;
                    }
                    const int p = rbase - lane;
                    const bool st = p >= first && !(pk < key[idx[p]]);
                    rmask = __ballot_sync(kFull, st);
                    rchunk = rbase;
                    rbase -= 32;
                }
                // the median of three leaves stoppers on both sides; running
                // out of either means a broken invariant, reported as failure
                if (rend) return false;
                // the t-th left stopper of lmask pairs with the t-th right
                // stopper of rmask while it lies left of it; those pairs form
                // a prefix of t and are swapped together, lane t taking pair t
                const int npair = lend ? 0 : min(__popc(lmask), __popc(rmask));
                int lp = 0x7fffffff, rp = -1;
                if (lane < npair) {
                    lp = lchunk + static_cast<int>(__fns(lmask, 0, lane + 1));
                    rp = rchunk - static_cast<int>(__fns(rmask, 0, lane + 1));
                }
                const bool swap = lane < npair && lp < rp;
                const int c = __popc(__ballot_sync(kFull, swap));
                if (swap) {
                    const int t = idx[lp];
                    idx[lp] = idx[rp];
                    idx[rp] = t;
                }
                __syncwarp();
                if (c > 0) prev_r = __shfl_sync(kFull, rp, c - 1);
                if (c == npair && !lend) {
                    // every pair of the round swapped: drop them, continue
                    for (int q = 0; q < c; ++q) {
                        lmask &= lmask - 1;
                        rmask &= rmask - 1;
                    }
                    continue;
                }
                // pair c crosses (or no left stopper is left)
                const int lpos = lend ? 0x7fffffff : __shfl_sync(kFull, lp, c);
                cut = prev_r < 0 ? lpos : min(lpos, prev_r);
                break;
            }
            __syncwarp();
            if (cut >= last) return false;
            if (cut < T) {
                if (top >= cap) return false;
                if (lane == 0) stack[top] = {cut, last, depth};
                ++top;
            }
            last = cut;
        }
        if (first < T && last > prefix_end) prefix_end = last;
    }
    __syncwarp();
    // insertion sort of [0, prefix_end) (at most a few dozen elements)
    if (lane == 0) {
        for (int i = 1; i < prefix_end; ++i) {
            const int v = idx[i];
            const float kv = key[v];
            int j = i;
            while (j > 0 && kv < key[idx[j - 1]]) {
                idx[j] = idx[j - 1];
                --j;
            }
            idx[j] = v;
        }
    }
    __syncwarp();
    return true;
}

template <int D>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kCtasPerSm) ksg_tie_kernel(KsgTieArgs A) {
    __shared__ SortSegment s_stack[kWarpsPerCta][kStack];
    const int lane = threadIdx.x & 31;
    const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    float* dz = A.dz + warp * A.stride;
    int* idx = A.idx + warp * A.stride;
    const int total = min(*A.tie_count, A.tie_cap);
    for (;;) {
        int e = 0;
        if (lane == 0) e = atomicAdd(A.tie_next, 1);
        e = __shfl_sync(kFull, e, 0);
        if (e >= total) return;
        const KsgTie t = A.ties[e];
        const KsgPairDesc P = A.pairs[t.pair];
        const int m = P.m, ld = P.ld;
        const int* __restrict__ fmap = P.fmap;
        const float* __restrict__ xa = P.xa;
        const float* __restrict__ xb = P.xb;
        if (P.m > A.stride) {  // the planner sizes rows for every pair
            if (lane == 0) atomicOr(A.fault, FAULT_BAD_INDEX);
            continue;
        }
        const int sq = tie_frame(fmap, t.q, ld, A.fault);
        float qa[D], qb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            qa[c] = __ldg(xa + (size_t)c * ld + sq);
            qb[c] = __ldg(xb + (size_t)c * ld + sq);
        }
        for (int j = lane; j < m; j += 32) {
            const int s = tie_frame(fmap, j, ld, A.fault);
            dz[j] = fmaxf(tie_marginal<D>(qa, xa, ld, s), tie_marginal<D>(qb, xb, ld, s));
            idx[j] = j;
        }
        __syncwarp();
        const int ok = sort_prefix_warp(dz, idx, m, A.k + 1, s_stack[threadIdx.x >> 5], kStack, lane) ? 1 : 0;
        __syncwarp();
        if (!ok) {
            if (lane == 0) atomicOr(A.fault, FAULT_TIE_UNRESOLVED);
            continue;
        }
        // eps over sorted positions 1..k (k can exceed the warp's 31 lanes)
        float ea = 0.f, eb = 0.f;
        for (int p = 1 + lane; p <= A.k; p += 32) {
            const int s = tie_frame(fmap, idx[p], ld, A.fault);
            ea = fmaxf(ea, tie_marginal<D>(qa, xa, ld, s));
            eb = fmaxf(eb, tie_marginal<D>(qb, xb, ld, s));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            ea = fmaxf(ea, __shfl_xor_sync(kFull, ea, off));
            eb = fmaxf(eb, __shfl_xor_sync(kFull, eb, off));
        }
        int ca = 0, cb = 0;
        for (int j0 = 0; j0 < m; j0 += 32) {
            const int j = j0 + lane;
            bool pa = false, pb = false;
            if (j < m) {
                const int s = tie_frame(fmap, j, ld, A.fault);
                pa = tie_marginal<D>(qa, xa, ld, s) <= ea;
                pb = tie_marginal<D>(qb, xb, ld, s) <= eb;
            }
            ca += __popc(__ballot_sync(kFull, pa));
            cb += __popc(__ballot_sync(kFull, pb));
        }
        if (lane == 0) {
            const long long o = P.scratch + t.q;
            const int nx = min(max(ca - 1, 0), m);
            const int ny = min(max(cb - 1, 0), m);
            A.psum[o] = __fadd_rn(__ldg(A.psi + nx), __ldg(A.psi + ny));
            if (A.nx) A.nx[o] = nx;
            if (A.ny) A.ny[o] = ny;
            if (A.eps_x) A.eps_x[o] = ea;
            if (A.eps_y) A.eps_y[o] = eb;
        }
        __syncwarp();
    }
}

}  // namespace

int ksg_tie_warps() { return sm_count() * kCtasPerSm * kWarpsPerCta; }

void ksg_launch_ties(const KsgTieArgs& a, int d, cudaStream_t st) {
    const int grid = sm_count() * kCtasPerSm;
    const int threads = kWarpsPerCta * 32;
    switch (d) {
        case 1: ksg_tie_kernel<1><<<grid, threads, 0, st>>>(a); break;
        case 2: ksg_tie_kernel<2><<<grid, threads, 0, st>>>(a); break;
        case 3: ksg_tie_kernel<3><<<grid, threads, 0, st>>>(a); break;
        default: fail(NSG_ERR_INVALID, "d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

// The same kernel on a caller-chosen number of CTAs (the caller's scratch
// holds kWarpsPerCta * ctas rows).
void ksg_launch_ties_ctas(const KsgTieArgs& a, int d, int ctas, cudaStream_t st) {
    const int threads = kWarpsPerCta * 32;
    switch (d) {
        case 1: ksg_tie_kernel<1><<<ctas, threads, 0, st>>>(a); break;
        case 2: ksg_tie_kernel<2><<<ctas, threads, 0, st>>>(a); break;
        case 3: ksg_tie_kernel<3><<<ctas, threads, 0, st>>>(a); break;
        default: fail(NSG_ERR_INVALID, "d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
