// KSG mutual-information count kernel (templated body; instantiated per
// dimension in ksg_d1.cu, ksg_d2.cu, ksg_d3.cu so the builds run in parallel).
//
// What one CTA does for a work item (pair p, query samples q0..q1):
//
//   * Each thread owns R query samples i (strided by the CTA size so that
//     neighbouring threads own neighbouring samples) and keeps their 2d
//     coordinates in registers.
//   * Pass 1 streams every frame j of the pair through a shared-memory tile
//     (structure-of-arrays: one row of `frames` floats per coordinate plane),
//     reads frames four at a time as float4 broadcasts, and forms the joint
//     Chebyshev distance dz = max(d_a, d_b). A per-sample ascending list of
//     the k smallest (dz, j) over the frames other than the sample itself
//     lives in registers, with a flag for a frame outside the list at the
//     k-th distance (see admit()); it is only touched when the minimum dz of
//     the four frames is at most the list's last entry, which after the
//     first few hundred frames is rare, and then by one branch-free bubble
//     step per candidate.
//   * eps_a / eps_b are the largest marginal distances over list positions
//     1..k (netcalc/src/mutual_information_cpu.cpp:54-77).
//   * Pass 2 streams the frames again and counts d_a <= eps_a and
//     d_b <= eps_b over all j (self included, then minus one,
//     netcalc/src/mutual_information_cpu.cpp:78-109).
//   * The sample's psi[n_x] + psi[n_y] (float add, :110) goes to the pair's
//     scratch row; ksg_final_kernel sums the row in sample order.
//
// Why the list needs no index tie-break: position 0 of the reference's sorted
// row holds a frame at distance 0 (the sample itself or an exact duplicate,
// all with zero marginals), and when the values at positions k and k+1
// differ, positions 1..k hold exactly the frames with dz <= that k-th value,
// whatever order equal values were offered in. Here position 0 is the first
// zero-distance frame offered, left out of the list, and `tied` says whether
// positions k and k+1 are equal. When they are (and non-zero) the
// reference's choice depends on its sort; the sample goes to the tie list
// and ksg_tie_kernel recomputes it. Frames past m are staged as +inf and
// are never offered.
//
// Runtime k with KMAX >= k+2: the list has KN = KMAX-2 slots, the first
// KN-k of them -inf sentinels that never move, so the live entries occupy the
// last k slots and the admission bound is always slot KN-1 (a static
// register index).
//
// Arithmetic: one rounded subtraction per coordinate, then exact abs/max, and
// exact compares, so distances, eps and counts are bit-identical to the
// reference CPU path.
#pragma once

#include "common.cuh"
#include "ksg.cuh"

namespace nsg {
namespace ksgk {

// Insert (v, j) into the ascending list (bd, bj), dropping its last entry;
// the caller has checked v < bd[KMAX-1]. Branch-free: every slot compares
// with v once; a slot holding a larger value takes its left neighbour, or v
// where that neighbour is not larger. v lands behind entries equal to it.
// Sentinel slots (-inf) never move.
template <int KMAX>
__device__ __forceinline__ void list_insert(float (&bd)[KMAX], int (&bj)[KMAX], float v, int j) {
    bool gt[KMAX];
#pragma unroll
    for (int s = 0; s < KMAX; ++s) gt[s] = v < bd[s];
#pragma unroll
    for (int s = KMAX - 1; s > 0; --s) {
        if (gt[s]) {
            bd[s] = gt[s - 1] ? bd[s - 1] : v;
            bj[s] = gt[s - 1] ? bj[s - 1] : j;
        }
    }
    if (gt[0]) {
        bd[0] = v;
        bj[0] = j;
    }
}

// Offer frame j at joint distance v to a sample's list of the KN nearest
// frames other than the sample itself (sorted; the last entry U bounds
// admission: a frame enters when strictly nearer). The first frame at
// distance 0 stands for the sample (self_seen) and is not listed: frames at
// distance 0 have both marginal distances 0, so which of them is left out
// changes neither eps nor the counts. `tied` records whether a frame outside
// the list lies at distance exactly U: one rejected at U, or evicted while U
// stayed the same. U only decreases, and no frame outside the list can lie at
// a new, smaller U, so a decrease clears the flag. Callers offer only frames
// with v <= U.
template <int KN>
__device__ __forceinline__ void admit(float (&bd)[KN], int (&bj)[KN], bool& self_seen, bool& tied,
                                      float v, int j) {
    const float u = bd[KN - 1];
    if (v == 0.f && !self_seen) {
        self_seen = true;
    } else if (v < u) {
        list_insert<KN>(bd, bj, v, j);
        tied = bd[KN - 1] == u;
    } else {
        tied = true;  // v == u
    }
}

// Variant 0: scalar subtractions, two-input max chain.
// Variant 1: packed f32x2 subtractions (two frames per instruction) and the
//            three-input max.
// Variant 2: packed f32x2 subtractions, two-input max chain.
template <int D, int VARIANT>
struct Marg {
    // Marginal Chebyshev distances of the four frames of a group (frames in
    // the x,y,z,w lanes of g[c]) from the query coordinates q[c].
    __device__ __forceinline__ static void four(const float (&q)[D], const float4 (&g)[D],
                                                float (&out)[4]) {
        if constexpr (VARIANT == 0) {
            float a[4] = {fabsf(q[0] - g[0].x), fabsf(q[0] - g[0].y), fabsf(q[0] - g[0].z),
                          fabsf(q[0] - g[0].w)};
#pragma unroll
            for (int c = 1; c < D; ++c) {
                a[0] = fmaxf(a[0], fabsf(q[c] - g[c].x));
                a[1] = fmaxf(a[1], fabsf(q[c] - g[c].y));
                a[2] = fmaxf(a[2], fabsf(q[c] - g[c].z));
                a[3] = fmaxf(a[3], fabsf(q[c] - g[c].w));
            }
#pragma unroll
            for (int f = 0; f < 4; ++f) out[f] = a[f];
        } else {
            float lo[D][4];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const float2 u = nsg_sub2(make_float2(q[c], q[c]), make_float2(g[c].x, g[c].y));
                const float2 v = nsg_sub2(make_float2(q[c], q[c]), make_float2(g[c].z, g[c].w));
                lo[c][0] = fabsf(u.x);
                lo[c][1] = fabsf(u.y);
                lo[c][2] = fabsf(v.x);
                lo[c][3] = fabsf(v.y);
            }
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if constexpr (D == 1) {
                    out[f] = lo[0][f];
                } else if constexpr (D == 2) {
                    out[f] = fmaxf(lo[0][f], lo[1][f]);
                } else {
                    if constexpr (VARIANT == 1) {
                        out[f] = nsg_max3(lo[0][f], lo[1][f], lo[2][f]);
                    } else {
                        out[f] = fmaxf(fmaxf(lo[0][f], lo[1][f]), lo[2][f]);
                    }
                }
            }
        }
    }
};

// Source frame of sample s: fmap[s] when a frame map is given. A map entry
// outside [0, ld) is recorded in the fault word and read as frame 0.
__device__ __forceinline__ int frame_of(const int* __restrict__ fmap, int s, int ld, int* fault) {
    if (!fmap) return s;
    const int f = __ldg(fmap + s);
    if (f < 0 || f >= ld) {
        atomicOr(fault, FAULT_BAD_INDEX);
        return 0;
    }
    return f;
}

template <int D>
__device__ __forceinline__ float marginal_at(const float (&q)[D], const float* __restrict__ x,
                                             int ld, int src) {
    float v = fabsf(q[0] - __ldg(x + src));
#pragma unroll
    for (int c = 1; c < D; ++c) v = fmaxf(v, fabsf(q[c] - __ldg(x + (size_t)c * ld + src)));
    return v;
}

// ---- per-tile pieces shared by the staged kernels -----------------------------

// Pass 1 over one tile: planes of the tile at tile[c*stride + f], frames
// j0 .. j0+jn-1 (frames past the pair's end hold +inf).
template <int D, int KN, int R, int VARIANT>
__device__ __forceinline__ void pass1_tile(const float* tile, int stride, int j0, int jn,
                                           const float (&qa)[R][D], const float (&qb)[R][D],
                                           float (&bd)[R][KN], int (&bj)[R][KN], bool (&self_seen)[R],
                                           bool (&tied)[R]) {
    const int ngroups = (jn + 3) >> 2;
    for (int g = 0; g < ngroups; ++g) {
        float4 ga[D], gb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            ga[c] = *reinterpret_cast<const float4*>(tile + c * stride + 4 * g);
            gb[c] = *reinterpret_cast<const float4*>(tile + (D + c) * stride + 4 * g);
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float da[4], db[4], dz[4];
            Marg<D, VARIANT>::four(qa[r], ga, da);
            Marg<D, VARIANT>::four(qb[r], gb, db);
#pragma unroll
            for (int f = 0; f < 4; ++f) dz[f] = fmaxf(da[f], db[f]);
            const float mn = nsg_min3(dz[0], dz[1], fminf(dz[2], dz[3]));
            if (mn <= bd[r][KN - 1]) {
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    if (dz[f] <= bd[r][KN - 1]) {
                        admit<KN>(bd[r], bj[r], self_seen[r], tied[r], dz[f], j0 + 4 * g + f);
                    }
                }
            }
        }
    }
}

// Pass 2 over one tile: marginal counts against eps, added up in floats
// from nsg_le_f32 within the tile (exact: at most J per lane) and then into
// the integer counts (7.6% less time per 8192-pair batch at m = 10000 than
// integer selects and adds). With CHECK, also
// looks at every frame whose joint distance equals a flagged sample's k-th
// distance wk and records in `mixed` whether any of them has marginals other
// than (ra, rb) -- the only case in which the reference's choice among tied
// frames can change eps.
template <int D, int R, int VARIANT, bool CHECK>
__device__ __forceinline__ void pass2_tile(const float* tile, int stride, int jn,
                                           const float (&qa)[R][D], const float (&qb)[R][D],
                                           const float (&ea)[R], const float (&eb)[R],
                                           int (&ca)[R], int (&cb)[R], const float (&wk)[R],
                                           const float (&ra)[R], const float (&rb)[R],
                                           bool (&mixed)[R]) {
    const int ngroups = (jn + 3) >> 2;
    float fa[R], fb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) fa[r] = fb[r] = 0.f;
    for (int g = 0; g < ngroups; ++g) {
        float4 ga[D], gb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            ga[c] = *reinterpret_cast<const float4*>(tile + c * stride + 4 * g);
            gb[c] = *reinterpret_cast<const float4*>(tile + (D + c) * stride + 4 * g);
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float da[4], db[4];
            Marg<D, VARIANT>::four(qa[r], ga, da);
            Marg<D, VARIANT>::four(qb[r], gb, db);
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                fa[r] += nsg_le_f32(da[f], ea[r]);
                fb[r] += nsg_le_f32(db[f], eb[r]);
                if constexpr (CHECK) {
                    if (fmaxf(da[f], db[f]) == wk[r] && (da[f] != ra[r] || db[f] != rb[r])) {
                        mixed[r] = true;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        ca[r] += static_cast<int>(fa[r]);
        cb[r] += static_cast<int>(fb[r]);
    }
}

// Query samples of this thread and their empty neighbour lists.
template <int D, int KN, int R, int NT>
__device__ __forceinline__ void load_queries(const KsgCountArgs& A, const KsgItem& w,
                                             const KsgPairDesc& P, int tid, float (&qa)[R][D],
                                             float (&qb)[R][D], int (&qi)[R],
                                             float (&bd)[R][KN], int (&bj)[R][KN], bool (&self_seen)[R],
                                             bool (&tied)[R]) {
    const float kInf = __int_as_float(0x7f800000);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        qi[r] = w.q0 + r * NT + tid;
        const bool valid = qi[r] < w.q1;
        const int src = valid ? frame_of(P.fmap, qi[r], P.ld, A.fault) : 0;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            qa[r][c] = valid ? __ldg(P.xa + (size_t)c * P.ld + src) : 0.f;
            qb[r][c] = valid ? __ldg(P.xb + (size_t)c * P.ld + src) : 0.f;
        }
    }
    // k live entries after nsent -inf sentinels: the k nearest frames other
    // than the sample (list positions 1..k of the reference's sorted row)
    const int nsent = KN - A.k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        self_seen[r] = false;
        tied[r] = false;
#pragma unroll
        for (int s = 0; s < KN; ++s) {
            bd[r][s] = s < nsent ? -kInf : kInf;
            bj[r][s] = -1;
        }
    }
}

// eps from list positions 1..k (slots nsent .. KN-1), and the tie test: a
// sample is flagged when another frame lies at its k-th distance wk (the flag
// `tied`) and wk is not zero; then the reference's choice among the frames at
// that distance comes from its sort. (ra, rb) are the marginals of the frame
// at position k; pass 2 checks whether every frame at distance wk has the
// same ones (for example copies of one frame in a bootstrap resample), in
// which case the choice cannot change eps and the flag is dropped.
template <int D, int KN, int R>
__device__ __forceinline__ void eps_and_ties(const KsgCountArgs& A, const KsgItem& w,
                                             const KsgPairDesc& P, const float (&qa)[R][D],
                                             const float (&qb)[R][D], const int (&qi)[R],
                                             const float (&bd)[R][KN], const int (&bj)[R][KN],
                                             const bool (&tied)[R], float (&ea)[R], float (&eb)[R],
                                             bool (&tie)[R], float (&wk)[R], float (&ra)[R], float (&rb)[R]) {
    const int nsent = KN - A.k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        ea[r] = 0.f;
        eb[r] = 0.f;
        ra[r] = 0.f;
        rb[r] = 0.f;
        const bool valid = qi[r] < w.q1;
        wk[r] = bd[r][KN - 1];
        tie[r] = valid && tied[r] && wk[r] > 0.f;
#pragma unroll
        for (int s = 0; s < KN; ++s) {
            const int j = bj[r][s];
            if (valid && s >= nsent && j >= 0 && j < P.m) {
                const int src = frame_of(P.fmap, j, P.ld, A.fault);
                const float da = marginal_at<D>(qa[r], P.xa, P.ld, src);
                const float db = marginal_at<D>(qb[r], P.xb, P.ld, src);
                ea[r] = fmaxf(ea[r], da);
                eb[r] = fmaxf(eb[r], db);
                if (s == KN - 1) {
                    ra[r] = da;
                    rb[r] = db;
                }
            }
        }
    }
}

// Samples whose tied frames differ in their marginals go to the tie list
// (ksg_tie_kernel recomputes them with the reference sort's order).
template <int R>
__device__ __forceinline__ void report_ties(const KsgCountArgs& A, const KsgItem& w,
                                            const int (&qi)[R], const bool (&tie)[R],
                                            const bool (&mixed)[R]) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (tie[r] && mixed[r]) {
            const int slot = atomicAdd(A.tie_count, 1);
            if (slot < A.tie_cap) {
                A.ties[slot] = KsgTie{w.pair, qi[r]};
            } else {
                atomicOr(A.fault, FAULT_TIE_OVERFLOW);
            }
        }
    }
}

template <int R>
__device__ __forceinline__ void write_outputs(const KsgCountArgs& A, const KsgItem& w,
                                              const KsgPairDesc& P, const int (&qi)[R],
                                              const float (&wk)[R], const float (&ea)[R],
                                              const float (&eb)[R], const int (&ca)[R],
                                              const int (&cb)[R]) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (qi[r] < w.q1) {
            const long long o = P.scratch + qi[r];
            // counts lie in [k, m-1] for finite inputs; the clamp keeps
            // non-finite inputs from indexing outside the psi table
            const int nx = min(max(ca[r] - 1, 0), P.m);
            const int ny = min(max(cb[r] - 1, 0), P.m);
            A.psum[o] = __fadd_rn(__ldg(A.psi + nx), __ldg(A.psi + ny));
            if (A.nx) A.nx[o] = nx;
            if (A.ny) A.ny[o] = ny;
            if (A.eps_x) A.eps_x[o] = ea[r];
            if (A.eps_y) A.eps_y[o] = eb[r];
            if (A.kdist) A.kdist[o] = wk[r];
        }
    }
}

// Staging with plain loads: every thread copies part of the tile
// (frame maps gathered here), frames past the pair's end set to +inf.
template <int D, int NT, int J>
__device__ __forceinline__ void stage_tile(float (&tile)[2 * D][J], const KsgPairDesc& P, int j0,
                                           int tid, int* fault) {
    const float kInf = __int_as_float(0x7f800000);
    for (int idx = tid; idx < 2 * D * J; idx += NT) {
        const int c = idx / J;
        const int f = idx - c * J;
        const int j = j0 + f;
        float v = kInf;
        if (j < P.m) {
            const int src = frame_of(P.fmap, j, P.ld, fault);
            v = c < D ? __ldg(P.xa + (size_t)c * P.ld + src)
                      : __ldg(P.xb + (size_t)(c - D) * P.ld + src);
        }
        tile[c][f] = v;
    }
}

template <int D, int KMAX, int R, int NT, int J, int VARIANT>
__global__ void __launch_bounds__(NT) ksg_count_kernel(KsgCountArgs A) {
    static_assert(J % (4 * 32) == 0, "tile must hold whole float4 groups");
    __shared__ __align__(16) float tile[2 * D][J];
    __shared__ int s_item;
    const int tid = threadIdx.x;

    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= A.nitems) return;
        const KsgItem w = A.items[item];
        const KsgPairDesc P = A.pairs[w.pair];
        const int m = P.m;

        float qa[R][D], qb[R][D];
        int qi[R];
        constexpr int KN = KMAX - 2;
        float bd[R][KN];
        int bj[R][KN];
        bool self_seen[R], tied[R];
        load_queries<D, KN, R, NT>(A, w, P, tid, qa, qb, qi, bd, bj, self_seen, tied);

        const int ntiles = (m + J - 1) / J;
        // ---- pass 1: k nearest joint neighbours ------------------------------
        for (int t = 0; t < ntiles; ++t) {
            const int j0 = t * J;
            __syncthreads();
            stage_tile<D, NT, J>(tile, P, j0, tid, A.fault);
            __syncthreads();
            pass1_tile<D, KN, R, VARIANT>(&tile[0][0], J, j0, min(J, m - j0), qa, qb, bd, bj, self_seen, tied);
        }
        float ea[R], eb[R], wk[R], ra[R], rb[R];
        bool tie[R], mixed[R];
        eps_and_ties<D, KN, R>(A, w, P, qa, qb, qi, bd, bj, tied, ea, eb, tie, wk, ra, rb);
        bool any_tie = false;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            mixed[r] = false;
            any_tie |= tie[r];
        }
        // warp-uniform: the tie-group check only runs in warps that need it
        any_tie = __any_sync(0xffffffffu, any_tie);

        // ---- pass 2: marginal counts ------------------------------------------
        int ca[R], cb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ca[r] = 0;
            cb[r] = 0;
        }
        for (int t = 0; t < ntiles; ++t) {
            const int j0 = t * J;
            if (ntiles > 1) {
                __syncthreads();
                stage_tile<D, NT, J>(tile, P, j0, tid, A.fault);
                __syncthreads();
            }
            if (any_tie) {
                pass2_tile<D, R, VARIANT, true>(&tile[0][0], J, min(J, m - j0), qa, qb, ea, eb, ca,
                                                cb, wk, ra, rb, mixed);
            } else {
                pass2_tile<D, R, VARIANT, false>(&tile[0][0], J, min(J, m - j0), qa, qb, ea, eb, ca,
                                                 cb, wk, ra, rb, mixed);
            }
        }
        report_ties<R>(A, w, qi, tie, mixed);
        write_outputs<R>(A, w, P, qi, wk, ea, eb, ca, cb);
    }
}

// Staging by bulk copies (TMA): two shared-memory stages, one elected
// thread issues one cp.async.bulk per coordinate plane per tile, completing
// on the stage's mbarrier, and the next-but-one tile is requested as soon as
// a stage has been read, so copies overlap the distance arithmetic. The
// copies move whole 16-byte groups; the last < 4 frames of a pair and the
// +inf padding of its last group are written by threads. Requires row
// starts 16-byte aligned, a plane stride that is a multiple of 4 and no frame
// map (the planner checks). Every wait is bounded: when one runs out the
// kernel records FAULT_WAIT_TIMEOUT, waits (bounded) for the copies it has
// in flight and returns.
constexpr unsigned kWaitPolls = 1u << 22;

template <int D, int KMAX, int R, int NT, int J, int VARIANT>
__global__ void __launch_bounds__(NT) ksg_count_kernel_tma(KsgCountArgs A) {
    static_assert(J % (4 * 32) == 0, "tile must hold whole float4 groups");
    constexpr int kStage = 2 * D * J;  // floats per stage
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) unsigned long long bars[2];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const float kInf = __int_as_float(0x7f800000);
    const uint32_t bar0 = nsg_smem_addr(&bars[0]);
    const uint32_t bar1 = nsg_smem_addr(&bars[1]);
    if (tid == 0) {
        nsg_mbar_init(bar0, 1);
        nsg_mbar_init(bar1, 1);
        nsg_fence_mbar_init();
    }
    __syncthreads();
    // phases consumed and copies in flight per stage (same in every thread);
    // scalars, not arrays, so they stay in registers
    unsigned phase0 = 0u, phase1 = 0u;
    int inflight0 = 0, inflight1 = 0;

    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= A.nitems) return;
        const KsgItem w = A.items[item];
        const KsgPairDesc P = A.pairs[w.pair];
        const int m = P.m;
        const int T = (m + J - 1) / J;
        const int nv = T == 1 ? 1 : 2 * T;  // pass-1 tiles, then pass-2 tiles

        // thread 0: request virtual tile v into stage v & 1
        auto issue = [&](int v) {
            const int st = v & 1;
            const int j0 = (v % T) * J;
            const int bulk = min(J, m - j0) & ~3;
            const uint32_t bar = st ? bar1 : bar0;
            nsg_fence_proxy_async();
            nsg_mbar_arrive_expect_tx(bar, static_cast<uint32_t>(2 * D * bulk * 4));
            if (bulk > 0) {
#pragma unroll
                for (int c = 0; c < 2 * D; ++c) {
                    const float* src = (c < D ? P.xa + (size_t)c * P.ld : P.xb + (size_t)(c - D) * P.ld) + j0;
                    nsg_bulk_load(nsg_smem_addr(smem + st * kStage + c * J), src,
                                  static_cast<uint32_t>(bulk * 4), bar);
                }
            }
        };
        if (tid == 0) {
            issue(0);
            if (nv > 1) issue(1);
        }
        inflight0 += 1;
        if (nv > 1) inflight1 += 1;

        float qa[R][D], qb[R][D];
        int qi[R];
        constexpr int KN = KMAX - 2;
        float bd[R][KN];
        int bj[R][KN];
        bool self_seen[R], tied[R];
        load_queries<D, KN, R, NT>(A, w, P, tid, qa, qb, qi, bd, bj, self_seen, tied);
        float ea[R], eb[R], wk[R], ra[R], rb[R];
        bool tie[R], mixed[R];
        bool any_tie = false;
        int ca[R], cb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ca[r] = 0;
            cb[r] = 0;
            mixed[r] = false;
        }

        for (int v = 0; v < nv; ++v) {
            const int st = v & 1;
            const int j0 = (v % T) * J;
            const int jn = min(J, m - j0);
            const unsigned ph = st ? phase1 : phase0;
            const bool ok = nsg_mbar_wait(st ? bar1 : bar0, ph & 1u, kWaitPolls);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(A.fault, FAULT_WAIT_TIMEOUT);
                // leave no copy in flight into shared memory we give up
                for (int u = 0; u < inflight0; ++u) nsg_mbar_wait(bar0, (phase0 + u) & 1u, kWaitPolls);
                for (int u = 0; u < inflight1; ++u) nsg_mbar_wait(bar1, (phase1 + u) & 1u, kWaitPolls);
                return;
            }
            if (st) {
                phase1 += 1;
                inflight1 -= 1;
            } else {
                phase0 += 1;
                inflight0 -= 1;
            }
            float* tile = smem + st * kStage;
            const int bulk = jn & ~3;
            if (bulk != jn || (jn & 3)) {
                // tail frames and the +inf padding of the last group
                const int tail_end = (jn + 3) & ~3;
                for (int idx = tid; idx < 2 * D * 4; idx += NT) {
                    const int c = idx >> 2;
                    const int f = bulk + (idx & 3);
                    if (f < tail_end) {
                        float val = kInf;
                        if (f < jn) {
                            val = c < D ? __ldg(P.xa + (size_t)c * P.ld + j0 + f)
                                        : __ldg(P.xb + (size_t)(c - D) * P.ld + j0 + f);
                        }
                        tile[c * J + f] = val;
                    }
                }
                // order these generic-proxy writes before a later bulk copy
                // into the same stage
                nsg_fence_proxy_async();
                __syncthreads();
            }
            if (v < T || T == 1) {
                pass1_tile<D, KN, R, VARIANT>(tile, J, j0, jn, qa, qb, bd, bj, self_seen, tied);
                if (v == T - 1) {
                    eps_and_ties<D, KN, R>(A, w, P, qa, qb, qi, bd, bj, tied, ea, eb, tie, wk, ra, rb);
#pragma unroll
                    for (int r = 0; r < R; ++r) any_tie |= tie[r];
                    any_tie = __any_sync(0xffffffffu, any_tie);
                }
            }
            if (v >= T || T == 1) {
                if (any_tie) {
                    pass2_tile<D, R, VARIANT, true>(tile, J, jn, qa, qb, ea, eb, ca, cb, wk, ra, rb,
                                                    mixed);
                } else {
                    pass2_tile<D, R, VARIANT, false>(tile, J, jn, qa, qb, ea, eb, ca, cb, wk, ra, rb,
                                                     mixed);
                }
            }
            __syncthreads();  // stage st fully read
            if (v + 2 < nv) {
                if (tid == 0) issue(v + 2);
                if (st) inflight1 += 1;
                else inflight0 += 1;
            }
        }
        report_ties<R>(A, w, qi, tie, mixed);
        write_outputs<R>(A, w, P, qi, wk, ea, eb, ca, cb);
    }
}

}  // namespace ksgk
}  // namespace nsg
