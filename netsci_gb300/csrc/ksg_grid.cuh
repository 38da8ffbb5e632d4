// KSG on cell grids: the same results as ksg_count_kernel with a fraction
// of the distance evaluations.
//
// Every frame a query can accept lies inside an axis-aligned box around it:
// pass 1 accepts frame j only when dz(i, j) <= the current (k+1)-th
// distance U_i, and dz >= |fl(x_c(i) - x_c(j))| for every coordinate c;
// pass 2 counts j only when d_a(i, j) <= eps_a(i), and d_a >= that
// coordinate difference for every coordinate of a. So frames are grouped
// into cells of a G x G grid over two coordinates, and a warp of 32
// neighbouring queries visits only the cells whose bounds can reach one of
// its queries. A cell [e_lo, e_hi) along coordinate c is skipped for query i
// when fl(q - e_hi) > U or fl(e_lo - q) > U: rounding is monotone, so every
// frame of the cell then has |fl(q - x)| > U. The test is exact, so the set
// of frames a query can accept, and with it eps, the counts and every
// output, equal the exhaustive kernel's.
//
// Grids:
//   * node grid (one per trajectory row): coordinates c1, c2 with the
//     widest spread, G-1 quantile edges on each, frames sorted by cell
//     (cell-major over c1, then c2), coordinates copied in that order;
//   * pair grid (one per pair and batch): cells over (c1 of a, c1 of b)
//     with the two nodes' edges, both nodes' coordinates copied in that
//     order with the frames' original indices.
//
// Warps, not CTAs, own queries: a warp takes frames consecutive in a query
// order as its queries (32 in pass 1, 16 at two lanes each in the counts).
// Where the batch builds query orders (ksg_grid.cu), pass 1 takes a block
// order (4 x 4 cell blocks in Z order, queries within a block by a size
// class of their box) and the counts a box order (the Z code of the cells
// their count box spans); else both take the Z order of the cells. The
// queries' boxes then overlap. The warp streams the
// frames of the cells it must visit through its own slice of shared memory,
// read back as float4 (pass 1) or float2 (counts) broadcasts.
// Pass 1 first scans the rectangle of cells its queries sit in (the seed,
// which fills the neighbour lists and bounds U), then cell rows outward,
// recomputing each row's column range from the current bounds and stopping
// in a direction at the first row no query can reach (rows further out have
// bounds further away). The counts use the fixed eps and visit the row and
// column ranges directly.
#pragma once

#include "common.cuh"
#include "ksg.cuh"
#include "ksg_grid.h"
#include "ksg_kernels.cuh"

namespace nsg {

namespace gridk {

__device__ __forceinline__ float inf_f() { return __int_as_float(0x7f800000); }

// Edge e[t] for t in [-1, G-1]: -inf below, +inf above.
__device__ __forceinline__ float edge_at(const float* e, int t, int G) {
    if (t < 0) return -inf_f();
    if (t >= G - 1) return inf_f();
    return e[t];
}

// Can a frame of bin t (values in [e[t-1], e[t])) lie within u of q?
__device__ __forceinline__ bool bin_reaches(const float* e, int t, int G, float q, float u) {
    return __fsub_rn(q, edge_at(e, t, G)) <= u && __fsub_rn(edge_at(e, t - 1, G), q) <= u;
}

// Range [lo, hi] of bins that can hold frames within u of q (lo > hi: none).
// Bins reachable form one interval: the first condition of bin_reaches holds
// from some bin on (edges ascend), the second up to some bin; both bounds by
// binary search.
__device__ __forceinline__ void bin_range(const float* e, int G, float q, float u, int& lo, int& hi) {
    int a = 0, b = G;  // first bin with fl(q - e[t]) <= u, G if none
    while (a < b) {
        const int mid = (a + b) >> 1;
        if (__fsub_rn(q, edge_at(e, mid, G)) <= u) b = mid;
        else a = mid + 1;
    }
    lo = a;
    a = 0;
    b = G - 1;  // last bin with fl(e[t-1] - q) <= u (bin 0 always qualifies)
    while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (__fsub_rn(edge_at(e, mid - 1, G), q) <= u) a = mid;
        else b = mid - 1;
    }
    hi = a;
}

// Largest of D non-negative values (three-input max for D = 3).
template <int D>
__device__ __forceinline__ float max_of(const float (&v)[D]) {
    if constexpr (D == 1) return v[0];
    else if constexpr (D == 2) return fmaxf(v[0], v[1]);
    else return nsg_max3(v[0], v[1], v[2]);
}

// Pair index and warp block of work item t (binary search over wprefix).
__device__ __forceinline__ void item_of(const int* wprefix, int npairs, int t, int& p, int& blk) {
    int lo = 0, hi = npairs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(wprefix + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    p = lo;
    blk = t - __ldg(wprefix + lo);
}

// Position (row-major storage) of the query of rank qi in a grid's query
// order: the last query-order cell starting at or before qi (it is not
// empty), then the offset within it.
__device__ __forceinline__ int query_position(const int* start, int G, int qi) {
    const int* qs = start + grid_qoff(G);
    const unsigned short* qc = reinterpret_cast<const unsigned short*>(qs + grid_qoff(G));
    int lo = 0, hi = G * G - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(qs + mid) <= qi) lo = mid;
        else hi = mid - 1;
    }
    return __ldg(start + __ldg(qc + lo)) + (qi - __ldg(qs + lo));
}

// Stage frames [base, base+n) of a sorted grid (planes of `stride` floats)
// into this warp's tile (NP planes of kGridChunk), +inf past n; with JT also
// their original indices.
template <int NP, bool JT>
__device__ __forceinline__ void stage(float* tile, int* jt, const float* sx, long long stride,
                                      const int* perm, int base, int n, int lane) {
#pragma unroll
    for (int t = 0; t < kGridChunk / 32; ++t) {
        const int f = lane + 32 * t;
        const bool in = f < n;
#pragma unroll
        for (int c = 0; c < NP; ++c) {
            tile[c * kGridChunk + f] = in ? __ldg(sx + c * stride + base + f) : inf_f();
        }
        if constexpr (JT) jt[f] = in ? __ldg(perm + base + f) : -1;
    }
}

// 4-byte asynchronous global -> shared copies (cp.async), grouped per call
// of stage_async and waited for with cp.async.wait_group.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Issue the copies of frames [base, base+n), n <= 64, into a half tile
// (planes of stride kGridChunk) with their indices in jt, as one group;
// slots past n are set to +inf (index -1) directly. Frames are single floats
// at arbitrary offsets, so the copies are 4 bytes each.
template <int NP>
__device__ __forceinline__ void stage_async(float* tile, int* jt, const float* sx, long long stride,
                                            const int* perm, int base, int n, int lane) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int f = lane + 32 * t;
        if (f < n) {
#pragma unroll
            for (int c = 0; c < NP; ++c) cp_async4(tile + c * kGridChunk + f, sx + c * stride + base + f);
            cp_async4(jt + f, perm + base + f);
        } else {
#pragma unroll
            for (int c = 0; c < NP; ++c) tile[c * kGridChunk + f] = inf_f();
            jt[f] = -1;
        }
    }
    cp_async_commit();
}

// What pass 1 knows about the frames outside a query's list at distance
// U = its last entry, kept in shared memory (rarely touched, so it costs no
// registers in the scan): tr[0] the U the record was made at, tr[kTieStride]
// and tr[2 * kTieStride] the marginal pair all those frames share, or
// kTieMixed (marginals are never negative) when they differ. U only
// decreases and no frame can lie outside the list at a new, smaller U; a
// record made at another U is stale. Every frame at the final U outside the
// final list was offered while U had that value (rejected at v == U, or
// pushed out of the last slot by a nearer frame with the last entry still
// at U), so at the end a record made at the final U covers all of them.
constexpr int kTieStride = 32 * kGridWarps;
constexpr float kTieMixed = -2.f;

__device__ __forceinline__ void tie_note(float* tr, float u, float va, float vb) {
    if (tr[0] != u) {
        tr[0] = u;
        tr[kTieStride] = va;
        tr[2 * kTieStride] = vb;
    } else if (va != tr[kTieStride] || vb != tr[2 * kTieStride]) {
        tr[kTieStride] = kTieMixed;
    }
}

// Offer frame j (joint distance v, marginals va, vb) to the list: the first
// frame at distance 0 stands for the query itself; a nearer frame enters
// (ksgk::list_insert); one at U is recorded. A frame pushed out of the list
// while U stays the same is recorded with its marginals read from the pair's
// original rows. Callers offer only frames with v <= U.
template <int D, int KN>
__device__ __forceinline__ void admit_rec(float (&bd)[KN], int (&bj)[KN], bool& self_seen, float* tr, float v,
                                          float va, float vb, int j, const float (&qa)[D], const float (&qb)[D],
                                          const KsgPairDesc* P) {
    const float u = bd[KN - 1];
    if (v == 0.f && !self_seen) {
        self_seen = true;
    } else if (v < u) {
        const int out = bj[KN - 1];
        ksgk::list_insert<KN>(bd, bj, v, j);
        if (bd[KN - 1] == u && out >= 0) {
            tie_note(tr, u, ksgk::marginal_at<D>(qa, P->xa, P->ld, out), ksgk::marginal_at<D>(qb, P->xb, P->ld, out));
        }
    } else {
        tie_note(tr, u, va, vb);
    }
}

// Pass 1 over a staged chunk: frames' original indices in jt. The list holds
// the KN nearest frames other than the query itself. Without REC the flag
// `tied` says whether a frame outside it lies at its last distance
// (ksgk::admit); with REC, tr records those frames' marginals (admit_rec).
template <int D, int KN, bool REC>
__device__ __forceinline__ void pass1_chunk(const float* tile, const int* jt, int n,
                                            const float (&qa)[D], const float (&qb)[D],
                                            float (&bd)[KN], int (&bj)[KN], bool& self_seen, bool& tied,
                                            float* tr, const KsgPairDesc* P) {
    const int ngroups = (n + 3) >> 2;
    for (int g = 0; g < ngroups; ++g) {
        float4 ga[D], gb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            ga[c] = *reinterpret_cast<const float4*>(tile + c * kGridChunk + 4 * g);
            gb[c] = *reinterpret_cast<const float4*>(tile + (D + c) * kGridChunk + 4 * g);
        }
        float da[4], db[4], dz[4];
        ksgk::Marg<D, 1>::four(qa, ga, da);
        ksgk::Marg<D, 1>::four(qb, gb, db);
#pragma unroll
        for (int f = 0; f < 4; ++f) dz[f] = fmaxf(da[f], db[f]);
        const float mn = nsg_min3(dz[0], dz[1], fminf(dz[2], dz[3]));
        if (mn <= bd[KN - 1]) {
            // In a pruned scan most frames are near the queries, so some lane
            // of the warp inserts in a large share of groups. Insert each
            // lane's nearest frame of the group first, in one shared step;
            // it lowers the bound, so the other frames rarely still pass.
            // (A loop offering the frames nearest first through one copy of
            // the insertion ran 10% slower.)
            int fm = 0;
            float vm = dz[0], am = da[0], bm = db[0];
#pragma unroll
            for (int f = 1; f < 4; ++f) {
                const bool lt = dz[f] < vm;
                vm = lt ? dz[f] : vm;
                fm = lt ? f : fm;
                if constexpr (REC) {
                    am = lt ? da[f] : am;
                    bm = lt ? db[f] : bm;
                }
            }
            if constexpr (REC) admit_rec<D, KN>(bd, bj, self_seen, tr, mn, am, bm, jt[4 * g + fm], qa, qb, P);
            else ksgk::admit<KN>(bd, bj, self_seen, tied, mn, jt[4 * g + fm]);
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if (f != fm && dz[f] <= bd[KN - 1]) {
                    if constexpr (REC) {
                        admit_rec<D, KN>(bd, bj, self_seen, tr, dz[f], da[f], db[f], jt[4 * g + f], qa, qb, P);
                    } else {
                        ksgk::admit<KN>(bd, bj, self_seen, tied, dz[f], jt[4 * g + f]);
                    }
                }
            }
        }
    }
}

// Counts over a staged chunk for up to kCountGroup pairs at once: one
// distance per frame, compared with each pair's eps (unused slots hold -inf).
// Two lanes share a query: the lane of parity `half` takes frames 4g + 2*half
// and 4g + 2*half + 1 of each group of four. The chunk's counts (at most 64
// per lane) add up in floats, exactly, from nsg_le_f32: 46-51 against 57-64
// ms per 8192-pair batch at m = 10000 for integer selects and adds.
template <int D>
__device__ __forceinline__ void count_chunk(const float* tile, int n, int half, const float (&q)[D],
                                            const float (&e)[kCountGroup], int (&cnt)[kCountGroup]) {
    const int ngroups = (n + 3) >> 2;
    float cf[kCountGroup];
#pragma unroll
    for (int p = 0; p < kCountGroup; ++p) cf[p] = 0.f;
    for (int g = 0; g < ngroups; ++g) {
        float dq0[D], dq1[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const float2 x = *reinterpret_cast<const float2*>(tile + c * kGridChunk + 4 * g + 2 * half);
            const float2 s2 = nsg_sub2(make_float2(q[c], q[c]), x);
            dq0[c] = fabsf(s2.x);
            dq1[c] = fabsf(s2.y);
        }
        const float d0 = max_of<D>(dq0), d1 = max_of<D>(dq1);
#pragma unroll
        for (int p = 0; p < kCountGroup; ++p) cf[p] += nsg_le_f32(d0, e[p]) + nsg_le_f32(d1, e[p]);
    }
#pragma unroll
    for (int p = 0; p < kCountGroup; ++p) cnt[p] += static_cast<int>(cf[p]);
}

// Tie check over a staged chunk (2d planes): the range of each marginal over
// the frames whose joint distance equals w (w < 0: no tie, nothing matches).
template <int D>
__device__ __forceinline__ void tie_chunk(const float* tile, int n, const float (&qa)[D], const float (&qb)[D],
                                          float w, float& lo_a, float& hi_a, float& lo_b, float& hi_b) {
    const int ngroups = (n + 3) >> 2;
    for (int g = 0; g < ngroups; ++g) {
        float4 ga[D], gb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            ga[c] = *reinterpret_cast<const float4*>(tile + c * kGridChunk + 4 * g);
            gb[c] = *reinterpret_cast<const float4*>(tile + (D + c) * kGridChunk + 4 * g);
        }
        float da[4], db[4];
        ksgk::Marg<D, 1>::four(qa, ga, da);
        ksgk::Marg<D, 1>::four(qb, gb, db);
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            if (fmaxf(da[f], db[f]) == w) {
                lo_a = fminf(lo_a, da[f]);
                hi_a = fmaxf(hi_a, da[f]);
                lo_b = fminf(lo_b, db[f]);
                hi_b = fmaxf(hi_b, db[f]);
            }
        }
    }
}

}  // namespace gridk

// ---- pass 1: joint k nearest neighbours, eps, ties -----------------------------
// REC: ties checked through the shared-memory tie record (gridk::tie_note)
// rather than by scanning the frames within the k-th distance again after
// the search. The record costs registers in the scan (7 ms more per
// 8192-pair batch at m = 10000), the scan costs little where ties are rare,
// so REC serves plans of resampled trajectories, where copies of one frame
// tie on a large share of samples (a quarter less search time there).
template <int D, int KMAX, bool REC>
__global__ void __launch_bounds__(32 * kGridWarps, (KMAX <= 8 ? 4 : 1)) ksg_grid_pass1_kernel(GridArgs A) {
    using namespace gridk;
    __shared__ __align__(16) float s_tile[kGridWarps][2 * D * kGridChunk];
    __shared__ int s_jt[kGridWarps][kGridChunk];
    __shared__ float s_tie[REC ? 3 * kTieStride : 1];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    float* tile = s_tile[wid];
    int* jt = s_jt[wid];
    const int total = __ldg(A.wprefix + A.npairs);
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(A.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) return;
        int p, blk;
        item_of(A.wprefix, A.npairs, t, p, blk);
        const KsgPairDesc* P = A.pairs + p;  // fields read where used
        const GridPair gp = A.gp[p];
        const GridNode na = A.nodes[gp.a];
        const GridNode nb = A.nodes[gp.b];
        const int m = P->m, G = na.G;
        const long long st = m;
        const int qi = blk * 32 + lane;  // query rank in the pair's search order
        const bool valid = qi < m;
        const int r = !valid ? 0 : A.search_order ? __ldg(gp.qpos + qi) : query_position(gp.start, G, qi);
        const int i = valid ? __ldg(gp.perm + r) : 0;
        float qa[D], qb[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            qa[c] = valid ? __ldg(gp.sx + c * st + r) : 0.f;
            qb[c] = valid ? __ldg(gp.sx + (D + c) * st + r) : 0.f;
        }
        // the k nearest frames other than the query, after nsent -inf
        // sentinels (list positions 1..k of the reference's sorted row)
        constexpr int KL = KMAX - 2;
        float bd[KL];
        int bj[KL];
        bool self_seen = false, tied = false;
        float* tr = s_tie + (REC ? threadIdx.x : 0);
        if constexpr (REC) tr[0] = -1.f;  // no record
        const int nsent = KMAX - (A.k + 2);
#pragma unroll
        for (int s = 0; s < KL; ++s) {
            bd[s] = s < nsent ? -inf_f() : inf_f();
            bj[s] = -1;
        }
        // cells of this warp's queries: row = bin of a on c1, column = bin of b on c1
        const int qrow = valid ? __ldg(na.cell + i) / G : 0;
        const int qcol = valid ? __ldg(nb.cell + i) / G : 0;
        const int rmin = __reduce_min_sync(0xffffffffu, valid ? qrow : G);
        const int rmax = __reduce_max_sync(0xffffffffu, valid ? qrow : -1);
        const int cmin = __reduce_min_sync(0xffffffffu, valid ? qcol : G);
        const int cmax = __reduce_max_sync(0xffffffffu, valid ? qcol : -1);
        // The seed is the rectangle of cells the queries span; where the
        // query order jumps between distant blocks, the cell of the first
        // query alone.
        int srow_lo = rmin, srow_hi = rmax, scol_lo = cmin, scol_hi = cmax;
        if ((rmax - rmin + 1) * (cmax - cmin + 1) > 16) {
            srow_lo = srow_hi = __shfl_sync(0xffffffffu, qrow, 0);
            scol_lo = scol_hi = __shfl_sync(0xffffffffu, qcol, 0);
        }
        // the seed rectangle packed in one register (bins are below 256)
        const unsigned seedbox = static_cast<unsigned>(srow_lo) | static_cast<unsigned>(srow_hi) << 8 |
                                 static_cast<unsigned>(scol_lo) << 16 | static_cast<unsigned>(scol_hi) << 24;
        const float qa1 = qa[na.c1], qb1 = qb[nb.c1];
        // Ranges to scan, produced by a small state machine so that the scan
        // body (with its unrolled list inserts) exists once in the kernel:
        // the seed rows, then the rows the queries sit in (minus the seeded
        // columns), then rows outward. Every query lies below row `up`
        // (above row `dn`), so row `up` can only be reached across its lower
        // edge, and if no query reaches that edge now, no row further up can
        // be reached later (bounds only shrink). A row minus the seeded
        // columns may leave two pieces.
        int phase = 0;  // 0 seed rows, 1 the queries' rows, 2 outward
        int cx = srow_lo, up = rmax + 1, dn = rmin - 1;
        bool prefer_up = true;
        int pend_lo = 0, pend_hi = 0;
        int scanned = 0;  // at most m: a frame is scanned once per warp
        for (;;) {
            int lo, hi;
            if (pend_hi > pend_lo) {
                lo = pend_lo;
                hi = pend_hi;
                pend_hi = pend_lo;
            } else if (phase == 0) {
                lo = __ldg(gp.start + cx * G + (seedbox >> 16 & 0xff));
                hi = __ldg(gp.start + cx * G + (seedbox >> 24) + 1);
                if (++cx > static_cast<int>(seedbox >> 8 & 0xff)) {
                    phase = 1;
                    cx = dn + 1;  // rmin: dn moves only in phase 2
                }
            } else {
                const float u = valid ? bd[KL - 1] : -inf_f();
                int row = -1;
                if (phase == 1) {
                    if (cx <= rmax) row = cx++;
                    else phase = 2;
                }
                if (phase == 2) {
                    const bool more_up = up < G && __any_sync(0xffffffffu, valid &&
                        __fsub_rn(edge_at(na.e1, up - 1, G), qa1) <= u);
                    const bool more_dn = dn >= 0 && __any_sync(0xffffffffu, valid &&
                        __fsub_rn(qa1, edge_at(na.e1, dn, G)) <= u);
                    if (!more_up && !more_dn) break;
                    if (more_up && (prefer_up || !more_dn)) row = up++;
                    else row = dn--;
                    prefer_up = !prefer_up;
                }
                const bool reach = valid && bin_reaches(na.e1, row, G, qa1, u);
                if (!__any_sync(0xffffffffu, reach)) continue;
                int clo = G, chi = -1;
                if (reach) bin_range(nb.e1, G, qb1, u, clo, chi);
                clo = __reduce_min_sync(0xffffffffu, clo);
                chi = __reduce_max_sync(0xffffffffu, chi);
                if (clo > chi) continue;
                int alo = clo, ahi = chi, blo = 1, bhi = 0;
                if (row >= static_cast<int>(seedbox & 0xff) && row <= static_cast<int>(seedbox >> 8 & 0xff)) {
                    ahi = min(chi, static_cast<int>(seedbox >> 16 & 0xff) - 1);
                    blo = max(clo, static_cast<int>(seedbox >> 24) + 1);
                    bhi = chi;
                    if (alo > ahi) {
                        alo = blo;
                        ahi = bhi;
                        blo = 1;
                        bhi = 0;
                    }
                    if (alo > ahi) continue;
                }
                lo = __ldg(gp.start + row * G + alo);
                hi = __ldg(gp.start + row * G + ahi + 1);
                if (blo <= bhi) {
                    pend_lo = __ldg(gp.start + row * G + blo);
                    pend_hi = __ldg(gp.start + row * G + bhi + 1);
                }
            }
            scanned += hi - lo;
            if (hi > lo) {
                // 64-frame halves of the tile, the next one loading while this one is scanned
                const int nc = (hi - lo + 63) >> 6;
                __syncwarp();
                stage_async<2 * D>(tile, jt, gp.sx, st, gp.perm, lo, min(64, hi - lo), lane);
                for (int ci = 0; ci < nc; ++ci) {
                    const int half = ci & 1;
                    if (ci + 1 < nc) {
                        const int nb = lo + 64 * (ci + 1);
                        stage_async<2 * D>(tile + 64 * (half ^ 1), jt + 64 * (half ^ 1), gp.sx, st, gp.perm, nb,
                                           min(64, hi - nb), lane);
                        cp_async_wait<1>();
                    } else {
                        cp_async_wait<0>();
                    }
                    __syncwarp();
                    pass1_chunk<D, KL, REC>(tile + 64 * half, jt + 64 * half, min(64, hi - lo - 64 * ci), qa, qb,
                                            bd, bj, self_seen, tied, tr, P);
                    __syncwarp();
                }
            }
        }
        if (A.evals && lane == 0) {
            atomicAdd(A.evals, static_cast<unsigned long long>(scanned) * min(32, m - blk * 32));
        }
        // eps from list positions 1..k (original rows), tie test
        float ea = 0.f, eb = 0.f;
        // wk: the k-th distance. A tie when another frame lies at wk too and
        // the frames at wk do not all have the same marginal pair; when they
        // do, whichever of them the reference's sort puts first gives the
        // same eps, and the search's result stands.
        const float wk = bd[KL - 1];
        bool tie = valid && (REC ? tr[0] == wk : tied) && wk > 0.f;
        if (valid) {
            const float ta = REC ? tr[kTieStride] : 0.f, tb = REC ? tr[2 * kTieStride] : 0.f;
            bool same = ta >= 0.f;
#pragma unroll
            for (int s = 0; s < KL; ++s) {
                const int j = bj[s];
                if (s >= nsent && j >= 0 && j < m) {
                    const float da = ksgk::marginal_at<D>(qa, P->xa, P->ld, j);
                    const float db = ksgk::marginal_at<D>(qb, P->xb, P->ld, j);
                    ea = fmaxf(ea, da);
                    eb = fmaxf(eb, db);
                    if (REC && bd[s] == wk) same = same && da == ta && db == tb;
                }
            }
            if (REC) tie = tie && !same;
            const long long o = P->scratch + i;
            A.eps_a[o] = ea;
            A.eps_b[o] = eb;
            if (A.eps_x) A.eps_x[o] = ea;
            if (A.eps_y) A.eps_y[o] = eb;
            if (A.kdist) A.kdist[o] = wk;
        }
        if constexpr (!REC) {
            if (__any_sync(0xffffffffu, tie)) {
                // Frames at distance wk lie in the cells within wk of the
                // sample: every tied lane takes the range of both marginals
                // over the frames at exactly wk.
                int qrlo = G, qrhi = -1, qclo = G, qchi = -1;
                if (tie) {
                    bin_range(na.e1, G, qa1, wk, qrlo, qrhi);
                    bin_range(nb.e1, G, qb1, wk, qclo, qchi);
                }
                const int rlo = __reduce_min_sync(0xffffffffu, qrlo);
                const int rhi = __reduce_max_sync(0xffffffffu, qrhi);
                float lo_a = inf_f(), hi_a = -inf_f(), lo_b = inf_f(), hi_b = -inf_f();
                for (int cx = rlo; cx <= rhi; ++cx) {
                    const bool in_row = cx >= qrlo && cx <= qrhi;
                    const int clo = __reduce_min_sync(0xffffffffu, in_row ? qclo : G);
                    const int chi = __reduce_max_sync(0xffffffffu, in_row ? qchi : -1);
                    if (clo > chi) continue;
                    const int lo = __ldg(gp.start + cx * G + clo);
                    const int hi = __ldg(gp.start + cx * G + chi + 1);
                    for (int base = lo; base < hi; base += kGridChunk) {
                        const int n = min(kGridChunk, hi - base);
                        __syncwarp();
                        stage<2 * D, false>(tile, nullptr, gp.sx, st, nullptr, base, n, lane);
                        __syncwarp();
                        tie_chunk<D>(tile, n, qa, qb, tie ? wk : -1.f, lo_a, hi_a, lo_b, hi_b);
                    }
                }
                tie = tie && !(lo_a == hi_a && lo_b == hi_b);
            }
        }
        // tied samples of the warp take consecutive slots of the tie list
        const unsigned tmask = __ballot_sync(0xffffffffu, tie);
        if (tmask) {
            int base = 0;
            if (lane == 0) base = atomicAdd(A.tie_count, __popc(tmask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (tie) {
                const int slot = base + __popc(tmask & ((1u << lane) - 1u));
                if (slot < A.tie_cap) A.ties[slot] = KsgTie{A.pair_base + p, i};
                else atomicOr(A.fault, FAULT_TIE_OVERFLOW);
            }
        }
    }
}

// ---- pass 2: marginal counts on a node grid -------------------------------------
// A work item is a count group (up to kCountGroup pairs that count the same
// node's variable) and a block of kCountQueries queries consecutive in the
// group's count order (A.corder, else the node grid's query order), two
// lanes per query. The warp visits the union of the queries' boxes for the
// largest of the pairs' eps, row by row over the columns of the boxes that
// hold the row, and counts every pair from one distance per frame.
template <int D>
__global__ void __launch_bounds__(32 * kGridWarps, 4) ksg_grid_count_kernel(GridArgs A) {
    using namespace gridk;
    __shared__ __align__(16) float s_tile[kGridWarps][D * kGridChunk];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    float* tile = s_tile[wid];
    const int total = __ldg(A.gprefix + A.ngroups);
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(A.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) return;
        int gi, blk;
        item_of(A.gprefix, A.ngroups, t, gi, blk);
        const CountGroup grp = A.groups[gi];
        const GridNode nd = A.nodes[grp.node];
        const float* eps = grp.side ? A.eps_b : A.eps_a;
        int* out = grp.side ? A.cnt_b : A.cnt_a;
        const int m = nd.m, G = nd.G;
        const long long st = m;
        const int half = lane & 1;  // two lanes per query
        const int qi = blk * kCountQueries + (lane >> 1);  // query rank in the group's count order
        const bool valid = qi < m;
        const int r = !valid ? 0
                      : A.corder ? __ldg(A.corder + static_cast<long long>(gi) * A.corder_ld + qi)
                                 : query_position(nd.start, G, qi);
        const int i = valid ? __ldg(nd.perm + r) : 0;
        float q[D];
#pragma unroll
        for (int c = 0; c < D; ++c) q[c] = valid ? __ldg(nd.sx + c * st + r) : 0.f;
        float e[kCountGroup];
        float emax = -inf_f();
#pragma unroll
        for (int p = 0; p < kCountGroup; ++p) {
            e[p] = (valid && p < grp.npairs) ? __ldg(eps + A.pairs[grp.pairs[p]].scratch + i) : -inf_f();
            emax = fmaxf(emax, e[p]);
        }
        const float q1 = q[nd.c1];
        const float q2 = nd.c2 >= 0 ? q[nd.c2] : 0.f;
        // each query's box of rows [qrlo, qrhi] and columns [qclo, qchi];
        // a row is scanned over the columns of the queries whose box holds it
        int qrlo = G, qrhi = -1, qclo = G, qchi = -1;
        if (valid) {
            bin_range(nd.e1, G, q1, emax, qrlo, qrhi);
            bin_range(nd.e2, G, q2, emax, qclo, qchi);
        }
        const int rlo = __reduce_min_sync(0xffffffffu, qrlo);
        const int rhi = __reduce_max_sync(0xffffffffu, qrhi);
        int cnt[kCountGroup];
#pragma unroll
        for (int p = 0; p < kCountGroup; ++p) cnt[p] = 0;
        long long scanned = 0;
        for (int cx = rlo; cx <= rhi; ++cx) {
            const bool in_row = cx >= qrlo && cx <= qrhi;
            const int clo = __reduce_min_sync(0xffffffffu, in_row ? qclo : G);
            const int chi = __reduce_max_sync(0xffffffffu, in_row ? qchi : -1);
            if (clo > chi) continue;
            const int lo = __ldg(nd.start + cx * G + clo);
            const int hi = __ldg(nd.start + cx * G + chi + 1);
            scanned += hi - lo;
            for (int base = lo; base < hi; base += kGridChunk) {
                const int n = min(kGridChunk, hi - base);
                __syncwarp();
                stage<D, false>(tile, nullptr, nd.sx, st, nullptr, base, n, lane);
                __syncwarp();
                count_chunk<D>(tile, n, half, q, e, cnt);
            }
        }
#pragma unroll
        for (int p = 0; p < kCountGroup; ++p) cnt[p] += __shfl_xor_sync(0xffffffffu, cnt[p], 1);
        if (valid && half == 0) {
#pragma unroll
            for (int p = 0; p < kCountGroup; ++p)
                if (p < grp.npairs) out[A.pairs[grp.pairs[p]].scratch + i] = cnt[p];
        }
        if (A.evals && lane == 0) {
            // one distance per (query, frame), compared with every pair's eps
            const unsigned long long ev =
                static_cast<unsigned long long>(scanned) * min(kCountQueries, m - blk * kCountQueries);
            atomicAdd(A.evals + 1, ev);
            atomicAdd(A.evals + 2, ev * grp.npairs);
        }
    }
}

}  // namespace nsg
