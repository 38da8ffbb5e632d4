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
//     the k+2 smallest (dz, j) -- the sample itself, whose dz is 0, and its
//     k+1 nearest -- lives in registers; it is only touched when the minimum
//     dz of the four frames is below the list's last entry, which after the
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
// Why the list needs no index tie-break: position 0 always holds a frame at
// distance 0 (the sample itself or an exact duplicate, all with zero
// marginals), and when the values at positions k and k+1 differ, positions
// 1..k hold exactly the frames with dz <= that k-th value, whatever order
// equal values were inserted in. When they are equal (and non-zero) the
// reference's choice depends on its sort; the sample goes to the tie list
// and ksg_tie_kernel recomputes it. Frames past m are staged as +inf and
// never pass the strict admission test.
//
// Runtime k with KMAX >= k+2: the first KMAX-k-2 slots hold -inf sentinels
// that never move, so the live entries occupy the last k+2 slots and the
// admission threshold is always slot KMAX-1 (a static register index).
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
// the caller has checked v < bd[KMAX-1]. Branch-free: place at the end,
// then one compare-and-swap per slot towards the front. Sentinel slots
// (-inf) never move.
template <int KMAX>
__device__ __forceinline__ void list_insert(float (&bd)[KMAX], int (&bj)[KMAX], float v, int j) {
    bd[KMAX - 1] = v;
    bj[KMAX - 1] = j;
#pragma unroll
    for (int s = KMAX - 1; s > 0; --s) {
        const bool sw = bd[s] < bd[s - 1];
        const float lo = sw ? bd[s] : bd[s - 1];
        const float hi = sw ? bd[s - 1] : bd[s];
        const int jl = sw ? bj[s] : bj[s - 1];
        const int jh = sw ? bj[s - 1] : bj[s];
        bd[s - 1] = lo;
        bd[s] = hi;
        bj[s - 1] = jl;
        bj[s] = jh;
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

template <int D, int KMAX, int R, int NT, int J, int VARIANT>
__global__ void __launch_bounds__(NT) ksg_count_kernel(KsgCountArgs A) {
    static_assert(J % (4 * 32) == 0, "tile must hold whole float4 groups");
    __shared__ __align__(16) float tile[2 * D][J];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const float kInf = __int_as_float(0x7f800000);

    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= A.nitems) return;
        const KsgItem w = A.items[item];
        const KsgPairDesc P = A.pairs[w.pair];
        const int m = P.m;
        const int ld = P.ld;
        const int* __restrict__ fmap = P.fmap;
        const float* __restrict__ xa = P.xa;
        const float* __restrict__ xb = P.xb;

        // query samples of this thread
        float qa[R][D], qb[R][D];
        int qi[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            qi[r] = w.q0 + r * NT + tid;
            const bool valid = qi[r] < w.q1;
            const int src = valid ? frame_of(fmap, qi[r], ld, A.fault) : 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                qa[r][c] = valid ? __ldg(xa + (size_t)c * ld + src) : 0.f;
                qb[r][c] = valid ? __ldg(xb + (size_t)c * ld + src) : 0.f;
            }
        }

        // k+2 live entries: the sample itself (distance 0), the k nearest and
        // the next one, so that a tie at the k-th distance is visible.
        float bd[R][KMAX];
        int bj[R][KMAX];
        const int nsent = KMAX - (A.k + 2);
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int s = 0; s < KMAX; ++s) {
                bd[r][s] = s < nsent ? -kInf : kInf;
                bj[r][s] = -1;
            }

        const int ntiles = (m + J - 1) / J;

        // ---- pass 1: k nearest joint neighbours ------------------------------
        for (int t = 0; t < ntiles; ++t) {
            const int j0 = t * J;
            __syncthreads();
            for (int idx = tid; idx < 2 * D * J; idx += NT) {
                const int c = idx / J;
                const int f = idx - c * J;
                const int j = j0 + f;
                float v = kInf;
                if (j < m) {
                    const int src = frame_of(fmap, j, ld, A.fault);
                    v = c < D ? __ldg(xa + (size_t)c * ld + src)
                              : __ldg(xb + (size_t)(c - D) * ld + src);
                }
                tile[c][f] = v;
            }
            __syncthreads();
            const int jn = min(J, m - j0);
            const int ngroups = (jn + 3) >> 2;
            for (int g = 0; g < ngroups; ++g) {
                float4 ga[D], gb[D];
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    ga[c] = *reinterpret_cast<const float4*>(&tile[c][4 * g]);
                    gb[c] = *reinterpret_cast<const float4*>(&tile[D + c][4 * g]);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    float da[4], db[4], dz[4];
                    Marg<D, VARIANT>::four(qa[r], ga, da);
                    Marg<D, VARIANT>::four(qb[r], gb, db);
#pragma unroll
                    for (int f = 0; f < 4; ++f) dz[f] = fmaxf(da[f], db[f]);
                    const float mn = nsg_min3(dz[0], dz[1], fminf(dz[2], dz[3]));
                    if (mn < bd[r][KMAX - 1]) {
#pragma unroll
                        for (int f = 0; f < 4; ++f) {
                            if (dz[f] < bd[r][KMAX - 1]) {
                                list_insert<KMAX>(bd[r], bj[r], dz[f], j0 + 4 * g + f);
                            }
                        }
                    }
                }
            }
        }

        // ---- eps from list positions 1..k ---------------------------------------
        // Position p is slot nsent+p; positions 1..k are slots nsent+1 ..
        // KMAX-2 and position k+1 is slot KMAX-1. When the k-th distance
        // equals the (k+1)-th (and is not zero) the reference's choice among
        // the equal frames depends on its sort; such samples go to the tie
        // list and ksg_tie_kernel recomputes them.
        float ea[R], eb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ea[r] = 0.f;
            eb[r] = 0.f;
            const bool valid = qi[r] < w.q1;
            if (valid && bd[r][KMAX - 2] == bd[r][KMAX - 1] && bd[r][KMAX - 2] > 0.f) {
                const int slot = atomicAdd(A.tie_count, 1);
                if (slot < A.tie_cap) {
                    A.ties[slot] = KsgTie{w.pair, qi[r]};
                } else {
                    atomicOr(A.fault, FAULT_TIE_OVERFLOW);
                }
            }
#pragma unroll
            for (int s = 1; s < KMAX - 1; ++s) {
                const int j = bj[r][s];
                if (valid && s > nsent && j >= 0 && j < m) {
                    const int src = frame_of(fmap, j, ld, A.fault);
                    ea[r] = fmaxf(ea[r], marginal_at<D>(qa[r], xa, ld, src));
                    eb[r] = fmaxf(eb[r], marginal_at<D>(qb[r], xb, ld, src));
                }
            }
        }

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
                for (int idx = tid; idx < 2 * D * J; idx += NT) {
                    const int c = idx / J;
                    const int f = idx - c * J;
                    const int j = j0 + f;
                    float v = kInf;
                    if (j < m) {
                        const int src = frame_of(fmap, j, ld, A.fault);
                        v = c < D ? __ldg(xa + (size_t)c * ld + src)
                                  : __ldg(xb + (size_t)(c - D) * ld + src);
                    }
                    tile[c][f] = v;
                }
                __syncthreads();
            }
            const int jn = min(J, m - j0);
            const int ngroups = (jn + 3) >> 2;
            for (int g = 0; g < ngroups; ++g) {
                float4 ga[D], gb[D];
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    ga[c] = *reinterpret_cast<const float4*>(&tile[c][4 * g]);
                    gb[c] = *reinterpret_cast<const float4*>(&tile[D + c][4 * g]);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    float da[4], db[4];
                    Marg<D, VARIANT>::four(qa[r], ga, da);
                    Marg<D, VARIANT>::four(qb[r], gb, db);
#pragma unroll
                    for (int f = 0; f < 4; ++f) {
                        ca[r] += da[f] <= ea[r] ? 1 : 0;
                        cb[r] += db[f] <= eb[r] ? 1 : 0;
                    }
                }
            }
        }

        // ---- per-sample outputs -----------------------------------------------
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (qi[r] < w.q1) {
                const long long o = P.scratch + qi[r];
                // counts lie in [k, m-1] for finite inputs; the clamp keeps
                // non-finite inputs from indexing outside the psi table
                const int nx = min(max(ca[r] - 1, 0), m);
                const int ny = min(max(cb[r] - 1, 0), m);
                A.psum[o] = __fadd_rn(__ldg(A.psi + nx), __ldg(A.psi + ny));
                if (A.nx) A.nx[o] = nx;
                if (A.ny) A.ny[o] = ny;
                if (A.eps_x) A.eps_x[o] = ea[r];
                if (A.eps_y) A.eps_y[o] = eb[r];
                if (A.kdist) A.kdist[o] = bd[r][KMAX - 2];
            }
        }
    }
}

}  // namespace ksgk
}  // namespace nsg
