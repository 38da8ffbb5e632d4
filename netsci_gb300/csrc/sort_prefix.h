// Order of equal keys under the reference CPU path's sort.
//
// The reference CPU estimator orders the candidate frames of each sample
// with std::sort over the frame indices 0..n-1, comparing joint distances
// with `<` (netcalc/src/mutual_information_cpu.cpp:48-53), and takes the
// neighbour set from sorted positions 1..k. When the k-th and (k+1)-th
// smallest distances are equal, which of the equal frames land in positions
// 1..k is decided by the sort's sequence of comparisons and swaps, not by
// the distances. To give the same neighbour sets as the reference on such
// samples, this routine follows the steps of the GNU libstdc++ std::sort
// (an introsort) on the index array, restricted to the segments that cover
// the positions that matter:
//
//   * segments longer than 16 are split by a median-of-three pivot (the
//     candidates at first+1, the middle, last-1, the median moved to first)
//     and an unguarded two-pointer partition of [first+1, last) around it;
//     the right part is split before the left part is continued, and a
//     recursion depth budget of 2*floor(log2 n) applies;
//   * segments of at most 16 elements are left for a final insertion sort,
//     which moves each element left past strictly greater ones, so elements
//     never cross a partition point and each final segment can be sorted on
//     its own.
//
//   * a segment on which the depth budget runs out is heapsorted, as the
//     library's partial sort with middle == last does it: a max-heap built
//     by sifting each parent down from the last one to the root, then the
//     root swapped with the last element of the shrinking heap and the
//     displaced element sifted back down. A sift-down first moves the hole
//     to a leaf along the larger children (the right child unless it is less
//     than the left one) and then lets the element rise from there while its
//     parent is less than it. Those steps decide where equal keys end up.
//
// Only segments that intersect [0, T) are followed, which makes the work
// O(n) instead of O(n log n), except on a heapsorted segment (O(L log L) for
// its L elements, only on inputs that defeat the median-of-three pivots).
//
// Written for both the host (tests compare it with std::sort) and the device
// (the tie-resolution kernel runs it per tied sample).
#pragma once

#ifdef __CUDACC__
#define NSG_HD __host__ __device__ __forceinline__
#else
#define NSG_HD inline
#endif

namespace nsg {

struct SortSegment {
    int first;
    int last;
    int depth;
};

// Sift-down of the heap v[0..len) (max at the root, by key[v[.]]) from the
// hole at `hole`, placing `value` (the element that was there).
NSG_HD void heap_sift_like_reference(const float* key, int* v, int hole, int len, int value) {
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (key[v[child]] < key[v[child - 1]]) --child;
        v[hole] = v[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        v[hole] = v[child - 1];
        hole = child - 1;
    }
    const float kv = key[value];
    int parent = (hole - 1) / 2;
    while (hole > top && key[v[parent]] < kv) {
        v[hole] = v[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    v[hole] = value;
}

// Heapsort of v[0..len) in the library's steps (heap build, then pops).
NSG_HD void heap_sort_like_reference(const float* key, int* v, int len) {
    if (len < 2) return;
    for (int parent = (len - 2) / 2;; --parent) {
        heap_sift_like_reference(key, v, parent, len, v[parent]);
        if (parent == 0) break;
    }
    for (int last = len - 1; last > 0; --last) {
        const int value = v[last];
        v[last] = v[0];
        heap_sift_like_reference(key, v, 0, last, value);
    }
}

// floor(log2(n)) for n >= 1
NSG_HD int floor_log2(int n) {
    int r = 0;
    while (n > 1) {
        n >>= 1;
        ++r;
    }
    return r;
}

// Rearranges idx[0..n) (initially 0..n-1) as the reference sort would, at
// least on positions [0, T). key[v] is the sort key of value v. `stack`
// must hold at least 2*floor(log2 n) + 2 segments. Returns false only when
// the stack is too small or a partition invariant breaks (neither happens
// with a large enough stack). *heapsorted (nullable) counts the segments
// that took the heapsort branch.
NSG_HD bool sort_prefix_like_reference(const float* key, int* idx, int n, int T,
                                       SortSegment* stack, int stack_cap, int* heapsorted = nullptr) {
    if (n <= 1) return true;
    constexpr int kThreshold = 16;
    int top = 0;
    stack[top++] = {0, n, 2 * floor_log2(n)};
    // final segments intersecting [0, T) in left-to-right order are not
    // needed explicitly: insertion-sorting [0, end) where end is the last
    // final segment's end gives the same prefix, since elements never cross
    // partition points.
    int prefix_end = 0;
    while (top > 0) {
        SortSegment s = stack[--top];
        int first = s.first, last = s.last, depth = s.depth;
        while (last - first > kThreshold) {
            if (depth == 0) {
                // depth budget spent: the segment is heapsorted and final
                heap_sort_like_reference(key, idx + first, last - first);
                if (heapsorted) ++*heapsorted;
                break;
            }
            --depth;
            // median of three moved to `first`
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
            {
                const int t = idx[first];
                idx[first] = idx[pick];
                idx[pick] = t;
            }
            // unguarded partition of [first+1, last) around key of idx[first]
            const float pk = key[idx[first]];
            int lo = first + 1, hi = last;
            for (;;) {
                // The median-of-three leaves an element >= and one <= the
                // pivot inside the range, so neither scan can leave it; the
                // bounds only turn a broken invariant into a reported failure.
                while (key[idx[lo]] < pk) {
                    if (++lo >= last) return false;
                }
                --hi;
                while (pk < key[idx[hi]]) {
                    if (--hi < first) return false;
                }
                if (!(lo < hi)) break;
                const int t = idx[lo];
                idx[lo] = idx[hi];
                idx[hi] = t;
                ++lo;
            }
            const int cut = lo;
            if (cut < T) {
                if (top >= stack_cap) return false;
                stack[top++] = {cut, last, depth};
            }
            last = cut;
        }
        if (first < T && last > prefix_end) prefix_end = last;
    }
    // insertion sort of [0, prefix_end): move each element left past
    // strictly greater keys
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
    return true;
}

}  // namespace nsg
