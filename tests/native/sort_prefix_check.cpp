// Compares nsg::sort_prefix_like_reference with std::sort on index arrays:
// positions [0, T) must hold the same indices in the same order.
//
//   * random arrays with many equal keys;
//   * inputs that defeat the median-of-three pivots, so that the sort's
//     depth budget runs out and it heapsorts segments: made with McIlroy's
//     adversary ("A killer adversary for quicksort", Software: Practice and
//     Experience 29(4), 1999), which fixes the keys lazily while std::sort
//     runs with them, then with ties planted among the adversarial keys;
//   * the heap steps alone (nsg::heap_sort_like_reference) against
//     std::make_heap + std::sort_heap on tie-heavy arrays.
//
// Prints "ok <cases> heapsorted <segments>" or the first mismatch. Built
// and run by tests/test_tie_order.py.
//
// With the arguments `adversary <n> <k>` it prints instead the number of
// segments the sort heapsorts among the first k+2 positions, then n integer
// keys: adversarial keys 0..n-1 with the key k+1 lowered to k, so that the
// k-th and (k+1)-th smallest keys tie (tests/test_tie_gpu.py turns them into
// the joint distances of one sample).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "sort_prefix.h"

namespace {

// McIlroy's adversary: every key starts as "gas"; when two gas keys are
// compared, one of them (the last gas element seen, if it is one of the
// two) is frozen to the next solid value. With `high` false gas is above
// every solid key and solid keys count up from 0, so pivots come out small
// and the long side of each partition is the right one; with `high` true
// gas is below every solid key and solid keys count down from n-1, so the
// long side is the left one, the side that holds the first positions.
struct Adversary {
    std::vector<int> val;
    int gas = 0, next = 0, step = 1, candidate = 0;
    bool less(int x, int y) {
        if (val[x] == gas && val[y] == gas) {
            if (x == candidate) val[x] = next;
            else val[y] = next;
            next += step;
        }
        if (val[x] == gas) candidate = x;
        else if (val[y] == gas) candidate = y;
        return val[x] < val[y];
    }
};

std::vector<float> adversarial_keys(int n, bool high = false) {
    Adversary a;
    a.gas = high ? -1 : n;
    a.next = high ? n - 1 : 0;
    a.step = high ? -1 : 1;
    a.val.assign(n, a.gas);
    std::vector<int> p(n);
    std::iota(p.begin(), p.end(), 0);
    std::sort(p.begin(), p.end(), [&](int x, int y) { return a.less(x, y); });
    std::vector<float> key(n);
    for (int i = 0; i < n; ++i) key[i] = static_cast<float>(a.val[i] < 0 ? 0 : a.val[i]);
    return key;
}

bool check(const std::vector<float>& key, int T, std::vector<nsg::SortSegment>& stack, int c,
           long& heapsorted) {
    const int n = static_cast<int>(key.size());
    std::vector<int> ref(n), got(n);
    std::iota(ref.begin(), ref.end(), 0);
    std::iota(got.begin(), got.end(), 0);
    std::sort(ref.begin(), ref.end(), [&](int a, int b) { return key[a] < key[b]; });
    int h = 0;
    const bool ok = nsg::sort_prefix_like_reference(key.data(), got.data(), n, T, stack.data(),
                                                    static_cast<int>(stack.size()), &h);
    heapsorted += h;
    if (!ok) {
        std::printf("UNRESOLVED case %d n=%d T=%d\n", c, n, T);
        return false;
    }
    for (int i = 0; i < std::min(T, n); ++i) {
        if (ref[i] != got[i]) {
            std::printf("MISMATCH case %d n=%d T=%d at %d: ref %d got %d\n", c, n, T, i, ref[i], got[i]);
            return false;
        }
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 4 && std::string(argv[1]) == "adversary") {
        const int n = std::atoi(argv[2]), k = std::atoi(argv[3]);
        std::vector<float> key = adversarial_keys(n, true);
        for (auto& v : key)
            if (v == static_cast<float>(k + 1)) v = static_cast<float>(k);
        std::vector<int> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        std::vector<nsg::SortSegment> st(128);
        int h = 0;
        nsg::sort_prefix_like_reference(key.data(), idx.data(), n, k + 2, st.data(), 128, &h);
        std::printf("%d\n", h);
        for (int i = 0; i < n; ++i) std::printf("%d\n", static_cast<int>(key[i]));
        return 0;
    }
    const int cases = argc > 1 ? std::atoi(argv[1]) : 2000;
    std::mt19937_64 rng(12345);
    std::vector<nsg::SortSegment> stack(128);
    long heapsorted = 0;
    for (int c = 0; c < cases; ++c) {
        const int n = 1 + static_cast<int>(rng() % (c < cases / 2 ? 400 : 20000));
        const int levels = 1 + static_cast<int>(rng() % (c % 3 == 0 ? 5 : 200));
        std::vector<float> key(n);
        for (auto& k : key) k = static_cast<float>(rng() % levels) * 0.25f;
        if (c % 7 == 0) key[rng() % n] = 0.0f;
        const int T = 1 + static_cast<int>(rng() % 40);
        if (!check(key, T, stack, c, heapsorted)) return 1;
    }
    // adversarial inputs: the depth budget runs out on segments that cover
    // the prefix
    long adv_heap = 0;
    for (int c = 0; c < 60; ++c) {
        const int n = 200 + static_cast<int>(rng() % 12000);
        std::vector<float> key = adversarial_keys(n, c % 2 == 1);
        // plant ties: a share of the keys rounded to coarse levels
        if (c % 3 != 0) {
            const int coarse = 2 + static_cast<int>(rng() % 64);
            for (auto& k : key)
                if (rng() % 4 == 0) k = static_cast<float>(static_cast<int>(k) / coarse * coarse);
        }
        for (int T : {1, 2, 7, 8, 33, n / 2, n}) {
            long h = 0;
            if (!check(key, T, stack, 100000 + c, h)) return 1;
            adv_heap += h;
        }
    }
    heapsorted += adv_heap;
    if (adv_heap == 0) {
        std::printf("the adversarial inputs never reached the heapsort branch\n");
        return 1;
    }
    // the heap steps alone against the library's heap algorithms
    for (int c = 0; c < 400; ++c) {
        const int n = 1 + static_cast<int>(rng() % 3000);
        const int levels = 1 + static_cast<int>(rng() % 30);
        std::vector<float> key(n);
        for (auto& k : key) k = static_cast<float>(rng() % levels);
        std::vector<int> ref(n), got(n);
        std::iota(ref.begin(), ref.end(), 0);
        std::shuffle(ref.begin(), ref.end(), rng);
        got = ref;
        auto less = [&](int a, int b) { return key[a] < key[b]; };
        std::make_heap(ref.begin(), ref.end(), less);
        std::sort_heap(ref.begin(), ref.end(), less);
        nsg::heap_sort_like_reference(key.data(), got.data(), n);
        if (ref != got) {
            std::printf("HEAP MISMATCH case %d n=%d\n", c, n);
            return 1;
        }
    }
    std::printf("ok %d heapsorted %ld\n", cases, heapsorted);
    return 0;
}
