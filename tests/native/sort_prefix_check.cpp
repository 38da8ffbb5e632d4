// Compares nsg::sort_prefix_like_reference with std::sort on random arrays
// with many equal keys: positions [0, T) must hold the same indices in the
// same order. Prints "ok <cases>" or the first mismatch. Built and run by
// tests/test_tie_order.py.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include "sort_prefix.h"

int main(int argc, char** argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 2000;
    std::mt19937_64 rng(12345);
    std::vector<nsg::SortSegment> stack(128);
    for (int c = 0; c < cases; ++c) {
        const int n = 1 + static_cast<int>(rng() % (c < cases / 2 ? 400 : 20000));
        const int levels = 1 + static_cast<int>(rng() % (c % 3 == 0 ? 5 : 200));
        std::vector<float> key(n);
        for (auto& k : key) k = static_cast<float>(rng() % levels) * 0.25f;
        if (c % 7 == 0) key[rng() % n] = 0.0f;
        const int T = 1 + static_cast<int>(rng() % 40);
        std::vector<int> ref(n), got(n);
        std::iota(ref.begin(), ref.end(), 0);
        std::iota(got.begin(), got.end(), 0);
        std::sort(ref.begin(), ref.end(), [&](int a, int b) { return key[a] < key[b]; });
        const bool ok = nsg::sort_prefix_like_reference(key.data(), got.data(), n, T, stack.data(),
                                                        static_cast<int>(stack.size()));
        if (!ok) {
            std::printf("unresolved case %d n=%d T=%d\n", c, n, T);
            continue;
        }
        for (int i = 0; i < std::min(T, n); ++i) {
            if (ref[i] != got[i]) {
                std::printf("MISMATCH case %d n=%d levels=%d T=%d at %d: ref %d got %d\n", c, n,
                            levels, T, i, ref[i], got[i]);
                return 1;
            }
        }
    }
    std::printf("ok %d\n", cases);
    return 0;
}
