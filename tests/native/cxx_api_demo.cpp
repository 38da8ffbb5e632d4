// A C++ host of the reference-signature API (include/cuarray.h,
// include/netcalc/*.h): the code a C++ user of netcalc compiles unchanged
// against these headers. CPU platform, so it runs without a GPU.
// Usage: cxx_api_demo <input.bin> (same format as cabi_host_demo)
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "cuarray.h"
#include "netcalc/generalized_correlation.h"
#include "netcalc/mutual_information.h"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    if (std::fread(hdr, sizeof(int), 3, f) != 3) return 2;
    const int N = hdr[0], n = hdr[1], k = hdr[2];
    std::vector<float> x(static_cast<size_t>(N) * n);
    if (std::fread(x.data(), sizeof(float), x.size(), f) != x.size()) return 2;
    std::fclose(f);
    CuArray<float> X;
    X.init(x.data(), N, n);
    CuArray<int> ab;
    ab.init(1, 2);
    ab.set(0, 0, 0);
    ab.set(1, 0, 1);
    CuArray<float> I, R;
    const int r1 = netcalc::mutualInformation(&X, &I, &ab, k, n, 2, 1, 1);
    const int r2 = netcalc::generalizedCorrelation(&X, &R, &ab, k, n, 2, 1, 1);
    std::printf("mi %.9g gc %.9g ret %d %d\n", I.get(0, 0), R.get(0, 0), r1, r2);
    try {
        netcalc::mutualInformation(&X, &I, &ab, k, n, 2, 1, 7);
        std::printf("invalid platform accepted\n");
        return 5;
    } catch (const std::runtime_error&) {
        std::printf("invalid platform throws\n");
    }
    return 0;
}
