// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own, unmodified GPU functions
// (netcalc/src/mutual_information_gpu.cu, generalized_correlation_gpu.cpp,
// hedetniemi_gpu.cu, math_utils_gpu.cu), compiled for sm_103a by
// oracle/Makefile (target `ref-gpu`) into oracle/_ref/libnetcalc_ref_gpu.so.
// Tests use them to pin the shortest-path solver and the row statistics
// against the reference kernels, and bench.py times them as the reference's
// GPU per-call path. Never linked by the product.

#include <cstring>

#include "cuarray.h"
#include "generalized_correlation.h"
#include "hedetniemi.h"
#include "math_utils.h"
#include "mutual_information.h"

namespace {
CuArray<float>* copy_in(const float* x, int rows, int cols) {
    auto* a = new CuArray<float>;
    a->init(rows, cols);
    std::memcpy(a->host(), x, sizeof(float) * (size_t)rows * cols);
    return a;
}
}  // namespace

extern "C" {

// netcalc::mutualInformationGpu (netcalc/src/mutual_information_gpu.cu:1007-1079):
// one blocking call per pair, with the reference's own device allocations.
float refgpu_mi(const float* xa, const float* xb, int n, int k, int d) {
    CuArray<float>* a = copy_in(xa, 1, d * n);
    CuArray<float>* b = copy_in(xb, 1, d * n);
    float r = netcalc::mutualInformationGpu(a, b, k, n, 2, d);
    delete a;
    delete b;
    return r;
}

// netcalc::generalizedCorrelationGpu (netcalc/src/generalized_correlation_gpu.cpp:8-32).
float refgpu_gc(const float* xa, const float* xb, int n, int k, int d) {
    CuArray<float>* a = copy_in(xa, 1, d * n);
    CuArray<float>* b = copy_in(xb, 1, d * n);
    float r = netcalc::generalizedCorrelationGpu(a, b, k, n, 2, d);
    delete a;
    delete b;
    return r;
}

// netcalc::hedetniemiAllShortestPathLengths on the GPU platform
// (netcalc/src/hedetniemi.cpp:39-54, hedetniemi_gpu.cu:109-146): A and H are
// n x n row-major; maxPathLength launches of the reference kernel.
void refgpu_apsp_lengths(const float* A, float* H, int n, int max_path_length) {
    CuArray<float>* a = copy_in(A, n, n);
    auto* h = new CuArray<float>;
    netcalc::hedetniemiAllShortestPathLengths(a, h, max_path_length, 0);
    std::memcpy(H, h->host(), sizeof(float) * (size_t)n * n);
    delete h;
    delete a;
}

// mean and standardDeviation on the GPU platform (netcalc/src/math_utils.cpp:6-36,
// math_utils_gpu.cu:22-198): a is m x n row-major; row means from both
// calls, population standard deviations from the second.
void refgpu_row_stats(const float* a, int m, int n, float* u_mean, float* u_sd, float* sigma) {
    CuArray<float>* A = copy_in(a, m, n);
    auto* u = new CuArray<float>;
    mean(A, u, m, n, 0);
    std::memcpy(u_mean, u->host(), sizeof(float) * (size_t)m);
    delete u;
    auto* u2 = new CuArray<float>;
    auto* s = new CuArray<float>;
    standardDeviation(A, u2, s, m, n, 0);
    std::memcpy(u_sd, u2->host(), sizeof(float) * (size_t)m);
    std::memcpy(sigma, s->host(), sizeof(float) * (size_t)m);
    delete s;
    delete u2;
    delete A;
}

}  // extern "C"
