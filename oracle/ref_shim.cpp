// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own, unmodified CPU functions, so that
// tests can pin the restatement in ksg_oracle.cpp against them. Compiled by
// oracle/Makefile (target `ref`) together with the reference sources, where
// they lie; the result goes to oracle/_ref/ and is never shipped or linked by
// the product.

#include <cstring>

#include "cuarray.h"
#include "generalized_correlation.h"
#include "mutual_information.h"
#include "psi.h"

namespace {
CuArray<float>* row_view(const float* x, int len) {
    auto* a = new CuArray<float>;
    a->init(1, len);
    std::memcpy(a->host(), x, sizeof(float) * (size_t)len);
    return a;
}
}  // namespace

extern "C" {

// netcalc::mutualInformationCpu (netcalc/src/mutual_information_cpu.cpp:6-121)
float ref_mi_cpu(const float* xa, const float* xb, int n, int k, int d) {
    CuArray<float>* a = row_view(xa, d * n);
    CuArray<float>* b = row_view(xb, d * n);
    float r = netcalc::mutualInformationCpu(a, b, k, n, 2, d);
    delete a;
    delete b;
    return r;
}

// netcalc::generalizedCorrelationCpu
// (netcalc/src/generalized_correlation_cpu.cpp:8-26)
float ref_gc_cpu(const float* xa, const float* xb, int n, int k, int d) {
    CuArray<float>* a = row_view(xa, d * n);
    CuArray<float>* b = row_view(xb, d * n);
    float r = netcalc::generalizedCorrelationCpu(a, b, k, n, 2, d);
    delete a;
    delete b;
    return r;
}

// generatePsi (netcalc/src/psi.cpp:6-20) into a caller buffer of n+1 floats.
void ref_psi(float* out, int n) {
    auto* p = new CuArray<float>;
    p->init(1, n + 1);
    generatePsi(p, n);
    std::memcpy(out, p->host(), sizeof(float) * (size_t)(n + 1));
    delete p;
}

}  // extern "C"
