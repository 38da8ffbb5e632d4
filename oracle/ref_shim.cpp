// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own, unmodified CPU functions, so that
// tests can pin the restatement in ksg_oracle.cpp against them. Compiled by
// oracle/Makefile (target `ref`) together with the reference sources, where
// they lie; the result goes to oracle/_ref/ and is never shipped or linked by
// the product.

#include <cstdio>
#include <cstring>
#include <limits>
#include <string>

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
CuArray<float>* matrix(const float* x, int rows, int cols) {
    auto* a = new CuArray<float>;
    a->init(rows, cols);
    std::memcpy(a->host(), x, sizeof(float) * (size_t)rows * cols);
    return a;
}

CuArray<int>* pair_list(const int* ab, int P) {
    auto* a = new CuArray<int>;
    a->init(P, 2);
    std::memcpy(a->host(), ab, sizeof(int) * 2 * (size_t)P);
    return a;
}
}  // namespace

// The pair-list drivers in mutual_information.cpp and generalized_correlation.cpp
// name the GPU per-pair functions; this library runs their CPU platform only,
// so those symbols are stubs that report the misuse and return NaN.
float netcalc::mutualInformationGpu(CuArray<float>*, CuArray<float>*, int, int, int, int) {
    std::fprintf(stderr, "liboracle_ref: GPU platform not built into this library\n");
    return std::numeric_limits<float>::quiet_NaN();
}

float netcalc::generalizedCorrelationGpu(CuArray<float>*, CuArray<float>*, int, int, int, int) {
    std::fprintf(stderr, "liboracle_ref: GPU platform not built into this library\n");
    return std::numeric_limits<float>::quiet_NaN();
}

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

// netcalc::mutualInformation / generalizedCorrelation with checkpointing
// (netcalc/src/mutual_information.cpp:8-101, generalized_correlation.cpp:8-102)
// on the CPU platform: X is N rows of d*n floats, ab P rows of (a, b). The
// checkpoint files are written where checkpointFileName says; out receives
// the P results. gc != 0 selects generalizedCorrelation. Returns the
// drivers' return value (the platform), or -1 on an exception.
int ref_pairs_checkpoint(const float* X, int N, int n, int d, const int* ab, int P, int k,
                         int gc, int frequency, const char* file_name, float* out) {
    CuArray<float>* Xc = matrix(X, N, d * n);
    CuArray<int>* abc = pair_list(ab, P);
    auto* R = new CuArray<float>;
    int rc = -1;
    try {
        if (gc)
            rc = netcalc::generalizedCorrelation(Xc, R, abc, k, n, 2, d, 1, frequency,
                                                 std::string(file_name));
        else
            rc = netcalc::mutualInformation(Xc, R, abc, k, n, 2, d, 1, frequency,
                                            std::string(file_name));
        std::memcpy(out, R->host(), sizeof(float) * (size_t)P);
    } catch (...) {
        rc = -1;
    }
    delete R;
    delete abc;
    delete Xc;
    return rc;
}

// netcalc::generateRestartAbFromCheckpointFile (mutual_information.cpp:174-201):
// the rows of ab after the last checkpointed index named in the file name.
// Writes at most cap rows to out and returns the restart list's row count.
int ref_restart_ab(const int* ab, int P, const char* checkpoint_file_name, int* out, int cap) {
    CuArray<int>* abc = pair_list(ab, P);
    auto* r = new CuArray<int>;
    netcalc::generateRestartAbFromCheckpointFile(abc, r, std::string(checkpoint_file_name));
    int m = r->m();
    int rows = m < cap ? m : cap;
    if (rows > 0) std::memcpy(out, r->host(), sizeof(int) * 2 * (size_t)rows);
    delete r;
    delete abc;
    return m;
}

}  // extern "C"
