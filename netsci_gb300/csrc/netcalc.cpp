// netcalc:: API over CuArray (include/netcalc/*.h).
//
// Signatures, argument meaning, return values and exception types follow
// the reference (netcalc/src/mutual_information.cpp, generalized_correlation
// .cpp, hedetniemi.cpp, psi.cpp). The GPU platform differs in structure:
// instead of one blocking device call per pair, X is uploaded once and all
// pairs of `ab` run through the KSG planner (engine.cpp).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "apsp.h"
#include "cuarray.h"
#include "engine.h"
#include "errors.h"
#include "ksg_cpu.h"
#include "netcalc/generalized_correlation.h"
#include "netcalc/hedetniemi.h"
#include "netcalc/mutual_information.h"
#include "netcalc/math_utils.h"
#include "netcalc/psi.h"
#include "rowstats.h"

namespace nsg {
namespace {

void check_variables(int xd, int d, int k, int n) {
    if (xd != 2) invalid("xd must be 2 (two random variables per pair)");
    if (d < 1 || d > 3) invalid("d must be 1, 2 or 3");
    if (n < 2) invalid("n must be at least 2");
    if (k < 1 || k >= n) invalid("k must satisfy 1 <= k < n");
}

// X of the pair-list calls: every node row must hold d*n values.
void check_rows(CuArray<float>* X, int d, int n, const char* what) {
    if (!X || !X->allocatedHost() || !X->host()) invalid(std::string(what) + " has no host data");
    if (X->n() < d * n) {
        invalid(std::string(what) + " rows hold " + std::to_string(X->n()) +
                " values; d*n = " + std::to_string(d * n) + " are needed");
    }
}

// Xa / Xb of the per-pair calls: the buffer is read as d planes of n values
// whatever its m x n shape (the reference indexes Xa[i + c*n] on the
// contiguous host buffer), so it must hold d*n values in total.
void check_variable(CuArray<float>* X, int d, int n, const char* what) {
    if (!X || !X->allocatedHost() || !X->host()) invalid(std::string(what) + " has no host data");
    if (X->size() < d * n) {
        invalid(std::string(what) + " holds " + std::to_string(X->size()) +
                " values; d*n = " + std::to_string(d * n) + " are needed");
    }
}

int round_up(int v, int q) { return (v + q - 1) / q * q; }

// Upload rows [r0, r0+rows) of X as d planes of n samples each, plane stride
// ld (a multiple of 64 floats, so every plane starts 256-byte aligned).
DeviceBuffer upload_rows(CuArray<float>* X, int rows, int d, int n, int* ld_out) {
    const int ld = round_up(n, 64);
    DeviceBuffer buf(static_cast<size_t>(rows) * d * ld * sizeof(float));
    const size_t row_stride = static_cast<size_t>(X->n());
    if (row_stride == static_cast<size_t>(d) * n) {
        NSG_CUDA(cudaMemcpy2D(buf.get(), ld * sizeof(float), X->host(), n * sizeof(float),
                              n * sizeof(float), static_cast<size_t>(rows) * d,
                              cudaMemcpyHostToDevice));
    } else {
        for (int r = 0; r < rows; ++r) {
            NSG_CUDA(cudaMemcpy2D(buf.as<float>() + static_cast<size_t>(r) * d * ld,
                                  ld * sizeof(float), X->host() + r * row_stride,
                                  n * sizeof(float), n * sizeof(float), d,
                                  cudaMemcpyHostToDevice));
        }
    }
    *ld_out = ld;
    return buf;
}

// MI of ab rows [first, first+count) on the GPU into host `out`, with X
// already resident as d planes of stride ld per node row.
void gpu_pair_list(const DeviceBuffer& xd, int ld, int nodes, CuArray<int>* ab, int first,
                   int count, int k, int n, int d, float* out) {
    if (count <= 0) return;
    std::vector<nsg_ksg_pair> pairs(count);
    for (int p = 0; p < count; ++p) {
        const int a = ab->get(first + p, 0);
        const int b = ab->get(first + p, 1);
        if (a < 0 || b < 0 || a >= nodes || b >= nodes) {
            invalid("ab row " + std::to_string(first + p) + " names a node outside X");
        }
        pairs[p] = {xd.as<float>() + static_cast<size_t>(a) * d * ld,
                    xd.as<float>() + static_cast<size_t>(b) * d * ld, nullptr, ld, n};
    }
    DeviceBuffer mi(sizeof(float) * count);
    KsgOutputs o;
    o.mi = mi.as<float>();
    KsgPlan plan(pairs, k, d, o, KsgPlanOptions{});
    plan.run(nullptr);
    NSG_CUDA(cudaMemcpy(out, mi.get(), sizeof(float) * count, cudaMemcpyDeviceToHost));
    raise_fault(plan.take_fault());
}

float gpu_single_pair(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int d) {
    const int ld = round_up(n, 64);
    DeviceBuffer buf(static_cast<size_t>(2) * d * ld * sizeof(float));
    NSG_CUDA(cudaMemcpy2D(buf.get(), ld * sizeof(float), Xa->host(), n * sizeof(float),
                          n * sizeof(float), d, cudaMemcpyHostToDevice));
    NSG_CUDA(cudaMemcpy2D(buf.as<float>() + static_cast<size_t>(d) * ld, ld * sizeof(float),
                          Xb->host(), n * sizeof(float), n * sizeof(float), d,
                          cudaMemcpyHostToDevice));
    std::vector<nsg_ksg_pair> pairs{
        {buf.as<float>(), buf.as<float>() + static_cast<size_t>(d) * ld, nullptr, ld, n}};
    DeviceBuffer mi(sizeof(float));
    KsgOutputs o;
    o.mi = mi.as<float>();
    KsgPlan plan(pairs, k, d, o, KsgPlanOptions{});
    plan.run(nullptr);
    float r = 0.f;
    NSG_CUDA(cudaMemcpy(&r, mi.get(), sizeof(float), cudaMemcpyDeviceToHost));
    raise_fault(plan.take_fault());
    return r;
}

std::string strip_npy(std::string name) {
    if (name.size() > 4 && name.substr(name.size() - 4) == ".npy") name = name.substr(0, name.size() - 4);
    return name;
}

// Shared driver of the four pair-list calls. netcalc/src/mutual_information
// .cpp:8-101, :103-172 and generalized_correlation.cpp:8-102, :104-173.
int pair_list(CuArray<float>* X, CuArray<float>* out, CuArray<int>* ab, int k, int n, int xd,
              int d, int platform, bool gc, int freq, const std::string* ckpt) {
    if (!ab || !out) invalid("null CuArray argument");
    std::string base;
    if (ckpt) {
        if (freq < 1) invalid("checkpointFrequency must be >= 1");
        base = strip_npy(*ckpt);
        ab->save(base + "_ab.npy");
    }
    const int P = ab->m();
    out->init(1, P);
    if (P == 0) return platform;
    if (platform != 0 && platform != 1) fail(NSG_ERR_PLATFORM, "Invalid platform");
    if (ab->n() < 2) invalid("ab must have two columns");
    check_variables(xd, d, k, n);
    check_rows(X, d, n, "X");
    float* res = out->host();
    DeviceBuffer xdev;
    int ld = 0;
    if (platform == 0) xdev = upload_rows(X, X->m(), d, n, &ld);
    auto finish = [&](int lo, int hi) {
        if (gc) for (int i = lo; i < hi; ++i) res[i] = gc_from_mi(res[i], d);
    };
    // Pairs are computed in segments that end where the reference writes a
    // checkpoint (after pair i with i % freq == 0), so each file holds the
    // same values as the reference's.
    int i = 0;
    while (i < P) {
        int hi = P;
        if (ckpt) {
            const int next = (i % freq == 0) ? i : (i / freq + 1) * freq;
            hi = std::min(P, next + 1);
        }
        if (platform == 0) {
            gpu_pair_list(xdev, ld, X->m(), ab, i, hi - i, k, n, d, res + i);
        } else {
            for (int p = i; p < hi; ++p) {
                const int a = ab->get(p, 0), b = ab->get(p, 1);
                if (a < 0 || b < 0 || a >= X->m() || b >= X->m()) {
                    invalid("ab row " + std::to_string(p) + " names a node outside X");
                }
                res[p] = ksg_cpu_pair(X->host() + static_cast<size_t>(a) * X->n(),
                                      X->host() + static_cast<size_t>(b) * X->n(), n, k, d);
            }
        }
        finish(i, hi);
        if (ckpt && (hi - 1) % freq == 0) {
            const int c = hi - 1;
            std::remove((base + "_" + std::to_string(c - freq) + ".npy").c_str());
            out->save(base + "_" + std::to_string(c) + ".npy");
        }
        i = hi;
    }
    return platform;
}

}  // namespace
}  // namespace nsg

// ---------------------------------------------------------------------------
// netcalc namespace
// ---------------------------------------------------------------------------
namespace netcalc {

int mutualInformation(CuArray<float>* X, CuArray<float>* I, CuArray<int>* ab, int k, int n,
                      int xd, int d, int platform, int checkpointFrequency,
                      std::string checkpointFileName) {
    return nsg::pair_list(X, I, ab, k, n, xd, d, platform, false, checkpointFrequency,
                          &checkpointFileName);
}

int mutualInformation(CuArray<float>* X, CuArray<float>* I, CuArray<int>* ab, int k, int n,
                      int xd, int d, int platform) {
    return nsg::pair_list(X, I, ab, k, n, xd, d, platform, false, 0, nullptr);
}

float mutualInformationGpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd, int d) {
    nsg::check_variables(xd, d, k, n);
    nsg::check_variable(Xa, d, n, "Xa");
    nsg::check_variable(Xb, d, n, "Xb");
    return nsg::gpu_single_pair(Xa, Xb, k, n, d);
}

float mutualInformationCpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd, int d) {
    nsg::check_variables(xd, d, k, n);
    nsg::check_variable(Xa, d, n, "Xa");
    nsg::check_variable(Xb, d, n, "Xb");
    return nsg::ksg_cpu_pair(Xa->host(), Xb->host(), n, k, d);
}

void generateRestartAbFromCheckpointFile(CuArray<int>* ab, CuArray<int>* restartAb,
                                         const std::string& checkpointFileName) {
    // netcalc/src/mutual_information.cpp:174-201: the pair index after the
    // last '_' of the file name (directory part ignored).
    std::string name = checkpointFileName;
    const size_t slash = name.find_last_of('/');
    if (slash != std::string::npos) name = name.substr(slash + 1);
    const size_t us = name.find_last_of('_');
    const int last = std::stoi(name.substr(us == std::string::npos ? 0 : us + 1));
    restartAb->fromCuArrayDeepCopy(ab, last + 1, ab->m() - 1, ab->m() - last - 1, 2);
}

int generalizedCorrelation(CuArray<float>* X, CuArray<float>* R, CuArray<int>* ab, int k, int n,
                           int xd, int d, int platform, int checkpointFrequency,
                           std::string checkpointFileName) {
    return nsg::pair_list(X, R, ab, k, n, xd, d, platform, true, checkpointFrequency,
                          &checkpointFileName);
}

int generalizedCorrelation(CuArray<float>* X, CuArray<float>* R, CuArray<int>* ab, int k, int n,
                           int xd, int d, int platform) {
    return nsg::pair_list(X, R, ab, k, n, xd, d, platform, true, 0, nullptr);
}

float generalizedCorrelationGpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd,
                                int d) {
    return nsg::gc_from_mi(mutualInformationGpu(Xa, Xb, k, n, xd, d), d);
}

float generalizedCorrelationCpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd,
                                int d) {
    return nsg::gc_from_mi(mutualInformationCpu(Xa, Xb, k, n, xd, d), d);
}

namespace {
void check_square(CuArray<float>* A) {
    if (!A || !A->allocatedHost() || !A->host()) nsg::invalid("A has no host data");
    if (A->m() != A->n()) nsg::invalid("A must be square");
}
}  // namespace

void hedetniemiAllShortestPaths(CuArray<float>* A, CuArray<float>* H, CuArray<int>* paths,
                                int maxPathLength, float tolerance, int platform) {
    H->init(A->m(), A->n());
    if (platform == 0) {
        hedetniemiAllShortestPathsGpu(A, H, paths, tolerance, maxPathLength);
    } else if (platform == 1) {
        hedetniemiAllShortestPathsCpu(A, H, paths, tolerance, maxPathLength);
    } else {
        throw std::invalid_argument("Invalid platform");
    }
}

void hedetniemiAllShortestPathsGpu(CuArray<float>* A, CuArray<float>* H, CuArray<int>* paths,
                                   float tolerance, int maxPathLength) {
    check_square(A);
    if (maxPathLength < 1) nsg::invalid("maxPathLength must be >= 1");
    const int n = A->n();
    const size_t nn = static_cast<size_t>(n) * n;
    H->init(n, n);
    paths->init(1, n * maxPathLength * n);
    nsg::DeviceBuffer a(nn * sizeof(float)), h(nn * sizeof(float));
    nsg::DeviceBuffer p(nn * maxPathLength * sizeof(int));
    NSG_CUDA(cudaMemcpy(a.get(), A->host(), nn * sizeof(float), cudaMemcpyHostToDevice));
    nsg::apsp_paths(a.as<float>(), h.as<float>(), p.as<int>(), n, maxPathLength, tolerance, nullptr);
    NSG_CUDA(cudaMemcpy(H->host(), h.get(), nn * sizeof(float), cudaMemcpyDeviceToHost));
    NSG_CUDA(cudaMemcpy(paths->host(), p.get(), nn * maxPathLength * sizeof(int),
                        cudaMemcpyDeviceToHost));
}

void hedetniemiAllShortestPathsCpu(CuArray<float>*, CuArray<float>*, CuArray<int>*, float, int) {
    // The reference CPU platform has no shortest-path solver
    // (netcalc/src/hedetniemi_cpu.cpp:5-16); same message, same no-op.
    std::cout << "Path finding on CPU is not implemented yet." << std::endl;
}

void hedetniemiAllShortestPathLengths(CuArray<float>* A, CuArray<float>* H, int maxPathLength,
                                      int platform) {
    H->init(A->m(), A->n());
    if (platform == 0) hedetniemiAllShortestPathLengthsGpu(A, H, maxPathLength);
}

void hedetniemiAllShortestPathLengthsGpu(CuArray<float>* A, CuArray<float>* H,
                                         int maxPathLength) {
    check_square(A);
    if (maxPathLength < 0) nsg::invalid("maxPathLength must be >= 0");
    const int n = A->n();
    const size_t nn = static_cast<size_t>(n) * n;
    H->init(n, n);
    nsg::DeviceBuffer a(nn * sizeof(float)), h(nn * sizeof(float));
    NSG_CUDA(cudaMemcpy(a.get(), A->host(), nn * sizeof(float), cudaMemcpyHostToDevice));
    nsg::apsp_lengths(a.as<float>(), h.as<float>(), n, maxPathLength, nullptr);
    NSG_CUDA(cudaMemcpy(H->host(), h.get(), nn * sizeof(float), cudaMemcpyDeviceToHost));
}

void correlationToAdjacency(CuArray<float>* A, CuArray<float>* C, int n, int platform) {
    A->init(n, n);
    if (platform == 0) correlationToAdjacencyGpu(A, C, n);
}

void correlationToAdjacencyGpu(CuArray<float>* A, CuArray<float>* C, int n) {
    if (n < 0) nsg::invalid("n must be >= 0");
    if (!C || !C->host() || C->size() < n * n) nsg::invalid("C must hold n*n values");
    if (A->m() != n || A->n() != n) A->init(n, n);
    const size_t nn = static_cast<size_t>(n) * n;
    if (nn == 0) return;
    nsg::DeviceBuffer c(nn * sizeof(float)), a(nn * sizeof(float));
    NSG_CUDA(cudaMemcpy(c.get(), C->host(), nn * sizeof(float), cudaMemcpyHostToDevice));
    nsg::corr_to_adjacency(c.as<float>(), a.as<float>(), n, 0, nullptr);
    NSG_CUDA(cudaMemcpy(A->host(), a.get(), nn * sizeof(float), cudaMemcpyDeviceToHost));
}

void recoverSingleShortestPath(int** NUMPY_ARRAY, int** NUMPY_ARRAY_DIM1, CuArray<int>* paths,
                               int maxPathLength, int i, int j) {
    // netcalc/src/hedetniemi.cpp:71-108: node sequence i, the distinct
    // stored nodes of cell (i, j) in order, then j.
    std::vector<int> path{i};
    const int n = static_cast<int>(std::sqrt(static_cast<double>(paths->n() / maxPathLength)));
    for (int p = 0; p < maxPathLength; ++p) {
        const int node = paths->get(0, i * maxPathLength * n + j * maxPathLength + p);
        if (std::find(path.begin(), path.end(), node) == path.end()) path.push_back(node);
    }
    if (std::find(path.begin(), path.end(), j) == path.end()) path.push_back(j);
    *NUMPY_ARRAY_DIM1 = new int[1];
    (*NUMPY_ARRAY_DIM1)[0] = static_cast<int>(path.size());
    *NUMPY_ARRAY = new int[path.size()];
    std::copy(path.begin(), path.end(), *NUMPY_ARRAY);
}

}  // namespace netcalc

void generatePsi(CuArray<float>* psi, int n) {
    // netcalc/src/psi.cpp:6-20, through set() so short tables are left as is.
    psi->set(static_cast<float>(-0.57721566490153), 0, 1);
    for (int i = 1; i < n; ++i) {
        const float inv = static_cast<float>(1.0 / static_cast<float>(i));
        psi->set(psi->get(0, i) + inv, 0, i + 1);
    }
}

// ---- row statistics (netcalc/src/math_utils.cpp:6-36, math_utils_gpu.cu:160-198) ----
namespace {
// Device copy of a (made from the host copy when a has none), u and sigma
// computed on the device and copied back to their host buffers.
void row_stats_cuarray(CuArray<float>* a, CuArray<float>* u, CuArray<float>* sigma, int m, int n) {
    if (!a || !u) nsg::invalid("a and u must be CuArrays");
    if (m < 0 || n < 1) nsg::invalid("row statistics need m >= 0 and n >= 1");
    if (static_cast<long long>(m) * n > a->size()) nsg::invalid("a holds fewer than m*n values");
    if (u->size() < m || (sigma && sigma->size() < m)) {
        nsg::invalid("u and sigma must hold m values (initialise them first)");
    }
    if (m == 0) return;
    if (!a->allocatedDevice()) {
        if (a->allocateDevice() || a->toDevice()) nsg::fail(NSG_ERR_CUDA, "cannot copy a to the device");
    }
    if (!u->allocatedDevice() && u->allocateDevice()) nsg::fail(NSG_ERR_CUDA, "cannot allocate u");
    if (sigma && !sigma->allocatedDevice() && sigma->allocateDevice()) {
        nsg::fail(NSG_ERR_CUDA, "cannot allocate sigma");
    }
    nsg::row_stats(a->device(), u->device(), sigma ? sigma->device() : nullptr, m, n, nullptr);
    NSG_CUDA(cudaDeviceSynchronize());
    if (u->toHost() || (sigma && sigma->toHost())) nsg::fail(NSG_ERR_CUDA, "cannot copy results back");
}
}  // namespace

void mean(CuArray<float>* a, CuArray<float>* u, int m, int n, int platform) {
    if (!a || !u) nsg::invalid("a and u must be CuArrays");
    if (n < 1) nsg::invalid("n must be >= 1");
    m = a->size() / n;
    u->init(1, m);
    if (platform == 0) meanGpu(a, u, m, n);
}

void meanGpu(CuArray<float>* a, CuArray<float>* u, int m, int n) {
    row_stats_cuarray(a, u, nullptr, m, n);
}

void standardDeviation(CuArray<float>* a, CuArray<float>* u, CuArray<float>* sigma, int m, int n,
                       int platform) {
    if (!a || !u || !sigma) nsg::invalid("a, u and sigma must be CuArrays");
    if (n < 1) nsg::invalid("n must be >= 1");
    m = a->size() / n;
    u->init(1, m);
    sigma->init(1, m);
    if (platform == 0) standardDeviationGpu(a, u, sigma, m, n);
}

void standardDeviationGpu(CuArray<float>* a, CuArray<float>* u, CuArray<float>* sigma, int m,
                          int n) {
    if (!sigma) nsg::invalid("sigma must be a CuArray");
    row_stats_cuarray(a, u, sigma, m, n);
}
