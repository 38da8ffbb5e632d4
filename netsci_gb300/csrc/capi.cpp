// extern "C" boundary (include/netsci_gb300.h). Every entry point catches
// C++ exceptions and returns a status; the message stays readable through
// nsg_last_error() on the calling thread.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <vector>

#include "apsp.h"
#include "cuarray.h"
#include "engine.h"
#include "serve.h"
#include "ksg.cuh"
#include "errors.h"
#include "netcalc/generalized_correlation.h"
#include "netcalc/hedetniemi.h"
#include "netcalc/mutual_information.h"
#include "netcalc/math_utils.h"
#include "netcalc/psi.h"
#include "netchem/network.h"
#include "dcd.h"
#include "rowstats.h"
#include "netsci_gb300.h"

struct nsg_cuarray {
    int dtype;
    void* obj;
};

struct nsg_ksg_plan {
    nsg::KsgPlan* plan;
};

struct nsg_server {
    nsg::Server* server;
};

namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f) {
    try {
        g_last_error.clear();
        f();
        return NSG_OK;
    } catch (const nsg::Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::invalid_argument& e) {
        g_last_error = e.what();
        return std::strcmp(e.what(), "Invalid platform") == 0 ? NSG_ERR_PLATFORM : NSG_ERR_INVALID;
    } catch (const std::bad_alloc& e) {
        g_last_error = std::string("host allocation failed: ") + e.what();
        return NSG_ERR_INVALID;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return NSG_ERR_INVALID;
    } catch (...) {
        g_last_error = "unknown error";
        return NSG_ERR_INVALID;
    }
}

template <typename T>
CuArray<T>* as(nsg_cuarray* a, const char* what) {
    if (!a || !a->obj) nsg::invalid(std::string(what) + " is null");
    const int want = std::is_same<T, float>::value ? NSG_DTYPE_FLOAT32
                     : std::is_same<T, int>::value ? NSG_DTYPE_INT32
                                                   : NSG_DTYPE_FLOAT64;
    if (a->dtype != want) nsg::invalid(std::string(what) + " has the wrong element type");
    return static_cast<CuArray<T>*>(a->obj);
}

// Dispatch a generic lambda over the handle's element type.
template <typename F>
void visit(nsg_cuarray* a, F&& f) {
    if (!a || !a->obj) nsg::invalid("CuArray handle is null");
    switch (a->dtype) {
        case NSG_DTYPE_FLOAT32: f(static_cast<CuArray<float>*>(a->obj)); break;
        case NSG_DTYPE_INT32: f(static_cast<CuArray<int>*>(a->obj)); break;
        case NSG_DTYPE_FLOAT64: f(static_cast<CuArray<double>*>(a->obj)); break;
        default: nsg::invalid("unknown CuArray element type");
    }
}

cudaStream_t stream_of(void* s) { return static_cast<cudaStream_t>(s); }

}  // namespace

extern "C" {

const char* nsg_last_error(void) { return g_last_error.c_str(); }
int nsg_version(void) { return 100; }

int nsg_release_cached_memory(void) {
    return guarded([&] { nsg::release_cached_device_blocks(); });
}
void nsg_free(void* p) { delete[] static_cast<int*>(p); }

// ---- CuArray ---------------------------------------------------------------
int nsg_cuarray_create(int dtype, nsg_cuarray** out) {
    return guarded([&] {
        if (!out) nsg::invalid("out is null");
        auto* h = new nsg_cuarray{dtype, nullptr};
        switch (dtype) {
            case NSG_DTYPE_FLOAT32: h->obj = new CuArray<float>(); break;
            case NSG_DTYPE_INT32: h->obj = new CuArray<int>(); break;
            case NSG_DTYPE_FLOAT64: h->obj = new CuArray<double>(); break;
            default: delete h; nsg::invalid("unknown dtype");
        }
        *out = h;
    });
}

int nsg_cuarray_destroy(nsg_cuarray* a) {
    return guarded([&] {
        if (!a) return;
        visit(a, [](auto* c) { delete c; });
        delete a;
    });
}

int nsg_cuarray_dtype(const nsg_cuarray* a) { return a ? a->dtype : -1; }

int nsg_cuarray_init(nsg_cuarray* a, int m, int n, int* err) {
    return guarded([&] { visit(a, [&](auto* c) { *err = c->init(m, n); }); });
}

int nsg_cuarray_init_from(nsg_cuarray* a, const void* host, int m, int n, int* err) {
    return guarded([&] {
        visit(a, [&](auto* c) {
            using T = std::remove_pointer_t<std::remove_reference_t<decltype(c->host())>>;
            *err = c->init(const_cast<T*>(static_cast<const T*>(host)), m, n);
        });
    });
}

int nsg_cuarray_from_cuarray_shallow(nsg_cuarray* a, nsg_cuarray* src, int start, int end, int m,
                                     int n, int* err) {
    return guarded([&] {
        if (!src || src->dtype != a->dtype) nsg::invalid("source CuArray type differs");
        visit(a, [&](auto* c) {
            *err = c->fromCuArrayShallowCopy(static_cast<decltype(c)>(src->obj), start, end, m, n);
        });
    });
}

int nsg_cuarray_from_cuarray_deep(nsg_cuarray* a, nsg_cuarray* src, int start, int end, int m,
                                  int n, int* err) {
    return guarded([&] {
        if (!src || src->dtype != a->dtype) nsg::invalid("source CuArray type differs");
        visit(a, [&](auto* c) {
            *err = c->fromCuArrayDeepCopy(static_cast<decltype(c)>(src->obj), start, end, m, n);
        });
    });
}

int nsg_cuarray_from_host(nsg_cuarray* a, const void* data, int m, int n, int* err) {
    return nsg_cuarray_init_from(a, data, m, n, err);
}

int nsg_cuarray_shape(const nsg_cuarray* a, int* m, int* n, int* size, size_t* bytes, int* owner,
                      int* ah, int* ad) {
    return guarded([&] {
        visit(const_cast<nsg_cuarray*>(a), [&](auto* c) {
            if (m) *m = c->m();
            if (n) *n = c->n();
            if (size) *size = c->size();
            if (bytes) *bytes = c->bytes();
            if (owner) *owner = c->owner();
            if (ah) *ah = c->allocatedHost();
            if (ad) *ad = c->allocatedDevice();
        });
    });
}

void* nsg_cuarray_host(nsg_cuarray* a) {
    void* p = nullptr;
    if (guarded([&] { visit(a, [&](auto* c) { p = c->host(); }); }) != NSG_OK) return nullptr;
    return p;
}

void* nsg_cuarray_device(nsg_cuarray* a) {
    void* p = nullptr;
    if (guarded([&] { visit(a, [&](auto* c) { p = c->device(); }); }) != NSG_OK) return nullptr;
    return p;
}

#define NSG_CUARRAY_OP(NAME, CALL)                                             \
    int NAME(nsg_cuarray* a, int* err) {                                       \
        return guarded([&] { visit(a, [&](auto* c) { *err = c->CALL(); }); }); \
    }
NSG_CUARRAY_OP(nsg_cuarray_allocate_host, allocateHost)
NSG_CUARRAY_OP(nsg_cuarray_allocate_device, allocateDevice)
NSG_CUARRAY_OP(nsg_cuarray_to_device, toDevice)
NSG_CUARRAY_OP(nsg_cuarray_to_host, toHost)
NSG_CUARRAY_OP(nsg_cuarray_deallocate_host, deallocateHost)
NSG_CUARRAY_OP(nsg_cuarray_deallocate_device, deallocateDevice)
#undef NSG_CUARRAY_OP

int nsg_cuarray_get(const nsg_cuarray* a, int i, int j, double* value) {
    return guarded([&] {
        visit(const_cast<nsg_cuarray*>(a), [&](auto* c) {
            if (!c->allocatedHost() || i < 0 || j < 0 || i >= c->m() || j >= c->n()) {
                nsg::invalid("CuArray index out of range");
            }
            *value = static_cast<double>(c->get(i, j));
        });
    });
}

int nsg_cuarray_set(nsg_cuarray* a, double value, int i, int j, int* err) {
    return guarded([&] {
        visit(a, [&](auto* c) {
            using T = std::remove_pointer_t<std::remove_reference_t<decltype(c->host())>>;
            *err = c->set(static_cast<T>(value), i, j);
        });
    });
}

int nsg_cuarray_load(nsg_cuarray* a, const char* path, int* err) {
    return guarded([&] {
        if (!path) nsg::invalid("path is null");
        visit(a, [&](auto* c) { *err = c->load(path); });
    });
}

int nsg_cuarray_save(nsg_cuarray* a, const char* path) {
    return guarded([&] {
        if (!path) nsg::invalid("path is null");
        visit(a, [&](auto* c) { c->save(path); });
    });
}

int nsg_cuarray_sort(nsg_cuarray* a, int i, nsg_cuarray** out) {
    return guarded([&] {
        visit(a, [&](auto* c) {
            if (i < 0 || i >= c->m()) nsg::invalid("row index out of range");
            *out = new nsg_cuarray{a->dtype, c->sort(i)};
        });
    });
}

int nsg_cuarray_argsort(nsg_cuarray* a, int i, nsg_cuarray** out) {
    return guarded([&] {
        visit(a, [&](auto* c) {
            if (i < 0 || i >= c->m()) nsg::invalid("row index out of range");
            *out = new nsg_cuarray{NSG_DTYPE_INT32, c->argsort(i)};
        });
    });
}

// ---- netcalc ---------------------------------------------------------------
int nsg_mutual_information(nsg_cuarray* X, nsg_cuarray* I, nsg_cuarray* ab, int k, int n, int xd,
                           int d, int platform, int* result) {
    return guarded([&] {
        *result = netcalc::mutualInformation(as<float>(X, "X"), as<float>(I, "I"),
                                             as<int>(ab, "ab"), k, n, xd, d, platform);
    });
}

int nsg_mutual_information_checkpointed(nsg_cuarray* X, nsg_cuarray* I, nsg_cuarray* ab, int k,
                                        int n, int xd, int d, int platform, int freq,
                                        const char* file, int* result) {
    return guarded([&] {
        if (!file) nsg::invalid("checkpoint file name is null");
        *result = netcalc::mutualInformation(as<float>(X, "X"), as<float>(I, "I"),
                                             as<int>(ab, "ab"), k, n, xd, d, platform, freq, file);
    });
}

int nsg_mutual_information_gpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd, int d,
                               float* result) {
    return guarded([&] {
        *result = netcalc::mutualInformationGpu(as<float>(Xa, "Xa"), as<float>(Xb, "Xb"), k, n,
                                                xd, d);
    });
}

int nsg_mutual_information_cpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd, int d,
                               float* result) {
    return guarded([&] {
        *result = netcalc::mutualInformationCpu(as<float>(Xa, "Xa"), as<float>(Xb, "Xb"), k, n,
                                                xd, d);
    });
}

int nsg_generalized_correlation(nsg_cuarray* X, nsg_cuarray* R, nsg_cuarray* ab, int k, int n,
                                int xd, int d, int platform, int* result) {
    return guarded([&] {
        *result = netcalc::generalizedCorrelation(as<float>(X, "X"), as<float>(R, "R"),
                                                  as<int>(ab, "ab"), k, n, xd, d, platform);
    });
}

int nsg_generalized_correlation_checkpointed(nsg_cuarray* X, nsg_cuarray* R, nsg_cuarray* ab,
                                             int k, int n, int xd, int d, int platform, int freq,
                                             const char* file, int* result) {
    return guarded([&] {
        if (!file) nsg::invalid("checkpoint file name is null");
        *result = netcalc::generalizedCorrelation(as<float>(X, "X"), as<float>(R, "R"),
                                                  as<int>(ab, "ab"), k, n, xd, d, platform, freq,
                                                  file);
    });
}

int nsg_generalized_correlation_gpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd,
                                    int d, float* result) {
    return guarded([&] {
        *result = netcalc::generalizedCorrelationGpu(as<float>(Xa, "Xa"), as<float>(Xb, "Xb"), k,
                                                     n, xd, d);
    });
}

int nsg_generalized_correlation_cpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd,
                                    int d, float* result) {
    return guarded([&] {
        *result = netcalc::generalizedCorrelationCpu(as<float>(Xa, "Xa"), as<float>(Xb, "Xb"), k,
                                                     n, xd, d);
    });
}

int nsg_generate_restart_ab_from_checkpoint_file(nsg_cuarray* ab, nsg_cuarray* restart,
                                                 const char* file) {
    return guarded([&] {
        if (!file) nsg::invalid("checkpoint file name is null");
        netcalc::generateRestartAbFromCheckpointFile(as<int>(ab, "ab"), as<int>(restart, "restartAb"),
                                                     file);
    });
}

int nsg_hedetniemi_all_shortest_paths(nsg_cuarray* A, nsg_cuarray* H, nsg_cuarray* paths, int L,
                                      float tol, int platform) {
    return guarded([&] {
        netcalc::hedetniemiAllShortestPaths(as<float>(A, "A"), as<float>(H, "H"),
                                            as<int>(paths, "paths"), L, tol, platform);
    });
}

int nsg_hedetniemi_all_shortest_paths_gpu(nsg_cuarray* A, nsg_cuarray* H, nsg_cuarray* paths,
                                          float tol, int L) {
    return guarded([&] {
        netcalc::hedetniemiAllShortestPathsGpu(as<float>(A, "A"), as<float>(H, "H"),
                                               as<int>(paths, "paths"), tol, L);
    });
}

int nsg_hedetniemi_all_shortest_path_lengths(nsg_cuarray* A, nsg_cuarray* H, int L,
                                             int platform) {
    return guarded([&] {
        netcalc::hedetniemiAllShortestPathLengths(as<float>(A, "A"), as<float>(H, "H"), L,
                                                  platform);
    });
}

int nsg_hedetniemi_all_shortest_path_lengths_gpu(nsg_cuarray* A, nsg_cuarray* H, int L) {
    return guarded([&] {
        netcalc::hedetniemiAllShortestPathLengthsGpu(as<float>(A, "A"), as<float>(H, "H"), L);
    });
}

int nsg_correlation_to_adjacency(nsg_cuarray* A, nsg_cuarray* C, int n, int platform) {
    return guarded([&] {
        netcalc::correlationToAdjacency(as<float>(A, "A"), as<float>(C, "C"), n, platform);
    });
}

int nsg_recover_single_shortest_path(nsg_cuarray* paths, int L, int i, int j, int** path,
                                     int* len) {
    return guarded([&] {
        CuArray<int>* p = as<int>(paths, "paths");
        if (L < 1) nsg::invalid("maxPathLength must be >= 1");
        const int n = static_cast<int>(std::sqrt(static_cast<double>(p->n() / L)));
        if (i < 0 || j < 0 || i >= n || j >= n) nsg::invalid("node index out of range");
        int* dim = nullptr;
        netcalc::recoverSingleShortestPath(path, &dim, p, L, i, j);
        *len = dim[0];
        delete[] dim;
    });
}

int nsg_generate_psi(nsg_cuarray* psi, int n) {
    return guarded([&] { generatePsi(as<float>(psi, "psi"), n); });
}

int nsg_mean(nsg_cuarray* a, nsg_cuarray* u, int m, int n, int platform) {
    return guarded([&] { mean(as<float>(a, "a"), as<float>(u, "u"), m, n, platform); });
}

int nsg_mean_gpu(nsg_cuarray* a, nsg_cuarray* u, int m, int n) {
    return guarded([&] { meanGpu(as<float>(a, "a"), as<float>(u, "u"), m, n); });
}

int nsg_standard_deviation(nsg_cuarray* a, nsg_cuarray* u, nsg_cuarray* sigma, int m, int n,
                           int platform) {
    return guarded([&] {
        standardDeviation(as<float>(a, "a"), as<float>(u, "u"), as<float>(sigma, "sigma"), m, n,
                          platform);
    });
}

int nsg_standard_deviation_gpu(nsg_cuarray* a, nsg_cuarray* u, nsg_cuarray* sigma, int m, int n) {
    return guarded([&] {
        standardDeviationGpu(as<float>(a, "a"), as<float>(u, "u"), as<float>(sigma, "sigma"), m, n);
    });
}

// ---- device-pointer entry points ----------------------------------------------
int nsg_ksg_pairs_device(const nsg_ksg_pair* pairs, int npairs, int k, int d, float* mi,
                         float* gc, float* w, void* stream) {
    return guarded([&] {
        if (npairs < 0 || (npairs && !pairs)) nsg::invalid("bad pair list");
        std::vector<nsg_ksg_pair> v(pairs, pairs + npairs);
        nsg::KsgOutputs o;
        o.mi = mi;
        o.gc = gc;
        o.w = w;
        nsg::KsgPlan plan(v, k, d, o, nsg::KsgPlanOptions{});
        plan.run(stream_of(stream));
        // the plan's descriptors and scratch are released on return
        NSG_CUDA(cudaStreamSynchronize(stream_of(stream)));
        nsg::raise_fault(plan.take_fault());
    });
}

int nsg_ksg_pair_detail_device(const float* xa, const float* xb, int ld, int m, int k, int d,
                               int* n_x, int* n_y, float* eps_x, float* eps_y, float* kdist,
                               float* mi, void* stream) {
    return guarded([&] {
        std::vector<nsg_ksg_pair> v{{xa, xb, nullptr, ld, m}};
        nsg::KsgOutputs o;
        o.mi = mi;
        o.nx = n_x;
        o.ny = n_y;
        o.eps_x = eps_x;
        o.eps_y = eps_y;
        o.kdist = kdist;
        nsg::KsgPlan plan(v, k, d, o, nsg::KsgPlanOptions{});
        plan.run(stream_of(stream));
        NSG_CUDA(cudaStreamSynchronize(stream_of(stream)));
        nsg::raise_fault(plan.take_fault());
    });
}

int nsg_ksg_pair_noalloc_device(const float* xa, const float* xb, int ld, int m, int k, int d,
                                float* mi, float* gc, void* stream) {
    return guarded([&] { nsg::ksg_pair_noalloc(xa, xb, ld, m, k, d, mi, gc, stream_of(stream)); });
}

int nsg_ksg_plan_create(const nsg_ksg_pair* pairs, int npairs, int k, int d, float* mi, float* gc,
                        float* w, int flags, nsg_ksg_plan** out) {
    return guarded([&] {
        if (!out) nsg::invalid("out is null");
        if (npairs < 0 || (npairs && !pairs)) nsg::invalid("bad pair list");
        std::vector<nsg_ksg_pair> v(pairs, pairs + npairs);
        nsg::KsgOutputs o;
        o.mi = mi;
        o.gc = gc;
        o.w = w;
        nsg::KsgPlanOptions opt;
        opt.graph = (flags & 1) != 0;
        opt.timing = (flags & 2) != 0;
        opt.autotune = (flags & 4) != 0;
        *out = new nsg_ksg_plan{new nsg::KsgPlan(v, k, d, o, opt)};
    });
}

int nsg_ksg_plan_run(nsg_ksg_plan* plan, void* stream) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        plan->plan->run(stream_of(stream));
    });
}

int nsg_ksg_plan_shape(const nsg_ksg_plan* plan, int* threads, int* r, int* frames,
                       int* variant) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        const nsg::KsgShape& s = plan->plan->shape();
        if (threads) *threads = s.threads;
        if (r) *r = s.r;
        if (frames) *frames = s.frames;
        if (variant) *variant = plan->plan->variant();
    });
}

int nsg_ksg_plan_staging(const nsg_ksg_plan* plan, int* staging) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        *staging = plan->plan->staging();
    });
}

int nsg_ksg_plan_search(const nsg_ksg_plan* plan, int* mode) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        *mode = plan->plan->search();
    });
}

int nsg_ksg_plan_evaluations(const nsg_ksg_plan* plan, unsigned long long* search,
                             unsigned long long* counts, unsigned long long* compares) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        if (!search || !counts) nsg::invalid("null output");
        plan->plan->evaluations(search, counts, compares);
    });
}

int nsg_ksg_plan_tied_samples(const nsg_ksg_plan* plan, long long* n) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        if (!n) nsg::invalid("null output");
        *n = plan->plan->tied_samples();
    });
}

int nsg_ksg_plan_kernel_ms(const nsg_ksg_plan* plan, float* search_ms, float* count_ms,
                           float* tie_ms) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        if (!search_ms || !count_ms) nsg::invalid("null output");
        plan->plan->kernel_ms(search_ms, count_ms, tie_ms);
    });
}

int nsg_ksg_plan_check(nsg_ksg_plan* plan) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        nsg::raise_fault(plan->plan->take_fault());
    });
}

int nsg_ksg_plan_prepare(nsg_ksg_plan* plan) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        plan->plan->prepare();
    });
}

int nsg_ksg_plan_launches(const nsg_ksg_plan* plan, int* launches) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        *launches = plan->plan->launches();
    });
}

int nsg_ksg_plan_count_ms(const nsg_ksg_plan* plan, float* ms) {
    return guarded([&] {
        if (!plan || !plan->plan) nsg::invalid("plan is null");
        *ms = plan->plan->count_ms();
    });
}

int nsg_ksg_plan_destroy(nsg_ksg_plan* plan) {
    return guarded([&] {
        if (!plan) return;
        delete plan->plan;
        delete plan;
    });
}

int nsg_ksg_set_shape(int threads, int r, int frames, int variant) {
    return guarded([&] { nsg::ksg_force_shape(threads, r, frames, variant); });
}

int nsg_ksg_set_staging(int staging) {
    return guarded([&] {
        if (staging < -1 || staging > 1) nsg::invalid("staging must be -1, 0 or 1");
        nsg::ksg_force_staging(staging);
    });
}

int nsg_ksg_set_search(int mode) {
    return guarded([&] {
        if (mode < -1 || mode > 1) nsg::invalid("search must be -1, 0 or 1");
        nsg::ksg_force_search(mode);
    });
}

int nsg_measure_issue_ceiling(int d, double* search_gops, double* count_gops) {
    return guarded([&] {
        if (!search_gops || !count_gops) nsg::invalid("null output");
        nsg::measure_issue_ceiling(d, search_gops, count_gops);
    });
}

int nsg_ksg_set_orders(int mode) {
    return guarded([&] {
        if (mode < -1 || mode > 1) nsg::invalid("orders must be -1, 0 or 1");
        nsg::ksg_force_orders(mode);
    });
}

int nsg_apsp_set_method(int method) {
    return guarded([&] { nsg::apsp_set_method(method); });
}

int nsg_apsp_lengths_device(const float* A, float* H, int n, int L, int* steps, void* stream) {
    return guarded([&] {
        const int s = nsg::apsp_lengths(A, H, n, L, stream_of(stream));
        if (steps) *steps = s;
    });
}

int nsg_apsp_paths_device(const float* A, float* H, int* paths, int n, int L, float tol,
                          void* stream) {
    return guarded([&] { nsg::apsp_paths(A, H, paths, n, L, tol, stream_of(stream)); });
}

int nsg_corr_to_adjacency_device(const float* C, float* A, int n, int mode, void* stream) {
    return guarded([&] {
        if (mode != 0 && mode != 1) nsg::invalid("mode must be 0 (1/r) or 1 (-ln r)");
        nsg::corr_to_adjacency(C, A, n, mode, stream_of(stream));
    });
}

int nsg_row_stats_device(const float* a, float* u, float* sigma, int m, int n, void* stream) {
    return guarded([&] {
        if (m > 0 && (!a || !u)) nsg::invalid("a and u must be device pointers");
        nsg::row_stats(a, u, sigma, m, n, stream_of(stream));
    });
}

// ---- serving ---------------------------------------------------------------
int nsg_server_create(size_t budget_bytes, double tick_ops, int max_m, nsg_server** out) {
    return guarded([&] {
        if (!out) nsg::invalid("out is null");
        nsg::ServerConfig c;
        if (budget_bytes) c.budget_bytes = budget_bytes;
        if (tick_ops > 0) c.tick_ops = tick_ops;
        if (max_m > 0) c.max_m = max_m;
        *out = new nsg_server{new nsg::Server(c)};
    });
}

int nsg_server_destroy(nsg_server* s) {
    return guarded([&] {
        if (!s) return;
        delete s->server;
        delete s;
    });
}

int nsg_server_register_trajectory(nsg_server* s, const float* X, int N, int m, int d, int* traj) {
    return guarded([&] { *traj = s->server->register_trajectory(X, N, m, d); });
}

int nsg_server_submit_gc(nsg_server* s, int traj, int k, float* out, long long* job) {
    return guarded([&] { *job = s->server->submit_gc(traj, k, out); });
}

int nsg_server_submit_mi(nsg_server* s, const float* x, const float* y, int n, int d, int k,
                         float* out, long long* job) {
    return guarded([&] { *job = s->server->submit_mi(x, y, n, d, k, out); });
}

int nsg_server_submit_apsp(nsg_server* s, const float* A, int N, int L, float* out,
                           long long* job) {
    return guarded([&] { *job = s->server->submit_apsp(A, N, L, out); });
}

int nsg_server_wait(nsg_server* s, long long job, double timeout_s, int* state) {
    return guarded([&] {
        s->server->wait(job, timeout_s);
        *state = s->server->state(job, nullptr);
        if (*state == nsg::JOB_FAILED) nsg::fail(NSG_ERR_CUDA, "job failed: " + s->server->error(job));
    });
}

int nsg_server_job_info(nsg_server* s, long long job, int* state, double* submit_s,
                        double* admit_s, double* done_s) {
    return guarded([&] {
        nsg::JobTimes t;
        const int st = s->server->state(job, &t);
        if (state) *state = st;
        if (submit_s) *submit_s = t.submit;
        if (admit_s) *admit_s = t.admit;
        if (done_s) *done_s = t.done;
    });
}

int nsg_server_stats(nsg_server* s, long long* jobs_done, long long* pairs_done,
                     long long* ticks, size_t* peak_bytes) {
    return guarded([&] { s->server->stats(jobs_done, pairs_done, ticks, peak_bytes); });
}

}  // extern "C"

// ---- netchem -----------------------------------------------------------------
struct nsg_network {
    Network net;
};

namespace {
Network& net_of(nsg_network* h) {
    if (!h) nsg::invalid("network is null");
    return h->net;
}

template <size_t N>
void put_str(char (&dst)[N], const std::string& s) {
    std::memset(dst, 0, N);
    std::memcpy(dst, s.data(), std::min(N - 1, s.size()));
}
}  // namespace

int nsg_network_create(nsg_network** out) {
    return guarded([&] {
        if (!out) nsg::invalid("out is null");
        *out = new nsg_network();
    });
}

int nsg_network_destroy(nsg_network* net) {
    return guarded([&] { delete net; });
}

int nsg_network_init(nsg_network* net, const char* trajectory_file, const char* topology_file,
                     int first_frame, int last_frame, int stride) {
    return guarded([&] {
        if (!trajectory_file || !topology_file) nsg::invalid("file name is null");
        net_of(net).init(trajectory_file, topology_file, first_frame, last_frame, stride);
    });
}

int nsg_network_parse_pdb(nsg_network* net, const char* topology_file) {
    return guarded([&] {
        if (!topology_file) nsg::invalid("file name is null");
        net_of(net).parsePdb(topology_file);
    });
}

int nsg_network_num_nodes(nsg_network* net, int* n) {
    return guarded([&] { *n = net_of(net).numNodes(); });
}

int nsg_network_num_frames(nsg_network* net, int* m) {
    return guarded([&] { *m = net_of(net).numFrames(); });
}

int nsg_network_num_atoms(nsg_network* net, int* n) {
    return guarded([&] { *n = net_of(net).atoms()->numAtoms(); });
}

int nsg_network_node_coordinates(nsg_network* net, nsg_cuarray* out) {
    return guarded([&] {
        CuArray<float>* src = net_of(net).nodeCoordinates();
        CuArray<float>* dst = as<float>(out, "out");
        if (src->size() == 0 || !src->host()) {
            dst->init(0, 0);
            return;
        }
        dst->init(src->host(), src->m(), src->n());
    });
}

int nsg_network_load_node_coordinates(nsg_network* net, const char* npy_file) {
    return guarded([&] {
        if (!npy_file) nsg::invalid("file name is null");
        net_of(net).nodeCoordinates(npy_file);
    });
}

int nsg_network_node(nsg_network* net, int node, nsg_node_info* out) {
    return guarded([&] {
        Network& n = net_of(net);
        if (node < 0 || node >= static_cast<int>(n.nodes().size())) nsg::invalid("node index out of range");
        Node* p = n.nodes()[node];
        out->index = static_cast<int>(p->index());
        out->num_atoms = static_cast<int>(p->numAtoms());
        out->total_mass = p->totalMass();
        out->hash = p->hash();
        put_str(out->tag, p->tag());
    });
}

int nsg_network_node_atoms(nsg_network* net, int node, int* atoms, int cap, int* count) {
    return guarded([&] {
        Network& n = net_of(net);
        if (node < 0 || node >= static_cast<int>(n.nodes().size())) nsg::invalid("node index out of range");
        const std::vector<Atom*> a = n.nodes()[node]->atoms();
        *count = static_cast<int>(a.size());
        for (int i = 0; i < *count && i < cap; ++i) atoms[i] = a[i]->index();
    });
}

int nsg_network_atom(nsg_network* net, int atom, nsg_atom_info* out) {
    return guarded([&] {
        Network& n = net_of(net);
        if (atom < 0 || atom >= n.atoms()->numAtoms()) nsg::invalid("atom index out of range");
        Atom* a = n.atoms()->at(atom);
        out->index = a->index();
        out->serial = a->serial();
        out->residue_id = a->residueId();
        out->occupancy = a->occupancy();
        out->temperature_factor = a->temperatureFactor();
        out->mass = a->mass();
        out->hash = a->hash();
        put_str(out->name, a->name());
        put_str(out->element, a->element());
        put_str(out->residue_name, a->residueName());
        put_str(out->chain_id, a->chainId());
        put_str(out->segment_id, a->segmentId());
        put_str(out->tag, a->tag());
    });
}

int nsg_network_node_from_atom(nsg_network* net, int atom, int* node) {
    return guarded([&] {
        Network& n = net_of(net);
        if (atom < 0 || atom >= n.atoms()->numAtoms()) nsg::invalid("atom index out of range");
        *node = static_cast<int>(n.nodeFromAtomIndex(atom)->index());
    });
}

int nsg_network_device_coordinates(nsg_network* net, const float** X, int* ld) {
    return guarded([&] {
        Network& n = net_of(net);
        *X = n.deviceCoordinates();
        *ld = n.deviceLd();
    });
}

int nsg_dcd_info(const char* path, int* natoms, int* nsets) {
    return guarded([&] {
        if (!path) nsg::invalid("path is null");
        nsg::DcdFile f(path);
        *natoms = f.info().natoms;
        *nsets = f.info().nsets;
    });
}

int nsg_dcd_read(const char* path, int first, int count, int stride, float* xyz) {
    return guarded([&] {
        if (!path) nsg::invalid("path is null");
        if (count < 0 || stride < 1) nsg::invalid("need count >= 0 and stride >= 1");
        nsg::DcdFile f(path);
        const nsg::DcdInfo& I = f.info();
        std::vector<unsigned char> buf(static_cast<size_t>(I.frame_bytes));
        for (int i = 0; i < count; ++i) {
            const long long fr = first + static_cast<long long>(i) * stride;
            if (fr < 0 || fr >= I.nsets) nsg::invalid("frame outside the file");
            f.read_frame(static_cast<int>(fr), buf.data());
            f.check_frame(buf.data(), static_cast<int>(fr));
            float* o = xyz + static_cast<size_t>(i) * 3 * I.natoms;
            f.coordinates(buf.data(), o, o + I.natoms, o + 2 * I.natoms);
        }
    });
}

