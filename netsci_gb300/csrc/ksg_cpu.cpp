// CPU platform of the KSG estimator: what netcalc's CPU_PLATFORM (1) runs.
// It is used only when a caller passes platform 1; the GPU platform never
// falls back to it.
//
// Same estimator and arithmetic as netcalc/src/mutual_information_cpu.cpp:
// 6-121 (joint Chebyshev distances, the k nearest, eps as the largest
// marginal distance over them, marginal counts minus one, float psi sum in
// sample order). The per-sample work selects the k+2 smallest joint
// distances instead of sorting all n; only when the k-th and (k+1)-th are
// equal (and non-zero), where the neighbour set depends on the order the
// reference's std::sort leaves equal distances in, is the full index array
// sorted with the reference's comparator. Samples are spread over host
// threads and their terms summed afterwards in sample order, so the result
// is the same float as the reference's sequential pass.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>
#include <vector>

#include "engine.h"
#include "ksg_cpu.h"

namespace nsg {

namespace {

inline float marg(const float* x, int n, int d, int i, int j) {
    float v = std::abs(x[i] - x[j]);
    for (int c = 1; c < d; ++c) v = std::max(v, std::abs(x[i + c * n] - x[j + c * n]));
    return v;
}

void samples_range(const float* xa, const float* xb, int n, int k, int d, const float* psi,
                   int i0, int i1, float* terms) {
    std::vector<float> dz(n);
    std::vector<int> idx(n);
    for (int i = i0; i < i1; ++i) {
        for (int j = 0; j < n; ++j) dz[j] = std::max(marg(xa, n, d, i, j), marg(xb, n, d, i, j));
        std::iota(idx.begin(), idx.end(), 0);
        auto less = [&](int a, int b) { return dz[a] < dz[b] || (dz[a] == dz[b] && a < b); };
        const int sel = std::min(n, k + 2);
        std::nth_element(idx.begin(), idx.begin() + (sel - 1), idx.end(), less);
        std::sort(idx.begin(), idx.begin() + sel, less);
        if (k + 1 < n && dz[idx[k]] == dz[idx[k + 1]] && dz[idx[k]] > 0.f) {
            std::iota(idx.begin(), idx.end(), 0);
            std::sort(idx.begin(), idx.end(), [&](int a, int b) { return dz[a] < dz[b]; });
        }
        float ex = 0.f, ey = 0.f;
        for (int q = 1; q <= k; ++q) {
            ex = std::max(ex, marg(xa, n, d, i, idx[q]));
            ey = std::max(ey, marg(xb, n, d, i, idx[q]));
        }
        int cx = 0, cy = 0;
        for (int j = 0; j < n; ++j) {
            if (marg(xa, n, d, i, j) <= ex) ++cx;
            if (marg(xb, n, d, i, j) <= ey) ++cy;
        }
        terms[i] = psi[cx - 1] + psi[cy - 1];
    }
}

}  // namespace

float ksg_cpu_pair(const float* xa, const float* xb, int n, int k, int d) {
    std::vector<float> psi(static_cast<size_t>(n) + 1);
    host_psi(psi.data(), n);
    std::vector<float> terms(n);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int threads = static_cast<int>(std::min<unsigned>(hw, std::max(1, n / 128)));
    if (threads <= 1) {
        samples_range(xa, xb, n, k, d, psi.data(), 0, n, terms.data());
    } else {
        std::vector<std::thread> pool;
        const int per = (n + threads - 1) / threads;
        for (int t = 0; t < threads; ++t) {
            const int i0 = t * per, i1 = std::min(n, i0 + per);
            if (i0 >= i1) break;
            pool.emplace_back(samples_range, xa, xb, n, k, d, psi.data(), i0, i1, terms.data());
        }
        for (auto& th : pool) th.join();
    }
    float average = 0.0f;
    for (int i = 0; i < n; ++i) average += terms[i];
    average /= static_cast<float>(n);
    return psi[n] + psi[k] - static_cast<float>(1.0 / static_cast<float>(k)) - average;
}

float gc_from_mi(float mi, int d) {
    if (mi <= 0.0) return 0.0f;
    return static_cast<float>(
        std::sqrt(1.0 - static_cast<float>(std::exp(-(2.0 / static_cast<float>(d)) * mi))));
}

}  // namespace nsg
