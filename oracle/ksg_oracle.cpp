// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference netcalc hot path (KSG mutual information,
// generalized correlation, psi table). It is the parity checker for the CUDA
// path and the "port" CPU baseline: only tests/, __graft_entry__.smoke() and
// bench.py's CPU legs load it. The product library never links or calls it.
//
// Each function names the reference file:line it restates (paths relative to
// the netsci project root). Parity of this restatement is pinned against the
// reference's own golden values (tests/netcalc/python/test_MutualInformation.py
// :37,64) and, where the reference sources are available, against the
// reference CPU functions compiled unmodified into oracle/_ref.
//
// Tie order. The reference orders each sample's candidates with std::sort
// over the frame indices, comparing joint distances with `<`
// (netcalc/src/mutual_information_cpu.cpp:48-53); equal distances end up
// in whatever order that sort leaves them. This restatement makes the same
// call with the same comparator on the same index array, so its neighbour
// sets, and therefore its counts and MI, equal the reference's on every
// input, tied distances included. oracle_mi_pair also reports how many
// samples have a tie at the k-th neighbour whose marginals differ (samples
// whose result depends on that order).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

// Chebyshev (max-abs) distance between samples i and j of one variable stored
// plane-major: x[c*n + s] is component c of sample s.
// netcalc/src/mutual_information_cpu.cpp:28-36 (and :57-65, :79-87).
inline float marginal(const float* x, int n, int d, int i, int j) {
    float v = std::abs(x[i] - x[j]);
    for (int c = 1; c < d; ++c) {
        v = std::max(v, std::abs(x[i + c * n] - x[j + c * n]));
    }
    return v;
}

struct Scratch {
    std::vector<float> dz;
    std::vector<int> order;
};

}  // namespace

extern "C" {

// psi table of n+1 floats: psi[0] = 0, psi[1] = -gamma (stored as float),
// psi[i+1] = psi[i] + (float)(1.0 / (float)i).
// netcalc/src/psi.cpp:6-20 (table sized n+1 by its callers, e.g.
// netcalc/src/mutual_information_cpu.cpp:14-16).
void oracle_psi(float* psi, int n) {
    for (int i = 0; i <= n; ++i) psi[i] = 0.0f;
    if (n >= 1) psi[1] = static_cast<float>(-0.57721566490153);
    for (int i = 1; i < n; ++i) {
        float inv = static_cast<float>(1.0 / static_cast<float>(i));
        psi[i + 1] = psi[i] + inv;
    }
}

// One sample's KSG terms: the joint-distance row, the reference's sort, eps
// over sorted positions 1..k and the marginal counts.
// netcalc/src/mutual_information_cpu.cpp:27-109 (one iteration of its loop
// over samples). Returns 1 when the sample's neighbour set is decided by the
// tie rule (equal k-th and (k+1)-th joint distances with different
// marginals), else 0.
static int sample_terms(const float* xa, const float* xb, int n, int k, int d, int i,
                        Scratch& s, int* cx_out, int* cy_out, float* ex_out, float* ey_out,
                        float* kd_out) {
    // joint distances, :27-47
    for (int j = 0; j < n; ++j) {
        float da = marginal(xa, n, d, i, j);
        float db = marginal(xb, n, d, i, j);
        s.dz[j] = std::max(da, db);
    }
    // ascending order, :48-53 (the reference's comparator)
    std::iota(s.order.begin(), s.order.end(), 0);
    const float* dz = s.dz.data();
    std::sort(s.order.begin(), s.order.end(), [dz](int a, int b) { return dz[a] < dz[b]; });
    // eps over sorted positions 1..k, :54-77
    float ex = 0.0f, ey = 0.0f;
    for (int q = 1; q < k + 1; ++q) {
        int j = s.order[q];
        ex = std::max(ex, marginal(xa, n, d, i, j));
        ey = std::max(ey, marginal(xb, n, d, i, j));
    }
    int tie = 0;
    if (k + 1 < n) {
        int jk = s.order[k], jn = s.order[k + 1];
        if (dz[jk] == dz[jn] &&
            (marginal(xa, n, d, i, jk) != marginal(xa, n, d, i, jn) ||
             marginal(xb, n, d, i, jk) != marginal(xb, n, d, i, jn))) {
            tie = 1;
        }
    }
    // marginal counts over all j (self included), then -1, :78-109
    int cx = 0, cy = 0;
    for (int j = 0; j < n; ++j) {
        if (marginal(xa, n, d, i, j) <= ex) ++cx;
        if (marginal(xb, n, d, i, j) <= ey) ++cy;
    }
    *cx_out = cx - 1;
    *cy_out = cy - 1;
    *ex_out = ex;
    *ey_out = ey;
    *kd_out = dz[s.order[k]];
    return tie;
}

// KSG (algorithm 2) mutual information of one variable pair, with the
// samples spread over `threads` host threads; the per-sample terms are
// summed afterwards in sample order, so the result does not depend on the
// thread count. netcalc/src/mutual_information_cpu.cpp:6-121.
//   xa, xb : d planes of n samples each (plane-major rows of X)
//   psi    : table from oracle_psi(psi, n)
// Optional per-sample outputs (may be null): n_x, n_y (marginal counts after
// the reference's "-1"), eps_x, eps_y (max marginal distance over the k
// nearest joint neighbours), kdist (k-th smallest joint distance, self
// excluded). ties (may be null) receives the number of samples whose
// neighbour set is decided by the tie rule.
float oracle_mi_pair_mt(const float* xa, const float* xb, int n, int k, int d,
                        const float* psi, int* n_x, int* n_y, float* eps_x,
                        float* eps_y, float* kdist, int* ties, int threads) {
    std::vector<int> cx(n), cy(n);
    std::vector<float> ex(n), ey(n), kd(n);
    std::atomic<int> tie_count(0);
    if (threads < 1) threads = 1;
    if (threads > n) threads = n > 0 ? n : 1;
    auto work = [&](int t) {
        Scratch s;
        s.dz.resize(n);
        s.order.resize(n);
        int local = 0;
        for (int i = t; i < n; i += threads) {
            local += sample_terms(xa, xb, n, k, d, i, s, &cx[i], &cy[i], &ex[i], &ey[i], &kd[i]);
        }
        tie_count += local;
    };
    if (threads == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(work, t);
        for (auto& th : pool) th.join();
    }
    // float accumulation in sample order, :110
    float average = 0.0f;
    for (int i = 0; i < n; ++i) average += (psi[cx[i]] + psi[cy[i]]);
    for (int i = 0; i < n; ++i) {
        if (n_x) n_x[i] = cx[i];
        if (n_y) n_y[i] = cy[i];
        if (eps_x) eps_x[i] = ex[i];
        if (eps_y) eps_y[i] = ey[i];
        if (kdist) kdist[i] = kd[i];
    }
    if (ties) *ties = tie_count.load();
    // :113-118
    average /= static_cast<float>(n);
    float mi = psi[n] + psi[k] - static_cast<float>(1.0 / static_cast<float>(k)) - average;
    return mi;
}

// The same on the calling thread only.
float oracle_mi_pair(const float* xa, const float* xb, int n, int k, int d,
                     const float* psi, int* n_x, int* n_y, float* eps_x,
                     float* eps_y, float* kdist, int* ties) {
    return oracle_mi_pair_mt(xa, xb, n, k, d, psi, n_x, n_y, eps_x, eps_y, kdist, ties, 1);
}

// MI from per-sample counts, in the reference's float summation order.
// netcalc/src/mutual_information_gpu.cu:1065-1074.
float oracle_mi_from_counts(const int* n_x, const int* n_y, int n, int k,
                            const float* psi) {
    float average = 0.0f;
    for (int i = 0; i < n; ++i) average += psi[n_x[i]] + psi[n_y[i]];
    average /= static_cast<float>(n);
    return psi[n] + psi[k] - static_cast<float>(1.0 / static_cast<float>(k)) - average;
}

// Generalized correlation of an MI value.
// netcalc/src/generalized_correlation_cpu.cpp:8-26.
float oracle_gc_from_mi(float mi, int d) {
    if (mi <= 0.0) return 0.0f;
    return static_cast<float>(
        std::sqrt(1.0 - static_cast<float>(std::exp(-(2.0 / static_cast<float>(d)) * mi))));
}

// Pair-list driver over a node-row matrix X (N rows of d*n floats), the loop
// of netcalc/src/mutual_information.cpp:103-172 and
// netcalc/src/generalized_correlation.cpp:104-173, spread over `threads`
// host threads (the per-pair function is re-entrant). gc != 0 applies the
// generalized-correlation transform.
void oracle_pairs(const float* X, int N, int n, int d, const int* ab, int P,
                  int k, int gc, float* out, int threads) {
    (void)N;
    std::vector<float> psi(n + 1);
    oracle_psi(psi.data(), n);
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    std::atomic<int>* next = new std::atomic<int>(0);
    auto work = [&]() {
        for (;;) {
            int p = next->fetch_add(1);
            if (p >= P) break;
            const float* xa = X + static_cast<size_t>(ab[2 * p]) * d * n;
            const float* xb = X + static_cast<size_t>(ab[2 * p + 1]) * d * n;
            float mi = oracle_mi_pair(xa, xb, n, k, d, psi.data(), nullptr, nullptr,
                                      nullptr, nullptr, nullptr, nullptr);
            out[p] = gc ? oracle_gc_from_mi(mi, d) : mi;
        }
    };
    for (int t = 0; t < threads; ++t) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    delete next;
}

}  // extern "C"
