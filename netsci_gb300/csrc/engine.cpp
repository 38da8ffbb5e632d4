// KSG planner (see engine.h).
#include "engine.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>

#include "errors.h"
#include "ksg_grid.h"
#include "ksg_registry.cuh"

namespace nsg {

// ---------------------------------------------------------------------------
// DeviceBuffer
// ---------------------------------------------------------------------------
// Freed blocks are kept per device, keyed by size, and handed out again for
// requests of at least half their size. A block is cached only after
// cudaDeviceSynchronize, the same device-wide wait cudaFree performs, so no
// kernel can still be using it when it is handed out. The cache holds at most
// kBlockCacheBytes per device; when cudaMalloc fails, every cached block is
// freed and the allocation retried.
namespace {

constexpr size_t kBlockCacheBytes = size_t(32) << 30;

struct BlockCache {
    std::mutex mu;
    std::map<int, std::multimap<size_t, void*>> blocks;  // device -> size -> block
    std::map<int, size_t> held;                           // device -> bytes cached
};

BlockCache& block_cache() {
    static BlockCache* c = new BlockCache();  // never destroyed: no frees at exit
    return *c;
}

}  // namespace

void release_cached_device_blocks() {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& [dev, m] : c.blocks) {
        cudaSetDevice(dev);
        for (auto& [sz, p] : m) cudaFree(p);
        m.clear();
        c.held[dev] = 0;
    }
    cudaSetDevice(cur);
}

DeviceBuffer::DeviceBuffer(size_t bytes) { reset(bytes); }
DeviceBuffer::~DeviceBuffer() { release(); }
DeviceBuffer::DeviceBuffer(DeviceBuffer&& o) noexcept
    : p_(o.p_), bytes_(o.bytes_), capacity_(o.capacity_), device_(o.device_) {
    o.p_ = nullptr;
    o.bytes_ = 0;
    o.capacity_ = 0;
    o.device_ = -1;
}
DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
        release();
        p_ = o.p_;
        bytes_ = o.bytes_;
        capacity_ = o.capacity_;
        device_ = o.device_;
        o.p_ = nullptr;
        o.bytes_ = 0;
        o.capacity_ = 0;
        o.device_ = -1;
    }
    return *this;
}

void DeviceBuffer::release() {
    if (!p_) return;
    BlockCache& c = block_cache();
    int cur = -1;
    cudaGetDevice(&cur);
    bool cached = false;
    if (cur == device_ && cudaDeviceSynchronize() == cudaSuccess) {
        std::lock_guard<std::mutex> lock(c.mu);
        if (c.held[device_] + capacity_ <= kBlockCacheBytes) {
            c.blocks[device_].emplace(capacity_, p_);
            c.held[device_] += capacity_;
            cached = true;
        }
    }
    if (!cached) cudaFree(p_);
    p_ = nullptr;
    bytes_ = 0;
    capacity_ = 0;
    device_ = -1;
}

void DeviceBuffer::reset(size_t bytes) {
    release();
    if (!bytes) return;
    int dev = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    BlockCache& c = block_cache();
    {
        std::lock_guard<std::mutex> lock(c.mu);
        auto& m = c.blocks[dev];
        auto it = m.lower_bound(bytes);
        if (it != m.end() && it->first / 2 <= bytes) {
            p_ = it->second;
            capacity_ = it->first;
            c.held[dev] -= it->first;
            m.erase(it);
        }
    }
    if (!p_) {
        cudaError_t e = cudaMalloc(&p_, bytes);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            release_cached_device_blocks();
            e = cudaMalloc(&p_, bytes);
        }
        if (e != cudaSuccess) {
            p_ = nullptr;
            NSG_CUDA(e);
        }
        capacity_ = bytes;
    }
    bytes_ = bytes;
    device_ = dev;
}

// ---------------------------------------------------------------------------
// psi tables
// ---------------------------------------------------------------------------
void host_psi(float* psi, int n) {
    for (int i = 0; i <= n; ++i) psi[i] = 0.0f;
    if (n >= 1) psi[1] = static_cast<float>(-0.57721566490153);
    for (int i = 1; i < n; ++i) {
        const float inv = static_cast<float>(1.0 / static_cast<float>(i));
        psi[i + 1] = psi[i] + inv;
    }
}

namespace {
std::mutex g_psi_mu;
struct PsiCache {
    int device = -1;
    int n = -1;
    std::shared_ptr<DeviceBuffer> buf;
};
PsiCache g_psi[16];

std::mutex g_shape_mu;
KsgShape g_forced{0, 0, 0};
int g_forced_variant = -1;
int g_forced_staging = -1;
int g_forced_search = -1;
int g_forced_orders = -1;
// Below this many samples per pair the exhaustive kernel is used: grids of
// a few cells per axis prune little (measured: 0.91x at m = 300, 1.08x at
// m = 1000, 1.28x at m = 2000, whole plans of 48-node trajectories).
constexpr int kGridMinSamples = 1000;
// Plans of a few pairs cannot fill the GPU and wait on launch and setup
// latency, where the grid's three extra launches cost more: one pair took
// 0.28 ms exhaustive against 0.33 ms on grids at m = 2000, and 0.90 against
// 0.72 ms at m = 10000.
constexpr int kGridFewPairs = 8;
constexpr int kGridMinSamplesFew = 4000;
// per batch: work-queue heads (two for the grid search), tie count, tie-kernel counter
constexpr int kCounters = 4;
}  // namespace

std::shared_ptr<const DeviceBuffer> device_psi(int n) {
    int dev = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_psi_mu);
    PsiCache& c = g_psi[dev & 15];
    if (c.device != dev || c.n < n || !c.buf) {
        // The recurrence is prefix-stable: a longer table serves every m below it.
        const int len = std::max(n, std::max(c.device == dev ? c.n : 0, 1024));
        std::vector<float> h(static_cast<size_t>(len) + 1);
        host_psi(h.data(), len);
        auto b = std::make_shared<DeviceBuffer>(h.size() * sizeof(float));
        NSG_CUDA(cudaMemcpy(b->get(), h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        c.device = dev;
        c.n = len;
        c.buf = b;
    }
    return c.buf;
}

void ksg_force_shape(int threads, int r, int frames, int variant) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_forced = {threads, r, frames};
    g_forced_variant = variant;
}

void ksg_force_search(int mode) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_forced_search = mode;
}

void ksg_force_orders(int mode) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_forced_orders = mode;
}

int ksg_forced_orders() {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    return g_forced_orders;
}

void ksg_force_staging(int staging) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_forced_staging = staging;
}

bool ksg_bulk_copy_ok(const std::vector<nsg_ksg_pair>& pairs) {
    for (const auto& p : pairs) {
        if (p.fmap) return false;
        if ((reinterpret_cast<uintptr_t>(p.xa) | reinterpret_cast<uintptr_t>(p.xb)) & 15u) return false;
        if (p.ld & 3) return false;
    }
    return !pairs.empty();
}

int sm_count() {
    static int cached[16] = {0};
    int dev = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    if (!cached[dev & 15]) {
        int v = 0;
        NSG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        cached[dev & 15] = v;
    }
    return cached[dev & 15];
}

// ---------------------------------------------------------------------------
// KsgPlan
// ---------------------------------------------------------------------------
namespace {

// Records `e` on `s`; while `s` is being captured the record becomes an
// event node of the graph (cudaEventRecordExternal), otherwise a plain record.
void record_event(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    NSG_CUDA(cudaStreamIsCapturing(s, &st));
    if (st == cudaStreamCaptureStatusActive) {
        NSG_CUDA(cudaEventRecordWithFlags(e, s, cudaEventRecordExternal));
    } else {
        NSG_CUDA(cudaEventRecord(e, s));
    }
}

long long count_items(const std::vector<nsg_ksg_pair>& pairs, int qc) {
    long long c = 0;
    for (const auto& p : pairs) c += (p.m + qc - 1) / qc;
    return c;
}

}  // namespace

// Timing events per batch: search begin, search end, counts begin (after
// the count-order kernel), counts end, tie kernel begin, tie kernel end.
constexpr int kEventsPerBatch = 6;

KsgPlan::KsgPlan(const std::vector<nsg_ksg_pair>& pairs_in, int k, int d, const KsgOutputs& out,
                 const KsgPlanOptions& opt)
    : d_(d), k_(k), kmax_(ksg_kmax_for(k)), timing_(opt.timing), out_(out), graph_(opt.graph) {
    if (d < 1 || d > 3) invalid("d must be 1, 2 or 3 (got " + std::to_string(d) + ")");
    if (k < 1) invalid("k must be >= 1");
    const int npairs = static_cast<int>(pairs_in.size());
    npairs_ = npairs;
    int maxm = 0;
    long long total_samples = 0;
    for (int p = 0; p < npairs; ++p) {
        const auto& q = pairs_in[p];
        if (!q.xa || !q.xb) invalid("pair " + std::to_string(p) + " has a null row pointer");
        if (q.m < k + 1) {
            invalid("pair " + std::to_string(p) + ": k must be smaller than the number of samples (k=" +
                    std::to_string(k) + ", m=" + std::to_string(q.m) + ")");
        }
        if (!q.fmap && q.ld < q.m) invalid("pair " + std::to_string(p) + ": ld < m");
        if (q.ld < 1) invalid("pair " + std::to_string(p) + ": ld < 1");
        maxm = std::max(maxm, q.m);
        total_samples += q.m;
    }
    if (kmax_ == 0) fail(NSG_ERR_UNSUPPORTED, "k > 62 is not supported by the GPU path");
    const bool per_sample = out.nx || out.ny || out.eps_x || out.eps_y || out.kdist;

    // ---- search: cell grids when every pair allows them -------------------
    int search = opt.search;
    bool tile_forced = opt.shape.threads != 0 || opt.staging == 1;
    {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        if (search < 0) search = g_forced_search;
        tile_forced = tile_forced || g_forced.threads != 0 || g_forced_staging == 1;
    }
    // a forced tile shape or bulk-copy staging asks for the exhaustive kernel
    if (search < 0 && tile_forced) search = 0;
    // Frame-mapped rows (bootstrap resamples) are copied out once per run for
    // the cell-grid search: one copy per distinct (row, map).
    struct RowKey {
        const float* x;
        const int* fmap;
        int m, ld;
        bool operator<(const RowKey& o) const {
            if (x != o.x) return x < o.x;
            if (fmap != o.fmap) return fmap < o.fmap;
            if (m != o.m) return m < o.m;
            return ld < o.ld;
        }
    };
    std::map<RowKey, size_t> mapped;  // row -> offset (floats) of its copy
    size_t mapped_floats = 0;
    double work = 0, work_large = 0;  // sum of m^2, and over pairs with m >= the grid's minimum
    const int grid_min_m = npairs < kGridFewPairs ? kGridMinSamplesFew : kGridMinSamples;
    for (const auto& q : pairs_in) {
        const double w = static_cast<double>(q.m) * q.m;
        work += w;
        if (q.m >= grid_min_m) work_large += w;
        if (!q.fmap) continue;
        for (const float* x : {q.xa, q.xb}) {
            if (mapped.emplace(RowKey{x, q.fmap, q.m, q.ld}, mapped_floats).second) {
                mapped_floats += static_cast<size_t>(d) * ((q.m + 63) / 64 * 64);
            }
        }
    }
    const bool grid_ok = npairs > 0 && mapped_floats * sizeof(float) <= (size_t(8) << 30);
    if (search == 1 && !grid_ok) {
        fail(NSG_ERR_UNSUPPORTED, "cell-grid search: copies of the frame-mapped rows exceed 8 GiB");
    }
    // automatic: grids when most of the work is in pairs large enough to prune
    if (search < 0) search = (grid_ok && work_large >= 0.5 * work) ? 1 : 0;
    search_ = search == 1 ? 1 : 0;
    std::vector<nsg_ksg_pair> eff;
    if (search_ && !mapped.empty()) {
        mapped_rows_.reset(mapped_floats * sizeof(float));
        std::vector<GatherRow> rows;
        for (const auto& kv : mapped) {
            rows.push_back({kv.first.x, kv.first.fmap, mapped_rows_.as<float>() + kv.second, kv.first.ld,
                            kv.first.m, (kv.first.m + 63) / 64 * 64});
        }
        gather_rows_.reset(rows.size() * sizeof(GatherRow));
        NSG_CUDA(cudaMemcpy(gather_rows_.get(), rows.data(), rows.size() * sizeof(GatherRow),
                            cudaMemcpyHostToDevice));
        ngather_ = static_cast<int>(rows.size());
        eff = pairs_in;
        for (auto& q : eff) {
            if (!q.fmap) continue;
            const int ld_out = (q.m + 63) / 64 * 64;
            q.xa = mapped_rows_.as<float>() + mapped.at(RowKey{q.xa, q.fmap, q.m, q.ld});
            q.xb = mapped_rows_.as<float>() + mapped.at(RowKey{q.xb, q.fmap, q.m, q.ld});
            q.fmap = nullptr;
            q.ld = ld_out;
        }
        bootstrap_ = true;
    }
    const std::vector<nsg_ksg_pair>& pairs = eff.empty() ? pairs_in : eff;

    // ---- tile shape -----------------------------------------------------
    // explicit per-plan shape, then the process-wide override, then the
    // autotuner, then the preference order below
    if (opt.shape.threads) {
        shape_ = opt.shape;
        variant_ = opt.variant;
    } else {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        if (g_forced.threads) {
            shape_ = g_forced;
            variant_ = g_forced_variant;
        }
    }
    int staging = opt.staging;
    if (staging < 0) {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        staging = g_forced_staging;
    }
    const bool bulk_ok = ksg_bulk_copy_ok(pairs);
    int tuned_staging = -1;
    if (!shape_.threads && opt.autotune && npairs > 0 && !search_) {
        const KsgTuned t = ksg_autotune(pairs, k, d);
        shape_ = t.shape;
        variant_ = t.variant;
        tuned_staging = t.staging;
    }
    if (shape_.threads) {
        if (!ksg_find_entry(d, kmax_, shape_.threads, shape_.r, shape_.frames, variant_, 0) &&
            !ksg_find_entry(d, kmax_, shape_.threads, shape_.r, shape_.frames, variant_, 1)) {
            fail(NSG_ERR_UNSUPPORTED, "requested KSG shape is not instantiated for this d/k");
        }
    } else {
        // Preference: one sample per thread, CTAs near 256 threads (the best
        // measured shapes at m = 10000); take the first preferred shape that
        // gives every resident CTA slot two work items, else the shape with
        // the smallest per-CTA sample block (small workloads).
        const KsgKernelEntry* cand[32];
        const int nc = std::min(32, ksg_list_entries(d, kmax_, cand, 32));
        std::vector<const KsgKernelEntry*> pref;
        for (int i = 0; i < nc; ++i) {
            if (cand[i]->variant == cand[0]->variant && cand[i]->tma == (staging == 1 && bulk_ok ? 1 : 0)) {
                pref.push_back(cand[i]);
            }
        }
        std::stable_sort(pref.begin(), pref.end(), [](const KsgKernelEntry* a, const KsgKernelEntry* b) {
            if (a->r != b->r) return a->r < b->r;
            return std::abs(a->threads - 256) < std::abs(b->threads - 256);
        });
        const int sms = sm_count();
        const KsgKernelEntry* best = nullptr;
        const KsgKernelEntry* smallest = nullptr;
        for (const KsgKernelEntry* e : pref) {
            const long long qc = static_cast<long long>(e->threads) * e->r;
            if (!smallest || qc < static_cast<long long>(smallest->threads) * smallest->r) smallest = e;
            const long long slots = static_cast<long long>(sms) * std::max(1, e->ctas_per_sm());
            if (!best && count_items(pairs, static_cast<int>(qc)) >= 2 * slots) best = e;
        }
        if (!best) best = smallest;
        if (!best) fail(NSG_ERR_UNSUPPORTED, "no KSG kernel for this d/k");
        shape_ = {best->threads, best->r, best->frames};
        variant_ = best->variant;
    }
    // staging: plain loads unless the plan option, the override or the
    // autotuner asks for bulk copies (which need aligned rows and no frame map)
    if (staging < 0) staging = tuned_staging;
    if (staging < 0) staging = 0;
    const KsgKernelEntry* entry = nullptr;
    if (staging != 0 && bulk_ok) {
        entry = ksg_find_entry(d, kmax_, shape_.threads, shape_.r, shape_.frames, variant_, 1);
    }
    if (staging == 1 && !entry) {
        fail(NSG_ERR_UNSUPPORTED, bulk_ok ? "no bulk-copy kernel for this shape"
                                          : "bulk-copy staging needs aligned rows and no frame map");
    }
    if (!entry) entry = ksg_find_entry(d, kmax_, shape_.threads, shape_.r, shape_.frames, variant_, 0);
    if (!entry) {
        fail(NSG_ERR_UNSUPPORTED, bulk_ok ? "KSG shape only has a bulk-copy kernel; staging was set to loads"
                                          : "KSG shape only has a bulk-copy kernel, which needs aligned rows and no frame map");
    }
    entry_ = entry;
    variant_ = entry->variant;
    const int qc = shape_.threads * shape_.r;

    // ---- order, batches, descriptors, items ------------------------------
    std::vector<int> order(npairs);
    std::iota(order.begin(), order.end(), 0);
    // longest pairs first (their count kernels take longest)
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return pairs[a].m > pairs[b].m; });
    std::vector<long long> prefix(npairs + 1, 0);
    for (int p = 0; p < npairs; ++p) prefix[p + 1] = prefix[p] + pairs[p].m;

    size_t budget = opt.scratch_budget_bytes ? opt.scratch_budget_bytes
                                             : (size_t(1) << (search_ ? 32 : 31));
    long long budget_floats = static_cast<long long>(budget / sizeof(float));
    // cell grids: eps and counts per sample plus the batch's pair grids
    // (2d coordinates and an index per sample) on top of the psi sums
    if (search_) budget_floats = static_cast<long long>(budget / (sizeof(float) * (5 + 2 * d + 1)));
    if (per_sample) budget_floats = std::max<long long>(budget_floats, total_samples);

    std::vector<KsgPairDesc> descs(npairs);
    std::vector<KsgItem> items;
    long long scratch_need = 0;
    int pos = 0;
    while (pos < npairs) {
        Batch b;
        b.pair0 = pos;
        b.item0 = static_cast<int>(items.size());
        long long used = 0;
        while (pos < npairs && (b.npairs == 0 || used + pairs[order[pos]].m <= budget_floats)) {
            const int src = order[pos];
            const auto& q = pairs[src];
            KsgPairDesc& dd = descs[pos];
            dd.xa = q.xa;
            dd.xb = q.xb;
            dd.fmap = q.fmap;
            dd.ld = q.ld;
            dd.m = q.m;
            dd.out = src;
            dd.pad = 0;
            dd.scratch = per_sample ? prefix[src] : used;
            if (!search_) {  // the exhaustive kernel's work queue (the grid kernels index blocks)
                for (int q0 = 0; q0 < q.m; q0 += qc) {
                    items.push_back({pos, q0, std::min(q.m, q0 + qc), 0});
                }
            }
            used += q.m;
            ++b.npairs;
            ++pos;
        }
        b.nitems = static_cast<int>(items.size()) - b.item0;
        const int slots = sm_count() * std::max(1, entry_->ctas_per_sm());
        b.grid = std::max(1, std::min(b.nitems, slots));
        scratch_need = std::max(scratch_need, per_sample ? total_samples : used);
        batches_.push_back(b);
    }

    if (npairs) {
        pairs_dev_.reset(descs.size() * sizeof(KsgPairDesc));
        NSG_CUDA(cudaMemcpy(pairs_dev_.get(), descs.data(), descs.size() * sizeof(KsgPairDesc),
                            cudaMemcpyHostToDevice));
        if (!items.empty()) {
            items_dev_.reset(items.size() * sizeof(KsgItem));
            NSG_CUDA(cudaMemcpy(items_dev_.get(), items.data(), items.size() * sizeof(KsgItem),
                                cudaMemcpyHostToDevice));
        }
        scratch_.reset(static_cast<size_t>(scratch_need) * sizeof(float));
        // per batch: work-queue head, tie count, tie-kernel work counter
        counters_.reset(kCounters * batches_.size() * sizeof(int));
        // Samples with an ambiguous tie are rare (about 1e-4 on trajectory
        // data), but nothing bounds them: the list holds every sample of the
        // largest batch, so it cannot overflow (8 bytes per sample, beside
        // the 4 bytes per sample of the psi terms).
        long long batch_samples = 0;
        for (const Batch& b : batches_) {
            long long sum = 0;
            for (int p = b.pair0; p < b.pair0 + b.npairs; ++p) sum += descs[p].m;
            batch_samples = std::max(batch_samples, sum);
        }
        tie_cap_ = static_cast<int>(std::min<long long>(std::max<long long>(1, batch_samples), 1LL << 30));
        ties_.reset(static_cast<size_t>(tie_cap_) * sizeof(KsgTie));
        tie_stride_ = maxm;
        tie_dz_.reset(static_cast<size_t>(ksg_tie_warps()) * tie_stride_ * sizeof(float));
        tie_idx_.reset(static_cast<size_t>(ksg_tie_warps()) * tie_stride_ * sizeof(int));
        fault_.reset(sizeof(int));
        NSG_CUDA(cudaMemset(fault_.get(), 0, sizeof(int)));
        psi_ = device_psi(maxm);
        if (search_) setup_grid(descs);
    }
    if (timing_) {
        events_.resize(kEventsPerBatch * batches_.size());
        for (auto& e : events_) NSG_CUDA(cudaEventCreate(&e));
    }
}

KsgPlan::~KsgPlan() {
    for (auto e : events_) cudaEventDestroy(e);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
}

void KsgPlan::enqueue(cudaStream_t s) {
    if (batches_.empty()) return;
    NSG_CUDA(cudaMemsetAsync(counters_.get(), 0, kCounters * batches_.size() * sizeof(int), s));
    if (search_) {
        enqueue_grid(s);
        return;
    }
    for (size_t bi = 0; bi < batches_.size(); ++bi) {
        const Batch& b = batches_[bi];
        int* ctr = counters_.as<int>() + kCounters * bi;
        KsgCountArgs a{};
        a.pairs = pairs_dev_.as<KsgPairDesc>();
        a.items = items_dev_.as<KsgItem>() + b.item0;
        a.nitems = b.nitems;
        a.k = k_;
        a.counter = ctr;
        a.fault = fault_.as<int>();
        a.ties = ties_.as<KsgTie>();
        a.tie_count = ctr + 1;
        a.tie_cap = tie_cap_;
        a.psi = psi_->as<float>();
        a.psum = scratch_.as<float>();
        a.nx = out_.nx;
        a.ny = out_.ny;
        a.eps_x = out_.eps_x;
        a.eps_y = out_.eps_y;
        a.kdist = out_.kdist;
        // Under capture, external records stay real event nodes in the graph.
        // The exhaustive kernel runs both passes: it is the search interval,
        // and the count interval is empty.
        cudaEvent_t* ev = events_.data() + kEventsPerBatch * bi;
        if (timing_) record_event(ev[0], s);
        entry_->launch(a, b.grid, s);
        NSG_CUDA(cudaGetLastError());
        if (timing_) {
            for (int j = 1; j < 5; ++j) record_event(ev[j], s);
        }
        KsgTieArgs t{};
        t.pairs = pairs_dev_.as<KsgPairDesc>();
        t.ties = ties_.as<KsgTie>();
        t.tie_count = ctr + 1;
        t.tie_cap = tie_cap_;
        t.tie_next = ctr + 2;
        t.k = k_;
        t.fault = fault_.as<int>();
        t.psi = psi_->as<float>();
        t.psum = scratch_.as<float>();
        t.nx = out_.nx;
        t.ny = out_.ny;
        t.eps_x = out_.eps_x;
        t.eps_y = out_.eps_y;
        t.dz = tie_dz_.as<float>();
        t.idx = tie_idx_.as<int>();
        t.stride = tie_stride_;
        ksg_launch_ties(t, d_, s);
        if (timing_) record_event(ev[5], s);
        KsgFinalArgs f{};
        f.pairs = pairs_dev_.as<KsgPairDesc>() + b.pair0;
        f.npairs = b.npairs;
        f.k = k_;
        f.d = d_;
        f.psi = psi_->as<float>();
        f.psum = scratch_.as<float>();
        f.mi = out_.mi;
        f.gc = out_.gc;
        f.w = out_.w;
        ksg_launch_final(f, s);
    }
}

// ---- cell-grid search ---------------------------------------------------------
struct KsgPlan::GridState {
    DeviceBuffer nodes, node_arena;       // GridNode[nnodes] and their buffers
    DeviceBuffer gps, pair_arena;         // GridPair per plan pair; pair grids of one batch
    std::vector<int> batch_maxm;          // largest m of each batch
    std::vector<char> batch_order;        // whether each batch builds query orders
    bool node_est = false;                // some batch does: nodes need scale estimates
    DeviceBuffer wprefix;                 // per batch: npairs+1 prefix of ceil(m/32)
    std::vector<long long> wprefix_off;   // offset of each batch's prefix
    DeviceBuffer groups, gprefix;         // count groups and their item prefix, per batch
    std::vector<long long> group_off, gprefix_off;
    std::vector<int> ngroups;
    DeviceBuffer corder;                  // count-query order: ngroups x largest m of a batch
    DeviceBuffer eps_a, eps_b, cnt_a, cnt_b;
    DeviceBuffer evals;                   // 3 counters per run (see GridArgs::evals)
    int nnodes = 0;
    int search_grid = 0, count_grid = 0;
};

void KsgPlan::setup_grid(const std::vector<KsgPairDesc>& descs) {
    auto g = std::make_shared<GridState>();
    // nodes: one per distinct (row, m, ld)
    struct Key {
        const float* x;
        int m, ld;
        bool operator<(const Key& o) const {
            if (x != o.x) return x < o.x;
            if (m != o.m) return m < o.m;
            return ld < o.ld;
        }
    };
    std::map<Key, int> ids;
    std::vector<GridNode> nodes;
    std::vector<size_t> node_off;
    size_t arena = 0;
    auto node_id = [&](const float* x, int m, int ld) {
        auto it = ids.find({x, m, ld});
        if (it != ids.end()) return it->second;
        const int id = static_cast<int>(nodes.size());
        ids.emplace(Key{x, m, ld}, id);
        GridNode n{};
        n.x = x;
        n.ld = ld;
        n.m = m;
        nodes.push_back(n);
        node_off.push_back(arena);
        arena += grid_node_bytes(m, d_);
        return id;
    };
    std::vector<GridPair> gps(descs.size());
    for (size_t p = 0; p < descs.size(); ++p) {
        gps[p].a = node_id(descs[p].xa, descs[p].m, descs[p].ld);
        gps[p].b = node_id(descs[p].xb, descs[p].m, descs[p].ld);
    }
    g->nnodes = static_cast<int>(nodes.size());
    g->node_arena.reset(std::max<size_t>(arena, 16));
    unsigned char* base = g->node_arena.as<unsigned char>();
    for (size_t i = 0; i < nodes.size(); ++i) {
        nodes[i] = grid_node_at(base + node_off[i], nodes[i].x, nodes[i].ld, nodes[i].m);
    }
    g->nodes.reset(nodes.size() * sizeof(GridNode));
    NSG_CUDA(cudaMemcpy(g->nodes.get(), nodes.data(), nodes.size() * sizeof(GridNode),
                        cudaMemcpyHostToDevice));

    // pair grids: every batch reuses one arena sized for the largest batch
    size_t pair_arena = 0;
    std::vector<int> wpre;
    for (const Batch& b : batches_) {
        size_t off = 0;
        g->wprefix_off.push_back(static_cast<long long>(wpre.size()));
        int acc = 0, maxm = 0;
        for (int p = b.pair0; p < b.pair0 + b.npairs; ++p) {
            maxm = std::max(maxm, descs[p].m);
            wpre.push_back(acc);
            acc += (descs[p].m + 31) / 32;
            off = grid_pair_place(gps[p], off, descs[p].m, d_);
        }
        wpre.push_back(acc);
        g->batch_maxm.push_back(maxm);
        const int forced = ksg_forced_orders();
        const bool order = forced >= 0 ? forced == 1 : grid_orders_pay(acc, sm_count());
        g->batch_order.push_back(order ? 1 : 0);
        g->node_est = g->node_est || order;
        pair_arena = std::max(pair_arena, off);
    }
    g->pair_arena.reset(std::max<size_t>(pair_arena, 16));
    for (auto& gp : gps) grid_pair_rebase(gp, g->pair_arena.get());
    // count groups: pairs of a batch that count the same node's variable
    {
        std::vector<CountGroup> groups;
        std::vector<int> gpre;
        for (const Batch& b : batches_) {
            g->group_off.push_back(static_cast<long long>(groups.size()));
            g->gprefix_off.push_back(static_cast<long long>(gpre.size()));
            const size_t first = groups.size();
            append_count_groups(gps.data() + b.pair0, b.npairs, groups);
            int acc = 0;
            for (size_t gi = first; gi < groups.size(); ++gi) {
                gpre.push_back(acc);
                acc += (nodes[groups[gi].node].m + kCountQueries - 1) / kCountQueries;
            }
            gpre.push_back(acc);
            g->ngroups.push_back(static_cast<int>(groups.size() - first));
        }
        size_t corder = 0;
        for (size_t bi = 0; bi < batches_.size(); ++bi) {
            if (g->batch_order[bi]) {
                corder = std::max(corder, static_cast<size_t>(g->ngroups[bi]) * g->batch_maxm[bi]);
            }
        }
        g->corder.reset(std::max<size_t>(1, corder) * sizeof(int));
        g->groups.reset(std::max<size_t>(1, groups.size()) * sizeof(CountGroup));
        if (!groups.empty()) {
            NSG_CUDA(cudaMemcpy(g->groups.get(), groups.data(), groups.size() * sizeof(CountGroup),
                                cudaMemcpyHostToDevice));
        }
        g->gprefix.reset(gpre.size() * sizeof(int));
        NSG_CUDA(cudaMemcpy(g->gprefix.get(), gpre.data(), gpre.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    g->gps.reset(gps.size() * sizeof(GridPair));
    NSG_CUDA(cudaMemcpy(g->gps.get(), gps.data(), gps.size() * sizeof(GridPair), cudaMemcpyHostToDevice));
    g->wprefix.reset(wpre.size() * sizeof(int));
    NSG_CUDA(cudaMemcpy(g->wprefix.get(), wpre.data(), wpre.size() * sizeof(int), cudaMemcpyHostToDevice));
    const size_t ns = scratch_.bytes() / sizeof(float);
    g->eps_a.reset(ns * sizeof(float));
    g->eps_b.reset(ns * sizeof(float));
    g->cnt_a.reset(ns * sizeof(int));
    g->cnt_b.reset(ns * sizeof(int));
    g->evals.reset(3 * sizeof(unsigned long long));
    g->search_grid = sm_count() * grid_search_ctas_per_sm(d_, kmax_);
    g->count_grid = sm_count() * grid_count_ctas_per_sm(d_);
    grid_ = std::move(g);
    shape_ = {32 * kGridWarps, 1, kGridChunk};
    variant_ = 1;
}

void KsgPlan::enqueue_grid(cudaStream_t s) {
    GridState& g = *grid_;
    NSG_CUDA(cudaMemsetAsync(g.evals.get(), 0, 3 * sizeof(unsigned long long), s));
    grid_launch_gather(gather_rows_.as<GatherRow>(), ngather_, d_, fault_.as<int>(), s);
    grid_launch_nodes(g.nodes.as<GridNode>(), g.nnodes, d_, g.node_est, s);
    for (size_t bi = 0; bi < batches_.size(); ++bi) {
        const Batch& b = batches_[bi];
        int* ctr = counters_.as<int>() + kCounters * bi;
        KsgPairDesc* bp = pairs_dev_.as<KsgPairDesc>() + b.pair0;
        GridPair* bg = g.gps.as<GridPair>() + b.pair0;
        const bool order = g.batch_order[bi] != 0;
        const int search_order =
            grid_launch_pairs(bp, bg, g.nodes.as<GridNode>(), b.npairs, g.batch_maxm[bi], d_, order, s);
        GridArgs a{};
        a.search_order = search_order;
        a.pairs = bp;
        a.gp = bg;
        a.nodes = g.nodes.as<GridNode>();
        a.wprefix = g.wprefix.as<int>() + g.wprefix_off[bi];
        a.groups = g.groups.as<CountGroup>() + g.group_off[bi];
        a.gprefix = g.gprefix.as<int>() + g.gprefix_off[bi];
        a.ngroups = g.ngroups[bi];
        a.npairs = b.npairs;
        a.pair_base = b.pair0;
        a.k = k_;
        a.counter = ctr;
        a.fault = fault_.as<int>();
        a.ties = ties_.as<KsgTie>();
        a.tie_count = ctr + 2;
        a.tie_cap = tie_cap_;
        a.eps_a = g.eps_a.as<float>();
        a.eps_b = g.eps_b.as<float>();
        a.cnt_a = g.cnt_a.as<int>();
        a.cnt_b = g.cnt_b.as<int>();
        a.evals = g.evals.as<unsigned long long>();
        a.eps_x = out_.eps_x;
        a.eps_y = out_.eps_y;
        a.kdist = out_.kdist;
        a.corder = order ? g.corder.as<int>() : nullptr;
        a.corder_ld = g.batch_maxm[bi];
        cudaEvent_t* ev = events_.data() + kEventsPerBatch * bi;
        if (timing_) record_event(ev[0], s);
        grid_launch_search(a, d_, kmax_, g.search_grid, bootstrap_, s);
        if (timing_) record_event(ev[1], s);
        a.counter = ctr + 1;
        const GridArgs c = grid_launch_count_order(a, s);
        if (timing_) record_event(ev[2], s);
        grid_launch_count_kernel(c, d_, g.count_grid, s);
        if (timing_) record_event(ev[3], s);
        grid_launch_combine(bp, b.npairs, g.cnt_a.as<int>(), g.cnt_b.as<int>(), psi_->as<float>(),
                            scratch_.as<float>(), out_.nx, out_.ny, s);
        KsgTieArgs t{};
        t.pairs = pairs_dev_.as<KsgPairDesc>();
        t.ties = ties_.as<KsgTie>();
        t.tie_count = ctr + 2;
        t.tie_cap = tie_cap_;
        t.tie_next = ctr + 3;
        t.k = k_;
        t.fault = fault_.as<int>();
        t.psi = psi_->as<float>();
        t.psum = scratch_.as<float>();
        t.nx = out_.nx;
        t.ny = out_.ny;
        t.eps_x = out_.eps_x;
        t.eps_y = out_.eps_y;
        t.dz = tie_dz_.as<float>();
        t.idx = tie_idx_.as<int>();
        t.stride = tie_stride_;
        if (timing_) record_event(ev[4], s);
        ksg_launch_ties(t, d_, s);
        if (timing_) record_event(ev[5], s);
        KsgFinalArgs f{};
        f.pairs = bp;
        f.npairs = b.npairs;
        f.k = k_;
        f.d = d_;
        f.psi = psi_->as<float>();
        f.psum = scratch_.as<float>();
        f.mi = out_.mi;
        f.gc = out_.gc;
        f.w = out_.w;
        ksg_launch_final(f, s);
    }
}

int KsgPlan::launches() const {
    const int nb = static_cast<int>(batches_.size());
    if (search_ != 1) return 3 * nb;
    if (!nb) return 0;
    // node grids (+ scale estimates), gather; per batch: pair grids, search,
    // counts, combine, ties, final sums (+ search and count orders)
    int n = 1 + (ngather_ ? 1 : 0) + 6 * nb;
    if (grid_) {
        if (grid_->node_est) ++n;
        for (size_t bi = 0; bi < grid_->batch_order.size(); ++bi) {
            if (grid_->batch_order[bi] && grid_->batch_maxm[bi] <= kOrderMaxM) n += 2;
        }
    }
    return n;
}

int KsgPlan::staging() const { return entry_ ? entry_->tma : 0; }

long long KsgPlan::tied_samples() const {
    if (batches_.empty()) return 0;
    std::vector<int> h(kCounters * batches_.size());
    NSG_CUDA(cudaMemcpy(h.data(), counters_.get(), h.size() * sizeof(int), cudaMemcpyDeviceToHost));
    long long n = 0;
    const int slot = search_ ? 2 : 1;  // the tie-list count of each batch
    for (size_t b = 0; b < batches_.size(); ++b) n += h[kCounters * b + slot];
    return n;
}

void KsgPlan::evaluations(unsigned long long* search, unsigned long long* counts,
                          unsigned long long* compares) const {
    *search = *counts = 0;
    if (compares) *compares = 0;
    if (!search_ || !grid_) return;
    unsigned long long h[3] = {0, 0, 0};
    NSG_CUDA(cudaMemcpy(h, grid_->evals.get(), sizeof(h), cudaMemcpyDeviceToHost));
    *search = h[0];
    *counts = h[1];
    if (compares) *compares = h[2];
}

int KsgPlan::take_fault() {
    if (!fault_.get()) return FAULT_NONE;
    int f = 0;
    NSG_CUDA(cudaMemcpy(&f, fault_.get(), sizeof(int), cudaMemcpyDeviceToHost));
    if (f) NSG_CUDA(cudaMemset(fault_.get(), 0, sizeof(int)));
    return f;
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mu;
std::map<std::string, KsgTuned> g_tune;
bool g_tune_loaded = false;

int bucket_pow2(long long v) {
    int b = 0;
    while ((1LL << b) < v) ++b;
    return b;
}

std::string tune_key(int d, int kmax, int maxm, long long npairs) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    return std::string(prop.name) + "|d" + std::to_string(d) + "|K" + std::to_string(kmax) + "|m" +
           std::to_string(bucket_pow2(maxm)) + "|p" + std::to_string(bucket_pow2(npairs));
}

void tune_load() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = std::getenv("NSG_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char key[512];
    KsgTuned t{};
    while (std::fscanf(f, "%511[^\t]\t%d %d %d %d %d %lf\n", key, &t.shape.threads, &t.shape.r,
                       &t.shape.frames, &t.variant, &t.staging, &t.gops) == 7) {
        g_tune[key] = t;
    }
    std::fclose(f);
}

void tune_store(const std::string& key, const KsgTuned& t) {
    const char* path = std::getenv("NSG_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s\t%d %d %d %d %d %.3f\n", key.c_str(), t.shape.threads, t.shape.r,
                 t.shape.frames, t.variant, t.staging, t.gops);
    std::fclose(f);
}
}  // namespace

KsgTuned ksg_autotune(const std::vector<nsg_ksg_pair>& pairs, int k, int d) {
    const int kmax = ksg_kmax_for(k);
    int maxm = 0;
    for (const auto& p : pairs) maxm = std::max(maxm, p.m);
    const std::string key = tune_key(d, kmax, maxm, static_cast<long long>(pairs.size()));
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
    // probe: the longest pairs first, up to 512 of them
    std::vector<nsg_ksg_pair> probe(pairs);
    std::stable_sort(probe.begin(), probe.end(),
                     [](const nsg_ksg_pair& a, const nsg_ksg_pair& b) { return a.m > b.m; });
    if (probe.size() > 512) probe.resize(512);
    double ops = 0;
    for (const auto& p : probe) ops += 8.0 * d * p.m * (p.m - 1.0);
    const KsgKernelEntry* cand[64];
    const int nc = std::min(64, ksg_list_entries(d, kmax, cand, 64));
    const bool bulk_ok = ksg_bulk_copy_ok(probe);
    DeviceBuffer out(sizeof(float) * probe.size());
    KsgTuned best{{0, 0, 0}, -1, 0, -1.0};
    for (int i = 0; i < nc; ++i) {
        if (cand[i]->tma && !bulk_ok) continue;
        KsgPlanOptions o;
        o.timing = true;
        o.shape = {cand[i]->threads, cand[i]->r, cand[i]->frames};
        o.variant = cand[i]->variant;
        o.staging = cand[i]->tma;
        KsgOutputs ko;
        ko.mi = out.as<float>();
        KsgPlan plan(probe, k, d, ko, o);
        plan.run(nullptr);
        NSG_CUDA(cudaDeviceSynchronize());
        plan.run(nullptr);
        NSG_CUDA(cudaDeviceSynchronize());
        const double ms = plan.count_ms();
        const double gops = ms > 0 ? ops / ms / 1e6 : 0;
        if (gops > best.gops) best = {o.shape, o.variant, o.staging, gops};
    }
    g_tune[key] = best;
    tune_store(key, best);
    return best;
}

float KsgPlan::count_ms() const {
    float search = 0.f, counts = 0.f;
    kernel_ms(&search, &counts, nullptr);
    return search + counts;
}

void KsgPlan::kernel_ms(float* search_ms, float* count_ms, float* tie_ms) const {
    if (!timing_) fail(NSG_ERR_INVALID, "plan was created without timing events");
    float search = 0.f, counts = 0.f, ties = 0.f;
    for (size_t b = 0; b < batches_.size(); ++b) {
        const cudaEvent_t* ev = events_.data() + kEventsPerBatch * b;
        NSG_CUDA(cudaEventSynchronize(ev[5]));
        float ms = 0.f;
        NSG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        search += ms;
        NSG_CUDA(cudaEventElapsedTime(&ms, ev[2], ev[3]));
        counts += ms;
        NSG_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
        ties += ms;
    }
    *search_ms = search;
    *count_ms = counts;
    if (tie_ms) *tie_ms = ties;
}

void KsgPlan::run(cudaStream_t s) {
    if (!graph_) {
        enqueue(s);
        return;
    }
    prepare();
    NSG_CUDA(cudaGraphLaunch(exec_, s));
}

void KsgPlan::prepare() {
    if (!graph_) return;
    if (!exec_) {
        NSG_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
        NSG_CUDA(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue(capture_stream_);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(capture_stream_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t g = nullptr;
        NSG_CUDA(cudaStreamEndCapture(capture_stream_, &g));
        const cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
        cudaGraphDestroy(g);
        NSG_CUDA(e);
    }
}

}  // namespace nsg
