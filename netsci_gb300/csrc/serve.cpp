// Serving loop (see serve.h).
#include "serve.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

#include "apsp.h"
#include "errors.h"
#include "ksg_registry.cuh"

namespace nsg {

// Device buffer allocated and freed in stream order (cudaMallocAsync /
// cudaFreeAsync), so job turnover never waits for other streams' kernels.
struct AsyncBuffer {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    void alloc(size_t bytes, cudaStream_t st) {
        release();
        s = st;
        NSG_CUDA(cudaMallocAsync(&p, bytes ? bytes : 1, st));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
    void* get() const { return p; }
    ~AsyncBuffer() { release(); }
};

struct Server::Traj {
    DeviceBuffer X;
    DeviceBuffer grid_arena;   // node grids of the rows
    int N = 0, m = 0, d = 0, ld = 0;
    int slot0 = 0;             // node-table slot of row 0
};

struct Server::Job {
    long long id = 0;
    int kind = JOB_GC;
    int state = JOB_PENDING;
    JobTimes t;
    std::string err;
    // inputs
    int traj = -1;                   // GC: registered trajectory
    const float* hx = nullptr;       // MI: host rows; APSP: host matrix
    const float* hy = nullptr;
    float* out = nullptr;            // host output
    int n = 0, d = 0, k = 0, N = 0, L = 0;
    size_t footprint = 0;
    bool admitted = false;           // footprint counted in used_bytes_
    // device state
    AsyncBuffer dx;                  // MI rows (2 x d x ld)
    AsyncBuffer res;                 // results (one float per pair)
    AsyncBuffer grid_arena;          // MI: node grids of the two rows
    int mi_slot = -1;                // MI: node-table slots mi_slot, mi_slot + 1
    int ld = 0;
    std::vector<nsg_ksg_pair> pairs;
    std::vector<std::pair<int, int>> slots;  // node-table slots of each pair's rows
    long long next_pair = 0, done_pairs = 0;
};

namespace {

double steady_seconds() {
    using namespace std::chrono;
    return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}

int round_up(int v, int q) { return (v + q - 1) / q * q; }

constexpr int kServeTieCtas = 32;    // 256 tie warps
constexpr int kServeTieWarps = kServeTieCtas * 8;
constexpr int kNodeSlots = 1 << 17;   // node-grid table entries
constexpr int kMiSlotPairs = 4096;    // concurrent MI jobs with node grids
constexpr int kGridTickPairs = 16384; // largest tick run on cell grids
constexpr int kGridMinSamples = 1000;

}  // namespace

double Server::now() const { return steady_seconds(); }

Server::Server(const ServerConfig& cfg) : cfg_(cfg) {
    NSG_CUDA(cudaGetDevice(&device_));
    NSG_CUDA(cudaStreamCreateWithFlags(&ksg_stream_, cudaStreamNonBlocking));
    NSG_CUDA(cudaStreamCreateWithFlags(&apsp_stream_, cudaStreamNonBlocking));
    NSG_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
    // Tick capacity: enough sample slots for tick_ops of work at the
    // smallest m that still costs something, bounded by memory.
    cap_samples_ = 1LL << 26;  // 64 Mi samples of psi terms (256 MB)
    cap_pairs_ = std::min<long long>(cfg.max_tick_pairs, 1 << 21);
    cap_items_ = cap_samples_ / 64 + cap_pairs_;
    d_pairs_.reset(sizeof(KsgPairDesc) * cap_pairs_);
    d_items_.reset(sizeof(KsgItem) * cap_items_);
    d_scratch_.reset(sizeof(float) * cap_samples_);
    d_counters_.reset(sizeof(int) * 64);
    d_fault_.reset(sizeof(int));
    NSG_CUDA(cudaMemset(d_fault_.get(), 0, sizeof(int)));
    // a tick holds at most cap_samples_ samples; the tie list holds them all,
    // so it cannot overflow
    tie_cap_ = static_cast<int>(cap_samples_);
    d_ties_.reset(sizeof(KsgTie) * tie_cap_);
    d_tie_dz_.reset(sizeof(float) * static_cast<size_t>(kServeTieWarps) * cfg.max_m);
    d_tie_idx_.reset(sizeof(int) * static_cast<size_t>(kServeTieWarps) * cfg.max_m);
    NSG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&h_pairs_), sizeof(KsgPairDesc) * cap_pairs_));
    NSG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&h_items_), sizeof(KsgItem) * cap_items_));
    d_gnodes_.reset(sizeof(GridNode) * kNodeSlots);
    d_gpairs_.reset(sizeof(GridPair) * kGridTickPairs);
    d_wpre_.reset(sizeof(int) * (kGridTickPairs + 1));
    d_groups_.reset(sizeof(CountGroup) * 2 * kGridTickPairs);
    d_gpre_.reset(sizeof(int) * (2 * kGridTickPairs + 1));
    NSG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&h_gpairs_), sizeof(GridPair) * kGridTickPairs));
    NSG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&h_wpre_), sizeof(int) * (kGridTickPairs + 1)));
    for (int i = kMiSlotPairs - 1; i >= 0; --i) free_mi_slots_.push_back(kNodeSlots - 2 * (i + 1));
    psi_ = device_psi(cfg.max_m);
    ksg_thread_ = std::thread([this] { ksg_loop(); });
    apsp_thread_ = std::thread([this] { apsp_loop(); });
}

Server::~Server() {
    stop_ = true;
    cv_.notify_all();
    if (ksg_thread_.joinable()) ksg_thread_.join();
    if (apsp_thread_.joinable()) apsp_thread_.join();
    cudaStreamSynchronize(ksg_stream_);
    cudaStreamSynchronize(apsp_stream_);
    cudaStreamSynchronize(copy_stream_);
    jobs_.clear();
    trajs_.clear();
    if (h_pairs_) cudaFreeHost(h_pairs_);
    if (h_items_) cudaFreeHost(h_items_);
    if (h_gpairs_) cudaFreeHost(h_gpairs_);
    if (h_wpre_) cudaFreeHost(h_wpre_);
    cudaStreamDestroy(ksg_stream_);
    cudaStreamDestroy(apsp_stream_);
    cudaStreamDestroy(copy_stream_);
}

int Server::register_trajectory(const float* X, int N, int m, int d) {
    if (!X || N < 1 || m < 2 || d < 1 || d > 3) invalid("bad trajectory");
    if (m > cfg_.max_m) invalid("m above the server's max_m");
    auto t = std::make_unique<Traj>();
    t->N = N;
    t->m = m;
    t->d = d;
    t->ld = round_up(m, 64);
    const size_t bytes = sizeof(float) * static_cast<size_t>(N) * d * t->ld;
    std::lock_guard<std::mutex> lk(mu_);
    if (used_bytes_ + bytes > cfg_.budget_bytes) fail(NSG_ERR_UNSUPPORTED, "trajectory exceeds the memory budget");
    NSG_CUDA(cudaSetDevice(device_));
    t->X.reset(bytes);
    NSG_CUDA(cudaMemcpy2D(t->X.get(), t->ld * sizeof(float), X, m * sizeof(float),
                          m * sizeof(float), static_cast<size_t>(N) * d, cudaMemcpyHostToDevice));
    // node grids of every row, built once: the cell-grid search of later ticks reads them
    size_t gbytes = 0;
    if (next_node_slot_ + N <= kNodeSlots - 2 * kMiSlotPairs) {
        const size_t per = grid_node_bytes(m, d);
        gbytes = per * N;
        t->grid_arena.reset(gbytes);
        t->slot0 = next_node_slot_;
        std::vector<GridNode> nodes(N);
        const size_t row = static_cast<size_t>(d) * t->ld;
        for (int a = 0; a < N; ++a) {
            nodes[a] = grid_node_at(t->grid_arena.as<unsigned char>() + per * a, t->X.as<float>() + a * row,
                                    t->ld, m);
        }
        GridNode* dst = d_gnodes_.as<GridNode>() + t->slot0;
        NSG_CUDA(cudaMemcpy(dst, nodes.data(), sizeof(GridNode) * N, cudaMemcpyHostToDevice));
        grid_launch_nodes(dst, N, d, true, nullptr);
        NSG_CUDA(cudaDeviceSynchronize());
        next_node_slot_ += N;
    } else {
        t->slot0 = -1;  // node table full: this trajectory runs the exhaustive search
    }
    used_bytes_ += bytes + gbytes;
    peak_bytes_ = std::max(peak_bytes_, used_bytes_);
    trajs_.push_back(std::move(t));
    return static_cast<int>(trajs_.size()) - 1;
}

long long Server::submit_gc(int traj, int k, float* out) {
    std::lock_guard<std::mutex> lk(mu_);
    if (traj < 0 || traj >= static_cast<int>(trajs_.size())) invalid("unknown trajectory");
    const Traj& T = *trajs_[traj];
    if (k < 1 || k >= T.m || !ksg_kmax_for(k)) invalid("bad k");
    if (!out) invalid("null output");
    auto j = std::make_unique<Job>();
    j->id = next_id_++;
    j->kind = JOB_GC;
    j->traj = traj;
    j->k = k;
    j->d = T.d;
    j->n = T.m;
    j->N = T.N;
    j->out = out;
    const long long P = static_cast<long long>(T.N) * (T.N - 1) / 2;
    j->footprint = sizeof(float) * static_cast<size_t>(std::max<long long>(P, 1));
    j->t.submit = now();
    const long long id = j->id;
    ksg_queue_.push_back(id);
    jobs_[id] = std::move(j);
    cv_.notify_all();
    return id;
}

long long Server::submit_mi(const float* x, const float* y, int n, int d, int k, float* out) {
    if (!x || !y || !out) invalid("null pointer");
    if (d < 1 || d > 3 || n < 2 || k < 1 || k >= n || !ksg_kmax_for(k)) invalid("bad sizes");
    if (n > cfg_.max_m) invalid("n above the server's max_m");
    std::lock_guard<std::mutex> lk(mu_);
    auto j = std::make_unique<Job>();
    j->id = next_id_++;
    j->kind = JOB_MI;
    j->hx = x;
    j->hy = y;
    j->n = n;
    j->d = d;
    j->k = k;
    j->out = out;
    j->ld = round_up(n, 64);
    j->footprint = sizeof(float) * (2 * static_cast<size_t>(d) * j->ld + 1);
    j->t.submit = now();
    const long long id = j->id;
    ksg_queue_.push_back(id);
    jobs_[id] = std::move(j);
    cv_.notify_all();
    return id;
}

long long Server::submit_apsp(const float* A, int N, int L, float* out) {
    if (!A || !out || N < 1 || L < 0) invalid("bad APSP job");
    std::lock_guard<std::mutex> lk(mu_);
    auto j = std::make_unique<Job>();
    j->id = next_id_++;
    j->kind = JOB_APSP;
    j->hx = A;
    j->N = N;
    j->L = L;
    j->out = out;
    j->footprint = 3 * sizeof(float) * static_cast<size_t>(N) * N;  // A, H, step buffer
    j->t.submit = now();
    const long long id = j->id;
    apsp_queue_.push_back(id);
    jobs_[id] = std::move(j);
    cv_.notify_all();
    return id;
}

int Server::state(long long id, JobTimes* t) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) invalid("unknown job");
    if (t) *t = it->second->t;
    return it->second->state;
}

const std::string& Server::error(long long id) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) invalid("unknown job");
    return it->second->err;
}

bool Server::wait(long long id, double timeout_s) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) invalid("unknown job");
    Job* j = it->second.get();
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                              std::chrono::duration<double>(timeout_s));
    while (j->state != JOB_DONE && j->state != JOB_FAILED) {
        if (done_cv_.wait_until(lk, deadline) == std::cv_status::timeout) break;
    }
    return j->state == JOB_DONE || j->state == JOB_FAILED;
}

void Server::stats(long long* jobs_done, long long* pairs_done, long long* ticks, size_t* peak) {
    std::lock_guard<std::mutex> lk(mu_);
    if (jobs_done) *jobs_done = jobs_done_;
    if (pairs_done) *pairs_done = pairs_done_;
    if (ticks) *ticks = ticks_;
    if (peak) *peak = peak_bytes_;
}

// Admission: device buffers for an arriving KSG job when its footprint fits.
bool Server::try_admit_locked(Job& j) {
    if (used_bytes_ + j.footprint > cfg_.budget_bytes) return false;
    used_bytes_ += j.footprint;
    peak_bytes_ = std::max(peak_bytes_, used_bytes_);
    j.admitted = true;
    if (j.kind == JOB_GC) {
        const Traj& T = *trajs_[j.traj];
        const long long P = static_cast<long long>(T.N) * (T.N - 1) / 2;
        j.res.alloc(sizeof(float) * std::max<long long>(P, 1), ksg_stream_);
        j.pairs.reserve(P);
        j.slots.reserve(T.slot0 >= 0 ? P : 0);
        const size_t row = static_cast<size_t>(T.d) * T.ld;
        for (int a = 0; a < T.N; ++a)
            for (int b = a + 1; b < T.N; ++b) {
                j.pairs.push_back({T.X.as<float>() + a * row, T.X.as<float>() + b * row, nullptr,
                                   T.ld, T.m});
                if (T.slot0 >= 0) j.slots.push_back({T.slot0 + a, T.slot0 + b});
            }
    } else {
        j.dx.alloc(sizeof(float) * 2 * static_cast<size_t>(j.d) * j.ld, ksg_stream_);
        j.res.alloc(sizeof(float), ksg_stream_);
        NSG_CUDA(cudaMemcpy2DAsync(j.dx.get(), j.ld * sizeof(float), j.hx, j.n * sizeof(float),
                                   j.n * sizeof(float), j.d, cudaMemcpyHostToDevice, ksg_stream_));
        NSG_CUDA(cudaMemcpy2DAsync(j.dx.as<float>() + static_cast<size_t>(j.d) * j.ld,
                                   j.ld * sizeof(float), j.hy, j.n * sizeof(float),
                                   j.n * sizeof(float), j.d, cudaMemcpyHostToDevice, ksg_stream_));
        j.pairs.push_back({j.dx.as<float>(), j.dx.as<float>() + static_cast<size_t>(j.d) * j.ld,
                           nullptr, j.ld, j.n});
        if (!free_mi_slots_.empty()) {
            j.mi_slot = free_mi_slots_.back();
            free_mi_slots_.pop_back();
            const size_t per = grid_node_bytes(j.n, j.d);
            j.grid_arena.alloc(2 * per, ksg_stream_);
            GridNode nodes[2];
            for (int r = 0; r < 2; ++r) {
                nodes[r] = grid_node_at(j.grid_arena.as<unsigned char>() + per * r,
                                        j.dx.as<float>() + static_cast<size_t>(r) * j.d * j.ld, j.ld, j.n);
            }
            GridNode* dst = d_gnodes_.as<GridNode>() + j.mi_slot;
            NSG_CUDA(cudaMemcpyAsync(dst, nodes, sizeof(nodes), cudaMemcpyHostToDevice, ksg_stream_));
            NSG_CUDA(cudaStreamSynchronize(ksg_stream_));  // the host descriptors go out of scope
            grid_launch_nodes(dst, 2, j.d, true, ksg_stream_);
            j.slots.push_back({j.mi_slot, j.mi_slot + 1});
        }
    }
    j.state = JOB_RUNNING;
    j.t.admit = now();
    return true;
}

void Server::release_locked(Job& j) {
    j.dx.release();
    j.res.release();
    j.grid_arena.release();
    if (j.mi_slot >= 0) free_mi_slots_.push_back(j.mi_slot);
    j.mi_slot = -1;
    j.pairs.clear();
    j.pairs.shrink_to_fit();
    j.slots.clear();
    j.slots.shrink_to_fit();
    if (j.admitted) used_bytes_ -= j.footprint;
    j.admitted = false;
}

// One tick over the given job slices (all of one (d, KMAX) group).
// A tick on cell grids when its pairs have node grids and most of its work
// is in pairs with m >= kGridMinSamples; false: the caller runs the
// exhaustive kernel.
bool Server::run_tick_grid(std::vector<std::pair<Job*, std::pair<long long, long long>>>& slices) {
    const int d = slices[0].first->d;
    const int k = slices[0].first->k;
    const int kmax = ksg_kmax_for(k);
    long long np = 0;
    double work = 0, work_large = 0;
    for (auto& sl : slices) {
        Job* j = sl.first;
        const long long cnt = sl.second.second - sl.second.first;
        if (static_cast<long long>(j->slots.size()) != static_cast<long long>(j->pairs.size())) return false;
        np += cnt;
        const double w = static_cast<double>(j->n) * j->n * cnt;
        work += w;
        if (j->n >= kGridMinSamples) work_large += w;
    }
    if (np > kGridTickPairs || work_large < 0.5 * work) return false;

    // descriptors, pair-grid arena offsets, warp-block prefix
    long long samples = 0, wacc = 0;
    int maxm = 0;
    size_t arena = 0;
    long long p = 0;
    std::vector<long long> slice_first(slices.size());
    for (size_t si = 0; si < slices.size(); ++si) {
        Job* j = slices[si].first;
        slice_first[si] = p;
        for (long long q = slices[si].second.first; q < slices[si].second.second; ++q, ++p) {
            const nsg_ksg_pair& pr = j->pairs[q];
            KsgPairDesc& dd = h_pairs_[p];
            dd.xa = pr.xa;
            dd.xb = pr.xb;
            dd.fmap = nullptr;
            dd.ld = pr.ld;
            dd.m = pr.m;
            dd.out = static_cast<int>(q);
            dd.pad = 0;
            dd.scratch = samples;
            samples += pr.m;
            GridPair& g = h_gpairs_[p];
            g.a = j->slots[q].first;
            g.b = j->slots[q].second;
            arena = grid_pair_place(g, arena, pr.m, d);
            h_wpre_[p] = static_cast<int>(wacc);
            wacc += (pr.m + 31) / 32;
            maxm = std::max(maxm, pr.m);
        }
    }
    h_wpre_[np] = static_cast<int>(wacc);
    cudaStream_t s = ksg_stream_;
    // buffers grow on demand (by a quarter more than asked, to grow rarely)
    auto ensure = [&](DeviceBuffer& b, size_t bytes) {
        if (b.bytes() < bytes) {
            NSG_CUDA(cudaStreamSynchronize(s));
            b.reset(bytes + bytes / 4);
        }
    };
    ensure(d_garena_, std::max<size_t>(arena, 16));
    ensure(d_eps_a_, sizeof(float) * samples);
    ensure(d_eps_b_, sizeof(float) * samples);
    ensure(d_cnt_a_, sizeof(int) * samples);
    ensure(d_cnt_b_, sizeof(int) * samples);
    for (long long i = 0; i < np; ++i) grid_pair_rebase(h_gpairs_[i], d_garena_.get());
    NSG_CUDA(cudaMemcpyAsync(d_pairs_.get(), h_pairs_, sizeof(KsgPairDesc) * np, cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemcpyAsync(d_gpairs_.get(), h_gpairs_, sizeof(GridPair) * np, cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemcpyAsync(d_wpre_.get(), h_wpre_, sizeof(int) * (np + 1), cudaMemcpyHostToDevice, s));
    // count groups: pairs of the tick that count the same node's variable
    std::vector<CountGroup> groups;
    append_count_groups(h_gpairs_, static_cast<int>(np), groups);
    std::vector<int> gpre(groups.size() + 1, 0);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        gpre[gi + 1] = gpre[gi] + (h_pairs_[groups[gi].pairs[0]].m + kCountQueries - 1) / kCountQueries;
    }
    const bool order = grid_orders_pay(wacc, sm_count());  // query orders for this tick
    if (order) ensure(d_corder_, sizeof(int) * std::max<size_t>(1, groups.size() * static_cast<size_t>(maxm)));
    NSG_CUDA(cudaMemcpyAsync(d_groups_.get(), groups.data(), sizeof(CountGroup) * groups.size(),
                             cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemcpyAsync(d_gpre_.get(), gpre.data(), sizeof(int) * gpre.size(), cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemsetAsync(d_counters_.get(), 0, sizeof(int) * 4, s));
    int* ctr = d_counters_.as<int>();
    KsgPairDesc* dp = d_pairs_.as<KsgPairDesc>();
    const int search_order = grid_launch_pairs(dp, d_gpairs_.as<GridPair>(), d_gnodes_.as<GridNode>(),
                                               static_cast<int>(np), maxm, d, order, s);
    GridArgs a{};
    a.search_order = search_order;
    a.pairs = dp;
    a.gp = d_gpairs_.as<GridPair>();
    a.nodes = d_gnodes_.as<GridNode>();
    a.wprefix = d_wpre_.as<int>();
    a.groups = d_groups_.as<CountGroup>();
    a.gprefix = d_gpre_.as<int>();
    a.ngroups = static_cast<int>(groups.size());
    a.npairs = static_cast<int>(np);
    a.pair_base = 0;
    a.k = k;
    a.counter = ctr;
    a.fault = d_fault_.as<int>();
    a.ties = d_ties_.as<KsgTie>();
    a.tie_count = ctr + 2;
    a.tie_cap = tie_cap_;
    a.eps_a = d_eps_a_.as<float>();
    a.eps_b = d_eps_b_.as<float>();
    a.cnt_a = d_cnt_a_.as<int>();
    a.cnt_b = d_cnt_b_.as<int>();
    a.corder = order ? d_corder_.as<int>() : nullptr;
    a.corder_ld = maxm;
    const int sms = sm_count();
    grid_launch_search(a, d, kmax, sms * grid_search_ctas_per_sm(d, kmax), false, s);
    a.counter = ctr + 1;
    grid_launch_counts(a, d, sms * grid_count_ctas_per_sm(d), s);
    grid_launch_combine(dp, static_cast<int>(np), a.cnt_a, a.cnt_b, psi_->as<float>(), d_scratch_.as<float>(),
                        nullptr, nullptr, s);
    KsgTieArgs t{};
    t.pairs = dp;
    t.ties = a.ties;
    t.tie_count = ctr + 2;
    t.tie_cap = tie_cap_;
    t.tie_next = ctr + 3;
    t.k = k;
    t.fault = a.fault;
    t.psi = psi_->as<float>();
    t.psum = d_scratch_.as<float>();
    t.dz = d_tie_dz_.as<float>();
    t.idx = d_tie_idx_.as<int>();
    t.stride = cfg_.max_m;
    ksg_launch_ties_ctas(t, d, kServeTieCtas, s);
    for (size_t si = 0; si < slices.size(); ++si) {
        Job* j = slices[si].first;
        KsgFinalArgs f{};
        f.pairs = dp + slice_first[si];
        f.npairs = static_cast<int>(slices[si].second.second - slices[si].second.first);
        f.k = k;
        f.d = d;
        f.psi = psi_->as<float>();
        f.psum = d_scratch_.as<float>();
        if (j->kind == JOB_GC) f.gc = j->res.as<float>();
        else f.mi = j->res.as<float>();
        ksg_launch_final(f, s);
    }
    NSG_CUDA(cudaStreamSynchronize(s));
    int fault = 0;
    NSG_CUDA(cudaMemcpy(&fault, d_fault_.get(), sizeof(int), cudaMemcpyDeviceToHost));
    if (fault) {
        NSG_CUDA(cudaMemset(d_fault_.get(), 0, sizeof(int)));
        raise_fault(fault);
    }
    return true;
}

void Server::run_tick(std::vector<std::pair<Job*, std::pair<long long, long long>>>& slices) {
    if (slices.empty()) return;
    if (run_tick_grid(slices)) return;
    const int d = slices[0].first->d;
    const int k = slices[0].first->k;
    const int kmax = ksg_kmax_for(k);
    // descriptors and items
    long long np = 0, ni = 0, samples = 0;
    long long total_items_256 = 0;
    for (auto& s : slices) {
        for (long long p = s.second.first; p < s.second.second; ++p) {
            total_items_256 += (s.first->pairs[p].m + 255) / 256;
        }
    }
    const int sms = sm_count();
    KsgShape shape = ksg_default_shape(d, kmax);
    const KsgKernelEntry* e = ksg_find_entry(d, kmax, shape.threads, shape.r, shape.frames, -1);
    if (total_items_256 < 2LL * sms * std::max(1, e->ctas_per_sm())) {
        const KsgKernelEntry* small = ksg_find_entry(d, kmax, 64, 1, 512, -1);
        if (small) {
            e = small;
            shape = {64, 1, 512};
        }
    }
    const int qc = shape.threads * shape.r;
    std::vector<long long> slice_first(slices.size());
    for (size_t si = 0; si < slices.size(); ++si) {
        Job* j = slices[si].first;
        slice_first[si] = np;
        for (long long p = slices[si].second.first; p < slices[si].second.second; ++p) {
            const nsg_ksg_pair& q = j->pairs[p];
            KsgPairDesc& dd = h_pairs_[np];
            dd.xa = q.xa;
            dd.xb = q.xb;
            dd.fmap = q.fmap;
            dd.ld = q.ld;
            dd.m = q.m;
            dd.out = static_cast<int>(p);
            dd.pad = 0;
            dd.scratch = samples;
            for (int q0 = 0; q0 < q.m; q0 += qc) h_items_[ni++] = {static_cast<int>(np), q0, std::min(q.m, q0 + qc), 0};
            samples += q.m;
            ++np;
        }
    }
    cudaStream_t s = ksg_stream_;
    NSG_CUDA(cudaMemcpyAsync(d_pairs_.get(), h_pairs_, sizeof(KsgPairDesc) * np, cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemcpyAsync(d_items_.get(), h_items_, sizeof(KsgItem) * ni, cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemsetAsync(d_counters_.get(), 0, sizeof(int) * 4, s));
    int* ctr = d_counters_.as<int>();
    KsgCountArgs a{};
    a.pairs = d_pairs_.as<KsgPairDesc>();
    a.items = d_items_.as<KsgItem>();
    a.nitems = static_cast<int>(ni);
    a.k = k;
    a.counter = ctr;
    a.fault = d_fault_.as<int>();
    a.ties = d_ties_.as<KsgTie>();
    a.tie_count = ctr + 1;
    a.tie_cap = tie_cap_;
    a.psi = psi_->as<float>();
    a.psum = d_scratch_.as<float>();
    const int grid = std::max(1, static_cast<int>(std::min<long long>(ni, static_cast<long long>(sms) * std::max(1, e->ctas_per_sm()))));
    e->launch(a, grid, s);
    NSG_CUDA(cudaGetLastError());
    KsgTieArgs t{};
    t.pairs = a.pairs;
    t.ties = a.ties;
    t.tie_count = ctr + 1;
    t.tie_cap = tie_cap_;
    t.tie_next = ctr + 2;
    t.k = k;
    t.fault = a.fault;
    t.psi = a.psi;
    t.psum = a.psum;
    t.dz = d_tie_dz_.as<float>();
    t.idx = d_tie_idx_.as<int>();
    t.stride = cfg_.max_m;
    ksg_launch_ties_ctas(t, d, kServeTieCtas, s);
    for (size_t si = 0; si < slices.size(); ++si) {
        Job* j = slices[si].first;
        KsgFinalArgs f{};
        f.pairs = d_pairs_.as<KsgPairDesc>() + slice_first[si];
        f.npairs = static_cast<int>(slices[si].second.second - slices[si].second.first);
        f.k = k;
        f.d = d;
        f.psi = a.psi;
        f.psum = a.psum;
        if (j->kind == JOB_GC) f.gc = j->res.as<float>();
        else f.mi = j->res.as<float>();
        ksg_launch_final(f, s);
    }
    NSG_CUDA(cudaStreamSynchronize(s));
    int fault = 0;
    NSG_CUDA(cudaMemcpy(&fault, d_fault_.get(), sizeof(int), cudaMemcpyDeviceToHost));
    if (fault) {
        NSG_CUDA(cudaMemset(d_fault_.get(), 0, sizeof(int)));
        raise_fault(fault);
    }
}

void Server::ksg_loop() {
    cudaSetDevice(device_);
    while (!stop_) {
        // ---- admission and tick selection (under the lock) ----------------
        std::map<std::pair<int, int>, std::vector<std::pair<Job*, std::pair<long long, long long>>>> groups;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait_for(lk, std::chrono::milliseconds(2), [this] { return stop_ || !ksg_queue_.empty(); });
            if (stop_) break;
            std::vector<Job*> active;
            for (long long id : ksg_queue_) {
                Job& j = *jobs_[id];
                if (j.state == JOB_PENDING) {
                    try {
                        try_admit_locked(j);
                    } catch (const std::exception& ex) {
                        j.state = JOB_FAILED;
                        j.err = ex.what();
                    }
                }
                if (j.state == JOB_RUNNING && j.next_pair < static_cast<long long>(j.pairs.size())) {
                    active.push_back(&j);
                }
            }
            if (active.empty()) continue;
            // Short jobs first: a job whose remaining work fits in a quarter
            // of the tick takes all of it, so short requests never wait behind
            // long ones. The rest of the tick goes to jobs in arrival order, so
            // the oldest long job advances at nearly the whole GPU's rate (as
            // if served alone) instead of sharing it with every later one.
            double used_ops = 0;
            long long used_pairs = 0, used_samples = 0;
            std::vector<long long> take(active.size(), 0);
            for (int pass = 0; pass < 2; ++pass) {
                for (size_t i = 0; i < active.size(); ++i) {
                    Job& j = *active[i];
                    const long long remaining = static_cast<long long>(j.pairs.size()) - j.next_pair - take[i];
                    if (remaining <= 0) continue;
                    // a pair's work; pairs searched on cell grids evaluate about 40% of it
                    const double per = 8.0 * j.d * j.n * (j.n - 1.0) *
                                       (j.slots.size() == j.pairs.size() && j.n >= kGridMinSamples ? 0.4 : 1.0);
                    long long t;
                    if (pass == 0) {
                        if (remaining * per > cfg_.tick_ops / 4 || used_ops + remaining * per > cfg_.tick_ops) continue;
                        t = remaining;
                    } else {
                        if (used_ops >= cfg_.tick_ops) break;
                        t = std::max<long long>(1, static_cast<long long>((cfg_.tick_ops - used_ops) / per));
                    }
                    t = std::min(t, remaining);
                    t = std::min(t, cap_pairs_ - used_pairs);
                    t = std::min(t, (cap_samples_ - used_samples) / std::max(1, j.n));
                    if (t <= 0) continue;
                    take[i] += t;
                    used_ops += t * per;
                    used_pairs += t;
                    used_samples += t * j.n;
                }
            }
            for (size_t i = 0; i < active.size(); ++i) {
                if (!take[i]) continue;
                Job& j = *active[i];
                groups[{j.d, ksg_kmax_for(j.k) * 1000 + j.k}].push_back({&j, {j.next_pair, j.next_pair + take[i]}});
                j.next_pair += take[i];
            }
        }
        // ---- run the tick (without the lock) ------------------------------
        std::vector<Job*> finished;
        for (auto& g : groups) {
            try {
                run_tick(g.second);
            } catch (const std::exception& ex) {
                std::lock_guard<std::mutex> lk(mu_);
                for (auto& s : g.second) {
                    s.first->state = JOB_FAILED;
                    s.first->err = ex.what();
                }
            }
            std::lock_guard<std::mutex> lk(mu_);
            ++ticks_;
            for (auto& s : g.second) {
                Job& j = *s.first;
                const long long cnt = s.second.second - s.second.first;
                j.done_pairs += cnt;
                pairs_done_ += cnt;
                if (j.state == JOB_RUNNING && j.done_pairs == static_cast<long long>(j.pairs.size())) {
                    finished.push_back(&j);
                }
            }
        }
        // ---- completions: results to the host, release -------------------------
        for (Job* j : finished) {
            const size_t bytes = sizeof(float) * j->pairs.size();
            cudaError_t e = cudaMemcpyAsync(j->out, j->res.get(), bytes, cudaMemcpyDeviceToHost, copy_stream_);
            if (e == cudaSuccess) e = cudaStreamSynchronize(copy_stream_);
            std::lock_guard<std::mutex> lk(mu_);
            if (e != cudaSuccess) {
                j->state = JOB_FAILED;
                j->err = cudaGetErrorString(e);
            } else {
                j->state = JOB_DONE;
            }
            j->t.done = now();
            ++jobs_done_;
            release_locked(*j);
            ksg_queue_.erase(std::remove(ksg_queue_.begin(), ksg_queue_.end(), j->id), ksg_queue_.end());
            done_cv_.notify_all();
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            // failed jobs leave the queue too
            for (auto it = ksg_queue_.begin(); it != ksg_queue_.end();) {
                Job& j = *jobs_[*it];
                if (j.state == JOB_FAILED) {
                    release_locked(j);
                    it = ksg_queue_.erase(it);
                    done_cv_.notify_all();
                } else {
                    ++it;
                }
            }
        }
    }
}

void Server::apsp_loop() {
    cudaSetDevice(device_);
    while (!stop_) {
        Job* j = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait_for(lk, std::chrono::milliseconds(2), [this] { return stop_ || !apsp_queue_.empty(); });
            if (stop_) break;
            for (long long id : apsp_queue_) {
                Job& c = *jobs_[id];
                if (c.state == JOB_PENDING && used_bytes_ + c.footprint <= cfg_.budget_bytes) {
                    used_bytes_ += c.footprint;
                    peak_bytes_ = std::max(peak_bytes_, used_bytes_);
                    c.state = JOB_RUNNING;
                    c.t.admit = now();
                    j = &c;
                    break;
                }
            }
        }
        if (!j) continue;
        std::string err;
        try {
            const size_t nn = static_cast<size_t>(j->N) * j->N;
            AsyncBuffer A, H;
            A.alloc(nn * sizeof(float), apsp_stream_);
            H.alloc(nn * sizeof(float), apsp_stream_);
            NSG_CUDA(cudaMemcpyAsync(A.get(), j->hx, nn * sizeof(float), cudaMemcpyHostToDevice, apsp_stream_));
            apsp_lengths(A.as<float>(), H.as<float>(), j->N, j->L, apsp_stream_);
            NSG_CUDA(cudaMemcpyAsync(j->out, H.get(), nn * sizeof(float), cudaMemcpyDeviceToHost, apsp_stream_));
            NSG_CUDA(cudaStreamSynchronize(apsp_stream_));
        } catch (const std::exception& ex) {
            err = ex.what();
        }
        std::lock_guard<std::mutex> lk(mu_);
        j->state = err.empty() ? JOB_DONE : JOB_FAILED;
        j->err = err;
        j->t.done = now();
        used_bytes_ -= j->footprint;
        ++jobs_done_;
        apsp_queue_.erase(std::remove(apsp_queue_.begin(), apsp_queue_.end(), j->id), apsp_queue_.end());
        done_cv_.notify_all();
    }
}

}  // namespace nsg
