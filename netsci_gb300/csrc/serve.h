// Serving loop: continuous batching of MI / GC / APSP jobs on one GPU.
//
// Jobs arrive through submit_*() from any thread. A scheduler thread admits
// them in arrival order whenever their device footprint fits the memory
// budget (a later, smaller job may be admitted while an earlier, larger one
// waits), and runs "ticks": each tick takes pairs from the admitted KSG jobs
// (first every job whose remaining work fits in a quarter of the tick, whole;
// then the rest of the tick in arrival order, so the oldest long job runs at
// nearly the full rate), puts them in one work queue and runs the count, tie
// and finalize kernels once over it. Jobs that arrive while a tick runs join
// the next one. APSP jobs run on their own stream and worker thread, so their
// kernels overlap the KSG ticks on the device. Trajectories can be
// registered once and stay resident in HBM for any number of jobs.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.h"
#include "ksg.cuh"
#include "ksg_grid.h"

namespace nsg {

struct ServerConfig {
    size_t budget_bytes = size_t(8) << 30;   // device memory for admitted jobs
    double tick_ops = 2.5e11;                // algorithmic ops per tick (~10 ms)
    long long max_tick_pairs = 1 << 20;
    int max_m = 1 << 15;                     // largest sample count a KSG job may have
};

struct JobTimes {
    double submit = 0, admit = 0, done = 0;  // seconds on the host steady clock
};

enum JobKind : int { JOB_GC = 0, JOB_MI = 1, JOB_APSP = 2 };
enum JobState : int { JOB_PENDING = 0, JOB_RUNNING = 1, JOB_DONE = 2, JOB_FAILED = 3 };

class Server {
public:
    explicit Server(const ServerConfig& cfg);
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    // Resident trajectory: N node rows of d planes of m samples (host
    // plane-major N x (d*m)); returns its id.
    int register_trajectory(const float* X, int N, int m, int d);
    // All pairs a < b of a registered trajectory -> out (host, N(N-1)/2
    // floats, row-major in a): generalized correlation.
    long long submit_gc(int traj, int k, float* out);
    // MI of one pair given on the host (x, y: d planes of n samples each).
    long long submit_mi(const float* x, const float* y, int n, int d, int k, float* out);
    // Shortest path lengths of an N x N host matrix into out (N*N floats).
    long long submit_apsp(const float* A, int N, int max_path_length, float* out);

    int state(long long id, JobTimes* t);
    bool wait(long long id, double timeout_s);
    // jobs completed, pairs computed, ticks run, peak device bytes in use
    void stats(long long* jobs_done, long long* pairs_done, long long* ticks, size_t* peak_bytes);
    const std::string& error(long long id);

private:
    struct Traj;
    struct Job;
    void ksg_loop();
    void apsp_loop();
    bool try_admit_locked(Job& j);
    void release_locked(Job& j);
    void run_tick(std::vector<std::pair<Job*, std::pair<long long, long long>>>& slices);
    bool run_tick_grid(std::vector<std::pair<Job*, std::pair<long long, long long>>>& slices);
    double now() const;

    ServerConfig cfg_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::condition_variable done_cv_;
    std::atomic<bool> stop_{false};
    std::map<long long, std::unique_ptr<Job>> jobs_;
    std::deque<long long> ksg_queue_;    // pending + admitted KSG jobs, arrival order
    std::deque<long long> apsp_queue_;
    std::vector<std::unique_ptr<Traj>> trajs_;
    long long next_id_ = 1;
    size_t used_bytes_ = 0, peak_bytes_ = 0;
    long long jobs_done_ = 0, pairs_done_ = 0, ticks_ = 0;
    cudaStream_t ksg_stream_ = nullptr, apsp_stream_ = nullptr, copy_stream_ = nullptr;
    int device_ = 0;

    // tick buffers (capacity-sized, reused)
    long long cap_pairs_ = 0, cap_items_ = 0, cap_samples_ = 0;
    DeviceBuffer d_pairs_, d_items_, d_scratch_, d_counters_, d_fault_, d_ties_, d_tie_dz_, d_tie_idx_;
    int tie_cap_ = 0;
    KsgPairDesc* h_pairs_ = nullptr;
    KsgItem* h_items_ = nullptr;
    // cell-grid search: one device table of node grids (trajectory rows from
    // the bottom, pairs of slots for MI jobs from a free list at the top),
    // and per-tick pair grids and scratch, grown on demand
    DeviceBuffer d_gnodes_, d_gpairs_, d_wpre_, d_garena_, d_eps_a_, d_eps_b_, d_cnt_a_, d_cnt_b_;
    DeviceBuffer d_groups_, d_gpre_;
    DeviceBuffer d_corder_;  // count-query order: groups x largest m of the tick
    GridPair* h_gpairs_ = nullptr;
    int* h_wpre_ = nullptr;
    int next_node_slot_ = 0;
    std::vector<int> free_mi_slots_;
    std::shared_ptr<const DeviceBuffer> psi_;
    std::thread ksg_thread_, apsp_thread_;
};

}  // namespace nsg
