// Host-side KSG planner: turns a list of variable pairs into device
// descriptors, a work queue and scratch, and runs it as one persistent
// count launch plus one finalize launch per batch (optionally captured in a
// CUDA graph).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "ksg.cuh"
#include "netsci_gb300.h"

namespace nsg {

// Device allocation owned by the library. Blocks come from, and go back to,
// a per-device cache of freed blocks (see engine.cpp), so plans built call
// after call with the same sizes do not map and unmap gigabytes each time.
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes);
    ~DeviceBuffer();
    DeviceBuffer(DeviceBuffer&& o) noexcept;
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    void* get() const { return p_; }
    template <typename T>
    T* as() const { return static_cast<T*>(p_); }
    size_t bytes() const { return bytes_; }
    void reset(size_t bytes);

private:
    void release();
    void* p_ = nullptr;
    size_t bytes_ = 0;     // requested
    size_t capacity_ = 0;  // size of the block
    int device_ = -1;
};

// Return every cached block to the driver (all devices).
void release_cached_device_blocks();

struct KsgOutputs {
    float* mi = nullptr;     // device, indexed by pair order of the input list
    float* gc = nullptr;
    float* w = nullptr;
    // optional per-sample outputs (device, length = total samples over pairs,
    // pair p's samples at the prefix offset of p in input order)
    int* nx = nullptr;
    int* ny = nullptr;
    float* eps_x = nullptr;
    float* eps_y = nullptr;
    float* kdist = nullptr;
};

struct KsgPlanOptions {
    bool graph = false;                  // capture each run in a CUDA graph
    bool timing = false;                 // CUDA events around each count launch
    bool autotune = false;               // time the instantiated shapes on a probe first
    KsgShape shape{0, 0, 0};             // explicit shape (threads == 0: choose)
    int variant = -1;
    int staging = -1;                    // -1 auto, 0 plain loads, 1 bulk copies (TMA)
    int search = -1;                     // -1 auto, 0 exhaustive, 1 cell grids
    size_t scratch_budget_bytes = 0;     // 0: library default
};

class KsgPlan {
public:
    KsgPlan(const std::vector<nsg_ksg_pair>& pairs, int k, int d, const KsgOutputs& out,
            const KsgPlanOptions& opt);
    ~KsgPlan();
    void run(cudaStream_t s);
    // Captures and instantiates the run's CUDA graph now (graph plans only).
    void prepare();
    // Kernel launches per run: count, tie resolution and finalize per batch
    // (exhaustive search); node grids once, then pair grids, search, counts,
    // combine, ties and finalize per batch (cell-grid search).
    int launches() const;
    // Device time of the count kernels of the last run (ms); needs timing.
    float count_ms() const;
    long long pairs() const { return npairs_; }
    // Reads (and clears) the device fault word; synchronizes with the device.
    int take_fault();
    const KsgShape& shape() const { return shape_; }
    int variant() const { return variant_; }
    int staging() const;  // 1: bulk-copy staged kernel, 0: plain loads
    int search() const { return search_; }  // 1: cell grids, 0: exhaustive
    // Query-frame evaluations of the last run's grid search (joint
    // distances), grid counts (one variable's distance, once per query and
    // frame) and the counts' eps comparisons (once per query, frame and pair
    // of a count group); 0 when exhaustive. compares may be null.
    // Synchronizes with the device.
    void evaluations(unsigned long long* search, unsigned long long* counts,
                     unsigned long long* compares = nullptr) const;
    // Samples the last run sent to the tie kernel (the reference sort's order
    // replayed); synchronizes with the device.
    long long tied_samples() const;
    // Device milliseconds of the last run's search kernels and count kernels
    // (the order kernels excluded), summed over batches; needs timing.
    void kernel_ms(float* search_ms, float* count_ms, float* tie_ms = nullptr) const;

private:
    struct Batch {
        int pair0 = 0, npairs = 0;
        int item0 = 0, nitems = 0;
        int grid = 0;
    };
    void enqueue(cudaStream_t s);
    void enqueue_grid(cudaStream_t s);
    void setup_grid(const std::vector<KsgPairDesc>& descs);

    int d_, k_, kmax_;
    long long npairs_ = 0;
    bool timing_ = false;
    std::vector<cudaEvent_t> events_;
    KsgShape shape_{};
    int variant_ = -1;
    const struct KsgKernelEntry* entry_ = nullptr;
    KsgOutputs out_;
    std::vector<Batch> batches_;
    DeviceBuffer pairs_dev_, items_dev_, scratch_, counters_, fault_;
    DeviceBuffer ties_, tie_dz_, tie_idx_;
    int tie_cap_ = 0;
    long long tie_stride_ = 0;
    int search_ = 0;
    bool bootstrap_ = false;             // frame-mapped rows copied for the grid search
    DeviceBuffer mapped_rows_, gather_rows_;
    int ngather_ = 0;
    struct GridState;
    std::shared_ptr<GridState> grid_;
    std::shared_ptr<const DeviceBuffer> psi_;
    bool graph_ = false;
    cudaGraphExec_t exec_ = nullptr;
    cudaStream_t capture_stream_ = nullptr;
};

// Device psi table with at least n+1 entries (shared, grown on demand).
std::shared_ptr<const DeviceBuffer> device_psi(int n);
// Host psi table of the reference recurrence (netcalc/src/psi.cpp:6-20).
void host_psi(float* psi, int n);

// Best shape for a pair list, measured on a probe of its first pairs and
// cached per (d, KMAX, m bucket, pair-count bucket); NSG_TUNE_CACHE names a
// file that keeps the cache across processes.
struct KsgTuned {
    KsgShape shape;
    int variant;
    int staging;
    double gops;
};
KsgTuned ksg_autotune(const std::vector<nsg_ksg_pair>& pairs, int k, int d);

// Shape override set by nsg_ksg_set_shape (threads == 0: automatic).
void ksg_force_shape(int threads, int r, int frames, int variant);
// Staging override set by nsg_ksg_set_staging (-1 automatic).
void ksg_force_staging(int staging);
// Search override set by nsg_ksg_set_search (-1 automatic, 0 exhaustive,
// 1 cell grids).
void ksg_force_search(int mode);
// Block-order override for cell-grid plans set by nsg_ksg_set_orders (-1
// automatic, 0 never, 1 always).
void ksg_force_orders(int mode);
int ksg_forced_orders();
// True when every pair allows bulk-copy staging (16-byte aligned rows,
// plane stride a multiple of 4, no frame map).
bool ksg_bulk_copy_ok(const std::vector<nsg_ksg_pair>& pairs);
int sm_count();
// Operation rates (Gop/s) of the cell-grid search and count kernels' inner
// loops alone, measured on the current device (ceiling.cu).
void measure_issue_ceiling(int d, double* search_gops, double* count_gops);

}  // namespace nsg
