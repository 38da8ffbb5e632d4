// KSG mutual information of one variable pair without any device allocation.
//
// Some callers cannot call cudaMalloc: an application that owns the GPU's
// memory (for example a simulation engine that hands this library its
// trajectory buffers through a plugin interface and keeps every byte of
// device memory in its own pool), or a loop whose latency budget does not
// allow the device-wide synchronisation an allocation can bring. For them,
// nsg_ksg_pair_noalloc_device computes one pair's MI (and optionally the
// generalized correlation) using only the caller's input rows and output
// slots plus a fixed scratch area compiled into this library.
//
// The scratch area is a file-scope __device__ array (g_noalloc_scratch):
// every GPU that loads the library holds its NSG_NOALLOC_SCRATCH_BYTES until
// the process exits. Host code never uses the array's name as a device
// address; the first call on each device (with that device current) asks
// the runtime for the array's device address with cudaGetSymbolAddress and
// keeps it. That first call also copies the psi table into the area, so it
// should be made before any stream capture. The address and the table are
// kept until the process exits; a device reset by the host application
// after the first call (cudaDeviceReset) is not supported, since it
// discards both. Every call uses the same area:
// calls whose work overlaps on the GPU (other streams, other threads) race
// and must be serialised by the caller. Sizes above the limit are rejected.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "ksg.cuh"
#include "ksg_registry.cuh"
#include "netsci_gb300.h"

namespace nsg {
namespace {

// Layout of the scratch area (byte offsets, each 256-byte aligned).
constexpr int kMaxSamples = NSG_NOALLOC_MAX_SAMPLES;
constexpr int kTieCtas = 2;           // tie-kernel CTAs (8 warps each)
constexpr int kTieWarps = kTieCtas * 8;
constexpr int kTieCap = kMaxSamples;  // every sample could be tied
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffPsi = 0;                                          // float[max+1]
constexpr size_t kOffPsum = align256(kOffPsi + sizeof(float) * (kMaxSamples + 1));
constexpr size_t kOffItems = align256(kOffPsum + sizeof(float) * kMaxSamples);
constexpr int kMaxItems = (kMaxSamples + 63) / 64;                     // smallest CTA block: 64
constexpr size_t kOffPair = align256(kOffItems + sizeof(KsgItem) * kMaxItems);
constexpr size_t kOffCounters = align256(kOffPair + sizeof(KsgPairDesc));
constexpr size_t kOffTies = align256(kOffCounters + sizeof(int) * 8);
constexpr size_t kOffTieDz = align256(kOffTies + sizeof(KsgTie) * kTieCap);
constexpr size_t kOffTieIdx = align256(kOffTieDz + sizeof(float) * kTieWarps * kMaxSamples);
constexpr size_t kScratchBytes = align256(kOffTieIdx + sizeof(int) * kTieWarps * kMaxSamples);
static_assert(kScratchBytes == NSG_NOALLOC_SCRATCH_BYTES,
              "NSG_NOALLOC_SCRATCH_BYTES in netsci_gb300.h must match the layout");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceArea {
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch
};

std::mutex g_setup_mu;
DeviceArea g_area[64];

// Device address of the scratch area on the current device; the first call
// per device also writes the psi table into it (synchronously).
unsigned char* area_for_current_device() {
    int dev = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) fail(NSG_ERR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceArea& a = g_area[dev];
    if (!a.base) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            fail(NSG_ERR_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch): ") +
                                   cudaGetErrorString(e));
        }
        std::vector<float> psi(static_cast<size_t>(kMaxSamples) + 1);
        host_psi(psi.data(), kMaxSamples);
        NSG_CUDA(cudaMemcpy(static_cast<unsigned char*>(p) + kOffPsi, psi.data(),
                            psi.size() * sizeof(float), cudaMemcpyHostToDevice));
        a.base = static_cast<unsigned char*>(p);
    }
    return a.base;
}

}  // namespace

void ksg_pair_noalloc(const float* xa, const float* xb, int ld, int m, int k, int d, float* mi,
                      float* gc, cudaStream_t s) {
    if (d < 1 || d > 3) invalid("d must be 1, 2 or 3");
    if (k < 1) invalid("k must be >= 1");
    if (m < k + 1) invalid("k must be smaller than the number of samples");
    if (m > kMaxSamples) {
        fail(NSG_ERR_UNSUPPORTED, "the no-allocation entry point handles at most " +
                                      std::to_string(kMaxSamples) + " samples (got " +
                                      std::to_string(m) + ")");
    }
    if (!xa || !xb || ld < m) invalid("bad row pointers or plane stride");
    if (!mi && !gc) invalid("no output requested");
    const int kmax = ksg_kmax_for(k);
    if (!kmax) fail(NSG_ERR_UNSUPPORTED, "k > 62 is not supported by the GPU path");

    unsigned char* base = area_for_current_device();
    // the smallest CTA block spreads one pair over as many SMs as possible
    const KsgKernelEntry* entry = ksg_find_entry(d, kmax, 64, 1, 512, -1);
    if (!entry) {
        const KsgShape sh = ksg_default_shape(d, kmax);
        entry = ksg_find_entry(d, kmax, sh.threads, sh.r, sh.frames, -1);
    }
    if (!entry) fail(NSG_ERR_UNSUPPORTED, "no KSG kernel for this d/k in the no-allocation path");
    const int qc = entry->threads * entry->r;
    const int nitems = (m + qc - 1) / qc;

    // Per-call descriptors go into the area by stream-ordered copies from
    // host values (no allocation on either side).
    KsgPairDesc desc{xa, xb, nullptr, 0, ld, m, 0, 0};
    std::vector<KsgItem> items(nitems);
    for (int i = 0; i < nitems; ++i) items[i] = {0, i * qc, std::min(m, (i + 1) * qc), 0};
    KsgPairDesc* d_pair = reinterpret_cast<KsgPairDesc*>(base + kOffPair);
    KsgItem* d_items = reinterpret_cast<KsgItem*>(base + kOffItems);
    int* counters = reinterpret_cast<int*>(base + kOffCounters);  // work, ties, tie work, fault
    NSG_CUDA(cudaMemcpyAsync(d_pair, &desc, sizeof(desc), cudaMemcpyHostToDevice, s));
    NSG_CUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(KsgItem) * nitems,
                             cudaMemcpyHostToDevice, s));
    // the area keeps the previous call's contents: zero the counters
    NSG_CUDA(cudaMemsetAsync(counters, 0, sizeof(int) * 8, s));

    KsgCountArgs a{};
    a.pairs = d_pair;
    a.items = d_items;
    a.nitems = nitems;
    a.k = k;
    a.counter = counters;
    a.fault = counters + 3;
    a.ties = reinterpret_cast<KsgTie*>(base + kOffTies);
    a.tie_count = counters + 1;
    a.tie_cap = kTieCap;
    a.psi = reinterpret_cast<const float*>(base + kOffPsi);
    a.psum = reinterpret_cast<float*>(base + kOffPsum);
    const int grid = std::max(1, std::min(nitems, sm_count() * std::max(1, entry->ctas_per_sm())));
    entry->launch(a, grid, s);
    NSG_CUDA(cudaGetLastError());

    KsgTieArgs t{};
    t.pairs = d_pair;
    t.ties = a.ties;
    t.tie_count = counters + 1;
    t.tie_cap = kTieCap;
    t.tie_next = counters + 2;
    t.k = k;
    t.fault = counters + 3;
    t.psi = a.psi;
    t.psum = a.psum;
    t.dz = reinterpret_cast<float*>(base + kOffTieDz);
    t.idx = reinterpret_cast<int*>(base + kOffTieIdx);
    t.stride = kMaxSamples;
    ksg_launch_ties_ctas(t, d, kTieCtas, s);

    KsgFinalArgs f{};
    f.pairs = d_pair;
    f.npairs = 1;
    f.k = k;
    f.d = d;
    f.psi = a.psi;
    f.psum = a.psum;
    f.mi = mi;
    f.gc = gc;
    ksg_launch_final(f, s);
    // read back the fault word to report frame-map and tie-list problems
    int fault = 0;
    NSG_CUDA(cudaMemcpyAsync(&fault, counters + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA(cudaStreamSynchronize(s));
    raise_fault(fault);
}

}  // namespace nsg
