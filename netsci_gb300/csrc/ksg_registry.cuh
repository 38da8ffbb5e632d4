// Registry of instantiated KSG count kernels: one entry per
// (d, KMAX, CTA size, samples per thread, tile frames, arithmetic variant).
// The planner and the autotuner pick from this table.
#pragma once

#include "ksg.cuh"

namespace nsg {

struct KsgKernelEntry {
    int d;
    int kmax;
    int threads;
    int r;
    int frames;
    int variant;
    int tma;              // 1: tiles staged by bulk copies (ksg_count_kernel_tma)
    void (*launch)(const KsgCountArgs&, int grid, cudaStream_t st);
    int (*ctas_per_sm)();
};

// Entries for one dimension (defined in ksg_d1.cu, ksg_d2.cu, ksg_d3.cu).
const KsgKernelEntry* ksg_entries_d1(int* count);
const KsgKernelEntry* ksg_entries_d2(int* count);
const KsgKernelEntry* ksg_entries_d3(int* count);

// variant < 0 / tma < 0: any; the plain-load kernels come first.
const KsgKernelEntry* ksg_find_entry(int d, int kmax, int threads, int r, int frames,
                                     int variant, int tma = 0);
// All entries for (d, kmax); returns the count.
int ksg_list_entries(int d, int kmax, const KsgKernelEntry** out, int cap);

}  // namespace nsg

#define NSG_KSG_ENTRY(D, KMAX, NT, R, J, V)                                                  \
    {D, KMAX, NT, R, J, V, 0,                                                               \
     [](const ::nsg::KsgCountArgs& a, int grid, cudaStream_t st) {                          \
         ::nsg::ksgk::ksg_count_kernel<D, KMAX, R, NT, J, V><<<grid, NT, 0, st>>>(a);       \
     },                                                                                     \
     []() {                                                                                 \
         int n = 0;                                                                         \
         cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                     \
             &n, ::nsg::ksgk::ksg_count_kernel<D, KMAX, R, NT, J, V>, NT, 0);               \
         return n;                                                                          \
     }}

// Bulk-copy staged instantiation: two stages of 2*D*J floats of dynamic
// shared memory (above the 48 KB default, so the limit is raised once).
#define NSG_KSG_ENTRY_TMA(D, KMAX, NT, R, J, V)                                              \
    {D, KMAX, NT, R, J, V, 1,                                                               \
     [](const ::nsg::KsgCountArgs& a, int grid, cudaStream_t st) {                          \
         constexpr int kSmem = 2 * 2 * D * J * 4;                                           \
         static const cudaError_t once = cudaFuncSetAttribute(                              \
             ::nsg::ksgk::ksg_count_kernel_tma<D, KMAX, R, NT, J, V>,                       \
             cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);                           \
         (void)once;                                                                        \
         ::nsg::ksgk::ksg_count_kernel_tma<D, KMAX, R, NT, J, V><<<grid, NT, kSmem, st>>>(a); \
     },                                                                                     \
     []() {                                                                                 \
         constexpr int kSmem = 2 * 2 * D * J * 4;                                           \
         cudaFuncSetAttribute(::nsg::ksgk::ksg_count_kernel_tma<D, KMAX, R, NT, J, V>,      \
                              cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);          \
         int n = 0;                                                                         \
         cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                     \
             &n, ::nsg::ksgk::ksg_count_kernel_tma<D, KMAX, R, NT, J, V>, NT, kSmem);       \
         return n;                                                                          \
     }}
#define NSG_KSG_FAMILY_TMA(D, KMAX, V)                                                      \
    NSG_KSG_ENTRY_TMA(D, KMAX, 256, 1, 1024, V), NSG_KSG_ENTRY_TMA(D, KMAX, 128, 1, 1024, V), \
        NSG_KSG_ENTRY_TMA(D, KMAX, 512, 1, 1024, V), NSG_KSG_ENTRY_TMA(D, KMAX, 256, 1, 512, V)

// Standard shape family for one (D, KMAX) with variant V.
#define NSG_KSG_FAMILY_SMALLK(D, KMAX, V)                                                   \
    NSG_KSG_ENTRY(D, KMAX, 256, 1, 1024, V), NSG_KSG_ENTRY(D, KMAX, 128, 1, 1024, V),       \
        NSG_KSG_ENTRY(D, KMAX, 128, 2, 1024, V), NSG_KSG_ENTRY(D, KMAX, 256, 2, 1024, V),   \
        NSG_KSG_ENTRY(D, KMAX, 64, 1, 512, V), NSG_KSG_ENTRY(D, KMAX, 512, 1, 1024, V)
#define NSG_KSG_FAMILY_K16(D, V) NSG_KSG_ENTRY(D, 16, 128, 1, 1024, V)
#define NSG_KSG_FAMILY_K32(D, V) NSG_KSG_ENTRY(D, 32, 128, 1, 1024, V)
#define NSG_KSG_FAMILY_K64(D, V) NSG_KSG_ENTRY(D, 64, 64, 1, 512, V)
