// KSG count kernels instantiated for d = 1 (one translation unit per d so the
// library builds in parallel).
#include "ksg_kernels.cuh"
#include "ksg_registry.cuh"

#ifndef NSG_KSG_VARIANT
#define NSG_KSG_VARIANT 1
#endif

namespace nsg {
namespace {
const KsgKernelEntry kEntries[] = {
    NSG_KSG_FAMILY_SMALLK(1, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_SMALLK(1, 8, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K16(1, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K32(1, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K64(1, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(1, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(1, 8, NSG_KSG_VARIANT),
};
}  // namespace

const KsgKernelEntry* ksg_entries_d1(int* count) {
    *count = static_cast<int>(sizeof(kEntries) / sizeof(kEntries[0]));
    return kEntries;
}
}  // namespace nsg
