// KSG count kernels instantiated for d = 2 (one translation unit per d so the
// library builds in parallel).
#include "ksg_kernels.cuh"
#include "ksg_registry.cuh"

#ifndef NSG_KSG_VARIANT
#define NSG_KSG_VARIANT 1
#endif

namespace nsg {
namespace {
const KsgKernelEntry kEntries[] = {
    NSG_KSG_FAMILY_SMALLK(2, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_SMALLK(2, 8, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K16(2, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K32(2, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K64(2, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(2, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(2, 8, NSG_KSG_VARIANT),
};
}  // namespace

const KsgKernelEntry* ksg_entries_d2(int* count) {
    *count = static_cast<int>(sizeof(kEntries) / sizeof(kEntries[0]));
    return kEntries;
}
}  // namespace nsg
