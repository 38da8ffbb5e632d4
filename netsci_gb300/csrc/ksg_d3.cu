// KSG count kernels instantiated for d = 3 (one translation unit per d so the
// library builds in parallel).
#include "ksg_kernels.cuh"
#include "ksg_registry.cuh"

#ifndef NSG_KSG_VARIANT
#define NSG_KSG_VARIANT 1
#endif

namespace nsg {
namespace {
const KsgKernelEntry kEntries[] = {
    NSG_KSG_FAMILY_SMALLK(3, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_SMALLK(3, 8, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K16(3, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K32(3, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_K64(3, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(3, 6, NSG_KSG_VARIANT),
    NSG_KSG_FAMILY_TMA(3, 8, NSG_KSG_VARIANT),
    // arithmetic variants of the d=3, k<=8 family, kept for the tuner
    NSG_KSG_FAMILY_SMALLK(3, 8, 0),
    NSG_KSG_FAMILY_SMALLK(3, 8, 2),
};
}  // namespace

const KsgKernelEntry* ksg_entries_d3(int* count) {
    *count = static_cast<int>(sizeof(kEntries) / sizeof(kEntries[0]));
    return kEntries;
}
}  // namespace nsg
