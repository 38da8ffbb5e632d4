// Platform selectors of the netcalc API (netcalc/include/platform.h:8-11).
#ifndef NETSCI_GB300_NETCALC_PLATFORM_H
#define NETSCI_GB300_NETCALC_PLATFORM_H
namespace netcalc {
const int GPU_PLATFORM = 0;
const int CPU_PLATFORM = 1;
}  // namespace netcalc
#endif
