// CPU platform KSG (ksg_cpu.cpp) and the host generalized-correlation
// transform shared by both platforms' per-pair calls.
#pragma once

namespace nsg {

// MI of one pair on the host (netcalc CPU_PLATFORM).
float ksg_cpu_pair(const float* xa, const float* xb, int n, int k, int d);
// r = sqrt(1 - exp(-2 I / d)) in double, rounded to float; 0 when I <= 0.
// netcalc/src/generalized_correlation_cpu.cpp:17-25.
float gc_from_mi(float mi, int d);

}  // namespace nsg
