// Row statistics (netcalc/include/math_utils.h:22-95). Same signatures.
//
// mean(): m is recomputed as a->size() / n and u is re-initialised to 1 x m
// (zeros); the values are computed only for platform 0 (GPU), as in the
// reference (netcalc/src/math_utils.cpp:6-36), which has no CPU version.
// meanGpu() / standardDeviationGpu() copy a to the device when it has no
// device copy yet (an existing device copy is used as it is), compute and copy
// u (and sigma) back to the host. sigma is the population standard deviation.
#ifndef NETSCI_GB300_NETCALC_MATH_UTILS_H
#define NETSCI_GB300_NETCALC_MATH_UTILS_H
#include "cuarray.h"
#include "netcalc/platform.h"

void mean(CuArray<float>* a, CuArray<float>* u, int m, int n, int platform);
void meanGpu(CuArray<float>* a, CuArray<float>* u, int m, int n);
void standardDeviation(CuArray<float>* a, CuArray<float>* u, CuArray<float>* sigma, int m, int n,
                       int platform);
void standardDeviationGpu(CuArray<float>* a, CuArray<float>* u, CuArray<float>* sigma, int m,
                          int n);
#endif
