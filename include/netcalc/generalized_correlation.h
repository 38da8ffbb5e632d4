// Generalized correlation r = sqrt(1 - exp(-2 I / d)), 0 where I <= 0
// (netcalc/include/generalized_correlation.h). Same signatures and return
// conventions as the mutual-information calls.
#ifndef NETSCI_GB300_NETCALC_GENERALIZED_CORRELATION_H
#define NETSCI_GB300_NETCALC_GENERALIZED_CORRELATION_H
#include <string>

#include "cuarray.h"
#include "netcalc/platform.h"

namespace netcalc {
int generalizedCorrelation(CuArray<float>* X, CuArray<float>* R, CuArray<int>* ab, int k, int n,
                           int xd, int d, int platform, int checkpointFrequency,
                           std::string checkpointFileName);
int generalizedCorrelation(CuArray<float>* X, CuArray<float>* R, CuArray<int>* ab, int k, int n,
                           int xd, int d, int platform);
float generalizedCorrelationGpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd,
                                int d);
float generalizedCorrelationCpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd,
                                int d);
}  // namespace netcalc
#endif
