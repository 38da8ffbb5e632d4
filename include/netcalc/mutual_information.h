// KSG mutual information (netcalc/include/mutual_information.h). Same
// signatures and return conventions: the pair-list calls return `platform`
// (0 GPU, 1 CPU) and throw std::runtime_error on any other platform.
//
// X is N x (d*n): row a holds node a's d coordinate planes of n samples
// each, plane-major. ab is P x 2 node indices; I is re-initialised to 1 x P.
// The GPU platform uploads X once and runs every pair in one persistent
// launch; per-pair results are bit-identical to the CPU platform on inputs
// whose (k+1)-th and (k+2)-th nearest joint distances differ.
#ifndef NETSCI_GB300_NETCALC_MUTUAL_INFORMATION_H
#define NETSCI_GB300_NETCALC_MUTUAL_INFORMATION_H
#include <string>

#include "cuarray.h"
#include "netcalc/platform.h"

namespace netcalc {
int mutualInformation(CuArray<float>* X, CuArray<float>* I, CuArray<int>* ab, int k, int n,
                      int xd, int d, int platform, int checkpointFrequency,
                      std::string checkpointFileName);
int mutualInformation(CuArray<float>* X, CuArray<float>* I, CuArray<int>* ab, int k, int n,
                      int xd, int d, int platform);
float mutualInformationGpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd, int d);
float mutualInformationCpu(CuArray<float>* Xa, CuArray<float>* Xb, int k, int n, int xd, int d);
void generateRestartAbFromCheckpointFile(CuArray<int>* ab, CuArray<int>* restartAb,
                                         const std::string& checkpointFileName);
}  // namespace netcalc
#endif
