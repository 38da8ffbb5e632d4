// Hedetniemi all-pairs shortest paths (netcalc/include/hedetniemi.h). Same
// signatures, including the (tolerance, maxPathLength) order of the *Gpu and
// *Cpu variants against (maxPathLength, tolerance) of the public call.
//
// Lengths: H_0 = A, H_{t+1}[i][j] = min_k A[j][k] + H_t[k][i], run until H
// stops changing or maxPathLength steps. A is N x N with +inf for missing
// edges and 0 on the diagonal.
// Paths: paths is re-initialised to 1 x (N * maxPathLength * N), laid out
// paths[i*L*N + j*L + p]; -1 marks unused cells.
// The CPU platform of the reference has no shortest-path implementation
// (netcalc/src/hedetniemi_cpu.cpp:5-16); the same holds here.
#ifndef NETSCI_GB300_NETCALC_HEDETNIEMI_H
#define NETSCI_GB300_NETCALC_HEDETNIEMI_H
#include "cuarray.h"
#include "netcalc/platform.h"

namespace netcalc {
void hedetniemiAllShortestPaths(CuArray<float>* A, CuArray<float>* H, CuArray<int>* paths,
                                int maxPathLength, float tolerance, int platform);
void hedetniemiAllShortestPathsGpu(CuArray<float>* A, CuArray<float>* H, CuArray<int>* paths,
                                   float tolerance, int maxPathLength);
void hedetniemiAllShortestPathsCpu(CuArray<float>* A, CuArray<float>* H, CuArray<int>* paths,
                                   float tolerance, int maxPathLength);
void hedetniemiAllShortestPathLengths(CuArray<float>* A, CuArray<float>* H, int maxPathLength,
                                      int platform);
void hedetniemiAllShortestPathLengthsGpu(CuArray<float>* A, CuArray<float>* H,
                                         int maxPathLength);
void correlationToAdjacency(CuArray<float>* A, CuArray<float>* C, int n, int platform);
void correlationToAdjacencyGpu(CuArray<float>* A, CuArray<float>* C, int n);
// New[]-allocated node sequence from i to j (duplicates removed) and its
// length in a new[]-allocated cell.
void recoverSingleShortestPath(int** NUMPY_ARRAY, int** NUMPY_ARRAY_DIM1, CuArray<int>* paths,
                               int maxPathLength, int i, int j);
}  // namespace netcalc
#endif
