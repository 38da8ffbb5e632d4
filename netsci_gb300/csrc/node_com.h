// Node centres of mass from raw DCD frames (node_com.cu).
#pragma once
#include <cuda_runtime.h>

namespace nsg {

struct NodeComArgs {
    const unsigned char* frames;   // device: nframes raw DCD frames
    long long frame_bytes;
    long long x_off, y_off, z_off; // payload offsets inside a frame
    int swap;                      // 1: file byte order differs
    int nframes;                   // frames in this batch
    int nnodes;
    const int* node_start;         // device [nnodes + 1], CSR into node_atoms
    const int* node_atoms;         // device, atoms of each node in index order
    const float* atom_mass;        // device [natoms]
    const float* node_mass;        // device [nnodes]
    float* out;                    // device: out[node*row_stride + c*plane_stride + frame0 + f]
    long long row_stride, plane_stride;
    int frame0;
};

void launch_node_com(const NodeComArgs& a, cudaStream_t st);
// x[r * ld + f] = +inf for every row r < rows and frame m <= f < ld.
void launch_pad_inf(float* x, long long rows, int m, int ld, cudaStream_t st);

}  // namespace nsg
