// Node centres of mass from raw DCD frames on the device.
//
// The frames arrive exactly as they lie in the file (record markers, unit
// cell and all), copied from pinned memory; the kernel reads each atom's
// x, y, z at the frame's payload offsets, byte-swapping when the file's order
// differs. One thread per (node, frame), frames fastest; a thread walks its
// node's atoms in index order (consecutive addresses, so its loads stay in
// one cache line for a run of atoms) and accumulates x * mass in float,
// then divides by the node's float total mass: the arithmetic of
// netchem/src/network.cpp:101-200, with every multiply and add rounded
// separately (no fused multiply-add).
#include <cuda_runtime.h>

#include "errors.h"
#include "node_com.h"

namespace nsg {
namespace {

__device__ __forceinline__ float load_coord(const unsigned char* p, int swap) {
    unsigned int v = *reinterpret_cast<const unsigned int*>(p);
    if (swap) v = __byte_perm(v, 0, 0x0123);
    return __uint_as_float(v);
}

__global__ void node_com_kernel(NodeComArgs A) {
    const long long total = static_cast<long long>(A.nnodes) * A.nframes;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int node = static_cast<int>(t / A.nframes);
        const int f = static_cast<int>(t - static_cast<long long>(node) * A.nframes);
        const unsigned char* fr = A.frames + static_cast<long long>(f) * A.frame_bytes;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int k = A.node_start[node]; k < A.node_start[node + 1]; ++k) {
            const int a = A.node_atoms[k];
            const float w = A.atom_mass[a];
            const long long o = 4LL * a;
            sx = __fadd_rn(sx, __fmul_rn(load_coord(fr + A.x_off + o, A.swap), w));
            sy = __fadd_rn(sy, __fmul_rn(load_coord(fr + A.y_off + o, A.swap), w));
            sz = __fadd_rn(sz, __fmul_rn(load_coord(fr + A.z_off + o, A.swap), w));
        }
        const float tm = A.node_mass[node];
        float* row = A.out + static_cast<long long>(node) * A.row_stride + A.frame0 + f;
        row[0] = __fdiv_rn(sx, tm);
        row[A.plane_stride] = __fdiv_rn(sy, tm);
        row[2 * A.plane_stride] = __fdiv_rn(sz, tm);
    }
}

__global__ void pad_inf_kernel(float* x, long long rows, int m, int ld) {
    const int pad = ld - m;
    const long long total = rows * pad;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long r = t / pad;
        x[r * ld + m + (t - r * pad)] = __int_as_float(0x7f800000);
    }
}

}  // namespace

void launch_pad_inf(float* x, long long rows, int m, int ld, cudaStream_t st) {
    const long long total = rows * (ld - m);
    if (total <= 0) return;
    const long long want = (total + 255) / 256;
    pad_inf_kernel<<<static_cast<int>(want < 4096 ? want : 4096), 256, 0, st>>>(x, rows, m, ld);
    NSG_CUDA(cudaGetLastError());
}

void launch_node_com(const NodeComArgs& a, cudaStream_t st) {
    const long long total = static_cast<long long>(a.nnodes) * a.nframes;
    if (total == 0) return;
    const int threads = 256;
    const long long want = (total + threads - 1) / threads;
    const int grid = static_cast<int>(want < (1 << 20) ? want : (1 << 20));
    node_com_kernel<<<grid, threads, 0, st>>>(a);
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
