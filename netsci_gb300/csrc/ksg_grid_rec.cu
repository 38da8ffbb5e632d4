// The cell-grid search with the tie record (ksg_grid_pass1_kernel<D, KMAX,
// true>), in a translation unit of its own so that it compiles in parallel
// with ksg_grid.cu.
#include <cuda_runtime.h>

#include "errors.h"
#include "ksg_grid.cuh"
#include "ksg_grid.h"

namespace nsg {
namespace {

template <int D>
void launch_pass1_rec(const GridArgs& a, int kmax, int grid, cudaStream_t st) {
    const dim3 b(32 * kGridWarps);
    switch (kmax) {
        case 6: ksg_grid_pass1_kernel<D, 6, true><<<grid, b, 0, st>>>(a); break;
        case 8: ksg_grid_pass1_kernel<D, 8, true><<<grid, b, 0, st>>>(a); break;
        case 16: ksg_grid_pass1_kernel<D, 16, true><<<grid, b, 0, st>>>(a); break;
        case 32: ksg_grid_pass1_kernel<D, 32, true><<<grid, b, 0, st>>>(a); break;
        case 64: ksg_grid_pass1_kernel<D, 64, true><<<grid, b, 0, st>>>(a); break;
        default: fail(NSG_ERR_UNSUPPORTED, "no grid kernel for this k");
    }
}

}  // namespace

void grid_launch_search_rec(const GridArgs& a, int d, int kmax, int grid, cudaStream_t st) {
    switch (d) {
        case 1: launch_pass1_rec<1>(a, kmax, grid, st); break;
        case 2: launch_pass1_rec<2>(a, kmax, grid, st); break;
        case 3: launch_pass1_rec<3>(a, kmax, grid, st); break;
        default: invalid("d must be 1, 2 or 3");
    }
    NSG_CUDA(cudaGetLastError());
}

}  // namespace nsg
