// Cell-grid KSG (ksg_grid.cu, ksg_grid.cuh): device descriptors and the
// host-side launchers the planner uses.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "ksg.cuh"

namespace nsg {

constexpr int kGridMaxG = 32;
constexpr int kGridChunk = 128;     // frames staged per warp step
constexpr int kGridWarps = 8;       // warps per CTA

// Cell index of a grid, one block of memory at `start`:
//   start[G*G+1]   first position of each cell, cells row-major (b1*G + b2);
//   qstart[G*G+1]  the same counts accumulated in query order;
//   qcell[G*G]     row-major cell of the t-th cell in query order.
// Query order is the Z (Morton) order of (b1, b2): a warp's 32 queries, taken
// consecutively in that order, sit in a compact block of cells rather than
// along one row, so the union of their search boxes is smaller. Frames stay
// stored row-major, which keeps a row's column range contiguous.
__host__ __device__ inline int grid_qoff(int G) { return (G * G + 1 + 3) & ~3; }
inline size_t grid_index_bytes(int G) {
    return sizeof(int) * 2 * static_cast<size_t>(grid_qoff(G)) +
           ((static_cast<size_t>(G) * G * sizeof(unsigned short) + 15) & ~static_cast<size_t>(15));
}

// Node grid of one trajectory row (device descriptor).
struct GridNode {
    const float* x;        // original row: x[c*ld + j]
    int ld, m, G;
    int c1, c2;            // c2 < 0 for d == 1
    float* e1;             // kGridMaxG floats: G-1 edges along c1, then +inf
    float* e2;             // likewise along c2 (all +inf when c2 < 0)
    unsigned short* cell;  // [m] cell of frame j: b1*G + b2
    int* perm;             // [m] frames in cell order
    int* start;            // cell index (grid_index_bytes(G)), see above
    float* sx;             // [d][m] coordinates in cell order (plane stride m)
    // [m] local scale of frame j: the distance to its kEstRank-th nearest
    // frame among those of the 3 x 3 cells around its own (+inf if fewer)
    float* est;
};

// Neighbour rank of the node scale estimate (GridNode::est).
constexpr int kEstRank = 6;

// Pair grid of one pair of a batch (device descriptor).
struct GridPair {
    int a, b;              // node indices
    int* perm;             // [m] frames in pair-cell order
    int* start;            // cell index (grid_index_bytes(G)), see above
    float* sx;             // [2d][m] coordinates of a then b in that order
    int* qpos;             // [m] search order: position of the query of each rank
};

// Pairs of a batch that count the same variable (node grid): their counts
// share every distance evaluation.
constexpr int kCountGroup = 4;
// Queries per warp in the counts: two lanes per query, each taking every
// other frame, so the union of the warp's query boxes is that of 16 queries.
constexpr int kCountQueries = 16;
struct CountGroup {
    int node;                      // node grid
    int side;                      // 0: variable a of the pairs, 1: variable b
    int npairs;                    // 1..kCountGroup
    int pairs[kCountGroup];        // batch-relative pair indices
};

struct GridArgs {
    const KsgPairDesc* pairs;   // batch pairs (scratch offsets, m, out)
    const GridPair* gp;         // same indexing as pairs
    const GridNode* nodes;
    const int* wprefix;         // [npairs+1] prefix of ceil(m/32) over the batch (search items)
    const CountGroup* groups;   // count groups of the batch
    const int* gprefix;         // [ngroups+1] prefix of ceil(m/32) over the groups (count items)
    int ngroups;
    int npairs;
    int pair_base;              // index of pairs[0] in the plan's pair array (tie entries)
    int k;
    int* counter;
    int* fault;
    KsgTie* ties;
    int* tie_count;
    int tie_cap;
    float* eps_a;               // scratch, per sample at pair.scratch + i
    float* eps_b;
    int* cnt_a;
    int* cnt_b;
    // query-frame evaluations done: [0] joint distances of the search,
    // [1] one-variable distances of the counts (one per query and frame,
    // shared by the group's pairs), [2] the counts' eps comparisons (one per
    // query, frame and pair of the group)
    unsigned long long* evals;
    // optional per-sample outputs
    float* eps_x;
    float* eps_y;
    float* kdist;
    // Count-query order per group (row gi at corder + gi * corder_ld, at
    // least m entries; nullptr: the node grids' own query order). Filled by
    // grid_launch_counts before the counts.
    int* corder;
    int corder_ld;
    // 1: pass 1 takes its queries in the pairs' search order (GridPair::qpos,
    // built by grid_launch_pairs); 0: in the grids' Z order of cells
    int search_order;
};

// Query orders, built when m <= kOrderMaxM (the keys of one grid fit in
// shared memory):
//   * counts: the queries of the node grid sorted by the Z code of the box
//     of cells their count box (the largest eps of the group's pairs)
//     overlaps, its four corner cells at kOrderBits bits each, so that a
//     warp's queries have boxes of nearly the same cells;
//   * search: the pair grid's cells in kOrderBlock x kOrderBlock blocks,
//     blocks in Z order, and within a block the queries by a size class of
//     the geometric mean of the two nodes' scale estimates.
constexpr int kOrderBits = 4;
constexpr int kOrderBlock = 4;
constexpr int kOrderMaxM = 40960;
// Orders are built for batches whose search runs at least this many waves
// of resident warps. Below that the batch is latency-bound, and the order
// kernels (one CTA per pair or group) sit on its critical path: one pair at
// m = 10000 took 1.4 ms per call with them against 0.95 ms without.
constexpr int kOrderMinWaves = 8;
bool grid_orders_pay(long long search_warps, int sms);

// A frame-mapped row copied out for the cell-grid search:
// out[c*ld_out + s] = x[c*ld + fmap[s]] for s < m, +inf up to ld_out.
struct GatherRow {
    const float* x;
    const int* fmap;
    float* out;
    int ld, m, ld_out;
};

// Appends the count groups of npairs pairs (descriptors with node indices a,
// b; pair indices relative to gps): for each side, the pairs that count the
// same node, in order, kCountGroup at a time.
void append_count_groups(const GridPair* gps, int npairs, std::vector<CountGroup>& out);

// Cells per axis for m samples (about ten frames per cell, at most kGridMaxG).
int grid_cells_per_axis(int m);
// Bytes of one node grid's buffers, and its descriptor with the buffers at
// `base` (16-byte aligned) for row x (stride ld) of m samples.
size_t grid_node_bytes(int m, int d);
GridNode grid_node_at(unsigned char* base, const float* x, int ld, int m);
// Places a pair grid's buffers at byte offset `off` of a batch arena
// (pointers hold offsets until grid_pair_rebase) and returns the end offset.
size_t grid_pair_place(GridPair& g, size_t off, int m, int d);
void grid_pair_rebase(GridPair& g, const void* base);
// Node grids (nodes: device array whose x, ld, m, G and buffers are set),
// with their scale estimates when `est` (needed by the search orders).
void grid_launch_nodes(GridNode* nodes, int nnodes, int d, bool est, cudaStream_t st);
// Pair grids of a batch (pairs, gps: device arrays of npairs) and, when
// `order` (the nodes carry scale estimates), their search orders. max_m: the
// largest m of the pairs (sizes the shared-memory staging). Returns
// GridArgs::search_order for the batch.
int grid_launch_pairs(const KsgPairDesc* pairs, GridPair* gps, const GridNode* nodes, int npairs,
                      int max_m, int d, bool order, cudaStream_t st);
// The search; tie_record: ties checked through a record kept during the
// scan (grid_launch_search_rec, ksg_grid_rec.cu) instead of a second scan of
// the frames within each tied query's k-th distance. Plans of resampled
// trajectories take it: copies of one frame tie on a large share of their
// samples.
void grid_launch_search(const GridArgs& a, int d, int kmax, int grid, bool tie_record, cudaStream_t st);
void grid_launch_search_rec(const GridArgs& a, int d, int kmax, int grid, cudaStream_t st);
void grid_launch_counts(const GridArgs& a, int d, int grid, cudaStream_t st);
// The two halves of grid_launch_counts: the count-order kernel (when the
// args carry a count order; returns the args the count kernel takes), then
// the count kernel itself.
GridArgs grid_launch_count_order(const GridArgs& a, cudaStream_t st);
void grid_launch_count_kernel(const GridArgs& c, int d, int grid, cudaStream_t st);
void grid_launch_combine(const KsgPairDesc* pairs, int npairs, const int* cnt_a, const int* cnt_b,
                         const float* psi, float* psum, int* nx, int* ny, cudaStream_t st);
// Copies frame-mapped rows (device array of nrows); a map entry outside
// [0, ld) sets FAULT_BAD_INDEX in *fault and reads frame 0.
void grid_launch_gather(const GatherRow* rows, int nrows, int d, int* fault, cudaStream_t st);
int grid_search_ctas_per_sm(int d, int kmax);
int grid_count_ctas_per_sm(int d);

}  // namespace nsg
