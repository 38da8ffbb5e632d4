// KSG mutual-information engine: device-side job layout shared by the
// kernels (ksg.cu) and the host planner (engine.cpp).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace nsg {

// One variable pair. Component c of sample s of variable a is
// xa[c*ld + f(s)], with f the identity or, for bootstrap resamples,
// f(s) = fmap[s]. This is the plane-major row layout of the reference's X
// (netchem/src/network.cpp:136-161, indexed as in
// netcalc/src/mutual_information_gpu.cu:454-459), with a plane stride.
struct KsgPairDesc {
    const float* xa;
    const float* xb;
    const int* fmap;      // null: identity
    long long scratch;    // offset of this pair's per-sample row in the scratch arrays
    int ld;               // plane stride in floats
    int m;                // samples
    int out;              // output slot of this pair
    int pad;
};

// A slice of one pair's query samples handled by one CTA pass.
struct KsgItem {
    int pair;
    int q0;
    int q1;
    int pad;
};

// A sample whose k-th and (k+1)-th nearest joint distances are equal.
struct KsgTie {
    int pair;             // index into the pair descriptor array
    int q;                // sample
};

struct KsgCountArgs {
    const KsgPairDesc* pairs;
    const KsgItem* items;
    int nitems;
    int k;
    int* counter;         // work-queue head, zero before launch
    int* fault;           // device fault word
    KsgTie* ties;         // tied samples, appended at tie_count
    int* tie_count;       // zero before launch
    int tie_cap;
    const float* psi;     // psi table, at least max(m)+1 entries
    float* psum;          // psi[n_x]+psi[n_y] per sample, at pair.scratch + q
    // optional per-sample outputs (null when unused), at pair.scratch + q
    int* nx;
    int* ny;
    float* eps_x;
    float* eps_y;
    float* kdist;
};

struct KsgTieArgs {
    const KsgPairDesc* pairs;
    const KsgTie* ties;
    const int* tie_count;
    int tie_cap;
    int* tie_next;        // work counter over tie entries, zero before launch
    int k;
    int* fault;
    const float* psi;
    float* psum;
    int* nx;
    int* ny;
    float* eps_x;
    float* eps_y;
    float* dz;            // per-warp scratch rows of `stride` floats
    int* idx;             // per-warp scratch rows of `stride` ints
    long long stride;
};

struct KsgFinalArgs {
    const KsgPairDesc* pairs;
    int npairs;
    int k;
    int d;
    const float* psi;
    const float* psum;
    float* mi;            // optional outputs indexed by pair.out (null when unused)
    float* gc;
    float* w;             // -ln(gc) edge weight, +inf when gc == 0
};

// Tile shape of one kernel instantiation.
struct KsgShape {
    int threads;          // CTA size
    int r;                // query samples per thread
    int frames;           // frames per shared-memory tile
};

int ksg_kmax_for(int k);                      // 0 when k is unsupported
KsgShape ksg_default_shape(int d, int kmax);
// Maximum resident CTAs per SM for the instantiation (occupancy query).
int ksg_ctas_per_sm(int d, int kmax, const KsgShape& s);
void ksg_launch_counts(const KsgCountArgs& a, int d, int kmax, const KsgShape& s, int grid,
                       cudaStream_t st);
void ksg_launch_final(const KsgFinalArgs& a, cudaStream_t st);
// Warps the tie kernel runs with (scratch rows needed).
int ksg_tie_warps();
void ksg_launch_ties(const KsgTieArgs& a, int d, cudaStream_t st);
void ksg_launch_ties_ctas(const KsgTieArgs& a, int d, int ctas, cudaStream_t st);
// One pair with all scratch in the library's static device area
// (ksg_noalloc.cu); synchronizes s.
void ksg_pair_noalloc(const float* xa, const float* xb, int ld, int m, int k, int d, float* mi,
                      float* gc, cudaStream_t s);
bool ksg_shape_supported(int d, int kmax, const KsgShape& s);

}  // namespace nsg
