/*
 * netsci_gb300 C ABI.
 *
 * The drop-in boundary for NetSci's netcalc hot path (KSG mutual
 * information, generalized correlation, Hedetniemi all-pairs shortest
 * paths) on one GB300 GPU. Plain C types only: opaque handles, pointers and
 * sizes. Every function returns an nsg status (NSG_OK == 0); on failure
 * nsg_last_error() gives a message for the calling thread.
 *
 * Three layers:
 *   1. CuArray handles: the reference's CuArray<T> container
 *      (cuarray/include/cuarray.h:23-489), for FFI callers (ctypes, cffi,
 *      SWIG-less bindings).
 *   2. netcalc calls over CuArray handles, one per reference function
 *      (netcalc/include/{mutual_information,generalized_correlation,
 *      hedetniemi,psi,math_utils}.h), same argument meaning, same return
 *      values, invalid platform -> NSG_ERR_PLATFORM.
 *   3. Device-pointer entry points (stream-explicit, caller-owned device
 *      buffers) for batched and resident workloads; these have no single
 *      reference counterpart and say which reference loop they replace.
 *
 * Device pointers are CUDA device addresses on the current device. Streams
 * are cudaStream_t passed as void* (NULL = legacy default stream).
 */
#ifndef NETSCI_GB300_H
#define NETSCI_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NSG_OK 0
#define NSG_ERR_INVALID 1       /* invalid argument                         */
#define NSG_ERR_CUDA 2          /* CUDA runtime error                       */
#define NSG_ERR_PLATFORM 3      /* platform not 0 (GPU) or 1 (CPU)          */
#define NSG_ERR_UNSUPPORTED 4   /* valid but not supported (e.g. k > 32)    */
#define NSG_ERR_DEVICE_FAULT 5  /* a kernel's bounded wait ran out          */
#define NSG_ERR_IO 6            /* file read/write failure                  */

#define NSG_DTYPE_FLOAT32 0
#define NSG_DTYPE_INT32 1
#define NSG_DTYPE_FLOAT64 2

/* Platform constants of netcalc/include/platform.h:8-11. */
#define NSG_GPU_PLATFORM 0
#define NSG_CPU_PLATFORM 1

/* Message of the last failed call on this thread ("" if none). */
const char* nsg_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int nsg_version(void);
/* Frees memory returned by the library (nsg_recover_single_shortest_path). */
void nsg_free(void* p);
/* Device memory the library has freed is kept in a per-device cache (at most
 * 32 GiB per device) and reused by later plans; it is returned to the driver
 * when an allocation of the library fails. This returns all of it now, for a
 * caller about to allocate device memory of its own. */
int nsg_release_cached_memory(void);

/* ---- 1. CuArray handles (cuarray/include/cuarray.h:23-489) -------------- */
typedef struct nsg_cuarray nsg_cuarray;

/* new CuArray<T>() / delete (cuarray/src/cuarray.cu:8-14, :65-73) */
int nsg_cuarray_create(int dtype, nsg_cuarray** out);
int nsg_cuarray_destroy(nsg_cuarray* a);
int nsg_cuarray_dtype(const nsg_cuarray* a);
/* init(m, n): zero-filled host buffer (cuarray.h:49) */
int nsg_cuarray_init(nsg_cuarray* a, int m, int n, int* cuarray_error);
/* init(host, m, n): copy of a host buffer (cuarray.h:68) */
int nsg_cuarray_init_from(nsg_cuarray* a, const void* host, int m, int n, int* cuarray_error);
/* fromCuArrayShallowCopy / fromCuArrayDeepCopy (cuarray.h:91, :116) */
int nsg_cuarray_from_cuarray_shallow(nsg_cuarray* a, nsg_cuarray* src, int start, int end,
                                     int m, int n, int* cuarray_error);
int nsg_cuarray_from_cuarray_deep(nsg_cuarray* a, nsg_cuarray* src, int start, int end, int m,
                                  int n, int* cuarray_error);
/* fromNumpy 1-D (m = 1) and 2-D (cuarray.h:297, :315): copies `data` */
int nsg_cuarray_from_host(nsg_cuarray* a, const void* data, int m, int n, int* cuarray_error);
/* m(), n(), size(), bytes(), owner(), allocatedHost(), allocatedDevice() */
int nsg_cuarray_shape(const nsg_cuarray* a, int* m, int* n, int* size, size_t* bytes,
                      int* owner, int* allocated_host, int* allocated_device);
/* host() / device() raw pointers (cuarray.h:190, :200) */
void* nsg_cuarray_host(nsg_cuarray* a);
void* nsg_cuarray_device(nsg_cuarray* a);
/* allocateHost, allocateDevice, toDevice, toHost, deallocateHost,
 * deallocateDevice (cuarray.h:211-282); *cuarray_error is the CuArrayError */
int nsg_cuarray_allocate_host(nsg_cuarray* a, int* cuarray_error);
int nsg_cuarray_allocate_device(nsg_cuarray* a, int* cuarray_error);
int nsg_cuarray_to_device(nsg_cuarray* a, int* cuarray_error);
int nsg_cuarray_to_host(nsg_cuarray* a, int* cuarray_error);
int nsg_cuarray_deallocate_host(nsg_cuarray* a, int* cuarray_error);
int nsg_cuarray_deallocate_device(nsg_cuarray* a, int* cuarray_error);
/* get(i, j) / set(value, i, j) (cuarray.h:365, :383); values as double */
int nsg_cuarray_get(const nsg_cuarray* a, int i, int j, double* value);
int nsg_cuarray_set(nsg_cuarray* a, double value, int i, int j, int* cuarray_error);
/* load / save .npy (cuarray.h:399, :410) */
int nsg_cuarray_load(nsg_cuarray* a, const char* path, int* cuarray_error);
int nsg_cuarray_save(nsg_cuarray* a, const char* path);
/* sort(i) (descending copy of row i) and argsort(i) (cuarray.h:422, :458) */
int nsg_cuarray_sort(nsg_cuarray* a, int i, nsg_cuarray** out);
int nsg_cuarray_argsort(nsg_cuarray* a, int i, nsg_cuarray** out);

/* ---- 2. netcalc over CuArray handles ------------------------------------ */
/* X: N x (d*n) float, plane-major node rows; ab: P x 2 int; I/R: re-inited
 * to 1 x P. *result is the reference's return value (the platform).       */
/* netcalc/include/mutual_information.h:34-43 (plain), :20-31 (checkpoint) */
int nsg_mutual_information(nsg_cuarray* X, nsg_cuarray* I, nsg_cuarray* ab, int k, int n,
                           int xd, int d, int platform, int* result);
int nsg_mutual_information_checkpointed(nsg_cuarray* X, nsg_cuarray* I, nsg_cuarray* ab, int k,
                                        int n, int xd, int d, int platform,
                                        int checkpoint_frequency,
                                        const char* checkpoint_file_name, int* result);
/* netcalc/include/mutual_information.h:45-66 (per-pair GPU / CPU) */
int nsg_mutual_information_gpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd, int d,
                               float* result);
int nsg_mutual_information_cpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd, int d,
                               float* result);
/* netcalc/include/generalized_correlation.h:55-64 (plain), :30-53 (ckpt) */
int nsg_generalized_correlation(nsg_cuarray* X, nsg_cuarray* R, nsg_cuarray* ab, int k, int n,
                                int xd, int d, int platform, int* result);
int nsg_generalized_correlation_checkpointed(nsg_cuarray* X, nsg_cuarray* R, nsg_cuarray* ab,
                                             int k, int n, int xd, int d, int platform,
                                             int checkpoint_frequency,
                                             const char* checkpoint_file_name, int* result);
/* netcalc/include/generalized_correlation.h:66-96 (per-pair GPU / CPU) */
int nsg_generalized_correlation_gpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd,
                                    int d, float* result);
int nsg_generalized_correlation_cpu(nsg_cuarray* Xa, nsg_cuarray* Xb, int k, int n, int xd,
                                    int d, float* result);
/* netcalc/include/mutual_information.h:68-80 */
int nsg_generate_restart_ab_from_checkpoint_file(nsg_cuarray* ab, nsg_cuarray* restart_ab,
                                                 const char* checkpoint_file_name);
/* netcalc/include/hedetniemi.h:31-38, :60-66, :106-111, :122-126 */
int nsg_hedetniemi_all_shortest_paths(nsg_cuarray* A, nsg_cuarray* H, nsg_cuarray* paths,
                                      int max_path_length, float tolerance, int platform);
int nsg_hedetniemi_all_shortest_paths_gpu(nsg_cuarray* A, nsg_cuarray* H, nsg_cuarray* paths,
                                          float tolerance, int max_path_length);
int nsg_hedetniemi_all_shortest_path_lengths(nsg_cuarray* A, nsg_cuarray* H,
                                             int max_path_length, int platform);
int nsg_hedetniemi_all_shortest_path_lengths_gpu(nsg_cuarray* A, nsg_cuarray* H,
                                                 int max_path_length);
/* netcalc/include/hedetniemi.h:139-160 */
int nsg_correlation_to_adjacency(nsg_cuarray* A, nsg_cuarray* C, int n, int platform);
/* netcalc/include/hedetniemi.h:173-180: *path (free with nsg_free), *len */
int nsg_recover_single_shortest_path(nsg_cuarray* paths, int max_path_length, int i, int j,
                                     int** path, int* len);
/* netcalc/include/psi.h:160-163 (generatePsi, table of n+1 floats) */
int nsg_generate_psi(nsg_cuarray* psi, int n);
/* netcalc/include/math_utils.h:22-95 (mean, meanGpu, standardDeviation,
 * standardDeviationGpu): row means / population standard deviations of a
 * row-major matrix; the platform calls re-initialise u (and sigma) to
 * 1 x (size/n) and compute only for platform 0, as the reference.          */
int nsg_mean(nsg_cuarray* a, nsg_cuarray* u, int m, int n, int platform);
int nsg_mean_gpu(nsg_cuarray* a, nsg_cuarray* u, int m, int n);
int nsg_standard_deviation(nsg_cuarray* a, nsg_cuarray* u, nsg_cuarray* sigma, int m, int n,
                           int platform);
int nsg_standard_deviation_gpu(nsg_cuarray* a, nsg_cuarray* u, nsg_cuarray* sigma, int m, int n);

/* ---- 3. device-pointer entry points -------------------------------------- */

/* One KSG variable pair on the device. Component c of sample s of variable
 * a is xa[c*ld + f(s)] with f the identity, or f(s) = fmap[s] (bootstrap
 * resample; fmap a device int array of m frame indices < ld).            */
typedef struct nsg_ksg_pair {
    const float* xa;
    const float* xb;
    const int* fmap;
    int ld;
    int m;
} nsg_ksg_pair;

/* All pairs of a list in one persistent launch plus a finalize launch.
 * Replaces the per-pair loop of netcalc/src/generalized_correlation.cpp:
 * 104-173 and netcalc/src/mutual_information.cpp:103-172 together with the
 * per-pair GPU call of netcalc/src/mutual_information_gpu.cu:1007-1079.
 * pairs: host array. mi / gc / w: device float[npairs] outputs, each
 * nullable (w = -ln(gc), +inf where gc == 0). Asynchronous on `stream`.  */
int nsg_ksg_pairs_device(const nsg_ksg_pair* pairs, int npairs, int k, int d, float* mi,
                         float* gc, float* w, void* stream);

/* One pair with per-sample outputs (device arrays of m, each nullable):
 * marginal counts n_x, n_y (after the reference's -1), eps_x, eps_y and the
 * k-th neighbour joint distance. mi: device float[1], nullable.            */
int nsg_ksg_pair_detail_device(const float* xa, const float* xb, int ld, int m, int k, int d,
                               int* n_x, int* n_y, float* eps_x, float* eps_y, float* kdist,
                               float* mi, void* stream);

/* Reusable plan: device descriptors, work queue and scratch built once;
 * each run is one captured CUDA graph (work-queue reset, count kernel,
 * finalize kernel per batch). Flags: bit 0 = capture a CUDA graph; bit 1 =
 * record CUDA events around every count launch (nsg_ksg_plan_count_ms);
 * bit 2 = pick the tile shape with the autotuner (each instantiated shape
 * timed on up to 512 of the pairs, longest first; the result is cached per
 * (GPU, d, k bucket, m bucket, pair-count bucket), in the file named by the
 * environment variable NSG_TUNE_CACHE when set).
 * The tile shape comes from the autotuner cache when one is loaded.       */
typedef struct nsg_ksg_plan nsg_ksg_plan;
int nsg_ksg_plan_create(const nsg_ksg_pair* pairs, int npairs, int k, int d, float* mi,
                        float* gc, float* w, int flags, nsg_ksg_plan** out);
int nsg_ksg_plan_run(nsg_ksg_plan* plan, void* stream);
/* Captures and instantiates a graph plan's CUDA graph without running it. */
int nsg_ksg_plan_prepare(nsg_ksg_plan* plan);
/* The tile shape a plan runs with (CTA threads, samples per thread, frames
 * per tile, arithmetic variant); each pointer nullable.                   */
int nsg_ksg_plan_shape(const nsg_ksg_plan* plan, int* threads, int* r, int* frames,
                       int* variant);
/* Tile staging a plan runs with: 1 bulk copies (TMA), 0 plain loads.      */
int nsg_ksg_plan_staging(const nsg_ksg_plan* plan, int* staging);
/* Raises NSG_ERR_DEVICE_FAULT when the runs so far recorded a device fault
 * (frame map entry out of range, tie list overflow); synchronizes.        */
int nsg_ksg_plan_check(nsg_ksg_plan* plan);
/* Kernel launches one run makes (count, tie resolution, finalize per batch). */
int nsg_ksg_plan_launches(const nsg_ksg_plan* plan, int* launches);
/* Device milliseconds of the count kernels in the last run (flag bit 1);
 * waits for that run's events.                                          */
int nsg_ksg_plan_count_ms(const nsg_ksg_plan* plan, float* ms);
int nsg_ksg_plan_destroy(nsg_ksg_plan* plan);

/* Force a KSG tile shape (CTA threads, samples per thread, frames per tile,
 * arithmetic variant; variant < 0 = any) for subsequent calls in this
 * process; threads == 0 restores automatic choice.                        */
int nsg_ksg_set_shape(int threads, int r, int frames, int variant);
/* Tile staging for subsequent plans: 1 = bulk copies (TMA) into shared
 * memory, 0 = plain loads, -1 = automatic (bulk copies when every pair has
 * 16-byte aligned rows, a plane stride that is a multiple of 4 and no
 * frame map).                                                             */
int nsg_ksg_set_staging(int staging);
/* Search for later plans: 1 cell grids (ksg_grid.cuh: only the frames whose
 * cells can reach a query are evaluated; same results), 0 exhaustive, -1
 * automatic (cell grids when at least half of the work, counted as m^2 per
 * pair, is in pairs with m >= 1000 (4000 for plans of fewer than 8 pairs)
 * and the copies of frame-mapped rows, which the grids search instead of
 * the maps, fit in 8 GiB). */
int nsg_ksg_set_search(int mode);
/* Query orders of later cell-grid plans: 1 = always build them (the search's
 * block order and the counts' box order of a batch), 0 = never (cells in Z
 * order),
 * -1 = automatic (only for batches whose search runs at least eight waves
 * of resident warps, where the order kernels pay for themselves). Orders
 * change which frames are visited first, never a result; m above 40960
 * always takes the Z order. Tuning knob with no reference counterpart.    */
int nsg_ksg_set_orders(int mode);
/* Issue ceilings of the cell-grid kernels, measured on the current device:
 * the operation rate (Gop/s) of the search kernel's and the count kernel's
 * inner loops alone (their own distance arithmetic on a staged tile, with no
 * memory traffic, no range setup and no neighbour-list updates), counted as
 * the kernels' rates are (search: 4d per joint distance; counts: 2d-1 per
 * one-variable distance plus one per eps comparison). A diagnostic for the
 * roofline of those kernels; no reference counterpart. Takes about 0.1 s. */
int nsg_measure_issue_ceiling(int d, double* search_gops, double* count_gops);
/* *mode = 1 when the plan uses cell grids, 0 when exhaustive. */
int nsg_ksg_plan_search(const nsg_ksg_plan* plan, int* mode);
/* Query-frame evaluations of the plan's last run with cell grids: *search
 * joint distances of the search, *counts one-variable distances of the
 * counts (one per query and frame, shared by the pairs of a count group),
 * *compares (may be null) the counts' eps comparisons (one per query, frame
 * and pair of the group). An exhaustive run evaluates m*m of each kind per
 * pair; 0 for exhaustive plans. Synchronizes with the device. */
int nsg_ksg_plan_evaluations(const nsg_ksg_plan* plan, unsigned long long* search,
                             unsigned long long* counts, unsigned long long* compares);
/* Device milliseconds of the last run's search kernels, count kernels and
 * tie kernels (tie_ms nullable; flag bit 1), summed over the plan's batches;
 * the order kernels are not included. An exhaustive plan's single kernel
 * counts as search. Waits for that run's events. */
int nsg_ksg_plan_kernel_ms(const nsg_ksg_plan* plan, float* search_ms, float* count_ms,
                           float* tie_ms);
/* Samples of the plan's last run whose k-th and (k+1)-th joint distances tie
 * between frames with different marginals, i.e. that went to the tie kernel
 * to replay the reference sort's order. Synchronizes with the device. */
int nsg_ksg_plan_tied_samples(const nsg_ksg_plan* plan, long long* n);

/* One pair's MI / GC without any device allocation. No counterpart in the
 * reference: it is for callers that cannot allocate device memory, such as
 * an application that owns the GPU's memory through its own pool and calls
 * this library as a plugin on its buffers, or a loop that cannot afford the
 * synchronisation an allocation may cause. All scratch lives in a fixed
 * NSG_NOALLOC_SCRATCH_BYTES device array inside the library, present on
 * every GPU that loads it until the process exits. The first call on each
 * device (with that device current) looks the array up and fills its psi
 * table, so make it before any stream capture. The address and the table
 * are kept for the life of the process: a host that resets the device
 * (cudaDeviceReset) after that first call cannot use this entry point any
 * more. Calls share the array: calls whose work overlaps on the GPU race.
 * m is at most
 * NSG_NOALLOC_MAX_SAMPLES (larger m: NSG_ERR_UNSUPPORTED). Rows as in
 * nsg_ksg_pair_detail_device; mi, gc: device float[1] each, one nullable.
 * Synchronizes `stream`.                                                  */
#define NSG_NOALLOC_MAX_SAMPLES 65536
#define NSG_NOALLOC_SCRATCH_BYTES 9454336
int nsg_ksg_pair_noalloc_device(const float* xa, const float* xb, int ld, int m, int k, int d,
                                float* mi, float* gc, void* stream);

/* Hedetniemi shortest path lengths on the device (A, H: n x n device
 * floats). H_{t+1}[i][j] = min_k A[j][k] + H_t[k][i] from H_0 = A, until H
 * stops changing or max_path_length steps. netcalc/src/hedetniemi_gpu.cu:
 * 109-146. Where max_path_length >= n-1 and A is symmetric with a zero
 * diagonal, no negative weight and integer weights whose path sums stay
 * below 2^24, the same fixed point is reached by repeated squaring
 * (H <- H (x) H, about log2 of the hop diameter products), bit for bit.
 * *steps (host, nullable) receives the min-plus products run (steps or
 * squarings). Synchronizes `stream` to read flags.                       */
int nsg_apsp_lengths_device(const float* A, float* H, int n, int max_path_length, int* steps,
                            void* stream);
/* Product schedule of later shortest-path solves: -1 automatic (squaring
 * only where it is bit-exact, as above), 0 Jacobi steps always (the
 * reference's association of every path sum), 1 squaring wherever the
 * fixed point of a symmetric, zero-diagonal, non-negative A is asked for
 * (float weights then agree with the reference within the rounding of a
 * path sum). Tuning knob with no reference counterpart.                  */
int nsg_apsp_set_method(int method);
/* Shortest paths with snapshots: paths device int[n*max_path_length*n],
 * layout paths[i*L*n + j*L + p]. netcalc/src/hedetniemi_gpu.cu:148-235. */
int nsg_apsp_paths_device(const float* A, float* H, int* paths, int n, int max_path_length,
                          float tolerance, void* stream);
/* Correlation -> adjacency on the device: mode 0 = 1/r with +inf for r == 0
 * (netcalc/src/hedetniemi_gpu.cu:10-26); mode 1 = -ln(r) with +inf for
 * r <= 0. Diagonal 0 in both.                                             */
int nsg_corr_to_adjacency_device(const float* C, float* A, int n, int mode, void* stream);
/* Row means (and, with sigma non-null, population standard deviations) of
 * a device row-major m x n matrix into device u[m], sigma[m]; the
 * summation order of netcalc/src/math_utils_gpu.cu:22-158.                 */
int nsg_row_stats_device(const float* a, float* u, float* sigma, int m, int n, void* stream);

/* ---- 4. serving: continuous batching of MI / GC / APSP jobs ------------- */
/* A request loop with no reference counterpart (the reference serves one
 * blocking call at a time). Jobs are submitted from any thread with host
 * input and output buffers that must stay valid until the job is done. A
 * scheduler thread admits jobs when their device footprint fits
 * budget_bytes and runs ticks of about tick_ops algorithmic operations, each
 * one persistent launch over pairs of the admitted MI/GC jobs: first every
 * job whose remaining work fits in a quarter of a tick, whole, then the rest
 * of the tick in arrival order; jobs that arrive meanwhile join the next
 * tick. APSP jobs run on their own stream.
 * Registered trajectories stay resident in HBM. Job states: 0 pending,
 * 1 running, 2 done, 3 failed. Times are seconds on the host steady clock. */
typedef struct nsg_server nsg_server;
int nsg_server_create(size_t budget_bytes, double tick_ops, int max_m, nsg_server** out);
int nsg_server_destroy(nsg_server* s);
/* X: host N x (d*m) plane-major rows, uploaded once and kept resident. */
int nsg_server_register_trajectory(nsg_server* s, const float* X, int N, int m, int d,
                                   int* traj);
/* GC of all pairs a < b of a trajectory into out (host, N(N-1)/2 floats). */
int nsg_server_submit_gc(nsg_server* s, int traj, int k, float* out, long long* job);
/* MI of one pair (host x, y: d planes of n samples) into out (host float). */
int nsg_server_submit_mi(nsg_server* s, const float* x, const float* y, int n, int d, int k,
                         float* out, long long* job);
/* Shortest path lengths of a host N x N matrix into out (host N*N floats). */
int nsg_server_submit_apsp(nsg_server* s, const float* A, int N, int max_path_length,
                           float* out, long long* job);
/* Waits up to timeout_s for the job; *state as above. */
int nsg_server_wait(nsg_server* s, long long job, double timeout_s, int* state);
int nsg_server_job_info(nsg_server* s, long long job, int* state, double* submit_s,
                        double* admit_s, double* done_s);
int nsg_server_stats(nsg_server* s, long long* jobs_done, long long* pairs_done,
                     long long* ticks, size_t* peak_bytes);

/* ---- 5. netchem: trajectory -> node coordinates --------------------------- */
/* netchem::Network (netchem/include/network.h:19-172) over an opaque handle.
 * nsg_network_init replaces Network::init (netchem/src/network.cpp:29-75):
 * PDB ATOM records grouped into nodes by residue tag, DCD frames first,
 * first + stride, ..., <= last (last == -1: the file's last frame), node
 * mass-weighted centres computed on the device. Atom and node fields are
 * those of netchem/include/atom.h:57-189 and node.h:39-88.                  */
typedef struct nsg_network nsg_network;
typedef struct nsg_atom_info {
    int index, serial, residue_id;
    float occupancy, temperature_factor, mass;
    unsigned int hash;
    char name[8], element[4], residue_name[8], chain_id[4], segment_id[8], tag[40];
} nsg_atom_info;
typedef struct nsg_node_info {
    int index, num_atoms;
    float total_mass;
    unsigned int hash;
    char tag[40];
} nsg_node_info;
int nsg_network_create(nsg_network** out);
int nsg_network_destroy(nsg_network* net);
int nsg_network_init(nsg_network* net, const char* trajectory_file, const char* topology_file,
                     int first_frame, int last_frame, int stride);
/* Network::parsePdb (netchem/src/network.cpp:258-278): appends the file's
 * ATOM records to the network's atoms (host only; init() calls it).        */
int nsg_network_parse_pdb(nsg_network* net, const char* topology_file);
int nsg_network_num_nodes(nsg_network* net, int* n);
int nsg_network_num_frames(nsg_network* net, int* m);
int nsg_network_num_atoms(nsg_network* net, int* n);
/* Copies Network::nodeCoordinates() (N x 3m) into the CuArray `out`. */
int nsg_network_node_coordinates(nsg_network* net, nsg_cuarray* out);
/* Network::nodeCoordinates(file): node coordinates from a .npy file. */
int nsg_network_load_node_coordinates(nsg_network* net, const char* npy_file);
int nsg_network_node(nsg_network* net, int node, nsg_node_info* out);
/* Atom indices of a node, in index order; *count = number of atoms (at most
 * cap are written).                                                        */
int nsg_network_node_atoms(nsg_network* net, int node, int* atoms, int cap, int* count);
int nsg_network_atom(nsg_network* net, int atom, nsg_atom_info* out);
int nsg_network_node_from_atom(nsg_network* net, int atom, int* node);
/* Device-resident node coordinates (valid until the next init or destroy):
 * row n at *X + n*3*(*ld), planes x, y, z of *ld floats, +inf past m. The
 * rows can be passed as nsg_ksg_pair.xa / .xb with d = 3.                  */
int nsg_network_device_coordinates(nsg_network* net, const float** X, int* ld);
/* DCD frames on the host (the reader under nsg_network_init): atom and
 * frame counts, and frames first, first + stride, ... (count of them) into
 * xyz[f][c][atom] (c = x, y, z). netchem/src/dcd/dcd.cpp:775-940.          */
int nsg_dcd_info(const char* path, int* natoms, int* nsets);
int nsg_dcd_read(const char* path, int first, int count, int stride, float* xyz);

#ifdef __cplusplus
}
#endif

#endif /* NETSCI_GB300_H */
