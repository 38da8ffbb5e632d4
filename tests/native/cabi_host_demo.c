/* A plain-C host of the C ABI (include/netsci_gb300.h), the way a non-Python
 * binding (cgo, JNI, FFI) drives it: CuArray handles, the netcalc pair-list
 * call on the CPU platform, a .npy round trip, the psi table, and the loud
 * failure of the GPU platform when no device is present.
 *
 * Usage: cabi_host_demo <input.bin> <out.npy>
 *   input.bin: int32 N, int32 n, int32 k, then N*n float32 (d = 1 rows).
 * Prints one line per pair "mi <a> <b> <value as %.9g>", then "psi <v>",
 * then "gpu_status <s>". */
#include <stdio.h>
#include <stdlib.h>

#include "netsci_gb300.h"

#define CHECK(call)                                                         \
    do {                                                                    \
        int st_ = (call);                                                   \
        if (st_ != NSG_OK) {                                                \
            fprintf(stderr, "%s failed (%d): %s\n", #call, st_, nsg_last_error()); \
            return 1;                                                       \
        }                                                                   \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    if (fread(hdr, sizeof(int), 3, f) != 3) return 2;
    const int N = hdr[0], n = hdr[1], k = hdr[2];
    float* x = (float*)malloc(sizeof(float) * (size_t)N * n);
    if (fread(x, sizeof(float), (size_t)N * n, f) != (size_t)N * n) return 2;
    fclose(f);

    nsg_cuarray *X = NULL, *I = NULL, *ab = NULL, *psi = NULL, *back = NULL;
    int err = 0, result = -1;
    CHECK(nsg_cuarray_create(NSG_DTYPE_FLOAT32, &X));
    CHECK(nsg_cuarray_create(NSG_DTYPE_FLOAT32, &I));
    CHECK(nsg_cuarray_create(NSG_DTYPE_INT32, &ab));
    CHECK(nsg_cuarray_from_host(X, x, N, n, &err));
    const int P = N * (N - 1) / 2;
    int* pairs = (int*)malloc(sizeof(int) * 2 * (size_t)P);
    int p = 0;
    for (int a = 0; a < N; ++a)
        for (int b = a + 1; b < N; ++b) {
            pairs[2 * p] = a;
            pairs[2 * p + 1] = b;
            ++p;
        }
    CHECK(nsg_cuarray_from_host(ab, pairs, P, 2, &err));
    CHECK(nsg_mutual_information(X, I, ab, k, n, 2, 1, NSG_CPU_PLATFORM, &result));
    if (result != NSG_CPU_PLATFORM) return 3;
    CHECK(nsg_cuarray_save(I, argv[2]));
    CHECK(nsg_cuarray_create(NSG_DTYPE_FLOAT32, &back));
    CHECK(nsg_cuarray_load(back, argv[2], &err));
    p = 0;
    for (int a = 0; a < N; ++a)
        for (int b = a + 1; b < N; ++b, ++p) {
            double v = 0, w = 0;
            CHECK(nsg_cuarray_get(I, 0, p, &v));
            CHECK(nsg_cuarray_get(back, 0, p, &w));
            if (v != w) return 4;
            printf("mi %d %d %.9g\n", a, b, v);
        }
    CHECK(nsg_cuarray_create(NSG_DTYPE_FLOAT32, &psi));
    CHECK(nsg_cuarray_init(psi, 1, n + 1, &err));
    CHECK(nsg_generate_psi(psi, n));
    double pv = 0;
    CHECK(nsg_cuarray_get(psi, 0, n, &pv));
    printf("psi %.9g\n", pv);
    /* the GPU platform reports an error status instead of falling back */
    printf("gpu_status %d\n", nsg_mutual_information(X, I, ab, k, n, 2, 1, NSG_GPU_PLATFORM, &result));
    nsg_cuarray_destroy(X);
    nsg_cuarray_destroy(I);
    nsg_cuarray_destroy(ab);
    nsg_cuarray_destroy(psi);
    nsg_cuarray_destroy(back);
    free(x);
    free(pairs);
    return 0;
}
