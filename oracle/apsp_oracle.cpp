// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's Hedetniemi all-pairs shortest-path
// solver and the adjacency transforms around it. The reference has no CPU
// implementation of these (netcalc/src/hedetniemi_cpu.cpp:5-16 only prints
// "not implemented") and no test, so parity of the APSP path is unpinned by
// the reference; this restatement follows the GPU kernels' arithmetic and is
// cross-checked by an independent Floyd-Warshall on integer weights.
//
// Iteration form. The reference kernel updates H in place
// (netcalc/src/hedetniemi_gpu.cu:28-45), so which neighbour values a thread
// reads depends on scheduling. This restatement runs the same update as a
// Jacobi step, H_{t+1}[i][j] = min_k fl(A[j][k] + H_t[k][i]), from H_0 = A,
// until H stops changing or maxPathLength steps have run. Both forms reach
// the same fixed point; before it, the in-place form can only be closer to
// it. Each entry is a minimum of single roundings, so the result does not
// depend on the order k is visited in.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

extern "C" {

// One Jacobi Hedetniemi step. netcalc/src/hedetniemi_gpu.cu:28-45.
static void hedetniemi_step(const float* A, const float* H, float* Hn, int n) {
    const float inf = std::numeric_limits<float>::infinity();
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            float c = inf;
            for (int k = 0; k < n; ++k) {
                float s = A[(size_t)j * n + k] + H[(size_t)k * n + i];
                if (s < c) c = s;
            }
            Hn[(size_t)i * n + j] = c;
        }
    }
}

// Shortest path lengths. netcalc/src/hedetniemi.cpp:39-54 with
// netcalc/src/hedetniemi_gpu.cu:109-146. Returns the number of steps run;
// *converged is set to 1 when the last step left H unchanged.
int oracle_apsp_lengths(const float* A, float* H, int n, int maxPathLength,
                        int* converged) {
    std::vector<float> cur(A, A + (size_t)n * n), nxt((size_t)n * n);
    int steps = 0;
    int conv = 0;
    for (int p = 0; p < maxPathLength; ++p) {
        hedetniemi_step(A, cur.data(), nxt.data(), n);
        ++steps;
        bool same = std::memcmp(cur.data(), nxt.data(), sizeof(float) * (size_t)n * n) == 0;
        cur.swap(nxt);
        if (same) {
            conv = 1;
            break;
        }
    }
    std::memcpy(H, cur.data(), sizeof(float) * (size_t)n * n);
    if (converged) *converged = conv;
    return steps;
}

// Floyd-Warshall over the same matrix, used only as an independent check of
// converged lengths (exact on integer weights).
void oracle_floyd_warshall(const float* A, float* D, int n) {
    std::memcpy(D, A, sizeof(float) * (size_t)n * n);
    for (int k = 0; k < n; ++k)
        for (int i = 0; i < n; ++i) {
            float dik = D[(size_t)i * n + k];
            for (int j = 0; j < n; ++j) {
                float s = dik + D[(size_t)k * n + j];
                if (s < D[(size_t)i * n + j]) D[(size_t)i * n + j] = s;
            }
        }
}

// Shortest paths with snapshots and back-walk.
// netcalc/src/hedetniemi_gpu.cu:148-235 (driver), :47-68 (step + snapshot),
// :70-107 (walk). Snapshots Hi[p] hold H before step p, p = 0..L-1, with the
// reference's L = maxPathLength steps always run. paths is n*L*n ints laid out
// as paths[i*L*n + j*L + p]. Off-diagonal cells follow the walk; each
// diagonal cell (i, i, p) holds i. (The reference writes the diagonal value
// to flat index j*n+i, outside this layout, racing with the thread that owns
// that cell; the intended "a vertex reaches itself" value is stored here.)
void oracle_apsp_paths(const float* A, float* H, int* paths, int n,
                       int maxPathLength, float tolerance) {
    const int L = maxPathLength;
    std::vector<float> Hi((size_t)L * n * n);
    std::vector<float> cur(A, A + (size_t)n * n), nxt((size_t)n * n);
    for (int p = 0; p < L; ++p) {
        std::memcpy(&Hi[(size_t)p * n * n], cur.data(), sizeof(float) * (size_t)n * n);
        hedetniemi_step(A, cur.data(), nxt.data(), n);
        cur.swap(nxt);
    }
    std::memcpy(H, cur.data(), sizeof(float) * (size_t)n * n);
    for (size_t t = 0; t < (size_t)n * L * n; ++t) paths[t] = -1;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            int* cell = paths + (size_t)i * L * n + (size_t)j * L;
            if (i == j) {
                for (int p = 0; p < L; ++p) cell[p] = i;
                continue;
            }
            float len = cur[(size_t)i * n + j];
            int k = j;
            for (int p = L - 1; p >= 0; --p) {
                const float* hp = &Hi[(size_t)p * n * n + (size_t)i * n];
                for (int q = 0; q < n; ++q) {
                    if (q == j) continue;
                    if (hp[q] + A[(size_t)q * n + k] - len < tolerance) {
                        len -= A[(size_t)q * n + k];
                        k = q;
                        break;
                    }
                }
                cell[p] = k;
            }
        }
    }
}

// 1/r adjacency. netcalc/src/hedetniemi_gpu.cu:10-26.
void oracle_corr_to_adj(const float* C, float* A, int n) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            float c = C[(size_t)i * n + j];
            float v;
            if (i == j) v = 0.0f;
            else if (c == 0.0f) v = std::numeric_limits<float>::infinity();
            else v = 1.0f / c;
            A[(size_t)i * n + j] = v;
        }
}

// -ln(r) adjacency used by the generalized-correlation network workloads:
// 0 on the diagonal, +inf where r <= 0, else -ln(r) evaluated in double and
// rounded to float.
void oracle_corr_to_neglog_adj(const float* C, float* A, int n) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            float c = C[(size_t)i * n + j];
            float v;
            if (i == j) v = 0.0f;
            else if (!(c > 0.0f)) v = std::numeric_limits<float>::infinity();
            else v = static_cast<float>(-std::log(static_cast<double>(c)));
            A[(size_t)i * n + j] = v;
        }
}

}  // extern "C"
