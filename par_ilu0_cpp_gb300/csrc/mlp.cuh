// Learned per-row diagonal shift: a 4 -> 16 -> 16 -> 1 MLP over per-row features.
//
// Features of row i (A's values on F's pattern, before factorisation):
//   x0 = log(|a_ii| / mean_j |a_jj|)          diagonal magnitude (relative to the matrix)
//   x1 = log(||a_i,off||_2 / mean_j |a_jj|)   off-diagonal row norm
//   x2 = min(|a_ii| / sum_j!=i |a_ij|, 4)     diagonal dominance ratio
//   x3 = depth_i / max(levels - 1, 1)         level depth in the lower dependency DAG
// Output y_i = softplus(MLP(x)) >= 0 is a relative shift: the factorisation uses
//   a_ii + sign(a_ii) * y_i * sum_j!=i |a_ij|.
// Parameter layout (FP32, kMlpParams values): W1[16][4], b1[16], W2[16][16], b2[16],
// W3[16], b3.
#pragma once

#include "common.cuh"

namespace gb300 {

constexpr int kMlpIn = 4;
constexpr int kMlpH = 16;
constexpr int kMlpParams = kMlpH * kMlpIn + kMlpH + kMlpH * kMlpH + kMlpH + kMlpH + 1;
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpH * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpH;
constexpr int kMlpB2 = kMlpW2 + kMlpH * kMlpH;
constexpr int kMlpW3 = kMlpB2 + kMlpH;
constexpr int kMlpB3 = kMlpW3 + kMlpH;
constexpr float kDominanceCap = 4.0f;

struct MlpAct {
    float h1[kMlpH];
    float h2[kMlpH];
    float z;
};

__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(__expf(z)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.f / (1.f + __expf(-z)); }

// Forward pass with the parameters in shared memory.
__device__ __forceinline__ float mlp_forward(const float* P, const float (&x)[kMlpIn], MlpAct& a) {
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) {
        float s = P[kMlpB1 + k];
#pragma unroll
        for (int m = 0; m < kMlpIn; ++m) s = fmaf(P[kMlpW1 + k * kMlpIn + m], x[m], s);
        a.h1[k] = tanhf(s);
    }
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) {
        float s = P[kMlpB2 + k];
#pragma unroll
        for (int j = 0; j < kMlpH; ++j) s = fmaf(P[kMlpW2 + k * kMlpH + j], a.h1[j], s);
        a.h2[k] = tanhf(s);
    }
    float z = P[kMlpB3];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z = fmaf(P[kMlpW3 + k], a.h2[k], z);
    a.z = z;
    return softplus(z);
}

// Per-row statistics of A on F's pattern: |a_ii|, sum of |a_ij| (j != i), off-diagonal
// 2-norm.  The diagonal is the entry at diag[i] (F always has it after SetupMatrix).
__device__ __forceinline__ void row_stats(int i, const int* rp, const int* ci, const double* v, const int* diag,
                                          double& d, double& offsum, double& off2) {
    d = 0.0;
    offsum = 0.0;
    off2 = 0.0;
    const int pd = diag ? diag[i] : -1;
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
        const double a = v[p];
        if (p == pd || (pd < 0 && ci[p] == i)) {
            d = fabs(a);
        } else {
            offsum += fabs(a);
            off2 = fma(a, a, off2);
        }
    }
    off2 = sqrt(off2);
}

__device__ __forceinline__ void make_features(double d, double offsum, double off2, double mean_d, int depth,
                                              int nlev, float (&x)[kMlpIn]) {
    const double md = mean_d > 0.0 ? mean_d : 1.0;
    x[0] = static_cast<float>(log(fmax(d, 1e-300) / md));
    x[1] = static_cast<float>(log(fmax(off2, 1e-300) / md));
    x[2] = static_cast<float>(
        fmin(offsum > 0.0 ? d / offsum : static_cast<double>(kDominanceCap), static_cast<double>(kDominanceCap)));
    x[3] = static_cast<float>(depth) / static_cast<float>(nlev > 1 ? nlev - 1 : 1);
}

}  // namespace gb300
