// Learned diagonal shift: the feature pre-pass fused with MLP inference (run right
// before the factorisation kernel), and the hand-written training kernels (forward,
// backward, Adam) used to fit the MLP on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "device_util.hpp"
#include "gmres_kernels.cuh"
#include "mlp.cuh"
#include "mlp_impl.hpp"

namespace gb300 {

constexpr int kPrepassThreads = 256;

// Sum of |a_ii| over rows (deterministic: per-block partials, last block adds them).
__global__ void __launch_bounds__(kPrepassThreads)
    shift_mean_diag_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                           const int* __restrict__ diag, double* partial, unsigned* counter, double* mean_out) {
    __shared__ double sred[kPrepassThreads / kWarp];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int pd = diag ? diag[i] : -1;
        if (pd >= 0) {
            s += fabs(v[pd]);
        } else {
            for (int p = rp[i]; p < rp[i + 1]; ++p)
                if (ci[p] == i) s += fabs(v[p]);
        }
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kPrepassThreads / kWarp; ++k) t += sred[k];
        partial[blockIdx.x] = t;
    }
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int b = 0; b < static_cast<int>(gridDim.x); ++b) t += __ldcg(partial + b);
        *mean_out = n > 0 ? t / n : 1.0;
    }
}

// Per row: features -> MLP -> shift = sign(a_ii) * y * sum_j!=i |a_ij| (0 when y is
// below min_shift).  Optionally also writes the features and y.
__global__ void __launch_bounds__(kPrepassThreads)
    shift_prepass_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                         const int* __restrict__ diag, const int* __restrict__ depth, int nlev,
                         const double* __restrict__ mean_d, const float* __restrict__ params, float min_shift,
                         double* __restrict__ shift_out, float* __restrict__ X_out, float* __restrict__ y_out) {
    __shared__ float P[kMlpParams];
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) P[k] = params ? params[k] : 0.f;
    __syncthreads();
    const double md = *mean_d;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d, offsum, off2;
        row_stats(i, rp, ci, v, diag, d, offsum, off2);
        float x[kMlpIn];
        make_features(d, offsum, off2, md, depth ? depth[i] : 0, nlev, x);
        if (X_out) {
#pragma unroll
            for (int m = 0; m < kMlpIn; ++m) X_out[static_cast<size_t>(i) * kMlpIn + m] = x[m];
        }
        if (params) {
            MlpAct a;
            const float y = mlp_forward(P, x, a);
            if (y_out) y_out[i] = y;
            if (shift_out) {
                const int pd = diag ? diag[i] : -1;
                const double aii = pd >= 0 ? v[pd] : 1.0;
                const double sgn = aii < 0.0 ? -1.0 : 1.0;
                shift_out[i] = y >= min_shift ? sgn * static_cast<double>(y) * offsum : 0.0;
            }
        }
    }
}

__global__ void __launch_bounds__(kPrepassThreads)
    mlp_forward_kernel(int n, const float* __restrict__ X, const float* __restrict__ params, float* __restrict__ y) {
    __shared__ float P[kMlpParams];
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) P[k] = params[k];
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float x[kMlpIn];
#pragma unroll
        for (int m = 0; m < kMlpIn; ++m) x[m] = X[static_cast<size_t>(i) * kMlpIn + m];
        MlpAct a;
        y[i] = mlp_forward(P, x, a);
    }
}

// One training step over `batch` samples (indices idx, or 0..batch-1): mean squared
// error between y = softplus(z) and the target t, gradient by backpropagation (chain
// rule through softplus, two tanh layers), accumulated in shared memory, reduced over
// blocks in block order by the last block, which then (apply != 0) takes one Adam step.
// grad_out receives the mean gradient, loss_out the mean loss.
__global__ void __launch_bounds__(kPrepassThreads)
    mlp_train_kernel(const float* __restrict__ X, const float* __restrict__ T, const int* __restrict__ idx, int batch,
                     float* params, float* partial, unsigned* counter, float* grad_out, double* loss_out, float* adam_m,
                     float* adam_v, int step, float lr, int apply) {
    __shared__ float P[kMlpParams];
    __shared__ float G[kMlpParams + 1];
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) P[k] = params[k];
    for (int k = threadIdx.x; k <= kMlpParams; k += blockDim.x) G[k] = 0.f;
    __syncthreads();
    const float inv_b = 1.f / static_cast<float>(batch);
    float loss = 0.f;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < batch; s += gridDim.x * blockDim.x) {
        const int i = idx ? idx[s] : s;
        float x[kMlpIn];
#pragma unroll
        for (int m = 0; m < kMlpIn; ++m) x[m] = X[static_cast<size_t>(i) * kMlpIn + m];
        MlpAct a;
        const float y = mlp_forward(P, x, a);
        const float diff = y - T[i];
        loss = fmaf(diff, diff, loss);
        const float dz = 2.f * diff * inv_b * sigmoid(a.z);
        atomicAdd(&G[kMlpB3], dz);
        float dh2[kMlpH];
#pragma unroll
        for (int k = 0; k < kMlpH; ++k) {
            atomicAdd(&G[kMlpW3 + k], dz * a.h2[k]);
            dh2[k] = dz * P[kMlpW3 + k] * (1.f - a.h2[k] * a.h2[k]);
        }
#pragma unroll
        for (int k = 0; k < kMlpH; ++k) {
            atomicAdd(&G[kMlpB2 + k], dh2[k]);
#pragma unroll
            for (int j = 0; j < kMlpH; ++j) atomicAdd(&G[kMlpW2 + k * kMlpH + j], dh2[k] * a.h1[j]);
        }
#pragma unroll
        for (int j = 0; j < kMlpH; ++j) {
            float g = 0.f;
#pragma unroll
            for (int k = 0; k < kMlpH; ++k) g = fmaf(dh2[k], P[kMlpW2 + k * kMlpH + j], g);
            const float dh1 = g * (1.f - a.h1[j] * a.h1[j]);
            atomicAdd(&G[kMlpB1 + j], dh1);
#pragma unroll
            for (int m = 0; m < kMlpIn; ++m) atomicAdd(&G[kMlpW1 + j * kMlpIn + m], dh1 * x[m]);
        }
    }
    atomicAdd(&G[kMlpParams], loss * inv_b);
    __syncthreads();
    for (int k = threadIdx.x; k <= kMlpParams; k += blockDim.x)
        partial[static_cast<size_t>(blockIdx.x) * (kMlpParams + 1) + k] = G[k];
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    constexpr float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int k = threadIdx.x; k <= kMlpParams; k += blockDim.x) {
        double g = 0.0;
        for (int b = 0; b < static_cast<int>(gridDim.x); ++b)
            g += __ldcg(partial + static_cast<size_t>(b) * (kMlpParams + 1) + k);
        if (k == kMlpParams) {
            *loss_out = g;
            continue;
        }
        grad_out[k] = static_cast<float>(g);
        if (apply) {
            const float gf = static_cast<float>(g);
            const float m = b1 * adam_m[k] + (1.f - b1) * gf;
            const float v = b2 * adam_v[k] + (1.f - b2) * gf * gf;
            adam_m[k] = m;
            adam_v[k] = v;
            const float mh = m / (1.f - powf(b1, static_cast<float>(step)));
            const float vh = v / (1.f - powf(b2, static_cast<float>(step)));
            params[k] = P[k] - lr * mh / (sqrtf(vh) + eps);
        }
    }
}

// ---------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------
void ShiftPrepass::ensure(int sms) {
    if (grid == 0) {
        grid = 4 * sms;
        partial.reserve(static_cast<size_t>(grid));
        counter.reserve(1);
        mean.reserve(1);
        GB_CUDA_CHECK(cudaMemset(counter.get(), 0, sizeof(unsigned)));
    }
}

void ShiftPrepass::run(cudaStream_t s, int sms, int n, const int* rp, const int* ci, const double* v, const int* diag,
                       const int* depth, int nlev, const float* params, float min_shift, double* shift_out,
                       float* X_out, float* y_out) {
    ensure(sms);
    if (n <= 0) return;
    shift_mean_diag_kernel<<<grid, kPrepassThreads, 0, s>>>(n, rp, ci, v, diag, partial.get(), counter.get(), mean.get());
    shift_prepass_kernel<<<grid, kPrepassThreads, 0, s>>>(n, rp, ci, v, diag, depth, nlev, mean.get(), params,
                                                          min_shift, shift_out, X_out, y_out);
    GB_CUDA_CHECK(cudaGetLastError());
}

ShiftTrainer::ShiftTrainer(unsigned seed) {
    dev = current_device();
    GB_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    grid = 2 * dev.sms;
    params.reserve(kMlpParams);
    adam_m.reserve(kMlpParams);
    adam_v.reserve(kMlpParams);
    grad.reserve(kMlpParams);
    partial.reserve(static_cast<size_t>(grid) * (kMlpParams + 1));
    counter.reserve(1);
    loss.reserve(1);
    GB_CUDA_CHECK(cudaMemsetAsync(counter.get(), 0, sizeof(unsigned), stream));
    // Glorot-uniform initialisation; the output bias starts at softplus^{-1}(0.01) so the
    // untrained network predicts a small shift.
    std::mt19937 rng(seed);
    std::vector<float> p(kMlpParams, 0.f);
    auto glorot = [&](int off, int fan_in, int fan_out) {
        std::uniform_real_distribution<float> u(-1.f, 1.f);
        const float a = std::sqrt(6.f / static_cast<float>(fan_in + fan_out));
        for (int k = 0; k < fan_in * fan_out; ++k) p[off + k] = a * u(rng);
    };
    glorot(kMlpW1, kMlpIn, kMlpH);
    glorot(kMlpW2, kMlpH, kMlpH);
    glorot(kMlpW3, kMlpH, 1);
    p[kMlpB3] = std::log(std::expm1(0.01f));
    set_params(p.data());
}

ShiftTrainer::~ShiftTrainer() {
    if (stream) cudaStreamDestroy(stream);
}

void ShiftTrainer::set_params(const float* host) {
    GB_CUDA_CHECK(cudaMemcpyAsync(params.get(), host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, stream));
    GB_CUDA_CHECK(cudaMemsetAsync(adam_m.get(), 0, sizeof(float) * kMlpParams, stream));
    GB_CUDA_CHECK(cudaMemsetAsync(adam_v.get(), 0, sizeof(float) * kMlpParams, stream));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
    step = 0;
}

void ShiftTrainer::get_params(float* host) {
    GB_CUDA_CHECK(cudaMemcpyAsync(host, params.get(), sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
}

void ShiftTrainer::set_data(const float* X_host, const float* T_host, int n_samples) {
    n = n_samples;
    X.upload(X_host, static_cast<size_t>(n) * kMlpIn, stream);
    T.upload(T_host, static_cast<size_t>(n), stream);
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
}

double ShiftTrainer::run(const int* idx_host, int batch, float lr, bool apply, float* grad_host) {
    if (n <= 0) throw std::runtime_error("trainer has no data");
    const int* d_idx = nullptr;
    if (idx_host) {
        idx.upload(idx_host, static_cast<size_t>(batch), stream);
        d_idx = idx.get();
    } else {
        batch = n;
    }
    if (apply) ++step;
    mlp_train_kernel<<<grid, kPrepassThreads, 0, stream>>>(X.get(), T.get(), d_idx, batch, params.get(), partial.get(),
                                                          counter.get(), grad.get(), loss.get(), adam_m.get(),
                                                          adam_v.get(), std::max(step, 1), lr, apply ? 1 : 0);
    GB_CUDA_CHECK(cudaGetLastError());
    double h_loss = 0.0;
    GB_CUDA_CHECK(cudaMemcpyAsync(&h_loss, loss.get(), sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (grad_host)
        GB_CUDA_CHECK(cudaMemcpyAsync(grad_host, grad.get(), sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
    return h_loss;
}

void ShiftTrainer::predict(float* y_host) {
    if (n <= 0) return;
    y.reserve(static_cast<size_t>(n));
    mlp_forward_kernel<<<grid, kPrepassThreads, 0, stream>>>(n, X.get(), params.get(), y.get());
    GB_CUDA_CHECK(cudaGetLastError());
    GB_CUDA_CHECK(cudaMemcpyAsync(y_host, y.get(), sizeof(float) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, stream));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
}

void shift_features_host(int n, const int* rp, const int* ci, const double* v, const int* depth, int nlev, float* X,
                         const float* params_host, float* y_host) {
    DeviceInfo dev = current_device();
    cudaStream_t s = nullptr;
    GB_CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    DeviceBuffer<int> d_rp, d_ci, d_depth;
    DeviceBuffer<double> d_v;
    DeviceBuffer<float> d_X, d_p, d_y;
    const long long nnz = rp[n];
    d_rp.upload(rp, static_cast<size_t>(n) + 1, s);
    d_ci.upload(ci, static_cast<size_t>(nnz), s);
    d_v.upload(v, static_cast<size_t>(nnz), s);
    if (depth) d_depth.upload(depth, static_cast<size_t>(n), s);
    d_X.reserve(static_cast<size_t>(std::max(n, 1)) * kMlpIn);
    if (params_host) {
        d_p.upload(params_host, kMlpParams, s);
        d_y.reserve(static_cast<size_t>(std::max(n, 1)));
    }
    ShiftPrepass pre;
    pre.run(s, dev.sms, n, d_rp.get(), d_ci.get(), d_v.get(), nullptr, depth ? d_depth.get() : nullptr, nlev,
            params_host ? d_p.get() : nullptr, 0.f, nullptr, d_X.get(), params_host ? d_y.get() : nullptr);
    if (n > 0) {
        GB_CUDA_CHECK(cudaMemcpyAsync(X, d_X.get(), sizeof(float) * static_cast<size_t>(n) * kMlpIn,
                                      cudaMemcpyDeviceToHost, s));
        if (params_host && y_host)
            GB_CUDA_CHECK(cudaMemcpyAsync(y_host, d_y.get(), sizeof(float) * static_cast<size_t>(n),
                                          cudaMemcpyDeviceToHost, s));
    }
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    cudaStreamDestroy(s);
}

}  // namespace gb300
