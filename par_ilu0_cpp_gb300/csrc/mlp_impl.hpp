// Host-side objects of the learned-shift MLP (see mlp.cuh / mlp.cu).
#pragma once

#include <cuda_runtime.h>

#include "device_util.hpp"

namespace gb300 {

// Feature pre-pass + MLP inference launched ahead of a factorisation.
struct ShiftPrepass {
    int grid = 0;
    DeviceBuffer<double> partial, mean;
    DeviceBuffer<unsigned> counter;
    void ensure(int sms);
    // shift_out (optional) receives the per-row diagonal shifts, X_out / y_out (optional)
    // the features and the MLP outputs.  params == nullptr computes features only.
    void run(cudaStream_t s, int sms, int n, const int* rp, const int* ci, const double* v, const int* diag,
             const int* depth, int nlev, const float* params, float min_shift, double* shift_out, float* X_out,
             float* y_out);
};

// GPU training state: parameters, Adam moments, dataset, reduction scratch.
struct ShiftTrainer {
    DeviceInfo dev;
    cudaStream_t stream = nullptr;
    int grid = 0;
    int n = 0;
    int step = 0;
    DeviceBuffer<float> params, adam_m, adam_v, grad, partial, X, T, y;
    DeviceBuffer<int> idx;
    DeviceBuffer<unsigned> counter;
    DeviceBuffer<double> loss;

    explicit ShiftTrainer(unsigned seed);
    ~ShiftTrainer();
    void set_params(const float* host);
    void get_params(float* host);
    void set_data(const float* X_host, const float* T_host, int n_samples);
    // One pass over `batch` samples (idx_host) or the whole data set (idx_host null);
    // apply = Adam step.  Returns the mean loss; grad_host (optional) gets the gradient.
    double run(const int* idx_host, int batch, float lr, bool apply, float* grad_host);
    void predict(float* y_host);
};

// Features (and, with params, MLP outputs) of a host CSR matrix, computed on the device.
void shift_features_host(int n, const int* rp, const int* ci, const double* v, const int* depth, int nlev, float* X,
                         const float* params_host, float* y_host);

}  // namespace gb300
