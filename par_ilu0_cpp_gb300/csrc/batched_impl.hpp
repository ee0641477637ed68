// Host driver of the batched persistent ILU(0) + GMRES solver (see batched.cuh).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "device_util.hpp"

namespace gb300 {

class BatchSolver {
public:
    // nsys systems; system s has n[s] rows; rp_all holds the systems' row pointers one
    // after the other (n[s] + 1 entries each, any base), ci_all / val_all their entries
    // (column indices local to the system, rows column-sorted with a diagonal).
    // fval_all (optional): the values to factorise, same layout as val_all (e.g. A plus a
    // diagonal shift); GMRES always iterates on val_all.
    BatchSolver(int nsys, const int* n, const int* rp_all, const int* ci_all, const double* val_all, int nrhs,
                int restart, double rtol, int maxit, const double* fval_all = nullptr);
    ~BatchSolver();
    BatchSolver(const BatchSolver&) = delete;
    BatchSolver& operator=(const BatchSolver&) = delete;

    void set_model(const float* params, float min_shift);
    void set_tau(double tau) { tau_ = tau; }
    // Tries launch shapes (right-hand sides per CTA x CTAs per SM) on a sample of the batch.
    void autotune();
    void set_shape(int ctas_per_sm, bool largest_first, int rhs_per_cta);
    // rhs_host: for every system, nrhs vectors of n[s] values (system-major); x_host the
    // same layout.  iters / resid / converged: nsys * nrhs entries (optional).
    float solve(const double* rhs_host, double* x_host, int* iters, double* resid, int* converged);

    struct Trial {
        int ctas_per_sm;
        int largest_first;
        int rhs_per_cta;
        float ms;
    };
    const std::vector<Trial>& trials() const { return tuned_; }
    int ctas_per_sm() const { return ctas_per_sm_; }
    bool largest_first() const { return largest_first_; }
    int rhs_per_cta() const { return rhs_per_cta_; }
    float last_ms() const { return last_ms_; }
    long long launches() const { return launches_; }
    long long total_unknowns() const { return total_rhs_; }

private:
    float launch(int ctas_per_sm, bool largest_first, int nsys_run, int rhs_per_cta);
    void ensure_workspace(int grid, int rhs_per_cta);
    size_t workspace_bytes(int grid, int rhs_per_cta) const;
    // largest workspace an autotuner trial may allocate (per-CTA Krylov bases)
    static constexpr size_t kBatchWorkspaceCap = size_t(48) << 30;
    // iterations per right-hand side in an autotuner trial
    static constexpr int kBatchTrialIterations = 40;
    bool trial_ = false;

    int nsys_ = 0, nrhs_ = 0, m_ = 0;
    double rtol_ = 1e-8, tau_ = 1e-6;
    int maxit_ = 1000;
    int nmax_ = 0;
    long long ws_ = 0, total_rows_ = 0, total_rhs_ = 0;
    std::vector<int> n_, order_;
    DeviceInfo dev_;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    int epoch_ = 0;
    int ctas_per_sm_ = 1;
    int rhs_per_cta_ = 1;
    bool largest_first_ = true;
    bool model_ = false;
    float min_shift_ = 0.f;
    float last_ms_ = 0.f;
    long long launches_ = 0;
    std::vector<Trial> tuned_;
    DeviceBuffer<int> d_n_, d_nlevL_, d_nlevU_, d_order_, d_rp_, d_ci_, d_diag_, d_ordL_, d_ordU_, d_lptrL_, d_lptrU_,
        d_depth_, d_iters_, d_conv_, d_shifted_, d_ready_, d_status_;
    DeviceBuffer<long long> d_rp_off_, d_nnz_off_, d_row_off_, d_lvl_off_, d_rhs_off_;
    DeviceBuffer<double> d_a64_, d_f64_, d_lu64_, d_rhs_, d_x_, d_resid_, d_xw_, d_rw_, d_H_;
    DeviceBuffer<float> d_a32_, d_lu32_, d_dinv_, d_mlp_, d_V_, d_Z_;
    DeviceBuffer<unsigned> d_ticket_;
};

}  // namespace gb300
