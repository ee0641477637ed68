// Internal state of lljbash::PreconditionedGmres.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "device_util.hpp"
#include "gmres.hpp"
#include "gmres_kernels.cuh"

namespace gb300 {

// Kernel categories timed in profiling mode.
enum KernelKind {
    kKResidual = 0,
    kKLower,
    kKUpper,
    kKSpmv,
    kKDot,
    kKAxpyDot,
    kKAxpyNorm,
    kKUpdate,
    kKKinds
};

// Word of PreconditionedGmres::Impl::counters that the structural check of a
// device-resident matrix reports into ([0] is the reductions' ticket counter).
constexpr int kCounterCheck = 3;

// Precision modes of Solve().
enum SolveMode { kModePlain = 0, kModeMixed = 1 };

struct SolveReport {
    int mode = 0;
    int iterations = 0;   // Arnoldi steps over all cycles
    int cycles = 0;       // restart cycles (outer refinement steps in mixed mode)
    int converged = 0;    // true FP64 residual <= tolerance at exit (when verified)
    double residual = -1; // ||b - A x||_2 in FP64 at exit (-1 when not computed)
    double solve_ms = 0;  // device time of the solve (events around the cycles)
};

// Identity of a captured cycle graph: the basis, the preconditioner's substitution data,
// its setup generation, the matrix values and the solution / right-hand side.
constexpr int kGraphKey = 6;

// The per-precision Krylov workspace and its captured cycle graph.
template <class T>
struct Krylov {
    DeviceBuffer<T> V, Z, y;
    long long ld = 0;
    int im = 0;
    int n = 0;
    cudaGraphExec_t graph = nullptr;
    const void* graph_key[kGraphKey] = {};
    long long graph_nodes = 0;
    ~Krylov() {
        if (graph) cudaGraphExecDestroy(graph);
    }
};

}  // namespace gb300

namespace lljbash {

struct PreconditionedGmres::Impl {
    gb300::DeviceInfo dev;
    cudaStream_t stream = nullptr;
    int n = 0;
    long long nnz = 0;
    gb300::DeviceBuffer<int> rp, ci;
    gb300::DeviceBuffer<double> a64, b, x;
    gb300::DeviceBuffer<float> a32;
    // Operands of the current solve: the buffers above (host-array entry point) or the
    // caller's device arrays (device-resident entry point).
    const int* rp_p = nullptr;
    const int* ci_p = nullptr;
    const double* a64_p = nullptr;
    const double* b_p = nullptr;
    double* x_p = nullptr;
    const double* a32_src = nullptr;  // a64 array that a32 was converted from
    long long launches = 0;           // kernels launched by solves (graph nodes included)
    gb300::Krylov<double> k64;
    gb300::Krylov<float> k32;
    gb300::DeviceBuffer<double> hh, h1, h2, partial;
    gb300::DeviceBuffer<unsigned> counters;  // [0] reductions, [kCounterCheck] CSR check
    gb300::DeviceBuffer<gb300::GmresCtl> ctl;
    gb300::GmresCtl* ctl_host = nullptr;  // pinned mirror
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int grid_spmv = 0, grid_blas = 0, grid_update = 0;
    int grid_blas64 = 0, grid_blas32 = 0;  // resident Gram-Schmidt blocks per value type

    // Gram-Schmidt grid for `nchunks` row chunks of value type T: at most the resident
    // blocks, and no more blocks than needed for every warp to take the same number of
    // chunks (a warp with one chunk more than the others would set the pass's length).
    template <class T>
    int cgs_grid(long long nchunks) const {
        const long long cap = sizeof(T) == 8 ? grid_blas64 : grid_blas32;
        const long long warps = cap * gb300::kBlasWarps;
        const long long per_warp = std::max<long long>(1, (nchunks + warps - 1) / warps);
        const long long g = (nchunks + per_warp * gb300::kBlasWarps - 1) / (per_warp * gb300::kBlasWarps);
        return static_cast<int>(std::max<long long>(1, std::min(g, cap)));
    }

    int mode = gb300::kModePlain;
    double tau = 1e-6;             // mixed mode: relative reduction per inner cycle
    bool use_graph = true;
    bool profile = false;          // time every kernel with events (no graph)
    bool keep_matrix = false;      // reuse the device copy of A from the previous Solve
    bool matrix_loaded = false;
    bool verify = true;            // compute the FP64 true residual at exit
    double kernel_ms[gb300::kKKinds] = {};
    long long kernel_launches[gb300::kKKinds] = {};
    gb300::SolveReport report;

    void init_once();
    ~Impl();
};

}  // namespace lljbash
