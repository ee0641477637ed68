// lljbash::PreconditionedGmres on GB300.  Replaces src/gmres.cpp:138-288: the restart
// cycle (residual, m Arnoldi steps with ILU preconditioning, CGS2, Givens, back
// substitution, solution update) is enqueued as one sequence of gated kernels and,
// by default, captured once as a CUDA graph that is replayed per cycle.  The host reads
// the device control record once per cycle to apply the reference's outer-loop rules.
//
// Modes:
//   plain (default): FP64 everywhere; the reference's algorithm and stopping rules.
//   mixed: FP32 Krylov cycles (FP32 SpMV, FP32 ILU factors and substitution, FP32
//          basis; dot products/norms/Hessenberg in FP64) inside FP64 iterative
//          refinement: every cycle starts from the FP64 residual b - A x and adds its
//          FP32 correction to the FP64 x; a cycle stops early once its residual estimate
//          fell by the factor tau, and only the FP64 residual can end the solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <climits>
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "device_util.hpp"
#include "analysis.hpp"
#include "gmres_impl.hpp"
#include "gmres_kernels.cuh"
#include "ilu_impl.hpp"

namespace lljbash {

using namespace gb300;

PreconditionedGmres::Impl::~Impl() {
    if (ctl_host) cudaFreeHost(ctl_host);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

PreconditionedGmres::Impl* PreconditionedGmres::impl_ensure() {
    if (!impl_) impl_ = new Impl;
    return impl_;
}

PreconditionedGmres::~PreconditionedGmres() {
    delete impl_;
    impl_ = nullptr;
}

namespace {

constexpr long long kLdAlign = 512;  // whole Gram-Schmidt chunks (at most 256 rows)

template <class T>
void ensure_krylov(Krylov<T>& K, int n, int im, cudaStream_t s, int sms) {
    const long long ld = std::max<long long>(kLdAlign, ceil_div<long long>(n, kLdAlign) * kLdAlign);
    if (K.n == n && K.im == im && K.ld == ld && K.V.get() != nullptr) return;
    K.V.release();
    K.Z.release();
    K.y.release();
    K.V.reserve(static_cast<size_t>((im + 1) * ld));
    K.Z.reserve(static_cast<size_t>(im * ld));
    K.y.reserve(static_cast<size_t>(ld));
    GB_CUDA_CHECK(cudaMemsetAsync(K.V.get(), 0, sizeof(T) * static_cast<size_t>((im + 1) * ld), s));
    const int threads = 256;
    const long long nz = static_cast<long long>(im) * ld;
    fill_sentinel_kernel<T><<<std::max(1, std::min<int>(static_cast<int>(ceil_div<long long>(nz, threads)), 8 * sms)),
                              threads, 0, s>>>(nz, K.Z.get());
    fill_sentinel_kernel<T><<<std::max(1, std::min<int>(static_cast<int>(ceil_div<long long>(ld, threads)), 8 * sms)),
                              threads, 0, s>>>(ld, K.y.get());
    GB_CUDA_CHECK(cudaGetLastError());
    K.n = n;
    K.im = im;
    K.ld = ld;
    if (K.graph) {
        cudaGraphExecDestroy(K.graph);
        K.graph = nullptr;
    }
}

template <class T>
struct ValueOf;
template <>
struct ValueOf<double> {
    static const double* get(const PreconditionedGmres::Impl& g) { return g.a64_p; }
};
template <>
struct ValueOf<float> {
    static const float* get(const PreconditionedGmres::Impl& g) { return g.a32.get(); }
};

struct Launcher {
    PreconditionedGmres::Impl& g;
    bool timed;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    long long count = 0;
    template <class F>
    void run(KernelKind kind, F&& f) {
        if (timed) GB_CUDA_CHECK(cudaEventRecord(e0, g.stream));
        f();
        count += (kind == kKUpdate) ? 2 : 1;
        GB_CUDA_CHECK(cudaGetLastError());
        if (timed) {
            GB_CUDA_CHECK(cudaEventRecord(e1, g.stream));
            GB_CUDA_CHECK(cudaEventSynchronize(e1));
            float ms = 0.f;
            GB_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
            g.kernel_ms[kind] += ms;
            g.kernel_launches[kind] += 1;
        }
    }
};

// Enqueues cycle pieces.  step == -1: residual / cycle start; step in [0, m): one
// Arnoldi step; step == m: back substitution + update.
template <class T>
void enqueue_piece(PreconditionedGmres::Impl& g, const IluSolver::Impl* ilu, Krylov<T>& K, int step, Launcher& L) {
    cudaStream_t st = g.stream;
    const int n = g.n;
    const long long ld = K.ld;
    GmresCtl* ctl = g.ctl.get();
    const int* gate = reinterpret_cast<const int*>(reinterpret_cast<const char*>(ctl) + offsetof(GmresCtl, gate));
    const double* inv_norm =
        reinterpret_cast<const double*>(reinterpret_cast<const char*>(ctl) + offsetof(GmresCtl, inv_norm));
    Hess H{g.hh.get(), K.im + 1};
    constexpr int R = kWarp * ChunkCfg<T>::RPL;
    const long long nchunks = ld / R;
    if (step < 0) {
        L.run(kKResidual, [&] {
            gmres_residual_kernel<T><<<g.grid_spmv, kSpmvWarps * kWarp, 0, st>>>(
                n, g.rp_p, g.ci_p, g.a64_p, g.b_p, g.x_p, K.V.get(), ctl, H, g.partial.get(), g.counters.get());
        });
        return;
    }
    if (step == K.im) {
        L.run(kKUpdate, [&] {
            gmres_backsolve_kernel<<<1, 256, sizeof(double) * static_cast<size_t>(K.im * K.im + K.im + 1), st>>>(ctl, H);
            gmres_update_kernel<T><<<g.grid_update, 256, 0, st>>>(n, ld, K.Z.get(), g.x_p, ctl, H);
        });
        return;
    }
    const int s = step;
    T* Vs = K.V.get() + s * ld;
    T* Zs = K.Z.get() + s * ld;
    T* W = K.V.get() + (s + 1) * ld;
    if (ilu) {
        L.run(kKLower, [&] { ilu->launch_lower<T>(st, Vs, inv_norm, K.y.get(), gate, s); });
        L.run(kKUpper, [&] { ilu->launch_upper<T>(st, K.y.get(), Zs, gate, s); });
    } else {
        L.run(kKLower, [&] {
            copy_scaled_kernel<T><<<g.grid_update, 256, 0, st>>>(n, Vs, inv_norm, Zs, gate, s);
        });
    }
    L.run(kKSpmv, [&] {
        spmv_kernel<T, T, T><<<g.grid_spmv, kSpmvWarps * kWarp, 0, st>>>(n, g.rp_p, g.ci_p, ValueOf<T>::get(g), Zs, W,
                                                                          gate, s, ilu ? K.y.get() : nullptr);
    });
    const int cgs_grid = g.cgs_grid<T>(nchunks);
    L.run(kKDot, [&] {
        cgs_dot_kernel<T><<<cgs_grid, kBlasThreads, 0, st>>>(nchunks, ld, K.V.get(), s, g.partial.get(), g.h1.get(),
                                                                g.counters.get(), gate);
    });
    L.run(kKAxpyDot, [&] {
        cgs_axpy_dot_kernel<T><<<cgs_grid, kBlasThreads, 0, st>>>(nchunks, ld, K.V.get(), s, g.h1.get(),
                                                                     g.partial.get(), g.h2.get(), g.counters.get(), gate);
    });
    L.run(kKAxpyNorm, [&] {
        cgs_axpy_norm_kernel<T><<<cgs_grid, kBlasThreads, 0, st>>>(nchunks, ld, K.V.get(), s, g.h1.get(), g.h2.get(),
                                                                      g.partial.get(), g.counters.get(), ctl, H, gate);
    });
}

template <class T>
void run_cycle(PreconditionedGmres::Impl& g, const IluSolver::Impl* ilu, Krylov<T>& K) {
    if (g.profile) {
        // Host-driven cycle with every kernel timed; stops launching once the gate closes.
        Launcher L{g, true, g.ev0, g.ev1};
        enqueue_piece<T>(g, ilu, K, -1, L);
        for (int s = 0; s < K.im; ++s) {
            GB_CUDA_CHECK(cudaMemcpyAsync(g.ctl_host, g.ctl.get(), sizeof(GmresCtl), cudaMemcpyDeviceToHost, g.stream));
            GB_CUDA_CHECK(cudaStreamSynchronize(g.stream));
            if (g.ctl_host->gate != s) break;
            enqueue_piece<T>(g, ilu, K, s, L);
        }
        enqueue_piece<T>(g, ilu, K, K.im, L);
        g.launches += L.count;
        return;
    }
    Launcher L{g, false};
    if (!g.use_graph) {
        for (int s = -1; s <= K.im; ++s) enqueue_piece<T>(g, ilu, K, s, L);
        g.launches += L.count;
        return;
    }
    const void* key[kGraphKey] = {K.V.get(),
                                  ilu ? ilu->subst_key<T>() : nullptr,
                                  ilu ? reinterpret_cast<const void*>(static_cast<uintptr_t>(ilu->setup_gen)) : nullptr,
                                  ValueOf<T>::get(g),
                                  g.x_p,
                                  g.b_p};
    bool same = K.graph != nullptr;
    for (int k = 0; k < kGraphKey && same; ++k) same = key[k] == K.graph_key[k];
    if (!same) {
        if (K.graph) {
            cudaGraphExecDestroy(K.graph);
            K.graph = nullptr;
        }
        cudaGraph_t graph = nullptr;
        GB_CUDA_CHECK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
        for (int s = -1; s <= K.im; ++s) enqueue_piece<T>(g, ilu, K, s, L);
        GB_CUDA_CHECK(cudaStreamEndCapture(g.stream, &graph));
        GB_CUDA_CHECK(cudaGraphInstantiate(&K.graph, graph, 0));
        cudaGraphDestroy(graph);
        for (int k = 0; k < kGraphKey; ++k) K.graph_key[k] = key[k];
        K.graph_nodes = L.count;
    }
    GB_CUDA_CHECK(cudaGraphLaunch(K.graph, g.stream));
    g.launches += K.graph_nodes;
}

template <class T>
std::pair<bool, int> solve_mode(PreconditionedGmres::Impl& g, const IluSolver::Impl* ilu, Krylov<T>& K,
                                const GmresParameters& prm) {
    GmresCtl h{};
    h.its = 0;
    h.i = -1;
    h.gate = -1;
    h.status = kCtlRunning;
    h.im = K.im;
    h.maxits = prm.max_iterations;
    h.tol = prm.tolerance;
    h.tau = g.mode == kModeMixed ? g.tau : 0.0;
    *g.ctl_host = h;
    GB_CUDA_CHECK(cudaMemcpyAsync(g.ctl.get(), g.ctl_host, sizeof(GmresCtl), cudaMemcpyHostToDevice, g.stream));
    GB_CUDA_CHECK(cudaEventRecord(g.ev0, g.stream));
    bool ok = true;
    bool converged_at_start = false;
    int cycles = 0;
    int its = 0;
    while (its < prm.max_iterations) {
        run_cycle<T>(g, ilu, K);
        GB_CUDA_CHECK(cudaMemcpyAsync(g.ctl_host, g.ctl.get(), sizeof(GmresCtl), cudaMemcpyDeviceToHost, g.stream));
        GB_CUDA_CHECK(cudaStreamSynchronize(g.stream));
        const GmresCtl c = *g.ctl_host;
        its = c.its;
        if (c.status == kCtlNan) {
            ok = false;
            break;
        }
        if (c.status == kCtlConverged) {
            converged_at_start = true;
            break;
        }
        ++cycles;
        if (g.mode == kModePlain && c.beta <= prm.tolerance) break;
        if (its > prm.max_iterations) {
            ok = false;
            break;
        }
    }
    GB_CUDA_CHECK(cudaEventRecord(g.ev1, g.stream));
    GB_CUDA_CHECK(cudaEventSynchronize(g.ev1));
    float ms = 0.f;
    GB_CUDA_CHECK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
    g.report = SolveReport{};
    g.report.mode = g.mode;
    g.report.iterations = its;
    g.report.cycles = cycles;
    g.report.solve_ms = ms;
    if (converged_at_start) {
        g.report.residual = g.ctl_host->beta;
        g.report.converged = 1;
    } else if (g.verify && g.n > 0) {
        Launcher L{g, false};
        enqueue_piece<T>(g, ilu, K, -1, L);
        g.launches += L.count;
        GB_CUDA_CHECK(cudaMemcpyAsync(g.ctl_host, g.ctl.get(), sizeof(GmresCtl), cudaMemcpyDeviceToHost, g.stream));
        GB_CUDA_CHECK(cudaStreamSynchronize(g.stream));
        g.report.residual = g.ctl_host->beta0;
        g.report.converged = g.ctl_host->beta0 <= prm.tolerance ? 1 : 0;
    }
    return {ok, its};
}

}  // namespace

void PreconditionedGmres::Impl::init_once() {
    if (stream) return;
    dev = current_device();
    GB_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    GB_CUDA_CHECK(cudaEventCreate(&ev0));
    GB_CUDA_CHECK(cudaEventCreate(&ev1));
    GB_CUDA_CHECK(cudaMallocHost(reinterpret_cast<void**>(&ctl_host), sizeof(GmresCtl)));
    grid_spmv = persistent_grid(spmv_kernel<double, double, double>, kSpmvWarps * kWarp, dev.sms, 16);
    // Gram-Schmidt grids per value type: the blocks all three kernels can keep resident
    // (FP32: 2 per SM, FP64: 1), so an FP32 pass is not held to the FP64 kernels' warps.
    auto resident = [&](auto k1, auto k2, auto k3) {
        int a = 0, b = 0, c = 0;
        GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k1, kBlasThreads, 0));
        GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k2, kBlasThreads, 0));
        GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k3, kBlasThreads, 0));
        return std::max(1, std::min({a, b, c, 2})) * dev.sms;
    };
    grid_blas64 = resident(cgs_dot_kernel<double>, cgs_axpy_dot_kernel<double>, cgs_axpy_norm_kernel<double>);
    grid_blas32 = resident(cgs_dot_kernel<float>, cgs_axpy_dot_kernel<float>, cgs_axpy_norm_kernel<float>);
    grid_blas = std::max(grid_blas64, grid_blas32);
    grid_update = 4 * dev.sms;
    GB_CUDA_CHECK(cudaFuncSetAttribute(gmres_backsolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(double) * (kMaxKrylov * kMaxKrylov + kMaxKrylov + 1))));
    counters.reserve(4);
    GB_CUDA_CHECK(cudaMemsetAsync(counters.get(), 0, sizeof(unsigned) * 4, stream));
    ctl.reserve(1);
    h1.reserve(kMaxKrylov + 1);
    h2.reserve(kMaxKrylov + 1);
    partial.reserve(static_cast<size_t>(std::max(grid_spmv, grid_blas)) * kPartialStride);
}

// Shared body of the host-array and device-array entry points: operands are in
// g.rp_p / ci_p / a64_p / b_p / x_p; a32 (mixed mode) is refreshed when needed.
static std::pair<bool, int> solve_core(PreconditionedGmres::Impl& g, IluSolver* ilu_solver, const GmresParameters& prm,
                                       GmresStat& stat, bool refresh_a32) {
    const int im = prm.krylov_subspace_dimension;
    if (im < 1 || im > kMaxKrylov) throw std::runtime_error("krylov_subspace_dimension must be in [1, 128]");
    IluSolver::Impl* ilu = ilu_solver ? ilu_solver->impl() : nullptr;
    if (ilu && (!ilu->factorized || ilu->n != g.n)) throw std::runtime_error("preconditioner not factorised for this size");
    cudaStream_t s = g.stream;
    const int n = g.n;
    const long long nnz = g.nnz;
    if (g.mode == kModeMixed && (refresh_a32 || g.a32_src != g.a64_p || g.a32.size() < static_cast<size_t>(nnz))) {
        g.a32.reserve(static_cast<size_t>(std::max<long long>(nnz, 1)));
        if (nnz > 0)
            convert_kernel<double, float><<<std::min<int>(8 * g.dev.sms, static_cast<int>(ceil_div<long long>(nnz, 256))),
                                            256, 0, s>>>(nnz, g.a64_p, g.a32.get());
        GB_CUDA_CHECK(cudaGetLastError());
        g.a32_src = g.a64_p;
        g.launches += 1;
    }
    g.hh.reserve(static_cast<size_t>(im + 1) * (im + 3));
    if (g.mode == kModeMixed) {
        ensure_krylov(g.k32, n, im, s, g.dev.sms);
    } else {
        ensure_krylov(g.k64, n, im, s, g.dev.sms);
    }
    const double mv0 = g.kernel_ms[kKSpmv] + g.kernel_ms[kKResidual];
    const double pc0 = g.kernel_ms[kKLower] + g.kernel_ms[kKUpper];
    std::pair<bool, int> ret{true, 0};
    if (n > 0) {
        ret = g.mode == kModeMixed ? solve_mode<float>(g, ilu, g.k32, prm) : solve_mode<double>(g, ilu, g.k64, prm);
        if (ilu) ilu->check_status(s);
    }
    stat.total_mv_time += (g.kernel_ms[kKSpmv] + g.kernel_ms[kKResidual] - mv0) * 1e-3;
    stat.total_precon_time += (g.kernel_ms[kKLower] + g.kernel_ms[kKUpper] - pc0) * 1e-3;
    return ret;
}

std::pair<bool, int> PreconditionedGmres::Solve(const CsrMatrix* mat, double* rhs, double* sol) {
    const auto wall0 = std::chrono::steady_clock::now();
    // bounds of the arrays first (no device work yet); the O(nnz) part of the check runs
    // below, while the copies are in flight
    const int n = mat ? mat->size : -1;
    if (n < 0 || (n > 0 && (mat->row_ptr == nullptr || mat->row_ptr[0] != 0 || mat->row_ptr[n] < 0 ||
                            (mat->max_nnz > 0 && mat->row_ptr[n] > mat->max_nnz))))
        validate_csr(n, mat ? mat->row_ptr : nullptr, mat ? mat->col_idx : nullptr, "GMRES matrix",
                     mat && mat->max_nnz > 0 ? mat->max_nnz : -1);
    Impl& g = *impl_ensure();
    g.init_once();
    const long long nnz = n > 0 ? mat->row_ptr[n] : 0;
    cudaStream_t s = g.stream;
    bool refresh = false;
    if (!(g.keep_matrix && g.matrix_loaded && g.n == n && g.nnz == nnz)) {
        // The structural check runs on the host while the copies are in flight; no
        // kernel touches the arrays before it has passed.
        g.matrix_loaded = false;
        g.rp.upload(mat->row_ptr, static_cast<size_t>(n) + 1, s);
        g.ci.upload(mat->col_idx, static_cast<size_t>(nnz), s);
        g.a64.upload(mat->value, static_cast<size_t>(nnz), s);
        try {
            validate_csr(n, mat->row_ptr, mat->col_idx, "GMRES matrix", mat->max_nnz > 0 ? mat->max_nnz : -1);
        } catch (...) {
            cudaStreamSynchronize(s);
            throw;
        }
        refresh = true;
    }
    g.matrix_loaded = true;
    g.n = n;
    g.nnz = nnz;
    const size_t nv = static_cast<size_t>(std::max(n, 1));
    g.b.reserve(nv);
    g.x.reserve(nv);
    if (n > 0) {
        GB_CUDA_CHECK(cudaMemcpyAsync(g.b.get(), rhs, sizeof(double) * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
        GB_CUDA_CHECK(cudaMemcpyAsync(g.x.get(), sol, sizeof(double) * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
    }
    g.rp_p = g.rp.get();
    g.ci_p = g.ci.get();
    g.a64_p = g.a64.get();
    g.b_p = g.b.get();
    g.x_p = g.x.get();
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    stat_.total_init_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    auto ret = solve_core(g, ilu_, param_, stat_, refresh);
    if (n > 0) {
        GB_CUDA_CHECK(cudaMemcpyAsync(sol, g.x.get(), sizeof(double) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, s));
        GB_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    stat_.total_fgmr_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    return ret;
}

std::pair<bool, int> PreconditionedGmres::SolveDevice(int n, const int* d_row_ptr, const int* d_col_idx,
                                                      const double* d_values, const double* d_rhs, double* d_sol) {
    const auto wall0 = std::chrono::steady_clock::now();
    Impl& g = *impl_ensure();
    g.init_once();
    long long nnz = 0;
    if (n < 0) throw std::runtime_error("invalid CSR matrix (GMRES matrix): negative size");
    if (n > 0) {
        int last = 0;
        GB_CUDA_CHECK(cudaMemcpy(&last, d_row_ptr + n, sizeof(int), cudaMemcpyDeviceToHost));
        nnz = last;
        if (nnz < 0) throw std::runtime_error("invalid CSR matrix (GMRES matrix): row_ptr[n] is negative");
        // structural check on the device before any kernel indexes with the arrays
        // (the device arrays are taken to hold n + 1 row pointers and row_ptr[n] entries)
        const int init = INT_MAX;
        int* flag = reinterpret_cast<int*>(g.counters.get() + kCounterCheck);
        GB_CUDA_CHECK(cudaMemcpyAsync(flag, &init, sizeof(int), cudaMemcpyHostToDevice, g.stream));
        const int grid = static_cast<int>(std::min<long long>(4ll * g.dev.sms, ceil_div<long long>(n, 256)));
        csr_check_kernel<<<grid, 256, 0, g.stream>>>(n, nnz, d_row_ptr, d_col_idx, flag);
        GB_CUDA_CHECK(cudaGetLastError());
        g.launches += 1;
        int bad = INT_MAX;
        GB_CUDA_CHECK(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, g.stream));
        GB_CUDA_CHECK(cudaStreamSynchronize(g.stream));
        if (bad != INT_MAX)
            throw std::runtime_error("invalid CSR matrix (GMRES matrix): row " + std::to_string(bad) +
                                     " has bad row pointers or column indices outside [0, n) or not ascending");
    }
    g.n = n;
    g.nnz = nnz;
    g.matrix_loaded = false;
    g.rp_p = d_row_ptr;
    g.ci_p = d_col_idx;
    g.a64_p = d_values;
    g.b_p = d_rhs;
    g.x_p = d_sol;
    auto ret = solve_core(g, ilu_, param_, stat_, !g.keep_matrix);
    GB_CUDA_CHECK(cudaStreamSynchronize(g.stream));
    stat_.total_fgmr_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    return ret;
}

}  // namespace lljbash
