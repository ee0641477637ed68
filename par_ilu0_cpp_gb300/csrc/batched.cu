// Batched persistent ILU(0) + GMRES(m) (see batched.cuh) and its host driver with the
// launch-shape autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "analysis.hpp"
#include "batched.cuh"
#include "batched_impl.hpp"
#include "common.cuh"
#include "device_util.hpp"
#include "ilu_kernels.cuh"
#include "mlp.cuh"

namespace gb300 {

namespace {

// Sum over the CTA of one double per thread (all threads must call it).
__device__ double block_sum(double v, double* red) {
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < kBatchWarps; ++k) t += red[k];
    __syncthreads();
    return t;
}

struct SysView {
    int n;
    const int* rp;
    const int* ci;
    const double* a64;
    float* a32;
    double* lu64;
    float* lu32;
    const int* diag;
    const int* ordL;
    const int* ordU;
    const int* lptrL;
    const int* lptrU;
    const int* depth;
    float* dinv;
    int nlevL, nlevU;
};

__device__ SysView sys_view(const BatchDesc& D, int s) {
    SysView v;
    v.n = D.n[s];
    v.rp = D.rp + D.rp_off[s];
    const long long z = D.nnz_off[s];
    v.ci = D.ci + z;
    v.a64 = D.a64 + z;
    v.a32 = D.a32 + z;
    v.lu64 = D.lu64 + z;
    v.lu32 = D.lu32 + z;
    const long long r = D.row_off[s];
    v.diag = D.diag + r;
    v.ordL = D.ordL + r;
    v.ordU = D.ordU + r;
    v.depth = D.depth + r;
    v.dinv = D.dinv + r;
    v.lptrL = D.lptrL + D.lvl_off[s];
    v.lptrU = D.lptrU + D.lvl_off[s];
    v.nlevL = D.nlevL[s];
    v.nlevU = D.nlevU[s];
    return v;
}

// Factorisation item: copy, learned shift, level-synchronous up-looking ILU(0) in FP64,
// FP32 factors and reciprocal diagonal, then publish.
__device__ void factor_system(const BatchDesc& D, int s, double* red, float* P) {
    const SysView S = sys_view(D, s);
    const int n = S.n;
    const long long nnz = S.rp[n];
    const double* fv = D.f64 ? D.f64 + D.nnz_off[s] : S.a64;
    for (long long p = threadIdx.x; p < nnz; p += blockDim.x) S.lu64[p] = fv[p];
    __syncthreads();
    bool shifted = false;
    if (D.mlp) {
        for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) P[k] = D.mlp[k];
        double sd = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) sd += fabs(S.a64[S.diag[i]]);
        const double md = block_sum(sd, red) / (n > 0 ? n : 1);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double d, offsum, off2;
            row_stats(i, S.rp, S.ci, S.a64, S.diag, d, offsum, off2);
            float x[kMlpIn];
            make_features(d, offsum, off2, md, S.depth[i], S.nlevL, x);
            MlpAct a;
            const float y = mlp_forward(P, x, a);
            if (y >= D.min_shift) {
                const double aii = S.a64[S.diag[i]];
                S.lu64[S.diag[i]] = aii + (aii < 0.0 ? -1.0 : 1.0) * static_cast<double>(y) * offsum;
            }
        }
        shifted = true;
        __syncthreads();
    }
    for (int l = 0; l < S.nlevL; ++l) {
        for (int q = S.lptrL[l] + threadIdx.x; q < S.lptrL[l + 1]; q += blockDim.x) {
            const int j = S.ordL[q];
            const int e = S.rp[j + 1];
            for (int p = S.rp[j]; p < S.diag[j]; ++p) {
                const int k = S.ci[p];
                const double lv = S.lu64[p] / S.lu64[S.diag[k]];
                S.lu64[p] = lv;
                int pj = p + 1;
                for (int qk = S.diag[k] + 1; qk < S.rp[k + 1]; ++qk) {
                    const int c = S.ci[qk];
                    while (pj < e && S.ci[pj] < c) ++pj;
                    if (pj < e && S.ci[pj] == c) S.lu64[pj] = fma(-S.lu64[qk], lv, S.lu64[pj]);
                }
            }
        }
        __syncthreads();
    }
    for (long long p = threadIdx.x; p < nnz; p += blockDim.x) {
        S.lu32[p] = static_cast<float>(S.lu64[p]);
        S.a32[p] = static_cast<float>(S.a64[p]);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) S.dinv[i] = static_cast<float>(1.0 / S.lu64[S.diag[i]]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        if (D.shifted) D.shifted[s] = shifted ? 1 : 0;
        st_release(D.ready + s, D.epoch);
    }
}

// Solve item: system s, right-hand sides r0 .. r0 + G - 1 (those below nrhs), solved in
// lockstep by one CTA.  Vectors are interleaved [row][G] and thread t works on right-hand
// side g = t % G of rows t / G, t / G + T / G, ...: each coefficient of L, U and A is
// loaded once for the G right-hand sides, the G threads reading it touch consecutive
// vector entries, and the level-synchronous sweeps pay their barriers once for G
// right-hand sides.  Each right-hand side keeps its own GMRES state (Hessenberg matrix in
// global workspace, rotations, residual, convergence); one that has converged or run out
// of iterations idles while the others continue.
__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the lanes of a warp that share g = lane % G (lanes g < G hold the sums).
template <int G, class V>
__device__ __forceinline__ V warp_sum_g(V v) {
#pragma unroll
    for (int o = 16; o >= G; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-right-hand-side sums over the CTA: every thread adds its value for g = tid % G into
// acc[g] (shared memory, zeroed by the caller before a barrier); a barrier follows.
template <int G>
__device__ __forceinline__ void group_sum(double v, double* acc) {
    v = warp_sum_g<G>(v);
    if ((threadIdx.x & 31) < G) atomicAdd(acc + (threadIdx.x & 31), v);
    __syncthreads();
}

// Per-item GMRES state of the G right-hand sides, carved from dynamic shared memory
// (sizes follow the restart length m): reductions acc [m + 1][G], and per right-hand side
// hc / cs / sn / rs [G][m + 2] (FP64), cf [G][m + 2] (FP32) and scalars.
struct GroupSmem {
    double* acc;
    double *hc, *cs, *sn, *rs;  // row g at g * ld
    float* cf;
    double *tol, *stop, *beta, *hnext;
    int *alive, *cyc, *its, *last, *conv;
    int* any;
    int* flag;
    int ld;
};

__host__ __device__ inline size_t group_smem_bytes(int m, int G) {
    const size_t ld = static_cast<size_t>(m) + 2;
    return sizeof(double) * (static_cast<size_t>(m + 1) * G + 4 * G * ld + 4 * G) + sizeof(float) * G * ld +
           sizeof(int) * (5 * G + 2) + 16;
}

__device__ inline GroupSmem group_smem(unsigned char* base, int m, int G) {
    GroupSmem S;
    S.ld = m + 2;
    double* d = reinterpret_cast<double*>(base);
    S.acc = d;
    d += (m + 1) * G;
    S.hc = d;
    d += G * S.ld;
    S.cs = d;
    d += G * S.ld;
    S.sn = d;
    d += G * S.ld;
    S.rs = d;
    d += G * S.ld;
    S.tol = d;
    S.stop = d + G;
    S.beta = d + 2 * G;
    S.hnext = d + 3 * G;
    d += 4 * G;
    float* f = reinterpret_cast<float*>(d);
    S.cf = f;
    f += G * S.ld;
    int* i = reinterpret_cast<int*>(f);
    S.alive = i;
    S.cyc = i + G;
    S.its = i + 2 * G;
    S.last = i + 3 * G;
    S.conv = i + 4 * G;
    S.any = i + 5 * G;
    S.flag = i + 5 * G + 1;
    return S;
}

template <int G>
__device__ void solve_group(const BatchDesc& D, int s, int r0, const GroupSmem& S2) {
    if (threadIdx.x == 0) *S2.flag = wait_flag(D.ready + s, D.epoch, D.status) ? 1 : 0;
    __syncthreads();
    const SysView S = sys_view(D, s);
    const int n = S.n;
    const int m = D.m;
    const long long ws = D.ws;
    const int tid = threadIdx.x;
    const int T = blockDim.x;
    const int g = tid % G;   // right-hand side of this thread
    const int rl = tid / G;  // first row of this thread
    const int RT = T / G;    // rows per round
    const int ng = min(G, D.nrhs - r0);
    float* V = D.V + static_cast<long long>(blockIdx.x) * (m + 1) * ws * G;  // V_k[row][g]
    float* Z = D.Z + static_cast<long long>(blockIdx.x) * m * ws * G;
    double* x = D.xw + static_cast<long long>(blockIdx.x) * ws * G;  // x[row][g]
    double* rw = D.rw + static_cast<long long>(blockIdx.x) * ws * G;
    const long long io = D.rhs_off[s] + static_cast<long long>(r0 + (g < ng ? g : 0)) * n;
    const double* b = D.rhs + io;
    const int out_base = s * D.nrhs + r0;
    if (!*S2.flag) {  // the factorisation never became ready: report and skip
        if (tid < ng) {
            D.iters[out_base + tid] = 0;
            D.resid[out_base + tid] = -1.0;
            D.converged[out_base + tid] = 0;
        }
        return;
    }
    auto vec = [&](float* base, int k, int row) -> float* { return base + (static_cast<long long>(k) * ws + row) * G + g; };
    if (tid < G) {
        S2.acc[tid] = 0.0;
        S2.its[tid] = 0;
        S2.conv[tid] = 0;
        S2.alive[tid] = tid < ng ? 1 : 0;
    }
    __syncthreads();
    double bb = 0.0;
    for (int i = rl; i < n; i += RT) {
        x[static_cast<long long>(i) * G + g] = 0.0;
        bb = fma(b[i], b[i], bb);
    }
    group_sum<G>(bb, S2.acc);
    if (tid < G) S2.tol[tid] = D.rtol * sqrt(S2.acc[tid]);
    while (true) {
        // FP64 residuals r_g = b_g - A x_g
        if (tid < G) S2.acc[tid] = 0.0;
        __syncthreads();
        double ss = 0.0;
        for (int i = rl; i < n; i += RT) {
            double acc = 0.0;
            for (int p = S.rp[i]; p < S.rp[i + 1]; ++p) acc = fma(S.a64[p], x[static_cast<long long>(S.ci[p]) * G + g], acc);
            const double ri = b[i] - acc;
            rw[static_cast<long long>(i) * G + g] = ri;
            ss = fma(ri, ri, ss);
        }
        group_sum<G>(ss, S2.acc);
        if (tid < G) {
            const double beta = sqrt(S2.acc[tid]);
            S2.beta[tid] = beta;
            if (S2.alive[tid]) {
                if (beta <= S2.tol[tid]) {
                    S2.conv[tid] = 1;
                    S2.alive[tid] = 0;
                } else if (S2.its[tid] >= D.maxit || isnan(beta)) {
                    S2.alive[tid] = 0;
                }
            }
            S2.cyc[tid] = S2.alive[tid];
            S2.last[tid] = -1;
            S2.stop[tid] = fmax(S2.tol[tid], D.tau * beta);
            S2.rs[(tid) * S2.ld + 0] = beta;
        }
        __syncthreads();
        if (tid == 0) {
            int a = 0;
            for (int q = 0; q < G; ++q) a |= S2.cyc[q];
            *S2.any = a;
        }
        __syncthreads();
        if (!*S2.any) break;
        {
            const double inv = S2.cyc[g] ? 1.0 / S2.beta[g] : 0.0;
            for (int i = rl; i < n; i += RT) *vec(V, 0, i) = static_cast<float>(rw[static_cast<long long>(i) * G + g] * inv);
        }
        __syncthreads();
        for (int i = 0; i < m; ++i) {
            if (tid < G && S2.cyc[tid]) ++S2.its[tid];
            // z = L^{-1} v (ascending entries), level by level
            for (int l = 0; l < S.nlevL; ++l) {
                for (int q = S.lptrL[l] + rl; q < S.lptrL[l + 1]; q += RT) {
                    const int row = S.ordL[q];
                    float t = *vec(V, i, row);
                    for (int p = S.rp[row]; p < S.diag[row]; ++p) t = fmaf(-S.lu32[p], *vec(Z, i, S.ci[p]), t);
                    *vec(Z, i, row) = t;
                }
                __syncthreads();
            }
            // z = U^{-1} z (descending entries), in place, level by level
            for (int l = 0; l < S.nlevU; ++l) {
                for (int q = S.lptrU[l] + rl; q < S.lptrU[l + 1]; q += RT) {
                    const int row = S.ordU[q];
                    float t = *vec(Z, i, row);
                    for (int p = S.rp[row + 1] - 1; p > S.diag[row]; --p) t = fmaf(-S.lu32[p], *vec(Z, i, S.ci[p]), t);
                    *vec(Z, i, row) = t * S.dinv[row];
                }
                __syncthreads();
            }
            // w = A z (FP32)
            for (int k = rl; k < n; k += RT) {
                float acc = 0.f;
                for (int p = S.rp[k]; p < S.rp[k + 1]; ++p) acc = fmaf(S.a32[p], *vec(Z, i, S.ci[p]), acc);
                *vec(V, i + 1, k) = acc;
            }
            // CGS2: two projections, per-warp partial sums in FP32, combined in FP64
            for (int pass = 0; pass < 2; ++pass) {
                for (int q = tid; q < (i + 1) * G; q += T) S2.acc[q] = 0.0;
                __syncthreads();
                for (int j = 0; j <= i; ++j) {
                    float part = 0.f;
                    for (int k = rl; k < n; k += RT) part = fmaf(*vec(V, j, k), *vec(V, i + 1, k), part);
                    part = warp_sum_g<G>(part);
                    if ((tid & 31) < G) atomicAdd(S2.acc + j * G + (tid & 31), static_cast<double>(part));
                }
                __syncthreads();
                for (int q = tid; q < (i + 1) * G; q += T) {
                    const int j = q / G, gg = q % G;
                    const double t = S2.acc[q];
                    if (pass == 0) {
                        S2.hc[(gg) * S2.ld + j] = t;
                    } else {
                        S2.hc[(gg) * S2.ld + j] += t;
                    }
                    S2.cf[(gg) * S2.ld + j] = static_cast<float>(t);  // this pass's coefficients
                }
                __syncthreads();
                for (int k = rl; k < n; k += RT) {
                    float a = *vec(V, i + 1, k);
                    for (int j = 0; j <= i; ++j) a = fmaf(-S2.cf[(g) * S2.ld + j], *vec(V, j, k), a);
                    *vec(V, i + 1, k) = a;
                }
                __syncthreads();
            }
            if (tid < G) S2.acc[tid] = 0.0;
            __syncthreads();
            {
                float nn = 0.f;
                for (int k = rl; k < n; k += RT) {
                    const float wv = *vec(V, i + 1, k);
                    nn = fmaf(wv, wv, nn);
                }
                group_sum<G>(static_cast<double>(nn), S2.acc);
            }
            if (tid < G && S2.cyc[tid]) {
                // Givens update of column i of right-hand side tid (src/gmres.cpp:238-256)
                const int q = tid;
                double* H = D.H + (static_cast<long long>(blockIdx.x) * G + q) * (kBatchMaxM + 1) * m;
                const double hnext = sqrt(S2.acc[q]);
                double* hc = S2.hc + q * S2.ld;
                double* cs = S2.cs + q * S2.ld;
                double* sn = S2.sn + q * S2.ld;
                double* rs = S2.rs + q * S2.ld;
                double prev = hc[0];
                for (int k = 1; k <= i; ++k) {
                    const double cur = hc[k];
                    hc[k - 1] = cs[k - 1] * prev + sn[k - 1] * cur;
                    prev = -sn[k - 1] * prev + cs[k - 1] * cur;
                }
                if (i >= 1) hc[i] = prev;
                double gam = sqrt(hc[i] * hc[i] + hnext * hnext);
                if (gam == 0.0) gam = 1e-16;
                cs[i] = hc[i] / gam;
                sn[i] = hnext / gam;
                rs[i + 1] = -sn[i] * rs[i];
                rs[i] = cs[i] * rs[i];
                hc[i] = cs[i] * hc[i] + sn[i] * hnext;
                for (int j = 0; j <= i; ++j) H[static_cast<long long>(i) * (kBatchMaxM + 1) + j] = hc[j];
                const double est = fabs(rs[i + 1]);
                S2.last[q] = i;
                S2.hnext[q] = hnext;
                if (hnext <= 1e-16 || est <= S2.stop[q] || isnan(est) || S2.its[q] >= D.maxit) S2.cyc[q] = 0;
            } else if (tid < G) {
                S2.hnext[tid] = 0.0;
            }
            __syncthreads();
            {
                const double hn = S2.hnext[g];
                if (hn > 1e-16) {
                    const float invn = static_cast<float>(1.0 / hn);
                    for (int k = rl; k < n; k += RT) *vec(V, i + 1, k) *= invn;
                }
            }
            if (tid == 0) {
                int a = 0;
                for (int q = 0; q < G; ++q) a |= S2.cyc[q];
                *S2.any = a;
            }
            __syncthreads();
            if (!*S2.any) break;
        }
        // least squares per right-hand side: rs[0..last] <- H^{-1} rs, then x += Z y (FP64)
        if (tid < G && S2.last[tid] >= 0) {
            const int q = tid;
            const int last = S2.last[q];
            const double* H = D.H + (static_cast<long long>(blockIdx.x) * G + q) * (kBatchMaxM + 1) * m;
            double* rs = S2.rs + q * S2.ld;
            rs[last] = rs[last] / H[static_cast<long long>(last) * (kBatchMaxM + 1) + last];
            for (int ii = last - 1; ii >= 0; --ii) {
                double t = rs[ii];
                for (int j = ii + 1; j <= last; ++j) t -= H[static_cast<long long>(j) * (kBatchMaxM + 1) + ii] * rs[j];
                rs[ii] = t / H[static_cast<long long>(ii) * (kBatchMaxM + 1) + ii];
            }
            for (int j = 0; j <= last; ++j) S2.cf[(q) * S2.ld + j] = static_cast<float>(rs[j]);
        }
        __syncthreads();
        {
            const int last = S2.last[g];
            for (int k = rl; k < n; k += RT) {
                float d = 0.f;
                for (int j = 0; j <= last; ++j) d = fmaf(S2.cf[(g) * S2.ld + j], *vec(Z, j, k), d);
                x[static_cast<long long>(k) * G + g] += static_cast<double>(d);
            }
        }
        __syncthreads();
    }
    if (g < ng)
        for (int k = rl; k < n; k += RT) D.x[io + k] = x[static_cast<long long>(k) * G + g];
    if (tid < ng) {
        D.iters[out_base + tid] = S2.its[tid];
        D.resid[out_base + tid] = S2.beta[tid];
        D.converged[out_base + tid] = S2.conv[tid];
    }
    __syncthreads();
}

}  // namespace

// Two CTAs per SM (64 registers per thread): the autotuner's two-CTA shapes must really
// be resident, and the solve items are latency-bound, so two per SM beat one.  G: right-
// hand sides per solve item.
template <int G>
__global__ void __launch_bounds__(kBatchThreads, 2) batched_ilu_gmres_kernel(BatchDesc D, int nsys_run) {
    __shared__ double red[kBatchWarps];
    __shared__ float P[kMlpParams];
    __shared__ int s_ticket;
    extern __shared__ __align__(16) unsigned char group_dyn[];
    const GroupSmem S2 = group_smem(group_dyn, D.m, G);
    const int groups = (D.nrhs + G - 1) / G;
    const int njobs = nsys_run + nsys_run * groups;
    for (int job = draw_block_ticket(D.ticket, njobs, &s_ticket); job < njobs;
         job = draw_block_ticket(D.ticket, njobs, &s_ticket)) {
        if (job < nsys_run) {
            factor_system(D, D.sys_of_slot[job], red, P);
        } else {
            const int k = job - nsys_run;
            solve_group<G>(D, D.sys_of_slot[k / groups], (k % groups) * G, S2);
        }
    }
}

// ---------------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------------
BatchSolver::BatchSolver(int nsys, const int* n, const int* rp_all, const int* ci_all, const double* val_all, int nrhs,
                         int restart, double rtol, int maxit, const double* fval_all)
    : nsys_(nsys), nrhs_(nrhs), m_(restart), rtol_(rtol), maxit_(maxit) {
    if (restart < 1 || restart > kBatchMaxM) throw std::runtime_error("batched restart must be in [1, 64]");
    if (nsys < 1 || nrhs < 1) throw std::runtime_error("batched solve needs systems and right-hand sides");
    // structural check of every system (row pointers local to the system, columns in
    // [0, n[s]), strictly ascending) before any device work
    {
        long long rpp = 0, srcp = 0;
        std::vector<int> rpl;
        for (int s = 0; s < nsys; ++s) {
            const int ns = n[s];
            const std::string what = "batched system " + std::to_string(s);
            if (ns < 0) throw std::runtime_error("invalid CSR matrix (" + what + "): negative size");
            const int* rp = rp_all + rpp;
            for (int i = 0; i < ns; ++i)
                if (rp[i + 1] < rp[i])
                    throw std::runtime_error("invalid CSR matrix (" + what + "): row_ptr decreases at row " +
                                             std::to_string(i));
            rpl.resize(static_cast<size_t>(ns) + 1);
            for (int i = 0; i <= ns; ++i) rpl[static_cast<size_t>(i)] = rp[i] - rp[0];
            validate_csr(ns, rpl.data(), ci_all + srcp, what.c_str());
            rpp += ns + 1;
            srcp += rpl[static_cast<size_t>(ns)];
        }
    }
    dev_ = current_device();
    GB_CUDA_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    GB_CUDA_CHECK(cudaEventCreate(&ev0_));
    GB_CUDA_CHECK(cudaEventCreate(&ev1_));
    // Per-system slices of the concatenated arrays start on 32-entry boundaries: arrays
    // written inside the kernel (factors, reciprocal diagonal) then never share a
    // 128-byte line between two systems, so no SM can hold a stale copy of another
    // system's freshly written factors in its L1.
    auto pad32 = [](long long v) { return (v + 31) / 32 * 32; };
    std::vector<long long> rp_off(nsys), nnz_off(nsys), row_off(nsys), lvl_off(nsys), rhs_off(nsys);
    std::vector<int> nlevL(nsys), nlevU(nsys), lptrL_all, lptrU_all;
    long long rp_pos = 0, nnz_pos = 0, row_pos = 0, lvl_pos = 0, rhs_pos = 0, src_nnz = 0;
    n_.assign(n, n + nsys);
    for (int s = 0; s < nsys; ++s) {
        rp_off[s] = rp_pos;
        nnz_off[s] = nnz_pos;
        row_off[s] = row_pos;
        const int ns = n[s];
        const long long nz = rp_all[rp_pos + ns] - rp_all[rp_pos];
        rp_pos += ns + 1;
        nnz_pos = pad32(nnz_pos + nz);
        row_pos = pad32(row_pos + ns);
        src_nnz += nz;
    }
    std::vector<int> ci_pad(static_cast<size_t>(std::max<long long>(nnz_pos, 1)), 0);
    std::vector<double> val_pad(static_cast<size_t>(std::max<long long>(nnz_pos, 1)), 0.0);
    std::vector<double> fval_pad(fval_all ? val_pad.size() : 0, 0.0);
    std::vector<int> diag_all(static_cast<size_t>(std::max<long long>(row_pos, 1)), 0);
    std::vector<int> ordL_all(diag_all.size(), 0), ordU_all(diag_all.size(), 0), depth_all(diag_all.size(), 0);
    std::vector<int> rp_local(static_cast<size_t>(rp_pos));
    long long src = 0;
    for (int s = 0; s < nsys; ++s) {
        const int ns = n[s];
        const int* rp = rp_all + rp_off[s];
        const long long base = rp[0];
        const long long nz = rp[ns] - base;
        for (int i = 0; i <= ns; ++i) rp_local[rp_off[s] + i] = static_cast<int>(rp[i] - base);
        std::copy(ci_all + src, ci_all + src + nz, ci_pad.begin() + nnz_off[s]);
        std::copy(val_all + src, val_all + src + nz, val_pad.begin() + nnz_off[s]);
        if (fval_all) std::copy(fval_all + src, fval_all + src + nz, fval_pad.begin() + nnz_off[s]);
        const int* rpl = rp_local.data() + rp_off[s];
        const int* ci = ci_all + src;
        std::vector<int> diag, depthL, depthU, ordL, ordU, lpL, lpU;
        diagonal_pointers(ns, rpl, ci, diag);
        nlevL[s] = level_sets(ns, DagView{rpl, ci, diag.data(), true}, depthL, ordL, lpL);
        nlevU[s] = level_sets(ns, DagView{rpl, ci, diag.data(), false}, depthU, ordU, lpU);
        const int nl = std::max(nlevL[s], nlevU[s]);
        lpL.resize(static_cast<size_t>(nl) + 1, lpL.back());
        lpU.resize(static_cast<size_t>(nl) + 1, lpU.back());
        std::copy(diag.begin(), diag.end(), diag_all.begin() + row_off[s]);
        std::copy(ordL.begin(), ordL.end(), ordL_all.begin() + row_off[s]);
        std::copy(ordU.begin(), ordU.end(), ordU_all.begin() + row_off[s]);
        std::copy(depthL.begin(), depthL.end(), depth_all.begin() + row_off[s]);
        lvl_off[s] = lvl_pos;
        lptrL_all.insert(lptrL_all.end(), lpL.begin(), lpL.end());
        lptrU_all.insert(lptrU_all.end(), lpU.begin(), lpU.end());
        lvl_pos += nl + 1;
        rhs_off[s] = rhs_pos;
        rhs_pos += static_cast<long long>(nrhs) * ns;
        nmax_ = std::max(nmax_, ns);
        src += nz;
    }
    (void)src_nnz;
    total_rows_ = row_pos;
    total_rhs_ = rhs_pos;
    cudaStream_t st = stream_;
    d_n_.upload(n, nsys, st);
    d_rp_off_.upload(rp_off.data(), nsys, st);
    d_nnz_off_.upload(nnz_off.data(), nsys, st);
    d_row_off_.upload(row_off.data(), nsys, st);
    d_lvl_off_.upload(lvl_off.data(), nsys, st);
    d_rhs_off_.upload(rhs_off.data(), nsys, st);
    d_nlevL_.upload(nlevL.data(), nsys, st);
    d_nlevU_.upload(nlevU.data(), nsys, st);
    d_rp_.upload(rp_local.data(), rp_local.size(), st);
    d_ci_.upload(ci_pad.data(), ci_pad.size(), st);
    d_a64_.upload(val_pad.data(), val_pad.size(), st);
    if (fval_all) d_f64_.upload(fval_pad.data(), fval_pad.size(), st);
    d_a32_.reserve(static_cast<size_t>(std::max<long long>(nnz_pos, 1)));
    d_lu64_.reserve(static_cast<size_t>(std::max<long long>(nnz_pos, 1)));
    d_lu32_.reserve(static_cast<size_t>(std::max<long long>(nnz_pos, 1)));
    d_diag_.upload(diag_all.data(), diag_all.size(), st);
    d_ordL_.upload(ordL_all.data(), ordL_all.size(), st);
    d_ordU_.upload(ordU_all.data(), ordU_all.size(), st);
    d_lptrL_.upload(lptrL_all.data(), lptrL_all.size(), st);
    d_lptrU_.upload(lptrU_all.data(), lptrU_all.size(), st);
    d_depth_.upload(depth_all.data(), depth_all.size(), st);
    d_dinv_.reserve(static_cast<size_t>(std::max<long long>(row_pos, 1)));
    d_rhs_.reserve(static_cast<size_t>(std::max<long long>(rhs_pos, 1)));
    d_x_.reserve(static_cast<size_t>(std::max<long long>(rhs_pos, 1)));
    const size_t njobs = static_cast<size_t>(nsys) * nrhs;
    d_iters_.reserve(njobs);
    d_resid_.reserve(njobs);
    d_conv_.reserve(njobs);
    d_shifted_.reserve(static_cast<size_t>(nsys));
    d_ready_.reserve(static_cast<size_t>(nsys));
    GB_CUDA_CHECK(cudaMemsetAsync(d_ready_.get(), 0, sizeof(int) * nsys, st));
    d_ticket_.reserve(1);
    GB_CUDA_CHECK(cudaMemsetAsync(d_ticket_.get(), 0, sizeof(unsigned), st));
    d_status_.reserve(kStatusWords);
    GB_CUDA_CHECK(cudaMemsetAsync(d_status_.get(), 0, sizeof(int) * kStatusWords, st));
    ws_ = std::max<long long>(256, ceil_div<long long>(nmax_, 256) * 256);
    order_.resize(nsys);
    std::iota(order_.begin(), order_.end(), 0);
    GB_CUDA_CHECK(cudaStreamSynchronize(st));
}

BatchSolver::~BatchSolver() {
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
}

void BatchSolver::set_model(const float* params, float min_shift) {
    if (!params) {
        model_ = false;
        return;
    }
    d_mlp_.upload(params, kMlpParams, stream_);
    GB_CUDA_CHECK(cudaStreamSynchronize(stream_));
    min_shift_ = min_shift;
    model_ = true;
}

void BatchSolver::ensure_workspace(int grid, int G) {
    const size_t vec = static_cast<size_t>(ws_) * G;
    d_V_.reserve(static_cast<size_t>(grid) * (m_ + 1) * vec);
    d_Z_.reserve(static_cast<size_t>(grid) * m_ * vec);
    d_xw_.reserve(static_cast<size_t>(grid) * vec);
    d_rw_.reserve(static_cast<size_t>(grid) * vec);
    d_H_.reserve(static_cast<size_t>(grid) * G * (kBatchMaxM + 1) * m_);
}

size_t BatchSolver::workspace_bytes(int grid, int G) const {
    const size_t vec = static_cast<size_t>(ws_) * G;
    return static_cast<size_t>(grid) * (sizeof(float) * (2 * m_ + 1) * vec + sizeof(double) * 2 * vec +
                                        sizeof(double) * G * (kBatchMaxM + 1) * m_);
}

// Right-hand sides for the autotuner's trials, b = A x with x deterministic in [-1, 1)
// (a hash of system, right-hand side and row), like the callers' b = A x_true: the
// trials need systems that iterate like real ones, and the caller's right-hand sides
// arrive only with solve().  One CTA per system.
__device__ __forceinline__ double trial_x(long long key) {
    unsigned long long h = static_cast<unsigned long long>(key) * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    return static_cast<double>(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void batch_trial_rhs_kernel(BatchDesc D, int nsys_run) {
    for (int q = blockIdx.x; q < nsys_run; q += gridDim.x) {
        const int s = D.sys_of_slot[q];
        const int n = D.n[s];
        const int* rp = D.rp + D.rp_off[s];
        const int* ci = D.ci + D.nnz_off[s];
        const double* a = D.a64 + D.nnz_off[s];
        for (int r = 0; r < D.nrhs; ++r) {
            double* b = const_cast<double*>(D.rhs) + D.rhs_off[s] + static_cast<long long>(r) * n;
            const long long key = (static_cast<long long>(s) * D.nrhs + r) << 32;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double acc = 0.0;
                for (int p = rp[i]; p < rp[i + 1]; ++p) acc = fma(a[p], trial_x(key + ci[p]), acc);
                b[i] = acc;
            }
        }
    }
}

template <int G>
static void launch_batched(int grid, const BatchDesc& D, int nsys_run, int m, cudaStream_t s) {
    const size_t smem = group_smem_bytes(m, G);
    GB_CUDA_CHECK(cudaFuncSetAttribute(batched_ilu_gmres_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
    batched_ilu_gmres_kernel<G><<<grid, kBatchThreads, smem, s>>>(D, nsys_run);
}

float BatchSolver::launch(int ctas_per_sm, bool largest_first, int nsys_run, int G) {
    const int grid = std::max(1, ctas_per_sm) * dev_.sms;
    ensure_workspace(grid, G);
    // the first nsys_run systems (input order), processed largest first or in input order
    order_.resize(nsys_run);
    std::iota(order_.begin(), order_.end(), 0);
    if (largest_first)
        std::stable_sort(order_.begin(), order_.end(), [&](int a, int b) { return n_[a] > n_[b]; });
    d_order_.upload(order_.data(), order_.size(), stream_);
    BatchDesc D;
    D.nsys = nsys_;
    D.nrhs = nrhs_;
    D.m = m_;
    D.maxit = maxit_;
    D.rtol = rtol_;
    D.tau = tau_;
    D.n = d_n_.get();
    D.rp_off = d_rp_off_.get();
    D.nnz_off = d_nnz_off_.get();
    D.row_off = d_row_off_.get();
    D.lvl_off = d_lvl_off_.get();
    D.nlevL = d_nlevL_.get();
    D.nlevU = d_nlevU_.get();
    D.rhs_off = d_rhs_off_.get();
    D.sys_of_slot = d_order_.get();
    D.rp = d_rp_.get();
    D.ci = d_ci_.get();
    D.a64 = d_a64_.get();
    D.f64 = d_f64_.size() ? d_f64_.get() : nullptr;
    D.a32 = d_a32_.get();
    D.lu64 = d_lu64_.get();
    D.lu32 = d_lu32_.get();
    D.diag = d_diag_.get();
    D.ordL = d_ordL_.get();
    D.ordU = d_ordU_.get();
    D.lptrL = d_lptrL_.get();
    D.lptrU = d_lptrU_.get();
    D.depth = d_depth_.get();
    D.dinv = d_dinv_.get();
    D.mlp = model_ ? d_mlp_.get() : nullptr;
    D.min_shift = min_shift_;
    D.rhs = d_rhs_.get();
    D.x = d_x_.get();
    D.iters = d_iters_.get();
    D.resid = d_resid_.get();
    D.converged = d_conv_.get();
    D.shifted = d_shifted_.get();
    D.ready = d_ready_.get();
    D.epoch = ++epoch_;
    D.ticket = d_ticket_.get();
    D.status = d_status_.get();
    D.V = d_V_.get();
    D.Z = d_Z_.get();
    D.xw = d_xw_.get();
    D.rw = d_rw_.get();
    D.H = d_H_.get();
    D.ws = ws_;
    if (trial_) {
        batch_trial_rhs_kernel<<<2 * dev_.sms, 256, 0, stream_>>>(D, nsys_run);
        GB_CUDA_CHECK(cudaGetLastError());
    }
    GB_CUDA_CHECK(cudaEventRecord(ev0_, stream_));
    switch (G) {
        case 1: launch_batched<1>(grid, D, nsys_run, m_, stream_); break;
        case 4: launch_batched<4>(grid, D, nsys_run, m_, stream_); break;
        case 16: launch_batched<16>(grid, D, nsys_run, m_, stream_); break;
        default: throw std::runtime_error("batched: right-hand sides per item must be 1, 4 or 16");
    }
    GB_CUDA_CHECK(cudaGetLastError());
    GB_CUDA_CHECK(cudaEventRecord(ev1_, stream_));
    GB_CUDA_CHECK(cudaEventSynchronize(ev1_));
    float ms = 0.f;
    GB_CUDA_CHECK(cudaEventElapsedTime(&ms, ev0_, ev1_));
    ++launches_;
    int h[kStatusWords];
    GB_CUDA_CHECK(cudaMemcpy(h, d_status_.get(), sizeof(h), cudaMemcpyDeviceToHost));
    if (h[kStatusTimeout] != 0) {
        GB_CUDA_CHECK(cudaMemset(d_status_.get(), 0, sizeof(int) * kStatusWords));
        throw std::runtime_error("batched solve: a factorisation wait timed out on the device");
    }
    return ms;
}

void BatchSolver::autotune() {
    // Launch shapes tried on the same sample (the first systems of the batch, largest
    // first): right-hand sides per CTA (G = 1, 4, 16: rows per CTA round T / G) x CTAs per
    // SM.  The fastest wins; every trial is kept (trials()).
    const int sample = std::min(nsys_, 2 * dev_.sms);
    float best = 1e30f;
    tuned_.clear();
    trial_ = true;  // right-hand sides b = A x of its own (below), iterations capped
    const int maxit = maxit_;
    maxit_ = std::min(maxit_, kBatchTrialIterations);
    for (int G : {1, 4, 16}) {
        if (G > 1 && G / 4 >= nrhs_) continue;  // no wider than the right-hand sides need
        for (int cps : {1, 2}) {
            if (workspace_bytes(cps * dev_.sms, G) > kBatchWorkspaceCap) continue;
            float ms = 0.f;
            try {
                ms = launch(cps, true, sample, G);
            } catch (...) {
                maxit_ = maxit;
                trial_ = false;
                throw;
            }
            tuned_.push_back({cps, 1, G, ms});
            if (ms < best) {
                best = ms;
                ctas_per_sm_ = cps;
                largest_first_ = true;
                rhs_per_cta_ = G;
            }
        }
    }
    maxit_ = maxit;
    trial_ = false;
}

void BatchSolver::set_shape(int ctas_per_sm, bool largest_first, int rhs_per_cta) {
    if (ctas_per_sm < 1 || ctas_per_sm > 2) throw std::runtime_error("batched: CTAs per SM must be 1 or 2");
    if (rhs_per_cta != 1 && rhs_per_cta != 4 && rhs_per_cta != 16)
        throw std::runtime_error("batched: right-hand sides per item must be 1, 4 or 16");
    ctas_per_sm_ = ctas_per_sm;
    largest_first_ = largest_first;
    rhs_per_cta_ = rhs_per_cta;
}

float BatchSolver::solve(const double* rhs_host, double* x_host, int* iters, double* resid, int* converged) {
    GB_CUDA_CHECK(cudaMemcpyAsync(d_rhs_.get(), rhs_host, sizeof(double) * static_cast<size_t>(total_rhs_),
                                  cudaMemcpyHostToDevice, stream_));
    const float ms = launch(ctas_per_sm_, largest_first_, nsys_, rhs_per_cta_);
    if (x_host)
        GB_CUDA_CHECK(cudaMemcpyAsync(x_host, d_x_.get(), sizeof(double) * static_cast<size_t>(total_rhs_),
                                      cudaMemcpyDeviceToHost, stream_));
    const size_t njobs = static_cast<size_t>(nsys_) * nrhs_;
    if (iters) GB_CUDA_CHECK(cudaMemcpyAsync(iters, d_iters_.get(), sizeof(int) * njobs, cudaMemcpyDeviceToHost, stream_));
    if (resid) GB_CUDA_CHECK(cudaMemcpyAsync(resid, d_resid_.get(), sizeof(double) * njobs, cudaMemcpyDeviceToHost, stream_));
    if (converged)
        GB_CUDA_CHECK(cudaMemcpyAsync(converged, d_conv_.get(), sizeof(int) * njobs, cudaMemcpyDeviceToHost, stream_));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream_));
    last_ms_ = ms;
    return ms;
}

}  // namespace gb300
