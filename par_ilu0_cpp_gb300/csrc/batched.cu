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

// Solve item (system s, right-hand side r).
__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The loops over a system's rows run in FP32 only (coefficients converted once into `cf`,
// per-thread and per-warp partial sums in FP32, warps combined in FP64): GB300's FP64
// pipe is far narrower than its FP32 one, and a conversion or FP64 add per element and
// basis vector set the pace of the Gram-Schmidt passes.
__device__ void solve_item(const BatchDesc& D, int s, int r, double* red, double* H, double* hc, double* cs,
                           double* sn, double* rs, float* cf, int* flag) {
    if (threadIdx.x == 0) *flag = wait_flag(D.ready + s, D.epoch, D.status) ? 1 : 0;
    __syncthreads();
    const SysView S = sys_view(D, s);
    const int n = S.n;
    const int m = D.m;
    const long long ws = D.ws;
    float* V = D.V + static_cast<long long>(blockIdx.x) * (m + 1) * ws;
    float* Z = D.Z + static_cast<long long>(blockIdx.x) * m * ws;
    double* x = D.xw + static_cast<long long>(blockIdx.x) * ws;
    double* rw = D.rw + static_cast<long long>(blockIdx.x) * ws;
    const long long io = D.rhs_off[s] + static_cast<long long>(r) * n;
    const double* b = D.rhs + io;
    const int tid = threadIdx.x;
    const int T = blockDim.x;
    if (!*flag) {  // the factorisation never became ready: report and skip
        if (tid == 0) {
            D.iters[s * D.nrhs + r] = 0;
            D.resid[s * D.nrhs + r] = -1.0;
            D.converged[s * D.nrhs + r] = 0;
        }
        return;
    }
    double bb = 0.0;
    for (int i = tid; i < n; i += T) {
        x[i] = 0.0;
        bb = fma(b[i], b[i], bb);
    }
    const double tol = D.rtol * sqrt(block_sum(bb, red));
    int its = 0;
    bool conv = false;
    double beta = 0.0;
    while (true) {
        // FP64 residual r = b - A x
        double ss = 0.0;
        for (int i = tid; i < n; i += T) {
            double acc = 0.0;
            for (int p = S.rp[i]; p < S.rp[i + 1]; ++p) acc = fma(S.a64[p], x[S.ci[p]], acc);
            const double ri = b[i] - acc;
            rw[i] = ri;
            ss = fma(ri, ri, ss);
        }
        beta = sqrt(block_sum(ss, red));
        if (beta <= tol) {
            conv = true;
            break;
        }
        if (its >= D.maxit || isnan(beta)) break;
        const double inv = 1.0 / beta;
        for (int i = tid; i < n; i += T) V[i] = static_cast<float>(rw[i] * inv);
        const double stop = fmax(tol, D.tau * beta);
        if (tid == 0) rs[0] = beta;
        __syncthreads();
        int i = 0;
        int last = -1;
        for (; i < m && its < D.maxit; ++i) {
            ++its;
            float* vi = V + static_cast<long long>(i) * ws;
            float* zi = Z + static_cast<long long>(i) * ws;
            float* w = V + static_cast<long long>(i + 1) * ws;
            // z = L^{-1} v (ascending entries), level by level
            for (int l = 0; l < S.nlevL; ++l) {
                for (int q = S.lptrL[l] + tid; q < S.lptrL[l + 1]; q += T) {
                    const int row = S.ordL[q];
                    float t = vi[row];
                    for (int p = S.rp[row]; p < S.diag[row]; ++p) t = fmaf(-S.lu32[p], zi[S.ci[p]], t);
                    zi[row] = t;
                }
                __syncthreads();
            }
            // z = U^{-1} z (descending entries), in place, level by level
            for (int l = 0; l < S.nlevU; ++l) {
                for (int q = S.lptrU[l] + tid; q < S.lptrU[l + 1]; q += T) {
                    const int row = S.ordU[q];
                    float t = zi[row];
                    for (int p = S.rp[row + 1] - 1; p > S.diag[row]; --p) t = fmaf(-S.lu32[p], zi[S.ci[p]], t);
                    zi[row] = t * S.dinv[row];
                }
                __syncthreads();
            }
            // w = A z (FP32)
            for (int k = tid; k < n; k += T) {
                float acc = 0.f;
                for (int p = S.rp[k]; p < S.rp[k + 1]; ++p) acc = fmaf(S.a32[p], zi[S.ci[p]], acc);
                w[k] = acc;
            }
            __syncthreads();
            // CGS2: two projections, dot products accumulated in FP64
            for (int pass = 0; pass < 2; ++pass) {
                for (int j = 0; j <= i; ++j) {
                    const float* vj = V + static_cast<long long>(j) * ws;
                    float part = 0.f;
                    for (int k = tid; k < n; k += T) part = fmaf(vj[k], w[k], part);
                    const float wsum = warp_sum_f32(part);
                    if ((tid & 31) == 0) red[(tid >> 5) * (kBatchMaxM + 1) + j] = static_cast<double>(wsum);
                }
                __syncthreads();
                for (int j = tid; j <= i; j += T) {
                    double t = 0.0;
                    for (int k = 0; k < kBatchWarps; ++k) t += red[k * (kBatchMaxM + 1) + j];
                    if (pass == 0) {
                        hc[j] = t;
                    } else {
                        hc[j] += t;
                    }
                    cf[j] = static_cast<float>(t);  // this pass's coefficients
                }
                __syncthreads();
                for (int k = tid; k < n; k += T) {
                    float a = w[k];
                    for (int j = 0; j <= i; ++j) a = fmaf(-cf[j], V[static_cast<long long>(j) * ws + k], a);
                    w[k] = a;
                }
                __syncthreads();
            }
            float nn = 0.f;
            for (int k = tid; k < n; k += T) nn = fmaf(w[k], w[k], nn);
            const double hnext = sqrt(block_sum(static_cast<double>(nn), red));
            if (tid == 0) {
                // Givens update of column i (src/gmres.cpp:238-256)
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
                for (int j = 0; j <= i; ++j) H[i * (kBatchMaxM + 1) + j] = hc[j];
                const double est = fabs(rs[i + 1]);
                flag[0] = (hnext <= 1e-16 || est <= stop || isnan(est)) ? 1 : 0;
            }
            __syncthreads();
            const bool done = flag[0] != 0;
            if (hnext > 1e-16) {
                const float invn = static_cast<float>(1.0 / hnext);
                for (int k = tid; k < n; k += T) w[k] *= invn;
            }
            last = i;
            __syncthreads();
            if (done) break;
        }
        if (last < 0) break;
        // least squares: rs[0..last] <- H^{-1} rs, then x += Z y in FP64
        if (tid == 0) {
            rs[last] = rs[last] / H[last * (kBatchMaxM + 1) + last];
            for (int ii = last - 1; ii >= 0; --ii) {
                double t = rs[ii];
                for (int j = ii + 1; j <= last; ++j) t -= H[j * (kBatchMaxM + 1) + ii] * rs[j];
                rs[ii] = t / H[ii * (kBatchMaxM + 1) + ii];
            }
            for (int j = 0; j <= last; ++j) cf[j] = static_cast<float>(rs[j]);
        }
        __syncthreads();
        for (int k = tid; k < n; k += T) {
            float d = 0.f;
            for (int j = 0; j <= last; ++j) d = fmaf(cf[j], Z[static_cast<long long>(j) * ws + k], d);
            x[k] += static_cast<double>(d);
        }
        __syncthreads();
    }
    for (int k = tid; k < n; k += T) D.x[io + k] = x[k];
    if (tid == 0) {
        D.iters[s * D.nrhs + r] = its;
        D.resid[s * D.nrhs + r] = beta;
        D.converged[s * D.nrhs + r] = conv ? 1 : 0;
    }
    __syncthreads();
}

}  // namespace

// Two CTAs per SM (64 registers per thread): the autotuner's two-CTA shape must really
// be resident, and the solve items are latency-bound, so two per SM beat one.
__global__ void __launch_bounds__(kBatchThreads, 2) batched_ilu_gmres_kernel(BatchDesc D, int nsys_run) {
    __shared__ double red[kBatchWarps * (kBatchMaxM + 1)];
    __shared__ double H[(kBatchMaxM + 1) * kBatchMaxM];
    __shared__ double hc[kBatchMaxM + 2];
    __shared__ double cs[2 * kBatchMaxM + 2];
    __shared__ double sn[kBatchMaxM + 1];
    __shared__ double rs[kBatchMaxM + 2];
    __shared__ float cf[kBatchMaxM + 2];
    __shared__ float P[kMlpParams];
    __shared__ int flag[2];
    __shared__ int s_ticket;
    const int njobs = nsys_run + nsys_run * D.nrhs;
    for (int job = draw_block_ticket(D.ticket, njobs, &s_ticket); job < njobs;
         job = draw_block_ticket(D.ticket, njobs, &s_ticket)) {
        if (job < nsys_run) {
            factor_system(D, D.sys_of_slot[job], red, P);
        } else {
            const int k = job - nsys_run;
            solve_item(D, D.sys_of_slot[k / D.nrhs], k % D.nrhs, red, H, hc, cs, sn, rs, cf, flag);
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

void BatchSolver::ensure_workspace(int grid) {
    const size_t vec = static_cast<size_t>(ws_);
    d_V_.reserve(static_cast<size_t>(grid) * (m_ + 1) * vec);
    d_Z_.reserve(static_cast<size_t>(grid) * m_ * vec);
    d_xw_.reserve(static_cast<size_t>(grid) * vec);
    d_rw_.reserve(static_cast<size_t>(grid) * vec);
}

float BatchSolver::launch(int ctas_per_sm, bool largest_first, int nsys_run) {
    const int grid = std::max(1, ctas_per_sm) * dev_.sms;
    ensure_workspace(grid);
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
    D.ws = ws_;
    GB_CUDA_CHECK(cudaEventRecord(ev0_, stream_));
    batched_ilu_gmres_kernel<<<grid, kBatchThreads, 0, stream_>>>(D, nsys_run);
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
    // Launch shapes tried on the same sample (the first systems of the batch): CTAs per
    // SM x system order (largest first / input order).  The fastest wins.
    const int sample = std::min(nsys_, 2 * dev_.sms);
    float best = 1e30f;
    for (int cps : {1, 2}) {
        for (bool lf : {true, false}) {
            const float ms = launch(cps, lf, sample);
            tuned_.push_back({cps, lf ? 1 : 0, ms});
            if (ms < best) {
                best = ms;
                ctas_per_sm_ = cps;
                largest_first_ = lf;
            }
        }
    }
}

float BatchSolver::solve(const double* rhs_host, double* x_host, int* iters, double* resid, int* converged) {
    GB_CUDA_CHECK(cudaMemcpyAsync(d_rhs_.get(), rhs_host, sizeof(double) * static_cast<size_t>(total_rhs_),
                                  cudaMemcpyHostToDevice, stream_));
    const float ms = launch(ctas_per_sm_, largest_first_, nsys_);
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
