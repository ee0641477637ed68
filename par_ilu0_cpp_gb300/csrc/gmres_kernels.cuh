// Restarted right-preconditioned GMRES(m) on the device: CSR SpMV, the fused CGS2
// Arnoldi step, Givens / Hessenberg least squares and the solution update.
//
// The control flow of the reference's Solve (src/gmres.cpp:138-288) is kept on the
// device in a GmresCtl record so that a whole restart cycle can be launched as one CUDA
// graph: the last block of the cycle-start and of each Arnoldi-step kernel evaluates the
// reference's loop conditions with a single thread and opens the gate of the next step
// (or closes the cycle); later kernels of the graph check the gate and return at once.
//
// Vector layout: Krylov bases V[0..m] and Z[0..m-1] are column blocks of one allocation
// with leading dimension ld = n rounded up to 512 entries; the padding entries of V are
// zero and never written with anything else, so whole chunks can be processed without
// bounds checks.  Basis type T is double (plain path) or float (mixed-precision inner
// cycles).  Norms accumulate in double from the first product.  Dot products (the
// Gram-Schmidt coefficients) accumulate in double for FP64 bases; for FP32 bases a warp
// sums its chunks' products in float (128 rows per chunk, a few chunks per warp) and
// those sums are added in double across warps and blocks.  The Hessenberg matrix,
// rotations and least-squares solution are double.
#pragma once

#include "common.cuh"
#include "ilu_kernels.cuh"

namespace gb300 {

constexpr int kMaxKrylov = 128;       // largest supported restart length m
constexpr int kBlasWarps = 16;        // warps per block of the vector kernels
constexpr int kBlasThreads = kBlasWarps * kWarp;
constexpr int kSpmvWarps = 4;
constexpr int kPartialStride = kMaxKrylov + 8;  // doubles per block in the partial buffers

enum CtlStatus { kCtlRunning = 0, kCtlConverged = 1, kCtlNan = 2 };

// Device-resident state of the reference's Solve loop.
struct GmresCtl {
    int its;          // Arnoldi steps over all restarts (reference `its`)
    int i;            // index of the current / last Arnoldi step of the cycle (`i`)
    int gate;         // = i while the inner loop continues with step i, else -1
    int status;       // CtlStatus
    int im;           // restart length m
    int maxits;       // max_iterations
    int steps;        // steps taken in the current cycle
    int happy;        // the last cycle ended with h_{i+1,i} <= 1e-16
    double tol;       // absolute tolerance (reference eps1 == tol)
    double tau;       // relative per-cycle stop (0 = none; mixed-precision inner cycles)
    double stop;      // per-cycle stop threshold max(tol, tau * beta0)
    double beta;      // residual norm (cycle start) / its estimate |rs[i+1]|
    double beta0;     // residual norm at the start of the current cycle
    double inv_norm;  // 1 / norm of the Krylov vector awaiting normalisation
};

// Hessenberg storage as in the reference (src/gmres.cpp:152-160): column-major
// hh[i * (m+1) + j] = H(j, i), followed by c[m+1], s[m+1], rs[m+1].
struct Hess {
    double* hh;
    int im1;
    __device__ double* c() const { return hh + im1 * (im1 - 1); }
    __device__ double* s() const { return c() + im1; }
    __device__ double* rs() const { return s() + im1; }
};

// ---------------------------------------------------------------------------------
// Block-level deterministic reductions through per-block partials: every block writes
// its partial sums, the last block to arrive (atomic counter) adds them up in block
// order, so results do not depend on scheduling.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Sums partial[b * kPartialStride + j] over blocks b for j < nv into out[j]; called by
// the last block only.  Warp w handles j = w, w + 32, ...; lanes stride over blocks.
__device__ __forceinline__ void reduce_partials(const double* partial, int nblocks, int nv, double* out) {
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    for (int j = w; j < nv; j += kBlasWarps) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += kWarp) s += __ldcg(partial + static_cast<size_t>(b) * kPartialStride + j);
        s = warp_sum(s);
        if (lane == 0) out[j] = s;
    }
}

// ---------------------------------------------------------------------------------
// CSR SpMV, one row per thread: each thread sums its row in column order (as CsrMatVec,
// src/csr_matrix.cpp:163-171) with the loads of up to 8 entries (columns, values, then
// the x gathers) in flight at once.  No shared memory, so 64 warps per SM stay resident;
// consecutive threads read consecutive rows, and their entry loads share cache lines.
// (A warp-per-32-row-chunk layout staged through shared memory ran at 38% of HBM peak:
// two dependent round trips per chunk and smem-limited occupancy.)
// ---------------------------------------------------------------------------------
// Row sums accumulate in the matrix's value type AT (FP64 for the plain path, FP32 for
// the mixed-precision inner cycles, whose SpMV is FP32 throughout).
template <class AT, class XT>
__device__ __forceinline__ AT spmv_row(const int* __restrict__ rp, const int* __restrict__ ci,
                                       const AT* __restrict__ av, const XT* __restrict__ x, int row) {
    const int pb = __ldg(rp + row);
    const int pe = __ldg(rp + row + 1);
    AT acc = AT(0);
#pragma unroll 8
    for (int p = pb; p < pe; ++p) acc = fma(__ldg(av + p), static_cast<AT>(__ldg(x + __ldg(ci + p))), acc);
    return acc;
}

// y = A x (gated when launched inside a cycle graph).  `reset` (optional) is set to the
// sentinel on rows [0, n): the forward-sweep vector of the preconditioner, which must hold
// the sentinel before the next forward substitution (done here, in a bandwidth-bound
// kernel, instead of inside the latency-bound backward substitution).
template <class AT, class XT, class YT>
__global__ void __launch_bounds__(kSpmvWarps * kWarp)
    spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const AT* __restrict__ av,
                const XT* __restrict__ x, YT* __restrict__ y, const int* gate, int step, YT* __restrict__ reset) {
    if (gate_closed(gate, step)) return;
    if (reset) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            reset[i] = Sentinel<YT>::value();
    }
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x)
        y[row] = static_cast<YT>(spmv_row(rp, ci, av, x, row));
}

// Cycle start: r = b - A x (FP64), v0 = r (unnormalised, type T), beta = ||r||_2, then
// the reference's restart logic (src/gmres.cpp:179-199): stop when beta <= tol,
// otherwise rs[0] = beta, i = -1 and the inner-loop condition
// (i < m-1) && (beta > eps1) && (its++ < maxits) opens step 0.
template <class T>
__global__ void __launch_bounds__(kSpmvWarps * kWarp)
    gmres_residual_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ av,
                          const double* __restrict__ b, const double* __restrict__ x, T* __restrict__ v0, GmresCtl* ctl,
                          Hess H, double* partial, unsigned* counter) {
    __shared__ double s_red[kSpmvWarps];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    double ss = 0.0;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        const double r = b[row] - spmv_row(rp, ci, av, x, row);
        v0[row] = static_cast<T>(r);
        ss = fma(r, r, ss);
    }
    ss = warp_sum(ss);
    if (lane == 0) s_red[w] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kSpmvWarps; ++k) t += s_red[k];
        partial[static_cast<size_t>(blockIdx.x) * kPartialStride] = t;
    }
    if (!arrive_last(counter)) return;
    __shared__ double s_norm;
    reduce_partials(partial, gridDim.x, 1, &s_norm);
    __syncthreads();
    if (threadIdx.x == 0) {
        const double beta = sqrt(s_norm);
        ctl->beta = beta;
        ctl->beta0 = beta;
        ctl->steps = 0;
        ctl->happy = 0;
        ctl->i = -1;
        ctl->gate = -1;
        ctl->stop = fmax(ctl->tol, ctl->tau * beta);
        if (beta <= ctl->tol) {
            ctl->status = kCtlConverged;
            return;
        }
        if (isnan(beta)) {
            ctl->status = kCtlNan;
            return;
        }
        ctl->inv_norm = 1.0 / beta;
        H.rs()[0] = beta;
        if (-1 < ctl->im - 1 && beta > ctl->stop && ctl->its++ < ctl->maxits) {
            ctl->i = 0;
            ctl->gate = 0;
        }
    }
}

// ---------------------------------------------------------------------------------
// Fused CGS2 Arnoldi step.  w = V[s+1] (the SpMV output), basis V[0..s].
//   dot1:        h1 = V^T w
//   axpy_dot:    w <- w - V h1;  h2 = V^T w
//   axpy_norm:   w <- w - V h2;  ||w||; then (last block) H(:,s) = h1 + h2,
//                H(s+1,s) = ||w||, Givens update and loop control.
// Work split: each warp owns chunks of R = 32 * RPL consecutive rows (128 FP32 / 256
// FP64), lane l the RPL contiguous rows [l RPL, (l+1) RPL) of a chunk, so every load of
// a basis vector is one fully coalesced 512 B / 2 KB access per warp.  The chunk of w
// stays in registers.  The basis is read JB vectors at a time, all loads of a batch in
// flight together; for the dots, the lane's RPL products of each vector are summed in
// registers and the JB sums are reduced across the warp together (warp_sum_batch), then
// added into a per-warp shared-memory row.  Short chunks keep the axpy_dot pass's second
// read of a warp's basis rows within L2's reach (2 KB chunks sent half of them to DRAM).
// FP32 bases keep the coefficients and the per-warp rows in FP32 (a warp adds a few
// chunk sums) and sum the rows over warps and blocks in FP64, so their per-basis-vector
// loops contain no FP64 instruction; the norm (once per step) accumulates in FP64.
// ---------------------------------------------------------------------------------
// Resident blocks per SM the Gram-Schmidt kernels are compiled for: two for FP32 (64
// registers per thread), one for FP64 (whose kernels are bound by the FP64 pipe).
template <class T>
constexpr int kBlasMinBlocks = sizeof(T) == 4 ? 2 : 1;

template <class T>
struct ChunkCfg;
// RPL: rows per lane (a chunk is 32 RPL rows, one 16-byte load per lane per 4 FP32 /
// 2 FP64 rows); JB / JBA: basis vectors loaded (and, for dots, reduced) as one batch in
// the dot pass / the passes with an axpy (smaller batches there stay clear of spills).
template <>
struct ChunkCfg<double> {
    static constexpr int RPL = 8;
    static constexpr int JB = 4;
    static constexpr int JBA = 2;
    using Acc = double;
};
template <>
struct ChunkCfg<float> {
    static constexpr int RPL = 4;
    static constexpr int JB = 8;
    static constexpr int JBA = 4;
    using Acc = float;
};

template <class T, int RPL>
__device__ __forceinline__ void load_rpl(const T* p, T (&v)[RPL]) {
    if constexpr (sizeof(T) == 4) {
        static_assert(RPL % 4 == 0, "whole float4 loads");
#pragma unroll
        for (int k = 0; k < RPL / 4; ++k) {
            const float4 t = reinterpret_cast<const float4*>(p)[k];
            v[4 * k] = t.x;
            v[4 * k + 1] = t.y;
            v[4 * k + 2] = t.z;
            v[4 * k + 3] = t.w;
        }
    } else {
        static_assert(RPL % 2 == 0, "whole double2 loads");
#pragma unroll
        for (int k = 0; k < RPL / 2; ++k) {
            const double2 t = reinterpret_cast<const double2*>(p)[k];
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    }
}
template <class T, int RPL>
__device__ __forceinline__ void store_rpl(T* p, const T (&v)[RPL]) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int k = 0; k < RPL / 4; ++k)
            reinterpret_cast<float4*>(p)[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < RPL / 2; ++k) reinterpret_cast<double2*>(p)[k] = make_double2(v[2 * k], v[2 * k + 1]);
    }
}

// Sums each of the JB per-lane values a[0..JB) over the warp (JB a power of two <= 32)
// with JB - 1 + log2(32 / JB) shuffles instead of 5 JB: each halving step keeps half of
// the values in each lane and adds the partner lane's copy of that half.  Lane l ends
// with the full sum of value batch_index<JB>(l); the lanes whose low log2(32 / JB) bits
// are zero hold distinct values.
template <int JB, class A>
__device__ __forceinline__ A warp_sum_batch(A (&a)[JB], int lane) {
#pragma unroll
    for (int h = JB / 2, o = 16; h >= 1; h >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const A send = up ? a[i] : a[i + h];
            const A keep = up ? a[i + h] : a[i];
            a[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    A v = a[0];
#pragma unroll
    for (int o = 16 / JB; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int JB>
__device__ __forceinline__ int batch_index(int lane) {
    int q = 0;
#pragma unroll
    for (int h = JB / 2, o = 16; h >= 1; h >>= 1, o >>= 1)
        if (lane & o) q += h;
    return q;
}

// Adds, for j < nv, the dot product of V[j] with the lane's chunk of w (wv, registers) to
// the warp's shared-memory row acc_row[j].  r0: the lane's first row.  The basis is read
// in batches of JB vectors (all loads of a batch in flight together) and each batch is
// reduced across the warp at once (warp_sum_batch).  The row has the accumulation type
// (FP32 for FP32 bases): the loop over the basis runs no FP64 instruction, GB300's FP64
// pipe being far narrower than its memory.
template <class T, int JB>
__device__ __forceinline__ void chunk_dots_rows(const T* __restrict__ V, long long ld, int nv, long long r0,
                                                const typename ChunkCfg<T>::Acc (&wv)[ChunkCfg<T>::RPL],
                                                typename ChunkCfg<T>::Acc* acc_row) {
    using Acc = typename ChunkCfg<T>::Acc;
    constexpr int RPL = ChunkCfg<T>::RPL;
    const int lane = threadIdx.x & 31;
    const int q = batch_index<JB>(lane);
    const bool writer = (lane & (32 / JB - 1)) == 0;
    for (int j0 = 0; j0 < nv; j0 += JB) {
        T v[JB][RPL];
#pragma unroll
        for (int b = 0; b < JB; ++b)
            if (j0 + b < nv) load_rpl<T, RPL>(V + static_cast<long long>(j0 + b) * ld + r0, v[b]);
        Acc p[JB];
#pragma unroll
        for (int b = 0; b < JB; ++b) {
            Acc t = Acc(0);
            if (j0 + b < nv) {
#pragma unroll
                for (int u = 0; u < RPL; ++u) t = fma(static_cast<Acc>(v[b][u]), wv[u], t);
            }
            p[b] = t;
        }
        const Acc tot = warp_sum_batch<JB>(p, lane);
        if (writer && j0 + q < nv) acc_row[j0 + q] += tot;
    }
}

// x -= sum_j sh[j] V[j] over the lane's rows (ascending j, the FMA order of a plain
// loop), the basis read in batches of JBA vectors.
template <class T>
__device__ __forceinline__ void chunk_axpy_rows(const T* __restrict__ V, long long ld, int nv, long long r0,
                                                const typename ChunkCfg<T>::Acc* sh,
                                                typename ChunkCfg<T>::Acc (&x)[ChunkCfg<T>::RPL]) {
    using Acc = typename ChunkCfg<T>::Acc;
    constexpr int RPL = ChunkCfg<T>::RPL;
    constexpr int JB = ChunkCfg<T>::JBA;
    for (int j0 = 0; j0 < nv; j0 += JB) {
        T v[JB][RPL];
#pragma unroll
        for (int b = 0; b < JB; ++b)
            if (j0 + b < nv) load_rpl<T, RPL>(V + static_cast<long long>(j0 + b) * ld + r0, v[b]);
#pragma unroll
        for (int b = 0; b < JB; ++b) {
            if (j0 + b < nv) {
                const Acc hj = sh[j0 + b];
#pragma unroll
                for (int u = 0; u < RPL; ++u) x[u] = fma(-hj, static_cast<Acc>(v[b][u]), x[u]);
            }
        }
    }
}

// Sums the per-warp rows acc_s[w][j] over warps, in FP64, into the block partials (all
// threads).
template <class Acc>
__device__ __forceinline__ void warp_rows_to_partial(Acc (*acc_s)[kMaxKrylov + 1], int nv, double* partial) {
    __syncthreads();
    for (int j = threadIdx.x; j < nv; j += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < kBlasWarps; ++k) s += static_cast<double>(acc_s[k][j]);
        partial[static_cast<size_t>(blockIdx.x) * kPartialStride + j] = s;
    }
}

template <class Acc>
__device__ __forceinline__ void zero_warp_rows(Acc (*acc_s)[kMaxKrylov + 1], int nv) {
    for (int e = threadIdx.x; e < kBlasWarps * (kMaxKrylov + 1); e += blockDim.x) (&acc_s[0][0])[e] = Acc(0);
    __syncthreads();
    (void)nv;
}

template <class T>
__global__ void __launch_bounds__(kBlasThreads, kBlasMinBlocks<T>)
    cgs_dot_kernel(long long nchunks, long long ld, const T* __restrict__ V, int s, double* partial, double* h1,
                   unsigned* counter, const int* gate) {
    if (gate_closed(gate, s)) return;
    using Acc = typename ChunkCfg<T>::Acc;
    constexpr int RPL = ChunkCfg<T>::RPL;
    constexpr int R = kWarp * RPL;
    __shared__ Acc acc_s[kBlasWarps][kMaxKrylov + 1];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nv = s + 1;
    zero_warp_rows(acc_s, nv);
    const T* wvec = V + static_cast<long long>(s + 1) * ld;
    for (long long c = blockIdx.x * static_cast<long long>(kBlasWarps) + w; c < nchunks;
         c += static_cast<long long>(gridDim.x) * kBlasWarps) {
        const long long r0 = c * R + lane * RPL;
        T a[RPL];
        load_rpl<T, RPL>(wvec + r0, a);
        Acc wv[RPL];
#pragma unroll
        for (int u = 0; u < RPL; ++u) wv[u] = static_cast<Acc>(a[u]);
        chunk_dots_rows<T, ChunkCfg<T>::JB>(V, ld, nv, r0, wv, acc_s[w]);
    }
    warp_rows_to_partial(acc_s, nv, partial);
    if (!arrive_last(counter)) return;
    reduce_partials(partial, gridDim.x, nv, h1);
}

template <class T>
__global__ void __launch_bounds__(kBlasThreads, kBlasMinBlocks<T>)
    cgs_axpy_dot_kernel(long long nchunks, long long ld, T* __restrict__ V, int s, const double* __restrict__ h1,
                        double* partial, double* h2, unsigned* counter, const int* gate) {
    if (gate_closed(gate, s)) return;
    using Acc = typename ChunkCfg<T>::Acc;
    constexpr int RPL = ChunkCfg<T>::RPL;
    constexpr int R = kWarp * RPL;
    __shared__ Acc acc_s[kBlasWarps][kMaxKrylov + 1];
    __shared__ Acc sh[kMaxKrylov + 1];  // coefficients in the accumulation type, converted once
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nv = s + 1;
    for (int j = threadIdx.x; j < nv; j += blockDim.x) sh[j] = static_cast<Acc>(__ldcg(h1 + j));
    zero_warp_rows(acc_s, nv);
    T* wvec = V + static_cast<long long>(s + 1) * ld;
    for (long long c = blockIdx.x * static_cast<long long>(kBlasWarps) + w; c < nchunks;
         c += static_cast<long long>(gridDim.x) * kBlasWarps) {
        const long long r0 = c * R + lane * RPL;
        T a[RPL];
        Acc x[RPL];
        load_rpl<T, RPL>(wvec + r0, a);
#pragma unroll
        for (int u = 0; u < RPL; ++u) x[u] = static_cast<Acc>(a[u]);
        chunk_axpy_rows<T>(V, ld, nv, r0, sh, x);
#pragma unroll
        for (int u = 0; u < RPL; ++u) {
            a[u] = static_cast<T>(x[u]);
            x[u] = static_cast<Acc>(a[u]);  // the dots use the stored (rounded) values
        }
        store_rpl<T, RPL>(wvec + r0, a);
        chunk_dots_rows<T, ChunkCfg<T>::JBA>(V, ld, nv, r0, x, acc_s[w]);
    }
    warp_rows_to_partial(acc_s, nv, partial);
    if (!arrive_last(counter)) return;
    reduce_partials(partial, gridDim.x, nv, h2);
}

// Givens update and loop control for step s.  Mirrors src/gmres.cpp:218-262 and the
// loop header at :199.  The block stages column s of H (h1 + h2), the rotations c, s
// and rs in shared memory; one thread then applies the rotations in order (a chain of
// dependent operations that runs on shared memory instead of global memory).
__device__ __forceinline__ void arnoldi_control(GmresCtl* ctl, Hess H, int s, const double* h1, const double* h2,
                                                double t) {
    __shared__ double col[kMaxKrylov + 2];
    __shared__ double cs[kMaxKrylov + 1];
    __shared__ double sn[kMaxKrylov + 1];
    constexpr double epsmac = 1e-16;
    const int im1 = H.im1;
    const int i = s;
    const int i1 = i + 1;
    double* hh = H.hh;
    double* c = H.c();
    double* sg = H.s();
    double* rs = H.rs();
    const int ptih = i * im1;
    for (int j = threadIdx.x; j <= i; j += blockDim.x) {
        col[j] = __ldcg(h1 + j) + __ldcg(h2 + j);
        cs[j] = c[j];
        sn[j] = sg[j];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    col[i1] = t;
    ctl->i = i;
    ctl->steps = i + 1;
    if (t <= epsmac) {  // happy breakdown: leave the inner loop before the rotation
        for (int j = 0; j <= i1; ++j) hh[ptih + j] = col[j];
        ctl->happy = 1;
        ctl->gate = -1;
        return;
    }
    ctl->inv_norm = 1.0 / t;
    double prev = col[0];
    for (int k = 1; k <= i; ++k) {
        const int k1 = k - 1;
        const double cur = col[k];
        col[k1] = cs[k1] * prev + sn[k1] * cur;
        prev = -sn[k1] * prev + cs[k1] * cur;
    }
    if (i >= 1) col[i] = prev;
    double gam = sqrt(col[i] * col[i] + col[i1] * col[i1]);
    if (gam == 0.0) gam = epsmac;
    const double ci = col[i] / gam;
    const double si = col[i1] / gam;
    c[i] = ci;
    sg[i] = si;
    const double rsi = rs[i];
    rs[i1] = -si * rsi;
    rs[i] = ci * rsi;
    col[i] = ci * col[i] + si * col[i1];
    for (int j = 0; j <= i1; ++j) hh[ptih + j] = col[j];
    const double beta = fabs(rs[i1]);
    ctl->beta = beta;
    if (isnan(beta)) {
        ctl->status = kCtlNan;
        ctl->gate = -1;
        return;
    }
    if (i < ctl->im - 1 && beta > ctl->stop && ctl->its++ < ctl->maxits) {
        ctl->i = i + 1;
        ctl->gate = i + 1;
    } else {
        ctl->gate = -1;
    }
}

template <class T>
__global__ void __launch_bounds__(kBlasThreads, kBlasMinBlocks<T>)
    cgs_axpy_norm_kernel(long long nchunks, long long ld, T* __restrict__ V, int s, const double* __restrict__ h1,
                         const double* __restrict__ h2, double* partial, unsigned* counter, GmresCtl* ctl, Hess H,
                         const int* gate) {
    if (gate_closed(gate, s)) return;
    using Acc = typename ChunkCfg<T>::Acc;
    constexpr int RPL = ChunkCfg<T>::RPL;
    constexpr int R = kWarp * RPL;
    __shared__ Acc sh[kMaxKrylov + 1];  // coefficients in the accumulation type, converted once
    __shared__ double s_red[kBlasWarps];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nv = s + 1;
    for (int j = threadIdx.x; j < nv; j += blockDim.x) sh[j] = static_cast<Acc>(__ldcg(h2 + j));
    __syncthreads();
    T* wv = V + static_cast<long long>(s + 1) * ld;
    double ss = 0.0;
    for (long long c = blockIdx.x * static_cast<long long>(kBlasWarps) + w; c < nchunks;
         c += static_cast<long long>(gridDim.x) * kBlasWarps) {
        const long long r0 = c * R + lane * RPL;
        T a[RPL];
        Acc x[RPL];
        load_rpl<T, RPL>(wv + r0, a);
#pragma unroll
        for (int u = 0; u < RPL; ++u) x[u] = static_cast<Acc>(a[u]);
        chunk_axpy_rows<T>(V, ld, nv, r0, sh, x);
        // the norm accumulates in double from the first product, also for FP32 bases
#pragma unroll
        for (int u = 0; u < RPL; ++u) {
            a[u] = static_cast<T>(x[u]);
            ss = fma(static_cast<double>(a[u]), static_cast<double>(a[u]), ss);
        }
        store_rpl<T, RPL>(wv + r0, a);
    }
    ss = warp_sum(ss);
    if (lane == 0) s_red[w] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kBlasWarps; ++k) t += s_red[k];
        partial[static_cast<size_t>(blockIdx.x) * kPartialStride] = t;
    }
    if (!arrive_last(counter)) return;
    __shared__ double s_norm;
    reduce_partials(partial, gridDim.x, 1, &s_norm);
    __syncthreads();
    arnoldi_control(ctl, H, s, h1, h2, sqrt(s_norm));
}

// Least-squares back substitution rs[0..i] <- H(0..i, 0..i)^{-1} rs (src/gmres.cpp:265-272).
// The block stages H's leading (i+1) x (i+1) triangle and rs in shared memory; one thread
// then runs the reference's loop in the same order.  Skipped when the cycle took no step
// or ended on NaN.
// Dynamic shared memory: (m * m + m + 1) doubles.
static __global__ void __launch_bounds__(256) gmres_backsolve_kernel(GmresCtl* ctl, Hess H) {
    extern __shared__ double bs_smem[];
    if (ctl->status != kCtlRunning || ctl->steps == 0) return;
    const int i = ctl->i;
    const int im1 = H.im1;
    const int w = i + 1;  // columns 0..i, rows 0..i
    double* sh = bs_smem;
    double* srs = bs_smem + (im1 - 1) * (im1 - 1);
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
        const int col = e / w;
        const int row = e - col * w;
        sh[col * w + row] = H.hh[col * im1 + row];
    }
    for (int j = threadIdx.x; j <= i; j += blockDim.x) srs[j] = H.rs()[j];
    __syncthreads();
    if (threadIdx.x != 0) return;
    srs[i] = srs[i] / sh[i * w + i];
    for (int ii = i - 1; ii >= 0; --ii) {
        double t = srs[ii];
        for (int j = ii + 1; j <= i; ++j) t -= sh[j * w + ii] * srs[j];
        srs[ii] = t / sh[ii * w + ii];
    }
    for (int j = 0; j <= i; ++j) H.rs()[j] = srs[j];
}

// x += sum_{j<=i} rs[j] Z[j] (src/gmres.cpp:274-276, j ascending) and Z[j] <- sentinel
// (the backward substitution of the next cycle waits on it).  Row-parallel.
template <class T>
__global__ void __launch_bounds__(256)
    gmres_update_kernel(int n, long long ld, T* __restrict__ Z, double* __restrict__ x, const GmresCtl* ctl, Hess H) {
    __shared__ double srs[kMaxKrylov];
    __shared__ float srs32[kMaxKrylov];  // FP32 path: the coefficients converted once
    if (ctl->status != kCtlRunning || ctl->steps == 0) return;
    const int nz = ctl->i + 1;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        srs[j] = H.rs()[j];
        srs32[j] = static_cast<float>(H.rs()[j]);
    }
    __syncthreads();
    // plain path: x += sum_j rs[j] z_j in FP64 in ascending j; mixed path: the
    // correction sum_j rs[j] z_j is formed in FP32 and added to the FP64 x.  Eight
    // independent loads are in flight per thread; the sentinel stores follow the loads.
    using Acc = typename ChunkCfg<T>::Acc;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        Acc d = Acc(0);
        double xv = x[r];
        int j = 0;
        for (; j + 8 <= nz; j += 8) {
            T z[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) z[u] = Z[static_cast<long long>(j + u) * ld + r];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if constexpr (sizeof(Acc) == sizeof(double)) {
                    xv = fma(srs[j + u], static_cast<double>(z[u]), xv);
                } else {
                    d = fma(srs32[j + u], static_cast<Acc>(z[u]), d);
                }
            }
        }
        for (; j < nz; ++j) {
            const T z = Z[static_cast<long long>(j) * ld + r];
            if constexpr (sizeof(Acc) == sizeof(double)) {
                xv = fma(srs[j], static_cast<double>(z), xv);
            } else {
                d = fma(srs32[j], static_cast<Acc>(z), d);
            }
        }
        x[r] = xv + static_cast<double>(d);
        for (j = 0; j < nz; ++j) Z[static_cast<long long>(j) * ld + r] = Sentinel<T>::value();
    }
}

// z = v for an unpreconditioned solve (identity preconditioner), gated.
template <class T>
__global__ void copy_scaled_kernel(int n, T* v, const double* scale, T* z, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const T sc = static_cast<T>(*scale);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const T a = v[r] * sc;
        v[r] = a;
        z[r] = a;
    }
}

template <class S, class D>
__global__ void convert_kernel(long long n, const S* __restrict__ s, D* __restrict__ d) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        d[i] = static_cast<D>(s[i]);
}

// Structural check of a device-resident CSR matrix of n rows and nnz entries (the row
// pointers hold n + 1 entries, the column indices nnz): row_ptr[0] == 0, row_ptr
// non-decreasing up to row_ptr[n] == nnz, columns in [0, n) and strictly ascending in
// each row.  *bad (INT_MAX on entry) receives the smallest offending row.  A row's
// columns are read only once its bounds have been checked, so no input makes the
// kernel read outside the two arrays.
static __global__ void csr_check_kernel(int n, long long nnz, const int* __restrict__ rp, const int* __restrict__ ci,
                                 int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long b = rp[i], e = rp[i + 1];
        bool ok = b >= 0 && e >= b && e <= nnz && (i != 0 || b == 0) && (i != n - 1 || e == nnz);
        if (ok) {
            int prev = -1;
            for (long long p = b; p < e; ++p) {
                const int c = ci[p];
                if (c < 0 || c >= n || c <= prev) {
                    ok = false;
                    break;
                }
                prev = c;
            }
        }
        if (!ok) atomicMin(bad, i);
    }
}

}  // namespace gb300
