// Sync-free ILU factorisation and triangular-substitution kernels.
//
// Scheduling (all kernels here): warps take work items from an atomic ticket counter in
// a fixed topological order — rows sorted by level of the dependency DAG, ascending row
// index inside a level (the reference's Levelization lset, src/subtree.hpp:524-551).
// An item only waits for items with smaller tickets; a ticket is only ever held by a
// running warp, and a warp processes its tickets in increasing order, so the warp
// holding the smallest unfinished ticket can always proceed: no deadlock, and no
// assumption that the whole grid is co-resident.  The next ticket is fetched before the
// current item is processed (its latency is hidden).  The last warp to fetch (it draws
// ticket ntask + W - 1, W = warps in the grid) resets the counter for the next launch.
// Every wait is bounded (common.cuh) and reports a timeout instead of hanging.  This
// replaces the reference's OpenMP subtree partition + spin-wait queue
// (src/ilu_solver.cpp:394-443).
#pragma once

#include "common.cuh"

namespace gb300 {

constexpr int kFactWarps = 8;    // warps per block of the factorisation kernel
constexpr int kFactCap = 256;    // row length staged in shared memory per warp
constexpr int kSolveWarps = 8;   // warps per block of the substitution kernels

// Binary search of c in the sorted s[lo, hi); returns the position or -1.
template <class P>
__device__ __forceinline__ int find_sorted(const P* s, int lo, int hi, int c) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int v = s[mid];
        if (v < c) {
            lo = mid + 1;
        } else if (v > c) {
            hi = mid;
        } else {
            return mid;
        }
    }
    return -1;
}

// Draws the warp's next ticket (lane 0 does the atomic); resets the counter when this is
// the grid's final draw.
__device__ __forceinline__ int draw_ticket(unsigned* counter, int ntask, int lane) {
    int t = 0;
    if (lane == 0) {
        t = static_cast<int>(atomicAdd(counter, 1u));
        const int nwarps = static_cast<int>(gridDim.x * (blockDim.x >> 5));
        if (t == ntask + nwarps - 1) atomicExch(counter, 0u);
    }
    return __shfl_sync(0xffffffffu, t, 0);
}

// Kernels launched inside a GMRES cycle graph carry a gate: they run only while
// *gate == step (the cycle is still active at that step).
__device__ __forceinline__ bool gate_closed(const int* gate, int step) {
    return gate != nullptr && *gate != step;
}

// Numeric ILU on a fixed pattern, one warp per row (the up-looking row elimination of
// src/ilu_solver.cpp:553-589).  For row j and each pivot column k of its strict-lower
// part in ascending order: l_jk = a_jk / u_kk, then a_jc -= u_kc * l_jk for every column
// c of row k's strict-upper part that is also in row j's pattern.  Lanes split row k's
// entries; every entry of row j therefore receives its updates in ascending k, the same
// sequence of operations as the reference.  Row j is staged in shared memory (global
// memory for rows longer than kFactCap).  Row k's values are read at L2 (ld.cg) after an
// acquire on row k's ready flag; row j publishes with fence + release.
// `shift` (optional) is added to the diagonal before elimination.
static __global__ void __launch_bounds__(kFactWarps * kWarp)
    ilu_factor_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const int* __restrict__ diag,
                      const int* __restrict__ order, double* lu, const double* __restrict__ shift, int* done,
                      int stamp, unsigned* counter, int* status) {
    __shared__ int s_col[kFactWarps][kFactCap];
    __shared__ double s_val[kFactWarps][kFactCap];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    int q = draw_ticket(counter, n, lane);
    while (q < n) {
        const int qn = draw_ticket(counter, n, lane);
        const int j = order[q];
        const int b = rp[j];
        const int len = rp[j + 1] - b;
        const int dloc = diag[j] - b;
        for (int t = lane; t < dloc; t += kWarp) wait_flag(done + ci[b + t], stamp, status);
        __syncwarp();
        if (len <= kFactCap) {
            int* scol = s_col[w];
            double* sval = s_val[w];
            for (int t = lane; t < len; t += kWarp) {
                scol[t] = ci[b + t];
                double v = lu[b + t];
                if (shift != nullptr && t == dloc) v += shift[j];
                sval[t] = v;
            }
            __syncwarp();
            for (int t = 0; t < dloc; ++t) {
                const int k = scol[t];
                const int kd = diag[k];
                const int ke = rp[k + 1];
                const double l = sval[t] / __ldcg(lu + kd);
                __syncwarp();
                if (lane == 0) sval[t] = l;
                for (int p = kd + 1 + lane; p < ke; p += kWarp) {
                    const int c = ci[p];
                    const int pos = find_sorted(scol, t + 1, len, c);
                    if (pos >= 0) sval[pos] = fma(-__ldcg(lu + p), l, sval[pos]);
                }
                __syncwarp();
            }
            for (int t = lane; t < len; t += kWarp) lu[b + t] = sval[t];
            if (lane == 0) {
                const double u = sval[dloc];
                if (!(fabs(u) > 0.0) || !isfinite(u)) {
                    atomicAdd(status + kStatusBreakdowns, 1);
                    atomicMin(status + kStatusFirstBreakdown, j);
                }
            }
        } else {
            const int* col = ci + b;
            double* val = lu + b;
            if (shift != nullptr && lane == 0) __stcg(val + dloc, __ldcg(val + dloc) + shift[j]);
            __syncwarp();
            for (int t = 0; t < dloc; ++t) {
                const int k = col[t];
                const int kd = diag[k];
                const int ke = rp[k + 1];
                const double l = __ldcg(val + t) / __ldcg(lu + kd);
                __syncwarp();
                if (lane == 0) __stcg(val + t, l);
                for (int p = kd + 1 + lane; p < ke; p += kWarp) {
                    const int pos = find_sorted(col, t + 1, len, ci[p]);
                    if (pos >= 0) __stcg(val + pos, fma(-__ldcg(lu + p), l, __ldcg(val + pos)));
                }
                __syncwarp();
            }
            if (lane == 0) {
                const double u = __ldcg(val + dloc);
                if (!(fabs(u) > 0.0) || !isfinite(u)) {
                    atomicAdd(status + kStatusBreakdowns, 1);
                    atomicMin(status + kStatusFirstBreakdown, j);
                }
            }
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(done + j, stamp);
        q = qn;
    }
}

// Level-ordered packed triangular factor (default substitution layout).  Rows are taken in the
// schedule order and grouped 32 to a task (one lane per row).  Task t owns slots
// [off[t], off[t] + 32 * len[t]); entry k of lane l sits at off[t] + 32 k + l, so a
// warp's loads of entry k are one coalesced 128/256-byte access.  Pad slots have
// col = -1.  L entries are stored in ascending column order and U entries in descending
// column order: the accumulation order of the reference's substitute_row_L / _U
// (src/ilu_solver.cpp:687-696, 719-729).
template <class T>
struct PackedTri {
    int ntask = 0;
    const int* rows = nullptr;   // [32 * ntask], -1 for padding
    const int* off = nullptr;    // [ntask]
    const int* len = nullptr;    // [ntask]
    const int* cols = nullptr;   // [slots]
    const T* vals = nullptr;     // [slots]
    const T* dvals = nullptr;    // [32 * ntask] diagonal (upper factor only)
};

constexpr int kLaneEntries = 8;  // rows with at most this many entries use the per-lane path

// Per-lane progressive solve of a warp's 32 rows (one per lane), for rows with at most
// kLaneEntries entries held in registers (c: column or -1, v: value).  Every round a
// lane issues the loads of all its pending dependencies at once, consumes the ready
// prefix in entry order (the reference's accumulation order, so the operations are the
// same as a sequential sweep) and publishes its row the moment its last entry is
// consumed.  A row therefore never waits for the slowest row of its warp; the warp
// leaves the loop when all 32 rows are published.  Rounds are bounded: past kSpinLimit
// (or once another wait has given up) the status word is set and the loop ends.
template <class T, bool UPPER>
__device__ __forceinline__ void progressive_rows(int row, int K, const int (&c)[kLaneEntries],
                                                 const T (&v)[kLaneEntries], T acc, T d, const T* dep, T* out,
                                                 int* status) {
    int k = 0;
    bool done = row < 0;
    long long rounds = 0;
    while (!__all_sync(0xffffffffu, done)) {
        if (!done) {
            T xs[kLaneEntries];
#pragma unroll
            for (int u = 0; u < kLaneEntries; ++u)
                xs[u] = (u >= k && u < K && c[u] >= 0) ? ld_relaxed(dep + c[u]) : T(0);
#pragma unroll
            for (int u = 0; u < kLaneEntries; ++u) {
                if (k == u && u < K) {
                    if (c[u] < 0) {
                        ++k;
                    } else if (!Sentinel<T>::is(xs[u])) {
                        acc = fma(-v[u], xs[u], acc);
                        ++k;
                    }
                }
            }
            if (k >= K) {
                // FP64: the reference's division; FP32 (mixed path): d holds 1 / u_ii
                const T r = UPPER ? (sizeof(T) == 8 ? acc / d : acc * d) : acc;
                st_relaxed(out + row, Sentinel<T>::canon(r));
                done = true;
            }
        }
        if (++rounds >= kSpinLimit) {
            if (!done) atomicExch(status + kStatusTimeout, 1);
            break;
        }
        if ((rounds & 1023) == 0 && ld_relaxed_int(status + kStatusTimeout) != 0) break;
    }
}

// Blocking solve of one row (any number of entries), the reference's entry order.
template <class T>
__device__ __forceinline__ T blocking_row(int off, int K, int lane, const int* cols, const T* vals, T acc, const T* dep,
                                          int* status) {
    for (int k0 = 0; k0 < K; k0 += 8) {
        int c[8];
        T v[8], x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int s = off + (k0 + u) * kWarp + lane;
            c[u] = (k0 + u < K) ? cols[s] : -1;
            v[u] = (k0 + u < K) ? vals[s] : T(0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = c[u] >= 0 ? ld_relaxed(dep + c[u]) : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (c[u] >= 0) {
                if (Sentinel<T>::is(x[u])) x[u] = wait_value(dep + c[u], status);
                acc = fma(-v[u], x[u], acc);
            }
        }
    }
    return acc;
}

// Forward substitution with the unit lower factor: y = L^{-1} (scale * b).
// With `scale` non-null, b is rescaled on the fly and the rescaled value is written back
// to b (GMRES uses this to normalise the new Krylov vector in the same pass).
// y must hold the sentinel everywhere on entry; each row publishes its value once.
template <class T>
__global__ void __launch_bounds__(kSolveWarps * kWarp)
    sptrsv_lower_kernel(PackedTri<T> L, T* b, const double* scale, T* y, unsigned* counter, int* status,
                        const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const int lane = threadIdx.x & 31;
    const T sc = scale ? static_cast<T>(*scale) : T(1);
    int t = draw_ticket(counter, L.ntask, lane);
    while (t < L.ntask) {
        const int tn = draw_ticket(counter, L.ntask, lane);
        const int row = L.rows[t * kWarp + lane];
        const int off = L.off[t];
        const int K = L.len[t];
        T acc = T(0);
        if (row >= 0) {
            acc = b[row];
            if (scale) acc = acc * sc;
        }
        const T acc0 = acc;
        if (K <= kLaneEntries) {
            int c[kLaneEntries];
            T v[kLaneEntries];
#pragma unroll
            for (int u = 0; u < kLaneEntries; ++u) {
                const int s = off + u * kWarp + lane;
                c[u] = (u < K) ? L.cols[s] : -1;
                v[u] = (u < K) ? L.vals[s] : T(0);
            }
            progressive_rows<T, false>(row, K, c, v, acc, T(1), y, y, status);
        } else {
            acc = blocking_row(off, K, lane, L.cols, L.vals, acc, y, status);
            if (row >= 0) st_relaxed(y + row, Sentinel<T>::canon(acc));
        }
        // the normalised Krylov vector is written back after the row is published: a
        // plain store ahead of the waits would delay them
        if (scale && row >= 0) b[row] = acc0;
        t = tn;
    }
}

// Backward substitution with the upper factor: x = U^{-1} y, waiting on x values of the
// rows it depends on.  x must hold the sentinel everywhere on entry.  y is left as it
// is (the caller resets it to the sentinel before the next forward sweep, off the
// dependency chain: a store into y here doubles this kernel's time).
template <class T>
__global__ void __launch_bounds__(kSolveWarps * kWarp)
    sptrsv_upper_kernel(PackedTri<T> U, T* y, T* x, unsigned* counter, int* status, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const int lane = threadIdx.x & 31;
    int t = draw_ticket(counter, U.ntask, lane);
    while (t < U.ntask) {
        const int tn = draw_ticket(counter, U.ntask, lane);
        const int q = t * kWarp + lane;
        const int row = U.rows[q];
        const int off = U.off[t];
        const int K = U.len[t];
        // the diagonal is loaded before the dependency waits: the waits are ordered
        // memory operations, so a load after them would add a full round trip per level
        const T d = U.dvals[q];
        const T acc = row >= 0 ? y[row] : T(0);
        if (K <= kLaneEntries) {
            int c[kLaneEntries];
            T v[kLaneEntries];
#pragma unroll
            for (int u = 0; u < kLaneEntries; ++u) {
                const int s = off + u * kWarp + lane;
                c[u] = (u < K) ? U.cols[s] : -1;
                v[u] = (u < K) ? U.vals[s] : T(0);
            }
            progressive_rows<T, true>(row, K, c, v, acc, d, x, x, status);
        } else {
            const T r = blocking_row(off, K, lane, U.cols, U.vals, acc, x, status);
            if (row >= 0) st_relaxed(x + row, Sentinel<T>::canon(sizeof(T) == 8 ? r / d : r * d));
        }
        t = tn;
    }
}

// Packed triangular factor for the substitution kernels (block-pipelined layout).
//
// Rows are cut into contiguous blocks of at most S rows; one CTA solves one block at a
// time and keeps the block's solution in shared memory.  Inside a block rows are grouped
// by their level in the block-internal dependency DAG (dependencies on rows of other
// blocks do not count) and a level is solved by the whole CTA between two barriers, so
// every block-internal dependency is a shared-memory read.  Dependencies on other blocks
// are read from the global solution with a value-as-flag wait; blocks are taken from a
// ticket counter in dependency order (ascending for L, descending for U), so a block
// only waits for blocks whose CTAs are already running: no deadlock, no co-residency
// assumption.  Only the critical path's block boundaries pay the global handoff.
//
// Task t (32 rows of one level, one lane per row) owns slots [off[t], off[t] + 32 len[t]):
// entry k of lane l sits at off[t] + 32 k + l (coalesced).  Entry codes: >= 0 global
// column (other block), <= -2 local row -2-code (this block), -1 padding.  L entries are
// kept in ascending column order and U entries in descending column order — the
// accumulation order of the reference's substitute_row_L / _U (src/ilu_solver.cpp:687-696,
// 719-729) — so the result is the same sequence of operations.
template <class T>
struct BlockTri {
    int nblk = 0;
    const int* blk_row = nullptr;   // [nblk + 1] first row of each block
    const int* blk_lvl = nullptr;   // [nblk + 1] first level (index into lvl_task) of each block
    const int* lvl_task = nullptr;  // [levels + 1] first task of each level
    const int* rows = nullptr;      // [32 * ntask], -1 for padding
    const int* off = nullptr;       // [ntask]
    const int* len = nullptr;       // [ntask]
    const int* codes = nullptr;     // [slots]
    const T* vals = nullptr;        // [slots]
    const T* dvals = nullptr;       // [32 * ntask] diagonal (upper factor only)
};

// Gathers packed values from the CSR factor values: dst[s] = src[s] >= 0 ? lu[src[s]] : 0.
template <class T>
__global__ void pack_gather_kernel(long long count, const int* __restrict__ src, const double* __restrict__ lu,
                                   T* __restrict__ dst) {
    for (long long s = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; s < count;
         s += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = src[s];
        dst[s] = p >= 0 ? static_cast<T>(lu[p]) : T(0);
    }
}

// FP32 diagonal of the upper factor stored as its reciprocal (computed in FP64, rounded
// once): the mixed-precision backward sweep multiplies instead of dividing.
static __global__ void pack_gather_recip_kernel(long long count, const int* __restrict__ src, const double* __restrict__ lu,
                                         float* __restrict__ dst) {
    for (long long s = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; s < count;
         s += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = src[s];
        dst[s] = p >= 0 ? static_cast<float>(1.0 / lu[p]) : 0.f;
    }
}

constexpr int kSolveThreads = kSolveWarps * kWarp;

// Draws the CTA's next block ticket (thread 0), broadcast through shared memory; the
// grid's final draw resets the counter.
__device__ __forceinline__ int draw_block_ticket(unsigned* counter, int nblk, int* s_slot) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const int t = static_cast<int>(atomicAdd(counter, 1u));
        if (t == nblk + static_cast<int>(gridDim.x) - 1) atomicExch(counter, 0u);
        *s_slot = t;
    }
    __syncthreads();
    return *s_slot;
}

// Forward (UPPER = false): out = L^{-1} (scale * in); with `scale`, in is rescaled in
//   place (GMRES normalises its new Krylov vector in the same pass).
// Backward (UPPER = true): out = U^{-1} in (in is left as it is).
// out must hold the sentinel for every row on entry.
template <class T, bool UPPER>
__global__ void __launch_bounds__(kSolveThreads)
    sptrsv_block_kernel(BlockTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                        const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    __shared__ int s_ticket;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const T sc = (!UPPER && scale) ? static_cast<T>(*scale) : T(1);
    for (int tk = draw_block_ticket(counter, P.nblk, &s_ticket); tk < P.nblk;
         tk = draw_block_ticket(counter, P.nblk, &s_ticket)) {
        const int c = UPPER ? P.nblk - 1 - tk : tk;
        const int base = P.blk_row[c];
        const int l0 = P.blk_lvl[c];
        const int l1 = P.blk_lvl[c + 1];
        for (int l = l0; l < l1; ++l) {
            const int t1 = P.lvl_task[l + 1];
            for (int t = P.lvl_task[l] + w; t < t1; t += kSolveWarps) {
                const int q = t * kWarp + lane;
                const int row = P.rows[q];
                const int o = P.off[t];
                const int K = P.len[t];
                const T d = UPPER ? P.dvals[q] : T(1);
                T acc = T(0);
                if (row >= 0) {
                    acc = in[row];
                    if (!UPPER && scale) {
                        acc = acc * sc;
                        in[row] = acc;
                    }
                }
                for (int k0 = 0; k0 < K; k0 += 8) {
                    int cd[8];
                    T v[8], x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int sidx = o + (k0 + u) * kWarp + lane;
                        cd[u] = (k0 + u < K) ? P.codes[sidx] : -1;
                        v[u] = (k0 + u < K) ? P.vals[sidx] : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        x[u] = cd[u] >= 0 ? ld_relaxed(out + cd[u]) : (cd[u] <= -2 ? xs[-2 - cd[u]] : T(0));
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if (cd[u] != -1) {
                            if (cd[u] >= 0 && Sentinel<T>::is(x[u])) x[u] = wait_value(out + cd[u], status);
                            acc = fma(-v[u], x[u], acc);
                        }
                    }
                }
                if (row >= 0) {
                    if (UPPER) acc = sizeof(T) == 8 ? acc / d : acc * d;
                    acc = Sentinel<T>::canon(acc);
                    xs[row - base] = acc;
                    st_relaxed(out + row, acc);
                }
            }
            __syncthreads();
        }
    }
}

// Fills n entries with the sentinel.
template <class T>
__global__ void fill_sentinel_kernel(long long n, T* p) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        p[i] = Sentinel<T>::value();
}

}  // namespace gb300
