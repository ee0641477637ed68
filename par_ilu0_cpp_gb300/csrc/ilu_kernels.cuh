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
constexpr int kFactCap = 128;    // row length staged in shared memory per warp
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
// sequence of operations as the reference.
//
// Row j is staged in shared memory together with, for every pivot k, diag[k], the end
// of row k and u_kk, all loaded in parallel once the pivots' ready flags are acquired;
// the strict-upper entries of the next pivot row are loaded into registers while the
// current pivot is eliminated.  The sequential chain per pivot is then one division
// (one lane) and a shared-memory search-and-update, instead of three dependent global
// round trips.  Rows longer than kFactCap are eliminated in global memory.  Row k's
// values are read at L2 (ld.cg) after an acquire on its ready flag; row j publishes
// with fence + release.  `shift` (optional) is added to the diagonal before elimination.
constexpr int kFactPre = 2;  // next-pivot entries per lane held in registers

static __global__ void __launch_bounds__(kFactWarps * kWarp)
    ilu_factor_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const int* __restrict__ diag,
                      const int* __restrict__ order, double* lu, const double* __restrict__ shift, int* done,
                      int stamp, unsigned* counter, int* status) {
    __shared__ int s_col[kFactWarps][kFactCap];
    __shared__ double s_val[kFactWarps][kFactCap];
    __shared__ int s_kd[kFactWarps][kFactCap];
    __shared__ int s_ke[kFactWarps][kFactCap];
    __shared__ double s_ukk[kFactWarps][kFactCap];
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
            int* skd = s_kd[w];
            int* ske = s_ke[w];
            double* sukk = s_ukk[w];
            for (int t = lane; t < len; t += kWarp) {
                const int c = ci[b + t];
                scol[t] = c;
                double v = lu[b + t];
                if (shift != nullptr && t == dloc) v += shift[j];
                sval[t] = v;
                if (t < dloc) {
                    const int kd = diag[c];
                    skd[t] = kd;
                    ske[t] = rp[c + 1];
                    sukk[t] = __ldcg(lu + kd);
                }
            }
            __syncwarp();
            // strict-upper entries of pivot row t held by this lane: p = kd + 1 + lane + 32 u
            int nc[kFactPre];
            double nv[kFactPre];
            auto load_pivot = [&](int t) {
                const int p0 = skd[t] + 1 + lane;
                const int pe = ske[t];
#pragma unroll
                for (int u = 0; u < kFactPre; ++u) {
                    const int p = p0 + u * kWarp;
                    nc[u] = p < pe ? ci[p] : -1;
                    nv[u] = p < pe ? __ldcg(lu + p) : 0.0;
                }
            };
            if (dloc > 0) load_pivot(0);
            for (int t = 0; t < dloc; ++t) {
                int cc[kFactPre];
                double cv[kFactPre];
#pragma unroll
                for (int u = 0; u < kFactPre; ++u) {
                    cc[u] = nc[u];
                    cv[u] = nv[u];
                }
                if (t + 1 < dloc) load_pivot(t + 1);
                double l = 0.0;
                if (lane == 0) {
                    l = sval[t] / sukk[t];
                    sval[t] = l;
                }
                l = __shfl_sync(0xffffffffu, l, 0);
#pragma unroll
                for (int u = 0; u < kFactPre; ++u) {
                    if (cc[u] >= 0) {
                        const int pos = find_sorted(scol, t + 1, len, cc[u]);
                        if (pos >= 0) sval[pos] = fma(-cv[u], l, sval[pos]);
                    }
                }
                // strict-upper entries beyond the register window (long pivot rows)
                for (int p = skd[t] + 1 + lane + kFactPre * kWarp; p < ske[t]; p += kWarp) {
                    const int pos = find_sorted(scol, t + 1, len, ci[p]);
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
// Automatic size of the level-ordered substitution grid: warps for this many levels of
// 32-row tasks (averaged over the factor), at most kSolveWarps per SM.
constexpr double kSolveLevelsAhead = 48.0;
constexpr double kSolveLevelsAheadLong = 4.0;  // factors whose rows average > kLaneEntries

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

// Solve of one long row (more than kLaneEntries entries), the reference's entry order.
// Entries are taken in chunks of 8, software-pipelined two deep: the columns, values and
// dependency loads of chunk i + 1 are in flight while chunk i is consumed, so a row pays
// about two memory round trips in total instead of two per chunk.  A dependency not yet
// published is waited for (bounded) when its chunk is consumed.
constexpr int kRowChunk = 8;

template <class T>
__device__ __forceinline__ void load_row_chunk(int off, int K, int k0, int lane, const int* cols, const T* vals,
                                               const T* dep, int (&c)[kRowChunk], T (&v)[kRowChunk],
                                               T (&x)[kRowChunk]) {
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) {
        const int s = off + (k0 + u) * kWarp + lane;
        c[u] = (k0 + u < K) ? cols[s] : -1;
        v[u] = (k0 + u < K) ? vals[s] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) x[u] = c[u] >= 0 ? ld_relaxed_nb(dep + c[u]) : T(0);
}

// Consumes chunk (c, v, x) in entry order.  Entries of the previous level are usually
// loaded before they are published, so several of a row's values can still hold the
// sentinel; after a wait ends, every later value of this chunk and of the other loaded
// chunk (co, xo; `other` = it is loaded) that still holds it is loaded again, all at
// once, so the row pays about one round trip per wait instead of one per entry.
template <class T>
__device__ __forceinline__ T consume_row_chunk(const int (&c)[kRowChunk], const T (&v)[kRowChunk], T (&x)[kRowChunk],
                                               const int (&co)[kRowChunk], T (&xo)[kRowChunk], bool other, T acc,
                                               const T* dep, int* status) {
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) {
        if (c[u] >= 0) {
            if (Sentinel<T>::is(x[u])) {
                x[u] = wait_value(dep + c[u], status);
#pragma unroll
                for (int w = u + 1; w < kRowChunk; ++w)
                    if (c[w] >= 0 && Sentinel<T>::is(x[w])) x[w] = ld_relaxed_nb(dep + c[w]);
                if (other) {
#pragma unroll
                    for (int w = 0; w < kRowChunk; ++w)
                        if (co[w] >= 0 && Sentinel<T>::is(xo[w])) xo[w] = ld_relaxed_nb(dep + co[w]);
                }
            }
            acc = fma(-v[u], x[u], acc);
        }
    }
    return acc;
}

template <class T>
__device__ __forceinline__ T blocking_row(int off, int K, int lane, const int* cols, const T* vals, T acc, const T* dep,
                                          int* status) {
    int cA[kRowChunk], cB[kRowChunk];
    T vA[kRowChunk], vB[kRowChunk], xA[kRowChunk], xB[kRowChunk];
    load_row_chunk(off, K, 0, lane, cols, vals, dep, cA, vA, xA);
    for (int k0 = 0; k0 < K; k0 += 2 * kRowChunk) {
        const bool hasB = k0 + kRowChunk < K;
        const bool hasA2 = k0 + 2 * kRowChunk < K;
        if (hasB) load_row_chunk(off, K, k0 + kRowChunk, lane, cols, vals, dep, cB, vB, xB);
        acc = consume_row_chunk(cA, vA, xA, cB, xB, hasB, acc, dep, status);
        if (hasA2) load_row_chunk(off, K, k0 + 2 * kRowChunk, lane, cols, vals, dep, cA, vA, xA);
        if (hasB) acc = consume_row_chunk(cB, vB, xB, cA, xA, hasA2, acc, dep, status);
    }
    return acc;
}

// Forward substitution with the unit lower factor: y = L^{-1} (scale * b).
// With `scale` non-null, b is rescaled on the fly and the rescaled value is written back
// to b (GMRES uses this to normalise the new Krylov vector in the same pass).
// y must hold the sentinel everywhere on entry; each row publishes its value once.
template <class T>
__global__ void __launch_bounds__(kSolveWarps * kWarp, 1)
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
__global__ void __launch_bounds__(kSolveWarps * kWarp, 1)
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

// ---------------------------------------------------------------------------------
// Block-pipelined substitution (TMA-fed).
//
// Rows are cut into contiguous blocks; one CTA solves one block at a time and keeps the
// block's right-hand side, overwritten in place by its solution, in shared memory.
// Inside a block rows are grouped by their level in the block-internal dependency DAG
// (dependencies on rows of other blocks do not count) and a level is solved by the whole
// CTA between two barriers, one thread per row, so every block-internal dependency is a
// shared-memory read.  Dependencies on other blocks are read from the global solution
// with a value-as-flag wait, their loads issued one level ahead.  Blocks are taken from
// a ticket counter in dependency order (ascending for L, descending for U), so a block
// only waits for blocks whose CTAs are already running: no deadlock, no co-residency
// assumption.  When the blocks follow the matrix's planes (a 3-D grid in natural order
// cut every nx*ny rows) the dependencies between blocks connect equal block-internal
// levels and the blocks run as a pipeline: the critical path crosses SMs once per
// block instead of once per level.
//
// The per-level data (a "slice") streams into a ring of shared-memory stages by 1-D
// bulk copies (cp.async.bulk, completed on one mbarrier per stage), `stages` levels
// ahead, so no level waits on a global load of its own row data.  Slice layout, every
// piece 16-byte aligned (Wp = W rounded up to 32):
//   int4 header {W, K, bytes of the slice `stages` levels later (0: none), Wp}
//   int  rows[Wp]          global row index of each position
//   int  codes[K * Wp]     entry k of position p at k * Wp + p: >= 0 global column (other
//                          block), <= -2 block-local row -2 - code, -1 padding (trailing)
//   T    vals[K * Wp]
//   T    diag[Wp]          upper factor only; FP32 stores 1 / u_ii
// L entries are in ascending and U entries in descending column order: the accumulation
// order of the reference's substitute_row_L / _U (src/ilu_solver.cpp:687-696, 719-729),
// so each row performs the same operations in the same order as a sequential sweep.
// ---------------------------------------------------------------------------------
constexpr int kBandThreadsMax = 512;
constexpr int kBandMaxStages = 16;
constexpr int kBandPre = 4;  // cross-block dependencies per row loaded ahead (registers)
#ifndef GB_BAND_AHEAD
#define GB_BAND_AHEAD 3
#endif
constexpr int kBandAhead = GB_BAND_AHEAD;  // levels between a prefetch and its use

template <class T>
struct BandTri {
    int nblk = 0;
    int stages = 0;           // ring depth (>= 2)
    unsigned stage_bytes = 0; // capacity of one ring stage (multiple of 128)
    unsigned xs_bytes = 0;    // shared bytes of the block vector (multiple of 128)
    const int* blk_row = nullptr;        // [nblk + 1] first row of each block
    const int* blk_lvl = nullptr;        // [nblk + 1] first level of each block
    const long long* blk_off = nullptr;  // [nblk] byte offset of each block's first slice
    const int* lvl_bytes = nullptr;      // [levels] bytes of each slice
    const unsigned char* data = nullptr; // slices, level order within block order
};

// Value-gather instructions of one slice of a block-pipelined factor: the slice's
// values (nvals) and diagonal (ndiag, right after them) take lu[src[src_off + i]]
// (0 for src < 0); an FP32 diagonal is stored as its reciprocal.
struct SliceGather {
    long long src_off;
    long long val_off;  // byte offset of vals[0] in the slice data
    int nvals;
    int ndiag;
};

// One warp per slice.
template <class T>
__global__ void band_gather_kernel(int levels, const SliceGather* __restrict__ gat, const int* __restrict__ src,
                                   const double* __restrict__ lu, unsigned char* __restrict__ data) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int l = blockIdx.x * wpb + (threadIdx.x >> 5); l < levels; l += gridDim.x * wpb) {
        const SliceGather gi = gat[l];
        T* dst = reinterpret_cast<T*>(data + gi.val_off);
        const int* sp = src + gi.src_off;
        const int total = gi.nvals + gi.ndiag;
        for (int i = lane; i < total; i += kWarp) {
            const int q = sp[i];
            double v = q >= 0 ? lu[q] : 0.0;
            if (sizeof(T) == 4 && i >= gi.nvals && q >= 0) v = 1.0 / v;
            dst[i] = static_cast<T>(v);
        }
    }
}

// The rare slow path (a value not yet published) stays out of line: the hot loop is
// unrolled several times and must fit the instruction cache.
template <class T>
__device__ __noinline__ T band_wait_value(const T* p, int* status) {
    return wait_value(p, status);
}

// Issues the loads of this thread's cross-block values of slice `sl` (first position).
// All shared-memory reads come first: a load with a compiler memory barrier between them
// would serialise them.
template <class T>
__device__ __forceinline__ void band_prefetch(const unsigned char* sl, int p, const T* out, T (&pre)[kBandPre]) {
    const int4 h = *reinterpret_cast<const int4*>(sl);
    const int* codes = reinterpret_cast<const int*>(sl + 16) + h.w;
    int cd[kBandPre];
#pragma unroll
    for (int k = 0; k < kBandPre; ++k) cd[k] = (p < h.x && k < h.y) ? codes[k * h.w + p] : -1;
#pragma unroll
    for (int k = 0; k < kBandPre; ++k) pre[k] = cd[k] >= 0 ? ld_relaxed_nb(out + cd[k]) : T(0);
}

// Reloads this thread's prefetched cross-block values of slice `sl` that still hold the
// sentinel.
template <class T>
__device__ __forceinline__ void band_repoll(const unsigned char* sl, int p, const T* out, T (&pre)[kBandPre]) {
    bool miss = false;
#pragma unroll
    for (int k = 0; k < kBandPre; ++k) miss |= Sentinel<T>::is(pre[k]);
    if (!miss) return;
    const int4 h = *reinterpret_cast<const int4*>(sl);
    const int* codes = reinterpret_cast<const int*>(sl + 16) + h.w;
#pragma unroll
    for (int k = 0; k < kBandPre; ++k) {
        if (Sentinel<T>::is(pre[k]) && p < h.x && k < h.y) {
            const int cd = codes[k * h.w + p];
            if (cd >= 0) pre[k] = ld_relaxed_nb(out + cd);
        }
    }
}

// Solves the rows of one slice (one block-internal level).  pre: this thread's
// prefetched cross-block values for its first position (p == threadIdx.x).  The
// shared-memory operands of a row are loaded together before any global access.
template <class T, bool UPPER>
__device__ __forceinline__ void band_solve_slice(const unsigned char* sl, const T (&pre)[kBandPre], T* xs, int base,
                                                 T* in, bool scaled, T sc, T* out, int* status) {
    const int4 h = *reinterpret_cast<const int4*>(sl);
    const int W = h.x, K = h.y, Wp = h.w;
    const int* rows = reinterpret_cast<const int*>(sl + 16);
    const int* codes = rows + Wp;
    const T* vals = reinterpret_cast<const T*>(codes + static_cast<size_t>(K) * Wp);
    const int tid = threadIdx.x;
    for (int p = tid; p < W; p += blockDim.x) {
        const int row = rows[p];
        int cd[kBandPre];
        T v[kBandPre], x[kBandPre];
#pragma unroll
        for (int k = 0; k < kBandPre; ++k) {
            cd[k] = k < K ? codes[k * Wp + p] : -1;
            v[k] = k < K ? vals[k * Wp + p] : T(0);
        }
        const T d = UPPER ? vals[static_cast<size_t>(K) * Wp + p] : T(1);
        T acc = xs[row - base];
#pragma unroll
        for (int k = 0; k < kBandPre; ++k) x[k] = cd[k] <= -2 ? xs[-2 - cd[k]] : (p == tid ? pre[k] : T(0));
        if (!UPPER && scaled) acc = acc * sc;
        const T acc0 = acc;
#pragma unroll
        for (int k = 0; k < kBandPre; ++k) {
            if (cd[k] >= 0) {
                if (p != tid) x[k] = ld_relaxed_nb(out + cd[k]);
                if (Sentinel<T>::is(x[k])) x[k] = band_wait_value(out + cd[k], status);
            }
        }
#pragma unroll
        for (int k = 0; k < kBandPre; ++k)
            if (cd[k] != -1) acc = fma(-v[k], x[k], acc);
        for (int k = kBandPre; k < K; ++k) {
            const int c = codes[k * Wp + p];
            if (c == -1) break;
            T xv;
            if (c <= -2) {
                xv = xs[-2 - c];
            } else {
                xv = ld_relaxed(out + c);
                if (Sentinel<T>::is(xv)) xv = band_wait_value(out + c, status);
            }
            acc = fma(-vals[k * Wp + p], xv, acc);
        }
        // FP64: the reference's division; FP32 (mixed path): d holds 1 / u_ii
        if (UPPER) acc = sizeof(T) == 8 ? acc / d : acc * d;
        acc = Sentinel<T>::canon(acc);
        xs[row - base] = acc;
        st_relaxed(out + row, acc);
        if (!UPPER && scaled) in[row] = acc0;
    }
}

// Forward (UPPER = false): out = L^{-1} (scale * in); with `scale`, in is rescaled in
//   place (GMRES normalises its new Krylov vector in the same pass).
// Backward (UPPER = true): out = U^{-1} in (in is left as it is).
// out must hold the sentinel for every row on entry.  Any block size (a multiple of 32,
// at most kBandThreadsMax); dynamic shared memory: xs_bytes + stages * stage_bytes, and
// stages >= kBandAhead + 2.
//
// Per level: solve the slice's rows, one CTA barrier, then issue the loads of the
// cross-block values of the slice kBandAhead levels later.  A block thereby trails the
// block it depends on by about one L2 round trip, and once the pipeline has filled its
// levels do not wait on global memory.  Thread 0 alone handles the slice ring: at the
// start of a level it refills the stage freed by the previous barrier and waits for the
// slice the next prefetch reads, so the barrier publishes that slice to every thread.
// The level loop is unrolled kBandAhead times so that every prefetch set stays in its
// own registers (a register move would wait for the load).
template <class T, bool UPPER>
__global__ void __launch_bounds__(kBandThreadsMax, 1)
    sptrsv_band_kernel(BandTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                       const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(128) unsigned char band_smem[];
    __shared__ __align__(8) unsigned long long bars[kBandMaxStages + 1];
    __shared__ int s_ticket;
    T* xs = reinterpret_cast<T*>(band_smem);
    unsigned char* ring = band_smem + P.xs_bytes;
    const unsigned D = static_cast<unsigned>(P.stages);
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (unsigned i = 0; i <= D; ++i) mbar_init(&bars[i], 1u);
        fence_mbar_init();
    }
    __syncthreads();
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    unsigned g0 = 0;     // ring slots consumed by this CTA so far (phase bookkeeping)
    unsigned xpar = 0;   // phase parity of the block-vector barrier
    auto slice = [&](unsigned g) { return ring + static_cast<size_t>(g % D) * P.stage_bytes; };
    // thread 0 only
    auto wait_slice = [&](unsigned g) { mbar_wait(&bars[g % D], (g / D) & 1u, status); };
    auto issue_slice = [&](unsigned g, unsigned nb, long long& off) {
        mbar_arrive_expect_tx(&bars[g % D], nb);
        bulk_copy_g2s(ring + static_cast<size_t>(g % D) * P.stage_bytes, P.data + off, nb, &bars[g % D]);
        off += nb;
    };
    for (int tk = draw_block_ticket(counter, P.nblk, &s_ticket); tk < P.nblk;
         tk = draw_block_ticket(counter, P.nblk, &s_ticket)) {
        const int c = UPPER ? P.nblk - 1 - tk : tk;
        const int base = P.blk_row[c];
        const int cnt = P.blk_row[c + 1] - base;
        const int lv0 = P.blk_lvl[c];
        const int nl = P.blk_lvl[c + 1] - lv0;
        const T* src = in + base;
        const unsigned xb =
            (reinterpret_cast<uintptr_t>(src) & 15u) == 0 ? (static_cast<unsigned>(cnt) * sizeof(T)) & ~15u : 0u;
        long long issue_off = 0;
        unsigned nb_prev = 0;  // thread 0: bytes of the slice that refills the stage freed last
        if (tid == 0) {
            if (xb) {
                mbar_arrive_expect_tx(&bars[D], xb);
                bulk_copy_g2s(xs, src, xb, &bars[D]);
            }
            issue_off = P.blk_off[c];
            const int first = min(static_cast<int>(D), nl);
            for (int i = 0; i < first; ++i)
                issue_slice(g0 + static_cast<unsigned>(i), static_cast<unsigned>(P.lvl_bytes[lv0 + i]), issue_off);
            for (int i = 0; i < kBandAhead && i < nl; ++i) wait_slice(g0 + static_cast<unsigned>(i));
            if (xb) mbar_wait(&bars[D], xpar, status);
        }
        if (xb) xpar ^= 1u;
        for (int i = static_cast<int>(xb / sizeof(T)) + tid; i < cnt; i += blockDim.x) xs[i] = src[i];
        __syncthreads();
        T pre[kBandAhead][kBandPre];
#pragma unroll
        for (int j = 0; j < kBandAhead; ++j)
            if (j < nl) band_prefetch<T>(slice(g0 + j), tid, out, pre[j]);
        for (int l = 0; l < nl; l += kBandAhead) {
#pragma unroll
            for (int j = 0; j < kBandAhead; ++j) {
                const int lj = l + j;
                if (lj < nl) {
                    const unsigned g = g0 + static_cast<unsigned>(lj);
                    if (tid == 0) {
                        // the barrier that ended level lj - 1 freed its stage: refill it
                        if (nb_prev != 0) issue_slice(g + D - 1, nb_prev, issue_off);
                        // the prefetch after this level's barrier reads slice lj + kBandAhead
                        if (lj + kBandAhead < nl) wait_slice(g + kBandAhead);
                    }
                    const unsigned char* sl = slice(g);
                    band_solve_slice<T, UPPER>(sl, pre[j], xs, base, in, scaled, sc, out, status);
                    if (tid == 0) nb_prev = static_cast<unsigned>(reinterpret_cast<const int4*>(sl)->z);
                    __syncthreads();
                    if (lj + kBandAhead < nl) band_prefetch<T>(slice(g + kBandAhead), tid, out, pre[j]);
                    // values of the next level that were not yet published when prefetched
                    // (the producing block runs just ahead): load them again now, a level
                    // before they are needed, instead of waiting a round trip then
                    if (kBandAhead > 1 && lj + 1 < nl) band_repoll<T>(slice(g + 1), tid, out, pre[(j + 1) % kBandAhead]);
                }
            }
        }
        g0 += static_cast<unsigned>(nl);
        // this block's generic writes of xs come before the next block's bulk copy into it
        // (once per block: a proxy fence waits for the thread's outstanding memory operations)
        fence_proxy_async_smem();
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
