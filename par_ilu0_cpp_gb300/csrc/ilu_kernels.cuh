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

constexpr int kFactWarps = 8;    // most warps per block of the factorisation kernel
constexpr int kFactCap = 128;    // least row length staged in shared memory per warp
constexpr int kFactEntryBytes = 2 * sizeof(double) + 3 * sizeof(int);  // staged bytes per entry
constexpr int kFactHashMin = 24;  // rows longer than this locate update positions by hashing
constexpr int kFactSmemMax = 200 * 1024;  // dynamic shared memory of one factorisation block
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
// the strict-upper entries of the next pivot row (PRE per lane: 2, or 8 for matrices
// whose rows have more than 64 entries above the diagonal) are loaded into registers
// while the current pivot is eliminated.  The sequential chain per pivot is then one
// division (one lane) and a shared-memory search-and-update, instead of three dependent
// global round trips.  The update position of a column in row j is found by binary
// search over the staged columns for short rows; rows longer than kFactHashMin entries
// build an open-addressing table (column -> position, hcap slots per warp, linear
// probing) once and look positions up in one or two probes: a binary search over tens
// of entries is a chain of dependent shared-memory loads and divergent branches per
// update, and it set the pace of 27-point ILU(k) rows with ~45 pivots.  Each warp stages
// up to `cap` entries (dynamic shared memory, kFactEntryBytes per entry plus 8 bytes per
// table slot and warp, sized by the host to the longest row where it fits); longer rows
// are eliminated in global memory.  Row k's values are read at L2 (ld.cg) after an
// acquire on its ready flag; row j publishes with fence + release.  `shift` (optional) is
// added to the diagonal before elimination.
// Per-warp shared-memory staging of ilu_factor_row (dynamic shared memory of the
// factorisation kernels, `cap` entries and `hcap` table slots per warp).
struct FactStage {
    double* sval;
    double* sukk;
    int* scol;
    int* skd;
    int* ske;
    int* hkey;
    int* hpos;
};

__device__ __forceinline__ FactStage fact_stage(double* fact_smem, int cap, int hcap) {
    const int w = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const size_t wc = static_cast<size_t>(w) * cap, nc_ = static_cast<size_t>(nw) * cap;
    FactStage st;
    st.sval = fact_smem + wc;
    st.sukk = fact_smem + nc_ + wc;
    int* ibase = reinterpret_cast<int*>(fact_smem + 2 * nc_);
    st.scol = ibase + wc;
    st.skd = ibase + nc_ + wc;
    st.ske = ibase + 2 * nc_ + wc;
    st.hkey = ibase + 3 * nc_ + static_cast<size_t>(w) * hcap;
    st.hpos = ibase + 3 * nc_ + static_cast<size_t>(nw) * hcap + static_cast<size_t>(w) * hcap;
    return st;
}

// Elimination of row j by one warp, every pivot row already final (see ilu_factor_kernel).
template <int PRE>
__device__ __forceinline__ void ilu_factor_row(int j, const int* __restrict__ rp, const int* __restrict__ ci,
                                               const int* __restrict__ diag, double* lu,
                                               const double* __restrict__ shift, int* status, int cap,
                                               const FactStage& st) {
    const int lane = threadIdx.x & 31;
    double* sval = st.sval;
    double* sukk = st.sukk;
    int* scol = st.scol;
    int* skd = st.skd;
    int* ske = st.ske;
    int* hkey = st.hkey;
    int* hpos = st.hpos;
    const int b = rp[j];
    const int len = rp[j + 1] - b;
    const int dloc = diag[j] - b;
    if (len <= cap) {
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
        // column -> position table of row j (long rows): hsize slots, a power of two
        // of at least twice the row length, keys -1 where empty
        const bool hashed = len > kFactHashMin;
        int hsize = 0, hshift = 0;
        if (hashed) {
            hsize = 64;
            while (hsize < 2 * len) hsize <<= 1;
            hshift = 32 - (31 - __clz(hsize));
            for (int h = lane; h < hsize; h += kWarp) hkey[h] = -1;
        }
        __syncwarp();
        if (hashed) {
            for (int t = lane; t < len; t += kWarp) {
                const int c = scol[t];
                unsigned h = (static_cast<unsigned>(c) * 0x9E3779B1u) >> hshift;
                while (atomicCAS(hkey + h, -1, c) != -1) h = (h + 1) & static_cast<unsigned>(hsize - 1);
                hpos[h] = t;
            }
            __syncwarp();
        }
        // position of column c in row j (c lies beyond position t), -1 if absent
        auto locate = [&](int c, int t) -> int {
            if (!hashed) return find_sorted(scol, t + 1, len, c);
            unsigned h = (static_cast<unsigned>(c) * 0x9E3779B1u) >> hshift;
            for (int probe = 0; probe < hsize; ++probe) {
                const int k = hkey[h];
                if (k == c) return hpos[h];
                if (k < 0) return -1;
                h = (h + 1) & static_cast<unsigned>(hsize - 1);
            }
            return -1;
        };
        // strict-upper entries of pivot row t held by this lane: p = kd + 1 + lane + 32 u
        int nc[PRE];
        double nv[PRE];
        auto load_pivot = [&](int t) {
            const int p0 = skd[t] + 1 + lane;
            const int pe = ske[t];
#pragma unroll
            for (int u = 0; u < PRE; ++u) {
                const int p = p0 + u * kWarp;
                nc[u] = p < pe ? ci[p] : -1;
                nv[u] = p < pe ? __ldcg(lu + p) : 0.0;
            }
        };
        if (dloc > 0) load_pivot(0);
        for (int t = 0; t < dloc; ++t) {
            int cc[PRE];
            double cv[PRE];
#pragma unroll
            for (int u = 0; u < PRE; ++u) {
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
            for (int u = 0; u < PRE; ++u) {
                if (cc[u] >= 0) {
                    const int pos = locate(cc[u], t);
                    if (pos >= 0) sval[pos] = fma(-cv[u], l, sval[pos]);
                }
            }
            // strict-upper entries beyond the register window (long pivot rows)
            for (int p = skd[t] + 1 + lane + PRE * kWarp; p < ske[t]; p += kWarp) {
                const int pos = locate(ci[p], t);
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
}

template <int PRE>
__global__ void __launch_bounds__(kFactWarps * kWarp)
    ilu_factor_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const int* __restrict__ diag,
                      const int* __restrict__ order, double* lu, const double* __restrict__ shift, int* done,
                      int stamp, unsigned* counter, int* status, int cap, int hcap) {
    extern __shared__ double fact_smem[];
    const int lane = threadIdx.x & 31;
    const FactStage st = fact_stage(fact_smem, cap, hcap);
    int q = draw_ticket(counter, n, lane);
    while (q < n) {
        const int qn = draw_ticket(counter, n, lane);
        const int j = order[q];
        const int b = rp[j];
        const int dloc = diag[j] - b;
        for (int t = lane; t < dloc; t += kWarp) wait_flag(done + ci[b + t], stamp, status);
        __syncwarp();
        ilu_factor_row<PRE>(j, rp, ci, diag, lu, shift, status, cap, st);
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(done + j, stamp);
        q = qn;
    }
}

// Subtree partitions of the elimination tree, one CTA each (the reference's subtree
// scheduler, src/subtree.hpp tree_schedule, run by src/ilu_solver.cpp:394-443): a row's
// pivots are its descendants in the elimination tree, so a partition made of whole
// subtrees depends on no other CTA.  The CTA takes its rows level by level (level groups
// of the partition, rows of a group independent), one warp per row, a barrier between
// groups: no ready flags are waited for.  Its rows' flags are set at the end for the
// separator rows, which ilu_factor_kernel then takes by tickets.  part_ptr[p] .. part_ptr[p+1]
// are partition p's groups in grp_ptr, whose rows are rows[grp_ptr[g] .. grp_ptr[g+1]).
constexpr int kSubtreeWarps = 32;  // most warps per CTA of the subtree factorisation kernel

template <int PRE>
__global__ void __launch_bounds__(kSubtreeWarps * kWarp)
    ilu_factor_subtree_kernel(const int* __restrict__ part_ptr, const int* __restrict__ grp_ptr,
                              const int* __restrict__ rows, const int* __restrict__ rp, const int* __restrict__ ci,
                              const int* __restrict__ diag, double* lu, const double* __restrict__ shift, int* done,
                              int stamp, int* status, int cap, int hcap) {
    extern __shared__ double fact_smem[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const FactStage st = fact_stage(fact_smem, cap, hcap);
    const int p = blockIdx.x;
    for (int gidx = part_ptr[p]; gidx < part_ptr[p + 1]; ++gidx) {
        for (int q = grp_ptr[gidx] + w; q < grp_ptr[gidx + 1]; q += nw)
            ilu_factor_row<PRE>(rows[q], rp, ci, diag, lu, shift, status, cap, st);
        // the group's rows (global memory, written by this CTA) before the next group reads them
        __syncthreads();
    }
    __threadfence();
    __syncthreads();
    const int r0 = grp_ptr[part_ptr[p]], r1 = grp_ptr[part_ptr[p + 1]];
    for (int q = r0 + threadIdx.x; q < r1; q += blockDim.x) done[rows[q]] = stamp;
    (void)lane;
}

// Level-ordered packed triangular factor (default substitution layout).  Rows are taken in the
// schedule order, G lanes per row (G = 1, 2, 4 .. 32, one value per factor), 32 / G rows
// to a task.  Task t owns slots [off[t], off[t] + 32 * len[t]); lane l = i G + j holds
// entries [j len[t], (j + 1) len[t]) of the task's row i, entry j len[t] + u at
// off[t] + 32 u + l, so a warp's loads of entry slot u are one coalesced 128/256-byte
// access.  Pad slots have col = -1.  L entries are stored in ascending column order and
// U entries in descending column order: the accumulation order of the reference's
// substitute_row_L / _U (src/ilu_solver.cpp:687-696, 719-729).
template <class T>
struct PackedTri {
    int ntask = 0;
    const int* rows = nullptr;   // [32 * ntask] row of each lane, -1 for padding
    const int* off = nullptr;    // [ntask]
    const int* len = nullptr;    // [ntask] entries per lane
    const int* cols = nullptr;   // [slots]
    const T* vals = nullptr;     // [slots]
    const T* dvals = nullptr;    // [32 * ntask] diagonal of each lane's row (upper factor only)
};

constexpr int kLaneEntries = 8;  // entries a lane holds in registers
constexpr int kRowLanesMax = 32;  // largest lane group per row (rows of up to 256 entries)
// Automatic size of the level-ordered substitution grid: warps for this many levels of
// tasks (averaged over the factor), at most kSolveWarps per SM.
constexpr double kSolveLevelsAhead = 48.0;      // one lane per row
constexpr double kSolveLevelsAheadGroup = 10.0;  // lane groups (long rows)
constexpr double kSolveLevelsAheadLong = 4.0;    // rows longer than kRowLanesMax * kLaneEntries

// Per-lane progressive solve of a warp's 32 rows (one per lane), for rows with at most
// kLaneEntries entries held in registers (c: column or -1, v: value).  Every round a
// lane issues the loads of all its pending dependencies at once, consumes the ready
// prefix in entry order (the reference's accumulation order, so the operations are the
// same as a sequential sweep) and publishes its row the moment its last entry is
// consumed.  A row therefore never waits for the slowest row of its warp; the warp
// leaves the loop when all 32 rows are published.  Rounds are bounded (WaitBudget): when
// the wait expires the status word is set and the loop ends.
template <class T, bool UPPER>
__device__ __forceinline__ void progressive_rows(int row, int K, const int (&c)[kLaneEntries],
                                                 const T (&v)[kLaneEntries], T acc, T d, const T* dep, T* out,
                                                 int* status) {
    int k = 0;
    bool done = row < 0;
    WaitBudget wb;
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
        if (wb.expired(status)) {
            if (!done) atomicExch(status + kStatusTimeout, 1);
            break;
        }
    }
}

// Progressive solve of rows of up to G * kLaneEntries entries with G lanes per row
// (G = 2 .. 32, a warp holds 32 / G rows).  Lane j of a row's group holds entries
// [j K, j K + K) of the row in registers (K = the task's entries per lane; columns -1
// pad the row's tail).  Every round each lane loads, all at once, the dependencies it
// holds that are still unconsumed and still read as the sentinel (published values
// never change, so a value once read is kept).  The running sum then travels along the
// group: the lane holding the first unconsumed entry (the owner) consumes its ready
// prefix in entry order and, once all its entries are consumed, hands the sum to the
// next lane by a shuffle; that lane goes on in the same round with the values it
// already holds.  So each entry is consumed in the reference's order (the operations of
// a sequential sweep), while a row waits about one round trip per wait instead of one
// per chunk of entries.  Lane 0 of the group publishes the row.  Rounds are bounded as
// in progressive_rows.
template <class T, bool UPPER, int G>
__device__ __forceinline__ void group_rows(int row, int K, int lane, const int (&c)[kLaneEntries],
                                           const T (&v)[kLaneEntries], T acc, T d, const T* dep, T* out,
                                           int* status) {
    const int j = lane & (G - 1);
    const int gb = lane - j;
    T x[kLaneEntries];
#pragma unroll
    for (int u = 0; u < kLaneEntries; ++u) x[u] = Sentinel<T>::value();
    int o = 0;  // owner: group position of the first unconsumed entry (G = row done)
    int k = 0;  // next entry of this lane to consume (meaningful in the owner)
    bool done = row < 0;
    WaitBudget wb;
    while (!__all_sync(0xffffffffu, done)) {
        if (!done && j >= o) {
            const int k0 = j == o ? k : 0;
#pragma unroll
            for (int u = 0; u < kLaneEntries; ++u)
                if (u >= k0 && u < K && c[u] >= 0 && Sentinel<T>::is(x[u])) x[u] = ld_relaxed_nb(dep + c[u]);
        }
#pragma unroll 1
        for (int step = 0; step < G; ++step) {
            bool fin = false;
            if (!done && j == o) {
#pragma unroll
                for (int u = 0; u < kLaneEntries; ++u) {
                    if (k == u && u < K) {
                        if (c[u] < 0) {
                            ++k;
                        } else if (!Sentinel<T>::is(x[u])) {
                            acc = fma(-v[u], x[u], acc);
                            ++k;
                        }
                    }
                }
                fin = k >= K;
            }
            const int src = gb + (o < G ? o : G - 1);
            const bool moved = __shfl_sync(0xffffffffu, fin, src);
            acc = __shfl_sync(0xffffffffu, acc, src);
            if (moved) {
                ++o;
                if (o == G) {
                    if (j == 0) {
                        // FP64: the reference's division; FP32 (mixed path): d holds 1 / u_ii
                        const T r = UPPER ? (sizeof(T) == 8 ? acc / d : acc * d) : acc;
                        st_relaxed(out + row, Sentinel<T>::canon(r));
                    }
                    done = true;
                }
            }
            if (!__any_sync(0xffffffffu, moved)) break;
        }
        if (wb.expired(status)) {
            if (!done) atomicExch(status + kStatusTimeout, 1);
            break;
        }
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

// Loads lane `lane`'s packed entries of task (off, K): columns (-1 past K) and values.
template <class T>
__device__ __forceinline__ void load_lane_entries(const PackedTri<T>& P, int off, int K, int lane,
                                                  int (&c)[kLaneEntries], T (&v)[kLaneEntries]) {
#pragma unroll
    for (int u = 0; u < kLaneEntries; ++u) {
        const int s = off + u * kWarp + lane;
        c[u] = (u < K) ? P.cols[s] : -1;
        v[u] = (u < K) ? P.vals[s] : T(0);
    }
}

// Forward substitution with the unit lower factor: y = L^{-1} (scale * b).
// With `scale` non-null, b is rescaled on the fly and the rescaled value is written back
// to b (GMRES uses this to normalise the new Krylov vector in the same pass).
// y must hold the sentinel everywhere on entry; each row publishes its value once.
// G lanes per row: 1 (rows of up to kLaneEntries entries progressive, longer rows
// blocking) or 2 .. 32 (group_rows; the packing guarantees K <= kLaneEntries).
template <class T, int G>
__global__ void __launch_bounds__(kSolveWarps * kWarp, 1)
    sptrsv_lower_kernel(PackedTri<T> L, T* b, const double* scale, T* y, unsigned* counter, int* status,
                        const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const int lane = threadIdx.x & 31;
    const bool lead = (lane & (G - 1)) == 0;  // the lane that owns the row's right-hand side
    const T sc = scale ? static_cast<T>(*scale) : T(1);
    int t = draw_ticket(counter, L.ntask, lane);
    while (t < L.ntask) {
        const int tn = draw_ticket(counter, L.ntask, lane);
        const int row = L.rows[t * kWarp + lane];
        const int off = L.off[t];
        const int K = L.len[t];
        T acc = T(0);
        if (row >= 0 && lead) {
            acc = b[row];
            if (scale) acc = acc * sc;
        }
        const T acc0 = acc;
        if (G > 1 || K <= kLaneEntries) {
            int c[kLaneEntries];
            T v[kLaneEntries];
            load_lane_entries(L, off, K, lane, c, v);
            if (G > 1)
                group_rows<T, false, G>(row, K, lane, c, v, acc, T(1), y, y, status);
            else
                progressive_rows<T, false>(row, K, c, v, acc, T(1), y, y, status);
        } else {
            acc = blocking_row(off, K, lane, L.cols, L.vals, acc, y, status);
            if (row >= 0) st_relaxed(y + row, Sentinel<T>::canon(acc));
        }
        // the normalised Krylov vector is written back after the row is published: a
        // plain store ahead of the waits would delay them
        if (scale && row >= 0 && lead) b[row] = acc0;
        t = tn;
    }
}

// Backward substitution with the upper factor: x = U^{-1} y, waiting on x values of the
// rows it depends on.  x must hold the sentinel everywhere on entry.  y is left as it
// is (the caller resets it to the sentinel before the next forward sweep, off the
// dependency chain: a store into y here doubles this kernel's time).
template <class T, int G>
__global__ void __launch_bounds__(kSolveWarps * kWarp, 1)
    sptrsv_upper_kernel(PackedTri<T> U, T* y, T* x, unsigned* counter, int* status, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const int lane = threadIdx.x & 31;
    const bool lead = (lane & (G - 1)) == 0;
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
        const T acc = (row >= 0 && lead) ? y[row] : T(0);
        if (G > 1 || K <= kLaneEntries) {
            int c[kLaneEntries];
            T v[kLaneEntries];
            load_lane_entries(U, off, K, lane, c, v);
            if (G > 1)
                group_rows<T, true, G>(row, K, lane, c, v, acc, d, x, x, status);
            else
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
// Block-local substitution (sync-free inside blocks and between them).
//
// Rows are cut into contiguous blocks; one CTA solves one block at a time and keeps the
// block's solution in shared memory, at the sentinel until written.  A block's rows are
// packed like PackedTri: 32-row tasks (one lane per row), rows in the order of the
// block-internal dependency DAG's levels, entry k of lane l at off[t] + 32 k + l.  Entry
// codes: >= 0 global column (a row of another block), <= -2 block-local row -2 - code,
// -1 padding.  Warp w of the CTA takes the block's tasks w, w + nwarps, ... and each lane
// solves its row with the per-lane progressive rounds of the level-ordered kernel,
// polling block-local dependencies in shared memory and the others in L2.  There is no
// barrier inside a block: a dependency handoff between two warps of the CTA costs one
// shared-memory round trip instead of an L2 one.  With the blocks cut at the matrix's
// planes (a 3-D grid in natural order, every nx*ny rows) the critical path crosses SMs
// once per block instead of once per level.
//
// Deadlock freedom: blocks are taken from a ticket counter in dependency order (ascending
// for L, descending for U), so a block only waits for blocks whose CTAs hold smaller
// tickets and are running; inside a block each warp takes its tasks in level order, so
// the earliest unfinished task always has all its dependencies in finished tasks or in
// lanes of its own warp, which progress independently.  All waits are bounded.
//
// The operations of each row are those of the level-ordered kernel (L ascending, U
// descending, src/ilu_solver.cpp:687-696, 719-729): results are identical.
// ---------------------------------------------------------------------------------
constexpr int kBlockWarpsMax = 16;
constexpr int kBlockCluster = 8;      // CTAs per cluster of the cluster variant (portable maximum)
constexpr int kBlockClusterBig = 16;  // non-portable cluster size, tried first where it can be scheduled
constexpr int kPubGlobal = 1 << 30;
constexpr int kPubSlotBits = 15;  // halo slot + 1 of a row, per distance d = 1, 2
constexpr int kPubSlotMask = (1 << kPubSlotBits) - 1;
constexpr int kHaloDepth = 2;     // positions ahead a row is pushed to (cluster variant)

template <class T>
struct BlockTri {
    int nblk = 0;
    int ntask = 0;
    long long slots = 0;
    const int* blk_row = nullptr;   // [nblk + 1] first row of each block
    const int* blk_task = nullptr;  // [nblk + 1] first task of each block
    const int* rows = nullptr;      // [32 * ntask] global row, -1 for padding
    const int* off = nullptr;       // [ntask]
    const int* len = nullptr;       // [ntask]
    const int* codes = nullptr;     // [slots]
    const T* vals = nullptr;        // [slots]
    const T* dvals = nullptr;       // [32 * ntask] diagonal (upper factor only; FP32: 1 / u_ii)
    // Per-row publication words: bit kPubGlobal = another block reads the row through L2
    // (store it to `out` as soon as it is computed; the others reach `out` in a coalesced
    // copy when their block is done); bits [15 (d - 1), 15 d) = halo slot + 1 of the row in
    // the CTA d = 1, 2 positions ahead (cluster variant: blocks at processing positions
    // q*cl .. q*cl + cl - 1 run on one cluster and the rows a position's block reads from
    // the two positions before it are pushed into its halo xs[block_rows + slot]).
    int block_rows = 0;
    int halo = 0;
    int cl = 0;
    const int* exps = nullptr;      // [32 * ntask]
};

// ---- thread-block cluster helpers (distributed shared memory) ----
__device__ __forceinline__ unsigned cluster_rank_u32() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size_u32() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// Address of `p` (this CTA's shared memory) in the shared memory of cluster CTA `rank`.
__device__ __forceinline__ unsigned map_shared_rank(const void* p, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(r)
                 : "r"(static_cast<unsigned>(__cvta_generic_to_shared(p))), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster(unsigned addr, float v) {
    asm volatile("st.relaxed.cluster.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(unsigned addr, double v) {
    asm volatile("st.relaxed.cluster.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(unsigned addr, int v) {
    asm volatile("st.relaxed.cluster.shared::cluster.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
// All threads of all CTAs of the cluster; release / acquire ordering of shared memory.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <class T>
__device__ __forceinline__ T ld_volatile_shared(const T* p) {
    return *reinterpret_cast<const volatile T*>(p);
}
template <class T>
__device__ __forceinline__ void st_volatile_shared(T* p, T v) {
    *reinterpret_cast<volatile T*>(p) = v;
}

// One dependency value of a block-local solve: block-local rows from shared memory,
// other rows from L2 (relaxed, GPU scope).
template <class T>
__device__ __forceinline__ T block_dep(int code, const T* xs, const T* out) {
    return code <= -2 ? ld_volatile_shared(xs + (-2 - code)) : ld_relaxed(out + code);
}

// Per-lane progressive solve of one task's rows (at most KM entries each);
// publishes each row to shared memory and to `out` the moment its last entry is consumed.
// Publishes row `row` (value r): the block's shared memory, the halos of the cluster
// CTAs one and two positions ahead (remote / remote2, 0 when none) where the row has a
// slot there, and `out` when another block reads it through L2.
template <class T>
__device__ __forceinline__ void block_publish(int row, T r, T* xs, int base, T* out, unsigned remote, unsigned remote2,
                                              int ex) {
    st_volatile_shared(xs + (row - base), r);
    const int s1 = (ex & kPubSlotMask) - 1;
    if (remote != 0u && s1 >= 0) st_cluster(remote + static_cast<unsigned>(s1) * sizeof(T), r);
    const int s2 = ((ex >> kPubSlotBits) & kPubSlotMask) - 1;
    if (remote2 != 0u && s2 >= 0) st_cluster(remote2 + static_cast<unsigned>(s2) * sizeof(T), r);
    if (ex & kPubGlobal) st_relaxed(out + row, r);
}

template <class T, bool UPPER, int KM>
__device__ __forceinline__ void block_progressive(int row, int K, const int (&c)[KM], const T (&v)[KM], T acc, T d,
                                                  T* xs, int base, T* out, unsigned remote, unsigned remote2, int ex,
                                                  int* status) {
    int k = 0;
    bool done = row < 0;
    WaitBudget wb;
    while (!__all_sync(0xffffffffu, done)) {
        if (!done) {
            T x[KM];
#pragma unroll
            for (int u = 0; u < KM; ++u)
                x[u] = (u >= k && u < K && c[u] != -1) ? block_dep(c[u], xs, out) : T(0);
#pragma unroll
            for (int u = 0; u < KM; ++u) {
                if (k == u && u < K) {
                    if (c[u] == -1) {
                        ++k;
                    } else if (!Sentinel<T>::is(x[u])) {
                        acc = fma(-v[u], x[u], acc);
                        ++k;
                    }
                }
            }
            if (k >= K) {
                // FP64: the reference's division; FP32 (mixed path): d holds 1 / u_ii
                const T r = Sentinel<T>::canon(UPPER ? (sizeof(T) == 8 ? acc / d : acc * d) : acc);
                block_publish(row, r, xs, base, out, remote, remote2, ex);
                done = true;
            }
        }
        if (wb.expired(status)) {
            if (!done) atomicExch(status + kStatusTimeout, 1);
            break;
        }
    }
}

// Solve of one long row (more than kLaneEntries entries) of a block-local task, entry by
// entry in order, each dependency waited for (bounded) when it is reached.
template <class T>
__device__ __noinline__ T block_long_row(int off, int K, int lane, const int* codes, const T* vals, T acc,
                                         const T* xs, const T* out, int* status) {
    for (int k = 0; k < K; ++k) {
        const int s = off + k * kWarp + lane;
        const int c = codes[s];
        if (c == -1) continue;
        T x = block_dep(c, xs, out);
        if (Sentinel<T>::is(x)) {
            if (c >= 0) {
                x = wait_value(out + c, status);
            } else {
                WaitBudget wb;
                while (Sentinel<T>::is(x) && !wb.expired(status)) x = ld_volatile_shared(xs + (-2 - c));
                if (Sentinel<T>::is(x)) {
                    atomicExch(status + kStatusTimeout, 1);
                    x = T(0);
                }
            }
        }
        acc = fma(-vals[s], x, acc);
    }
    return acc;
}

// One lane's share of a block-local task: its row, entries (registers), right-hand side
// and diagonal.
template <class T, int KM>
struct BlockTask {
    int row, off, K, ex;
    int c[KM];
    T v[KM];
    T b, d;
};

template <class T, bool UPPER, int KM, bool FIXED>
__device__ __forceinline__ void load_block_task(const BlockTri<T>& P, int t, int lane, const T* in,
                                                BlockTask<T, KM>& s) {
    s.row = P.rows[t * kWarp + lane];
    if constexpr (FIXED) {
        s.off = t * (KM * kWarp);  // compile-time task length: no off / len loads, fixed loop bounds
        s.K = KM;
    } else {
        s.off = P.off[t];
        s.K = P.len[t];
    }
#pragma unroll
    for (int u = 0; u < KM; ++u) {
        const int sidx = s.off + u * kWarp + lane;
        s.c[u] = (u < s.K) ? P.codes[sidx] : -1;
        s.v[u] = (u < s.K) ? P.vals[sidx] : T(0);
    }
    s.b = s.row >= 0 ? in[s.row] : T(0);
    s.d = UPPER ? P.dvals[t * kWarp + lane] : T(1);
    s.ex = P.exps[t * kWarp + lane];
}

template <class T, bool UPPER, int KM>
__device__ __forceinline__ void solve_block_task(const BlockTri<T>& P, const BlockTask<T, KM>& s, int lane,
                                                 bool scaled, T sc, T* in, T* xs, int base, T* out, unsigned remote,
                                                 unsigned remote2, int* status) {
    T acc = scaled ? s.b * sc : s.b;
    if (s.K <= KM) {
        block_progressive<T, UPPER, KM>(s.row, s.K, s.c, s.v, acc, s.d, xs, base, out, remote, remote2, s.ex,
                                        status);
    } else {
        acc = block_long_row(s.off, s.K, lane, P.codes, P.vals, acc, xs, out, status);
        if (s.row >= 0) {
            const T r = Sentinel<T>::canon(UPPER ? (sizeof(T) == 8 ? acc / s.d : acc * s.d) : acc);
            block_publish(s.row, r, xs, base, out, remote, remote2, s.ex);
        }
    }
}

// Solves block `blk` (its solution xs[0 .. rows) already at the sentinel).
template <class T, bool UPPER, int KM, bool FIXED>
__device__ __forceinline__ void solve_block(const BlockTri<T>& P, int blk, T* in, bool scaled, T sc, T* xs, T* out,
                                            unsigned remote, unsigned remote2, int* status) {
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int base = P.blk_row[blk];
    const int t1 = P.blk_task[blk + 1];
    // Task data is loaded one task ahead (the block's packed data was streamed into L2
    // when the block was taken; loading two tasks ahead measured slower by ~2%).
    BlockTask<T, KM> A;
    int t = P.blk_task[blk] + w;
    if (t < t1) load_block_task<T, UPPER, KM, FIXED>(P, t, lane, in, A);
    while (t < t1) {
        const BlockTask<T, KM> cur = A;
        const int tn = t + nw;
        if (tn < t1) load_block_task<T, UPPER, KM, FIXED>(P, tn, lane, in, A);
        solve_block_task<T, UPPER, KM>(P, cur, lane, scaled, sc, in, xs, base, out, remote, remote2, status);
        t = tn;
    }
}

// Once every row of the block is solved: GMRES normalises its new Krylov vector in the
// forward sweep, so the block's slice of `in` is rescaled in one coalesced pass (the same
// product b * scale the rows used), off the dependency chain.
// Also the block's solution reaches `out` here, copied from shared memory (rows that
// other blocks read were stored when computed and are stored again, unchanged).
template <class T>
__device__ __forceinline__ void finish_block(const BlockTri<T>& P, int blk, T* in, bool scaled, T sc, const T* xs,
                                             T* out) {
    __syncthreads();
    const int base = P.blk_row[blk];
    const int cnt = P.blk_row[blk + 1] - base;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        out[base + i] = xs[i];
        if (scaled) in[base + i] = in[base + i] * sc;
    }
}

// Streams block `blk`'s packed task data and right-hand side into L2 (first warp):
// between sweeps the Krylov vectors evict them, and the warps' own loads run only two
// tasks ahead.
template <class T, bool UPPER>
__device__ __forceinline__ void prefetch_block(const BlockTri<T>& P, int blk, const T* in) {
    if (threadIdx.x >= kWarp) return;
    const int lane = threadIdx.x;
    const int base = P.blk_row[blk];
    const int cnt = P.blk_row[blk + 1] - base;
    const int t0 = P.blk_task[blk];
    const int t1 = P.blk_task[blk + 1];
    const long long s0 = P.off[t0];
    const long long s1 = t1 < P.ntask ? P.off[t1] : P.slots;
    prefetch_l2_range(P.codes + s0, (s1 - s0) * 4, lane);
    prefetch_l2_range(P.vals + s0, (s1 - s0) * static_cast<long long>(sizeof(T)), lane);
    prefetch_l2_range(P.rows + static_cast<long long>(t0) * kWarp, (t1 - t0) * 128ll, lane);
    if (UPPER)
        prefetch_l2_range(P.dvals + static_cast<long long>(t0) * kWarp,
                          (t1 - t0) * static_cast<long long>(kWarp * sizeof(T)), lane);
    // right-hand side rows [base, base + cnt): whole 16-byte pieces inside the range
    const unsigned long long ib = reinterpret_cast<unsigned long long>(in + base);
    const unsigned long long ie = reinterpret_cast<unsigned long long>(in + base + cnt);
    const unsigned long long a16 = (ib + 15) & ~15ull;
    if (ie > a16)
        prefetch_l2_range(reinterpret_cast<const void*>(a16), static_cast<long long>((ie - a16) & ~15ull), lane);
}

// Forward (UPPER = false): out = L^{-1} (scale * in); with `scale`, in is rescaled in
//   place (GMRES normalises its new Krylov vector in the same pass).
// Backward (UPPER = true): out = U^{-1} in (in is left as it is).
// out must hold the sentinel for every row on entry.  Dynamic shared memory: the
// largest block's rows x sizeof(T).
// KM: entries per row held in registers (3 or 4 when no row of the factor has more, else
// kLaneEntries); longer rows take the entry-by-entry path.  FIXED: every task holds KM
// entries per lane (factors whose rows fit in registers), so the task layout and the
// loops over a lane's entries have compile-time bounds (7% faster FP32 7-point sweeps
// than per-task lengths loaded from off / len).
template <class T, bool UPPER, int KM, bool FIXED>
__global__ void __launch_bounds__(kBlockWarpsMax * kWarp, 1)
    sptrsv_block_kernel(BlockTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                        const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char blk_smem[];
    T* xs = reinterpret_cast<T*>(blk_smem);
    __shared__ int s_ticket;
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    for (int tk = draw_block_ticket(counter, P.nblk, &s_ticket); tk < P.nblk;
         tk = draw_block_ticket(counter, P.nblk, &s_ticket)) {
        const int blk = UPPER ? P.nblk - 1 - tk : tk;
        const int cnt = P.blk_row[blk + 1] - P.blk_row[blk];
        prefetch_block<T, UPPER>(P, blk, in);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) xs[i] = Sentinel<T>::value();
        __syncthreads();
        solve_block<T, UPPER, KM, FIXED>(P, blk, in, scaled, sc, xs, out, 0u, 0u, status);
        finish_block(P, blk, in, scaled, sc, xs, out);
    }
}

// Cluster variant: launched with clusters of P.cl CTAs.  The cluster's CTA of rank r takes
// processing position q * cl + r of the cluster's ticket q (tickets in dependency order:
// no co-residency assumption between clusters; the CTAs of one cluster are co-scheduled
// by the hardware).  Each CTA pushes the rows that the blocks one and two positions
// ahead read into those CTAs' shared-memory halos (xs[block_rows + slot], distributed
// shared memory), where the consumers' entry codes point: in-cluster handoffs never
// touch L2.  Sources outside the cluster are read from L2 as in the plain variant.
// Dynamic shared memory: (block_rows + halo) x sizeof(T).
template <class T, bool UPPER, int KM, bool FIXED>
__global__ void __launch_bounds__(kBlockWarpsMax * kWarp, 1)
    sptrsv_block_cluster_kernel(BlockTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                                const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char blk_smem[];
    T* xs = reinterpret_cast<T*>(blk_smem);
    __shared__ int s_ticket;
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    const unsigned rank = cluster_rank_u32();
    const unsigned CL = cluster_size_u32();
    const int nq = (P.nblk + static_cast<int>(CL) - 1) / static_cast<int>(CL);
    const int nclusters = static_cast<int>(gridDim.x / CL);
    for (;;) {
        // the previous round is complete in every CTA of the cluster (no remote store in
        // flight) before the ticket and the halos are reset
        cluster_sync_all();
        if (rank == 0 && threadIdx.x == 0) {
            const int q = static_cast<int>(atomicAdd(counter, 1u));
            if (q == nq + nclusters - 1) atomicExch(counter, 0u);
            for (unsigned r = 0; r < CL; ++r) st_cluster(map_shared_rank(&s_ticket, r), q);
        }
        cluster_sync_all();
        const int q = *reinterpret_cast<volatile int*>(&s_ticket);
        if (q >= nq) break;
        const int pos = q * static_cast<int>(CL) + static_cast<int>(rank);
        const bool active = pos < P.nblk;
        const int blk = UPPER ? P.nblk - 1 - pos : pos;
        if (active) {
            const int cnt = P.blk_row[blk + 1] - P.blk_row[blk];
            prefetch_block<T, UPPER>(P, blk, in);
            for (int i = threadIdx.x; i < cnt; i += blockDim.x) xs[i] = Sentinel<T>::value();
            for (int i = threadIdx.x; i < P.halo; i += blockDim.x) xs[P.block_rows + i] = Sentinel<T>::value();
        }
        __syncthreads();
        // every halo is at the sentinel before any CTA of the cluster pushes into it
        cluster_sync_all();
        if (active) {
            const bool push = rank + 1 < CL && pos + 1 < P.nblk;
            const bool push2 = rank + 2 < CL && pos + 2 < P.nblk;
            const unsigned remote = push ? map_shared_rank(xs + P.block_rows, rank + 1) : 0u;
            const unsigned remote2 = push2 ? map_shared_rank(xs + P.block_rows, rank + 2) : 0u;
            solve_block<T, UPPER, KM, FIXED>(P, blk, in, scaled, sc, xs, out, remote, remote2, status);
        }
        if (active) finish_block(P, blk, in, scaled, sc, xs, out);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------
// Level-synchronous substitution (the reference's USE_LEVEL variant,
// src/ilu_solver.cpp:482-511, src/subtree.hpp:516-575): the rows of one level of the
// dependency DAG are solved by all warps of the grid at once, without waits, and a grid
// barrier separates consecutive levels.  Launched cooperatively (all CTAs resident).
// Packed like PackedTri with one lane per row, but tasks never straddle two levels:
// ltask[l] .. ltask[l + 1] are the tasks of level l.  Dependencies are read at L2 (ld.cg):
// they were written by other SMs before the barrier.  Operations per row as the other
// kernels (L ascending, U descending, FP64 division / FP32 reciprocal): identical results.
// ---------------------------------------------------------------------------------

// Grid barrier over all CTAs of a cooperative launch: bar[0] arrivals, bar[1] generation.
// The last CTA to arrive resets the count and advances the generation; the others wait
// (bounded) for the generation to change.  Returns false when the wait gave up.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        s_ok = 1;
        const int gen = ld_acquire(reinterpret_cast<const int*>(bar + 1));
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(bar, 0u);
            __threadfence();
            st_release(reinterpret_cast<int*>(bar + 1), gen + 1);
        } else {
            WaitBudget wb;
            while (ld_acquire(reinterpret_cast<const int*>(bar + 1)) == gen) {
                if (wb.expired(status)) {
                    atomicExch(status + kStatusTimeout, 1);
                    s_ok = 0;
                    break;
                }
            }
        }
    }
    __syncthreads();
    return s_ok != 0;
}

template <class T, bool UPPER>
__global__ void __launch_bounds__(kSolveWarps * kWarp)
    sptrsv_levelsync_kernel(PackedTri<T> P, const int* __restrict__ ltask, int nlev, T* in, const double* scale,
                            T* out, unsigned* bar, int* status, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    const int lane = threadIdx.x & 31;
    const int gw = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int l = 0; l < nlev; ++l) {
        for (int t = ltask[l] + gw; t < ltask[l + 1]; t += nw) {
            const int row = P.rows[t * kWarp + lane];
            if (row < 0) continue;
            T acc = in[row];
            if (scaled) {
                acc = acc * sc;
                in[row] = acc;
            }
            const int off = P.off[t];
            const int K = P.len[t];
            for (int k = 0; k < K; ++k) {
                const int c = P.cols[off + k * kWarp + lane];
                if (c >= 0) acc = fma(-P.vals[off + k * kWarp + lane], __ldcg(out + c), acc);
            }
            if (UPPER) {
                const T d = P.dvals[t * kWarp + lane];
                acc = sizeof(T) == 8 ? acc / d : acc * d;  // FP32: d holds 1 / u_ii
            }
            out[row] = Sentinel<T>::canon(acc);
        }
        if (l + 1 < nlev && !grid_barrier(bar, status)) return;
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
