// Lane-per-row sync-free ILU factorisation for factors with short rows (at most
// kLaneRowMax entries), the counterpart of the lane-per-row triangular sweeps.
//
// Each lane factorises one row with the reference's up-looking row elimination
// (src/ilu_solver.cpp:553-589): for every pivot column k of its strict-lower part in
// ascending order, l_jk = a_jk / u_kk, then a_jc -= u_kc * l_jk for every column c of
// row k's strict-upper part that lies in row j's pattern.  The operations and their order
// per entry are those of the warp-per-row kernel (ilu_factor_kernel): identical factors.
//
// Publication is value-as-flag: a finished row k writes u_kk and its strict-upper entries
// into its slots of `pub` (all at the sentinel before the launch); a row waiting for pivot
// k polls exactly the slots it needs (u_kk and the u_kc of its updates).  No fence or
// ready flag sits on the dependency chain.  Rows are taken in level order by 32-row
// tickets (one lane per row); a lane only waits for rows with smaller tickets, lanes of a
// warp progress independently in rounds, so the grid needs no co-residency; every wait is
// bounded (WaitBudget).  A row is staged in the warp's shared memory (32 x kLaneRowMax
// values) because updates address its entries by position.
#pragma once

#include "common.cuh"
#include "ilu_kernels.cuh"

namespace gb300 {

constexpr int kLaneRowMax = 16;     // most entries of a row handled by this kernel
constexpr int kLaneFactWarps = 8;   // warps per CTA

// Update lists of the lower entries: for lower entry p of row j (pivot k = ci[p]),
// upd[upd_ptr[p] .. upd_ptr[p+1]) holds (offset of the updated entry in row j,
// pub slot of u_kc) pairs in ascending column c.
struct LaneFactor {
    int n = 0;
    int ntask = 0;
    const int* rows = nullptr;     // [32 * ntask] row of each lane, -1 for padding (level order)
    const int* rp = nullptr;
    const int* ci = nullptr;
    const int* diag = nullptr;
    const int* pub_off = nullptr;  // [n] first pub slot of each row (u_kk, then its upper entries)
    const int* upd_ptr = nullptr;  // [nnz + 1]
    const int2* upd = nullptr;     // (offset in row j, pub slot)
};

static __global__ void __launch_bounds__(kLaneFactWarps * kWarp)
    ilu_factor_lane_kernel(LaneFactor F, double* lu, const double* __restrict__ shift, double* pub, unsigned* counter,
                           int* status) {
    __shared__ double srow[kLaneFactWarps][kWarp][kLaneRowMax + 1];  // +1: no bank conflicts between lanes
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    double* s = srow[w][lane];
    int q = draw_ticket(counter, F.ntask, lane);
    while (q < F.ntask) {
        const int qn = draw_ticket(counter, F.ntask, lane);
        const int j = F.rows[q * kWarp + lane];
        int b = 0, dl = 0, e = 0, t = 0;
        bool done = j < 0;
        if (!done) {
            b = F.rp[j];
            dl = F.diag[j];
            e = F.rp[j + 1];
            for (int p = b; p < e; ++p) s[p - b] = __ldcg(lu + p);
            if (shift != nullptr) s[dl - b] += shift[j];
            t = b;
        }
        WaitBudget wb;
        while (!__all_sync(0xffffffffu, done)) {
            if (!done) {
                // advance through every pivot whose values are published
                while (t < dl) {
                    const int k = F.ci[t];
                    const double ukk = ld_relaxed(pub + F.pub_off[k]);
                    if (Sentinel<double>::is(ukk)) break;
                    const int u0 = F.upd_ptr[t], u1 = F.upd_ptr[t + 1];
                    bool ready = true;
                    for (int u = u0; u < u1 && ready; ++u) ready = !Sentinel<double>::is(ld_relaxed(pub + F.upd[u].y));
                    if (!ready) break;
                    const double l = s[t - b] / ukk;
                    s[t - b] = l;
                    for (int u = u0; u < u1; ++u) {
                        const int2 d = F.upd[u];
                        s[d.x] = fma(-ld_relaxed(pub + d.y), l, s[d.x]);
                    }
                    ++t;
                }
                if (t == dl) {
                    for (int p = b; p < e; ++p) lu[p] = s[p - b];
                    const double ujj = s[dl - b];
                    if (!(fabs(ujj) > 0.0) || !isfinite(ujj)) {
                        atomicAdd(status + kStatusBreakdowns, 1);
                        atomicMin(status + kStatusFirstBreakdown, j);
                    }
                    // publish the upper entries, then u_jj (each slot is its own flag)
                    const int po = F.pub_off[j];
                    for (int p = dl + 1; p < e; ++p) st_relaxed(pub + po + (p - dl), Sentinel<double>::canon(s[p - b]));
                    st_relaxed(pub + po, Sentinel<double>::canon(ujj));
                    done = true;
                }
            }
            if (wb.expired(status)) {
                if (!done) atomicExch(status + kStatusTimeout, 1);
                break;
            }
        }
        q = qn;
    }
}

}  // namespace gb300
