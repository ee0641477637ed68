// lljbash::IluSolver on GB300: host analysis of the pattern (bit-exact with the
// reference), sync-free ILU factorisation and sync-free triangular substitution on the
// device.  Replaces src/ilu_solver.cpp (SetupMatrix :225-373, Factorize :616-671,
// Substitute :736-831).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <array>
#include <climits>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "analysis.hpp"
#include "common.cuh"
#include "device_util.hpp"
#include "ilu_impl.hpp"
#include "ilu_kernels.cuh"
#include "mlp.cuh"
#include "tree_schedule.hpp"

namespace gb300 {

// Lanes per row of the level-ordered kernels for a triangle whose rows have at most
// `kmax` entries: 1 while a row fits one lane's registers, else the smallest group that
// holds kmax entries in kLaneEntries per lane; rows too long for kRowLanesMax lanes keep
// one lane per row (blocking path).  `requested`: 1 forces one lane per row, > 1 raises
// the group to at least that many lanes.
static int row_lanes_for(int kmax, int requested) {
    if (requested == 1) return 1;
    int g = 1;
    while (g < kRowLanesMax && ceil_div(kmax, g) > kLaneEntries) g *= 2;
    if (ceil_div(kmax, g) > kLaneEntries) return 1;
    while (g < requested && g < kRowLanesMax) g *= 2;
    return g;
}

// Position of column c in the sorted ci[lo, hi), -1 if absent.
static int find_sorted_host(const int* ci, int lo, int hi, int c) {
    const int* it = std::lower_bound(ci + lo, ci + hi, c);
    return (it != ci + hi && *it == c) ? static_cast<int>(it - ci) : -1;
}

// Host construction of a packed factor from a schedule `order` (rows in level order),
// `group` lanes per row (PackedTri layout).  lower: entries [rp[r], diag[r]) ascending;
// upper: entries (diag[r], rp[r+1]) descending plus the diagonal position.
static void build_level_pack(int n, const int* rp, const int* ci, const std::vector<int>& diag,
                             const std::vector<int>& order, bool lower, int group, LevelPack& P, cudaStream_t s) {
    const int per_task = kWarp / group;  // rows per task
    const int ntask = ceil_div(n, per_task);
    std::vector<int> rows(static_cast<size_t>(ntask) * kWarp, -1);
    std::vector<int> off(ntask), len(ntask);
    std::vector<int> dsrc(lower ? 0 : static_cast<size_t>(ntask) * kWarp, -1);
    auto count = [&](int r) { return lower ? diag[r] - rp[r] : rp[r + 1] - diag[r] - 1; };
    long long slots = 0;
    for (int t = 0; t < ntask; ++t) {
        int k = 0;
        for (int i = 0; i < per_task; ++i) {
            const long long q = static_cast<long long>(t) * per_task + i;
            if (q >= n) break;
            const int r = order[q];
            k = std::max(k, count(r));
            for (int j = 0; j < group; ++j) {
                rows[static_cast<size_t>(t) * kWarp + i * group + j] = r;
                if (!lower) dsrc[static_cast<size_t>(t) * kWarp + i * group + j] = diag[r];
            }
        }
        off[t] = static_cast<int>(slots);
        len[t] = ceil_div(k, group);
        if (group > 1 && len[t] > kLaneEntries) throw std::runtime_error("lane group too small for the row length");
        slots += static_cast<long long>(len[t]) * kWarp;
        if (slots > INT_MAX) throw std::runtime_error("triangular factor too large for 32-bit slot offsets");
    }
    std::vector<int> cols(static_cast<size_t>(slots), -1), src(static_cast<size_t>(slots), -1);
    for (int t = 0; t < ntask; ++t) {
        for (int i = 0; i < per_task; ++i) {
            const long long q = static_cast<long long>(t) * per_task + i;
            if (q >= n) break;
            const int r = order[q];
            int e = 0;  // entry index within the row, in accumulation order
            auto put = [&](int p) {
                const int l = i * group + e / len[t];
                const size_t sidx = static_cast<size_t>(off[t]) + static_cast<size_t>(e % len[t]) * kWarp + l;
                cols[sidx] = ci[p];
                src[sidx] = p;
                ++e;
            };
            if (lower) {
                for (int p = rp[r]; p < diag[r]; ++p) put(p);
            } else {
                for (int p = rp[r + 1] - 1; p > diag[r]; --p) put(p);
            }
        }
    }
    P.ntask = ntask;
    P.group = group;
    P.slots = slots;
    P.rows.upload(rows.data(), rows.size(), s);
    P.off.upload(off.data(), off.size(), s);
    P.len.upload(len.data(), len.size(), s);
    P.cols.upload(cols.data(), cols.size(), s);
    P.src.upload(src.data(), src.size(), s);
    if (!lower) P.dsrc.upload(dsrc.data(), dsrc.size(), s);
    P.v64.reserve(static_cast<size_t>(slots));
    P.v32.reserve(static_cast<size_t>(slots));
    if (!lower) {
        P.d64.reserve(static_cast<size_t>(ntask) * kWarp);
        P.d32.reserve(static_cast<size_t>(ntask) * kWarp);
    }
    // host vectors must outlive the asynchronous copies
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
}

// Host construction of a level-synchronous pack: rows in level order (order / lptr:
// the level sets), one lane per row, 32 rows per task, a new task at every level
// boundary; ltask[l] = first task of level l.  Entry layout as build_level_pack.
static void build_levelsync_pack(int n, const int* rp, const int* ci, const std::vector<int>& diag,
                                 const std::vector<int>& order, const std::vector<int>& lptr, int nlev, bool lower,
                                 LevelPack& P, cudaStream_t s) {
    std::vector<int> rows, off, len, dsrc, ltask(static_cast<size_t>(nlev) + 1, 0);
    auto count = [&](int r) { return lower ? diag[r] - rp[r] : rp[r + 1] - diag[r] - 1; };
    long long slots = 0;
    for (int l = 0; l < nlev; ++l) {
        ltask[static_cast<size_t>(l)] = static_cast<int>(off.size());
        for (int q0 = lptr[static_cast<size_t>(l)]; q0 < lptr[static_cast<size_t>(l) + 1]; q0 += kWarp) {
            int K = 0;
            for (int u = 0; u < kWarp; ++u) {
                const int q = q0 + u;
                const int r = q < lptr[static_cast<size_t>(l) + 1] ? order[static_cast<size_t>(q)] : -1;
                rows.push_back(r);
                if (!lower) dsrc.push_back(r >= 0 ? diag[r] : -1);
                if (r >= 0) K = std::max(K, count(r));
            }
            off.push_back(static_cast<int>(slots));
            len.push_back(K);
            slots += static_cast<long long>(K) * kWarp;
            if (slots > INT_MAX) throw std::runtime_error("triangular factor too large for 32-bit slot offsets");
        }
    }
    ltask[static_cast<size_t>(nlev)] = static_cast<int>(off.size());
    const int ntask = static_cast<int>(off.size());
    std::vector<int> cols(static_cast<size_t>(slots), -1), src(static_cast<size_t>(slots), -1);
    for (int t = 0; t < ntask; ++t)
        for (int l = 0; l < kWarp; ++l) {
            const int r = rows[static_cast<size_t>(t) * kWarp + l];
            if (r < 0) continue;
            int k = 0;
            auto put = [&](int p) {
                const size_t sidx = static_cast<size_t>(off[static_cast<size_t>(t)]) + static_cast<size_t>(k++) * kWarp + l;
                cols[sidx] = ci[p];
                src[sidx] = p;
            };
            if (lower) {
                for (int p = rp[r]; p < diag[r]; ++p) put(p);
            } else {
                for (int p = rp[r + 1] - 1; p > diag[r]; --p) put(p);
            }
        }
    P.ntask = ntask;
    P.group = 1;
    P.slots = slots;
    P.nlev = nlev;
    P.rows.upload(rows.data(), rows.size(), s);
    P.off.upload(off.data(), off.size(), s);
    P.len.upload(len.data(), len.size(), s);
    P.cols.upload(cols.data(), cols.size(), s);
    P.src.upload(src.data(), src.size(), s);
    P.ltask.upload(ltask.data(), ltask.size(), s);
    if (!lower) P.dsrc.upload(dsrc.data(), dsrc.size(), s);
    P.v64.reserve(static_cast<size_t>(std::max<long long>(slots, 1)));
    P.v32.reserve(static_cast<size_t>(std::max<long long>(slots, 1)));
    if (!lower) {
        P.d64.reserve(static_cast<size_t>(std::max(ntask, 1)) * kWarp);
        P.d32.reserve(static_cast<size_t>(std::max(ntask, 1)) * kWarp);
    }
    GB_CUDA_CHECK(cudaStreamSynchronize(s));  // host vectors must outlive the copies
}

template <class T, bool UPPER>
static void launch_levelsync(const LevelPack& P, int grid, cudaStream_t s, T* in, const double* scale, T* out,
                             unsigned* bar, int* status, const int* gate, int step) {
    if (P.ntask == 0) return;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    cfg.blockDim = dim3(kSolveWarps * kWarp);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CUDA_CHECK(cudaLaunchKernelEx(&cfg, sptrsv_levelsync_kernel<T, UPPER>, P.view<T>(),
                                     static_cast<const int*>(P.ltask.get()), P.nlev, in, scale, out, bar, status, gate,
                                     step));
}

// Host construction of the lane-per-row factorisation (factor_lane.cuh): 32-row tasks in
// the order `order` (level order: topological), every row's pub slots (u_kk, then its
// strict-upper entries), and for every strict-lower entry p of row j (pivot k) the
// updates (offset of c in row j, pub slot of u_kc) for c in row k's strict-upper part and
// in row j's pattern, ascending c.  False when a row is longer than kLaneRowMax.
static bool build_lane_factor(int n, const int* rp, const int* ci, const std::vector<int>& diag,
                              const std::vector<int>& order, lljbash::IluSolver::Impl& im, cudaStream_t s) {
    for (int r = 0; r < n; ++r)
        if (rp[r + 1] - rp[r] > kLaneRowMax) return false;
    const long long nnz = rp[n];
    std::vector<int> pub_off(static_cast<size_t>(n));
    long long slots = 0;
    for (int r = 0; r < n; ++r) {
        pub_off[static_cast<size_t>(r)] = static_cast<int>(slots);
        slots += rp[r + 1] - diag[static_cast<size_t>(r)];  // u_rr and the strict-upper entries
    }
    if (slots > INT_MAX) return false;
    std::vector<int> upd_ptr(static_cast<size_t>(nnz) + 1, 0);
    std::vector<int2> upd;
    for (int j = 0; j < n; ++j) {
        for (int p = rp[j]; p < rp[j + 1]; ++p) {
            upd_ptr[static_cast<size_t>(p)] = static_cast<int>(upd.size());
            if (p >= diag[static_cast<size_t>(j)]) continue;
            const int k = ci[p];
            for (int qk = diag[static_cast<size_t>(k)] + 1; qk < rp[k + 1]; ++qk) {
                const int pos = find_sorted_host(ci, rp[j], rp[j + 1], ci[qk]);
                if (pos >= 0)
                    upd.push_back(make_int2(pos - rp[j], pub_off[static_cast<size_t>(k)] + (qk - diag[static_cast<size_t>(k)])));
            }
        }
    }
    upd_ptr[static_cast<size_t>(nnz)] = static_cast<int>(upd.size());
    const int ntask = ceil_div(n, kWarp);
    std::vector<int> rows(static_cast<size_t>(ntask) * kWarp, -1);
    for (int q = 0; q < n; ++q) rows[static_cast<size_t>(q)] = order[static_cast<size_t>(q)];
    im.lf_rows.upload(rows.data(), rows.size(), s);
    im.lf_pub_off.upload(pub_off.data(), pub_off.size(), s);
    im.lf_upd_ptr.upload(upd_ptr.data(), upd_ptr.size(), s);
    if (upd.empty()) upd.push_back(make_int2(0, 0));
    im.lf_upd.upload(upd.data(), upd.size(), s);
    im.lf_pub.reserve(static_cast<size_t>(std::max<long long>(slots, 1)));
    im.lf_pub_len = slots;
    im.lf_ntask = ntask;
    // one CTA (8 warps) per SM, as the level-ordered sweeps: more warps only poll further
    // ahead of the dependency chain and slow its L2 handoffs
    im.grid_lane_fact = std::max(1, std::min(im.dev.sms, ntask));
    GB_CUDA_CHECK(cudaStreamSynchronize(s));  // host vectors must outlive the copies
    return true;
}

// Level-ordered sweeps, dispatched on the factor's lanes per row.
template <class T>
static void launch_level_lower(const LevelPack& L, int grid, int threads, cudaStream_t s, T* b, const double* scale,
                               T* y, unsigned* counter, int* status, const int* gate, int step) {
    const PackedTri<T> P = L.view<T>();
    switch (L.group) {
        case 1: sptrsv_lower_kernel<T, 1><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        case 2: sptrsv_lower_kernel<T, 2><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        case 4: sptrsv_lower_kernel<T, 4><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        case 8: sptrsv_lower_kernel<T, 8><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        case 16: sptrsv_lower_kernel<T, 16><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        case 32: sptrsv_lower_kernel<T, 32><<<grid, threads, 0, s>>>(P, b, scale, y, counter, status, gate, step); break;
        default: throw std::runtime_error("unsupported lanes per row");
    }
}

template <class T>
static void launch_level_upper(const LevelPack& U, int grid, int threads, cudaStream_t s, T* y, T* x,
                               unsigned* counter, int* status, const int* gate, int step) {
    const PackedTri<T> P = U.view<T>();
    switch (U.group) {
        case 1: sptrsv_upper_kernel<T, 1><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        case 2: sptrsv_upper_kernel<T, 2><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        case 4: sptrsv_upper_kernel<T, 4><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        case 8: sptrsv_upper_kernel<T, 8><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        case 16: sptrsv_upper_kernel<T, 16><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        case 32: sptrsv_upper_kernel<T, 32><<<grid, threads, 0, s>>>(P, y, x, counter, status, gate, step); break;
        default: throw std::runtime_error("unsupported lanes per row");
    }
}

static void gather_level_pack(const LevelPack& P, bool lower, const double* lu, cudaStream_t s, int sms) {
    const int threads = 256;
    auto grid_for = [&](long long count) {
        long long g = ceil_div<long long>(count, threads);
        return static_cast<int>(std::max<long long>(1, std::min<long long>(g, 8LL * sms)));
    };
    if (P.slots > 0) {
        pack_gather_kernel<double><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v64.get());
        pack_gather_kernel<float><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v32.get());
    }
    if (!lower) {
        const long long nd = static_cast<long long>(P.ntask) * kWarp;
        pack_gather_kernel<double><<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d64.get());
        pack_gather_recip_kernel<<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d32.get());
    }
    GB_CUDA_CHECK(cudaGetLastError());
}

// Block-internal levels of rows [lo, hi): dependencies on rows outside the block do
// not count.  depth[r - lo] receives the level of row r; returns the level count.
static int block_levels(int lo, int hi, bool lower, const int* rp, const int* ci, const std::vector<int>& diag,
                        std::vector<int>& depth) {
    int nlev = 0;
    for (int s2 = 0; s2 < hi - lo; ++s2) {
        const int r = lower ? lo + s2 : hi - 1 - s2;
        int d = 0;
        const int b0 = lower ? rp[r] : diag[r] + 1;
        const int b1 = lower ? diag[r] : rp[r + 1];
        for (int p = b0; p < b1; ++p) {
            const int col = ci[p];
            if (col >= lo && col < hi) d = std::max(d, depth[col - lo] + 1);
        }
        depth[r - lo] = d;
        nlev = std::max(nlev, d + 1);
    }
    return nlev;
}

// ---- choice of the substitution schedule ----------------------------------------
// Model constants, measured on GB300 with the 128^3 7-point and 256^2 5-point factors:
// one block-internal level of the block-local kernel, one cross-block handoff, and the
// level-ordered kernel's cost per level (a fixed handoff plus a term per row).
constexpr double kModelBlockLevelUs = 0.35;
constexpr double kModelBlockHopUs = 2.0;
constexpr double kModelClusterHopUs = 0.5;  // handoff into a halo of the same cluster
constexpr double kModelLevelUs = 0.6;
constexpr double kModelLevelRowUs = 9e-5;

// Plane size of a matrix from a structured grid in natural order: the most frequent
// offset r - c of the strict-lower entries among those at least half the largest one
// (nx * ny for a 3-D grid, nx for a 2-D one), provided it occurs in a quarter of the
// rows; 0 otherwise.
static int plane_offset(int n, const int* rp, const int* ci, const std::vector<int>& diag) {
    int max_off = 0;
    for (int r = 0; r < n; ++r)
        if (diag[r] > rp[r]) max_off = std::max(max_off, r - ci[rp[r]]);
    if (max_off <= 0) return 0;
    const int lo = (max_off + 1) / 2;
    std::vector<int> count(static_cast<size_t>(max_off - lo) + 1, 0);
    for (int r = 0; r < n; ++r)
        for (int p = rp[r]; p < diag[r]; ++p)
            if (r - ci[p] >= lo) ++count[r - ci[p] - lo];
    int best = 0, best_cnt = 0;
    for (int o = lo; o <= max_off; ++o) {
        if (count[o - lo] > best_cnt) {
            best_cnt = count[o - lo];
            best = o;
        }
    }
    return 4ll * best_cnt >= n ? best : 0;
}

// Modelled critical path (us) of the forward sweep with the block-local kernel and
// blocks of B rows: every row finishes one block-level after its latest dependency,
// plus a handoff when that dependency lies in another block.
// R: CTAs resident at once; block b starts only once block b - R is done (blocks go to
// CTAs by tickets in order), which bounds schedules with more blocks than CTAs.
static double block_schedule_model(int n, const int* rp, const int* ci, const std::vector<int>& diag, int B, int cl,
                                   int R) {
    std::vector<double> t(static_cast<size_t>(n));
    std::vector<double> bend(static_cast<size_t>(ceil_div(n, B)), 0.0);
    double T = 0.0;
    for (int r = 0; r < n; ++r) {
        const int br = r / B;
        double m = br >= R ? bend[static_cast<size_t>(br - R)] : 0.0;
        for (int p = rp[r]; p < diag[r]; ++p) {
            const int c = ci[p];
            const int bc = c / B;
            const double hop = bc == br ? 0.0
                               : (cl > 1 && br - bc <= kHaloDepth && br / cl == bc / cl) ? kModelClusterHopUs
                                                                                          : kModelBlockHopUs;
            m = std::max(m, t[c] + hop);
        }
        t[r] = m + kModelBlockLevelUs;
        bend[static_cast<size_t>(br)] = std::max(bend[static_cast<size_t>(br)], t[r]);
        T = std::max(T, t[r]);
    }
    return T;
}

// Halo rows a CTA of the cluster variant needs: the most distinct rows that a block reads
// from the blocks 1 .. kHaloDepth positions before it in its cluster (lower triangle).
static int halo_rows_needed(int n, const int* rp, const int* ci, const std::vector<int>& diag, int B, int cl) {
    int H = 0;
    std::vector<int> mark(static_cast<size_t>(n), -1);
    for (int b = 1; b * static_cast<long long>(B) < n; ++b) {
        if (b % cl == 0) continue;
        int cnt = 0;
        const int lo = b * B, hi = std::min(n, lo + B);
        const int src_lo = std::max((b / cl) * cl, b - kHaloDepth) * B;
        for (int r = lo; r < hi; ++r)
            for (int p = rp[r]; p < diag[r]; ++p) {
                const int c = ci[p];
                if (c >= src_lo && c < lo && mark[c] != b) {
                    mark[c] = b;
                    ++cnt;
                }
            }
        H = std::max(H, cnt);
    }
    return H;
}

// Block-local schedules for values of `elem` bytes, cheapest first by the cost model
// (block_schedule_model), those the model expects to beat the level-ordered kernel only
// (empty: keep the level kernel).  Candidates: multiples of the plane size that fit in
// shared memory, each with clusters (block + halo must fit) and without.  Rows with more than kLaneEntries entries take the block kernel's slow path,
// so such factors keep the level kernel.
struct BlockChoice {
    int rows;
    int cl;
    double us;
};

static std::vector<BlockChoice> choose_block_schedules(int n, const int* rp, const int* ci,
                                                       const std::vector<int>& diag, int nlev, int elem,
                                                       size_t smem_budget, size_t smem_per_sm, int sms) {
    std::vector<BlockChoice> out;
    if (n <= 0) return out;
    int kmax = 0;
    for (int r = 0; r < n; ++r) kmax = std::max({kmax, diag[r] - rp[r], rp[r + 1] - diag[r] - 1});
    if (kmax > kLaneEntries) return out;
    const long long max_rows = static_cast<long long>(smem_budget / static_cast<size_t>(elem));
    const double level_us =
        std::max(1, nlev) * (kModelLevelUs + kModelLevelRowUs * static_cast<double>(n) / std::max(1, nlev));
    // resident CTAs: by shared memory per SM; clusters of cl CTAs sit within one GPC,
    // and about 80% of the SMs can hold whole clusters of 8 (15 on 152 SMs, measured)
    auto resident = [&](long long bytes, int cl) {
        const int per_sm = std::max<int>(1, static_cast<int>(smem_per_sm / static_cast<size_t>(std::max<long long>(bytes, 1))));
        return cl > 1 ? std::max(cl, (sms * 4 / 5 / cl) * cl) * per_sm : sms * per_sm;
    };
    if (n <= max_rows) {
        const double us = block_schedule_model(n, rp, ci, diag, n, 0, 1);
        if (us < level_us) out.push_back({n, 0, us});
        return out;
    }
    const int P = plane_offset(n, rp, ci, diag);
    if (P <= 0) return out;
    // (Half-plane blocks, whose halos reach two positions back, were tried for FP64 on
    // 128^3, where a plane plus a one-plane halo does not fit: twice the blocks, more
    // than stay resident at once, and 7% slower sweeps than one-plane blocks without
    // clusters; they stay available through LLJBASH_ILU_OPT_BLOCK_ROWS.)
    std::vector<long long> sizes;
    for (long long B = P; B <= max_rows && B < n; B *= 2) sizes.push_back(B);
    for (long long B : sizes) {
        if (B > max_rows || B >= n) continue;
        for (int cl : {kBlockClusterBig, kBlockCluster, 0}) {
            const long long H = cl > 0 ? halo_rows_needed(n, rp, ci, diag, static_cast<int>(B), cl) : 0;
            if (B + H > max_rows) continue;
            const int R = resident((B + H) * elem, cl);
            const double us = block_schedule_model(n, rp, ci, diag, static_cast<int>(B), cl, R);
            if (us < level_us) out.push_back({static_cast<int>(B), cl, us});
        }
    }
    std::sort(out.begin(), out.end(), [](const BlockChoice& a, const BlockChoice& b) { return a.us < b.us; });
    return out;
}

// Entries per lane held in registers by the block-local kernel for rows of at most
// `row_max` entries (the kernel specialisations: 3, 4, kLaneEntries).
static int block_km_for(int row_max) { return row_max <= 3 ? 3 : (row_max <= 4 ? 4 : kLaneEntries); }

// Host construction of a block-local packed factor (see BlockTri): contiguous blocks of
// `block_rows` rows; inside a block the rows in block-internal level order (ascending row
// index inside a level), 32 to a task, tasks never crossing a block.  lower: entries
// [rp[r], diag[r]) ascending; upper: entries (diag[r], rp[r+1]) descending plus the
// diagonal position.  A value type is marked as fitting when the largest block's
// solution fits in `smem_budget` bytes of shared memory.
static void build_block_pack(int n, const int* rp, const int* ci, const std::vector<int>& diag, bool lower,
                             int block_rows, int elem, size_t smem_budget, int cl, BlockPack& P, cudaStream_t s) {
    const int S = std::max(1, std::min(block_rows, std::max(n, 1)));
    const int nblk = n > 0 ? ceil_div(n, S) : 0;
    auto ebeg = [&](int r) { return lower ? rp[r] : diag[r] + 1; };
    auto eend = [&](int r) { return lower ? diag[r] : rp[r + 1]; };
    std::vector<int> blk_row(static_cast<size_t>(nblk) + 1), blk_task(static_cast<size_t>(nblk) + 1, 0);
    std::vector<int> rows, off, len, dsrc;
    std::vector<int> depth(static_cast<size_t>(S)), cnt, ord;
    long long slots = 0;
    int max_level_tasks = 1;
    // Factors whose rows fit a lane's registers get one task length for all tasks: the
    // register count of the kernel that solves them (block_km_for), so that task t's
    // slots start at t * stride * 32 and the kernel's loops have compile-time bounds.
    int row_max = 0;
    for (int r = 0; r < n; ++r) row_max = std::max(row_max, eend(r) - ebeg(r));
    const int stride = row_max <= kLaneEntries ? block_km_for(row_max) : 0;
    for (int c = 0; c < nblk; ++c) {
        const int lo = c * S;
        const int hi = std::min(n, lo + S);
        blk_row[c] = lo;
        blk_task[c] = static_cast<int>(off.size());
        const int nlev = block_levels(lo, hi, lower, rp, ci, diag, depth);
        cnt.assign(static_cast<size_t>(nlev) + 1, 0);
        for (int r = lo; r < hi; ++r) ++cnt[depth[r - lo] + 1];
        for (int l = 0; l < nlev; ++l) {
            max_level_tasks = std::max(max_level_tasks, ceil_div(cnt[l + 1], kWarp));
            cnt[l + 1] += cnt[l];
        }
        ord.assign(static_cast<size_t>(hi - lo), 0);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int r = lo; r < hi; ++r) ord[fill[depth[r - lo]]++] = r;
        // tasks never straddle two levels: a task's rows are independent of each other,
        // so a warp finishes its task in one level-time
        for (int l = 0; l < nlev; ++l) {
            for (int q0 = cnt[l]; q0 < cnt[l + 1]; q0 += kWarp) {
                int K = 0;
                for (int u = 0; u < kWarp; ++u) {
                    const int q = q0 + u;
                    if (q < cnt[l + 1]) {
                        const int r = ord[q];
                        rows.push_back(r);
                        K = std::max(K, eend(r) - ebeg(r));
                        if (!lower) dsrc.push_back(diag[r]);
                    } else {
                        rows.push_back(-1);
                        if (!lower) dsrc.push_back(-1);
                    }
                }
                if (stride > 0) K = stride;
                off.push_back(static_cast<int>(slots));
                len.push_back(K);
                slots += static_cast<long long>(K) * kWarp;
                if (slots > INT_MAX) throw std::runtime_error("triangular factor too large for 32-bit slot offsets");
            }
        }
    }
    blk_row[nblk] = n;
    blk_task[nblk] = static_cast<int>(off.size());
    const int ntask = static_cast<int>(off.size());
    std::vector<int> codes(static_cast<size_t>(slots), -1), src(static_cast<size_t>(slots), -1);
    for (int t = 0; t < ntask; ++t) {
        for (int l = 0; l < kWarp; ++l) {
            const int r = rows[static_cast<size_t>(t) * kWarp + l];
            if (r < 0) continue;
            const int lo = (r / S) * S;
            const int hi = std::min(n, lo + S);
            int k = 0;
            auto put = [&](int p) {
                const size_t sidx = static_cast<size_t>(off[t]) + static_cast<size_t>(k) * kWarp + l;
                const int col = ci[p];
                codes[sidx] = (col >= lo && col < hi) ? -2 - (col - lo) : col;
                src[sidx] = p;
                ++k;
            };
            if (lower) {
                for (int p = rp[r]; p < diag[r]; ++p) put(p);
            } else {
                for (int p = rp[r + 1] - 1; p > diag[r]; --p) put(p);
            }
        }
    }
    P.nblk = nblk;
    P.block_rows = S;
    P.ntask = ntask;
    P.stride = stride;
    P.kmax = len.empty() ? 0 : *std::max_element(len.begin(), len.end());
    P.slots = slots;
    // two tasks in flight per level of the widest block level, 4 .. kBlockWarpsMax warps
    P.threads = kWarp * std::max(4, std::min(kBlockWarpsMax, 2 * max_level_tasks));
    // Cluster halos (cl > 0): the block at processing position p (ascending blocks for L,
    // descending for U) reads the rows of positions p - 1 .. p - kHaloDepth that it depends
    // on from its shared-memory halo when those positions are in its cluster
    // (p - d >= cl * (p / cl)).  Halo slots: the rows of p - 1 in ascending row order, then
    // those of p - 2; the producer's rows carry their slot for the block d positions
    // ahead in `exps` (kPubSlotBits bits per distance).
    std::vector<int> exps(rows.size(), 0);
    int H = 0;
    bool halo_ok = true;
    if (cl > 1) {
        std::vector<int> slot_of(static_cast<size_t>(S), -1), used;
        for (int pos = 1; pos < nblk; ++pos) {
            if (pos % cl == 0) continue;
            const int cb = lower ? pos : nblk - 1 - pos;
            int base = 0;
            for (int d = 1; d <= kHaloDepth && pos % cl >= d; ++d) {
                const int pb = lower ? pos - d : nblk - 1 - (pos - d);
                const int plo = blk_row[pb], phi = blk_row[pb + 1];
                used.clear();
                for (int t = blk_task[cb]; t < blk_task[cb + 1]; ++t)
                    for (long long q = off[t]; q < off[t] + static_cast<long long>(len[t]) * kWarp; ++q) {
                        const int col = codes[static_cast<size_t>(q)];
                        if (col >= plo && col < phi && slot_of[col - plo] < 0) {
                            slot_of[col - plo] = 0;
                            used.push_back(col);
                        }
                    }
                std::sort(used.begin(), used.end());
                for (size_t k = 0; k < used.size(); ++k) slot_of[used[k] - plo] = base + static_cast<int>(k);
                for (int t = blk_task[cb]; t < blk_task[cb + 1]; ++t)
                    for (long long q = off[t]; q < off[t] + static_cast<long long>(len[t]) * kWarp; ++q) {
                        int& code = codes[static_cast<size_t>(q)];
                        if (code >= plo && code < phi) code = -2 - (S + slot_of[code - plo]);
                    }
                for (int t = blk_task[pb]; t < blk_task[pb + 1]; ++t)
                    for (int l = 0; l < kWarp; ++l) {
                        const int r = rows[static_cast<size_t>(t) * kWarp + l];
                        if (r >= 0 && slot_of[r - plo] >= 0)
                            exps[static_cast<size_t>(t) * kWarp + l] |= (slot_of[r - plo] + 1) << (kPubSlotBits * (d - 1));
                    }
                for (int col : used) slot_of[col - plo] = -1;
                base += static_cast<int>(used.size());
            }
            H = std::max(H, base);
        }
        if (H >= (1 << kPubSlotBits) - 1) halo_ok = false;  // slots + 1 must fit their fields
    }
    // Per-row publication word (`pub`): bit kPubGlobal = some block reads the row through
    // L2 (a code >= 0 names it), so its value is stored to `out` the moment it is
    // computed; then for d = 1, 2 a field of kPubSlotBits bits = the halo slot + 1 of the
    // row in the CTA d positions ahead (0: none).  Rows without kPubGlobal reach `out` in
    // one coalesced copy when their block is done.
    {
        std::vector<unsigned char> global_read(static_cast<size_t>(n), 0);
        for (int code : codes)
            if (code >= 0) global_read[static_cast<size_t>(code)] = 1;
        for (size_t q = 0; q < rows.size(); ++q) {
            const int r = rows[q];
            if (r >= 0 && global_read[static_cast<size_t>(r)]) exps[q] |= kPubGlobal;
        }
    }
    P.cl = cl > 1 ? cl : 0;
    P.halo = H;
    P.elem = elem;
    P.smem = static_cast<size_t>(elem) * (static_cast<size_t>(S) + static_cast<size_t>(H));
    P.fits = P.smem <= smem_budget && halo_ok;
    P.exps.upload(exps.data(), exps.size(), s);
    P.blk_row.upload(blk_row.data(), blk_row.size(), s);
    P.blk_task.upload(blk_task.data(), blk_task.size(), s);
    P.rows.upload(rows.data(), rows.size(), s);
    P.off.upload(off.data(), off.size(), s);
    P.len.upload(len.data(), len.size(), s);
    P.codes.upload(codes.data(), codes.size(), s);
    P.src.upload(src.data(), src.size(), s);
    if (!lower) P.dsrc.upload(dsrc.data(), dsrc.size(), s);
    if (elem == 8) {
        P.v64.reserve(static_cast<size_t>(slots));
        if (!lower) P.d64.reserve(rows.size());
    } else {
        P.v32.reserve(static_cast<size_t>(slots));
        if (!lower) P.d32.reserve(rows.size());
    }
    // host vectors must outlive the asynchronous copies
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
}

static void gather_block(const BlockPack& P, bool lower, const double* lu, cudaStream_t s, int sms) {
    const int threads = 256;
    auto grid_for = [&](long long count) {
        long long g = ceil_div<long long>(count, threads);
        return static_cast<int>(std::max<long long>(1, std::min<long long>(g, 8LL * sms)));
    };
    if (P.slots > 0) {
        if (P.elem == 8)
            pack_gather_kernel<double><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v64.get());
        else
            pack_gather_kernel<float><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v32.get());
    }
    if (!lower && P.ntask > 0) {
        const long long nd = static_cast<long long>(P.ntask) * kWarp;
        if (P.elem == 8)
            pack_gather_kernel<double><<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d64.get());
        else
            pack_gather_recip_kernel<<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d32.get());
    }
    GB_CUDA_CHECK(cudaGetLastError());
}

// Raises the kernel's dynamic shared-memory limit to the pack's footprint for type T and
// records the number of resident CTAs.
// Launch configuration of the cluster variant (clusters of P.cl CTAs along x).
static cudaLaunchConfig_t cluster_launch_config(const BlockPack& P, int grid, size_t smem, cudaStream_t s,
                                                cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    cfg.blockDim = dim3(static_cast<unsigned>(P.threads));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(P.cl);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// Raises the kernel's dynamic shared-memory limit to the pack's footprint and records how
// many CTAs to launch: the resident CTAs (plain variant) or the resident clusters times
// the cluster size (cluster variant; 0 when a cluster cannot be scheduled).
template <class T, bool UPPER, int KM, bool FIXED>
static void configure_block_km(BlockPack& P, int sms) {
    const int bytes = static_cast<int>(std::max<size_t>(P.smem, 16));
    if (P.cl) {
        auto* kern = sptrsv_block_cluster_kernel<T, UPPER, KM, FIXED>;
        GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        // clusters above the portable 8 CTAs (clusters of 16: 2% faster 128^3 FP32 sweeps
        // than 8, fewer handoffs through L2); where they cannot be scheduled the
        // occupancy query below reports 0 and the next schedule candidate is used
        GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                           P.cl > kBlockCluster ? 1 : 0));
        const int nq = ceil_div(P.nblk, P.cl);
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = cluster_launch_config(P, nq * P.cl, static_cast<size_t>(bytes), nullptr, attr);
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            nclusters = 0;
        }
        P.grid = std::min(nclusters, nq) * P.cl;
        return;
    }
    GB_CUDA_CHECK(cudaFuncSetAttribute(sptrsv_block_kernel<T, UPPER, KM, FIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       bytes));
    int per_sm = 0;
    GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sptrsv_block_kernel<T, UPPER, KM, FIXED>, P.threads,
                                                               static_cast<size_t>(bytes)));
    P.grid = std::max(1, per_sm) * sms;
}

template <class T, bool UPPER>
static void configure_block(BlockPack& P, int sms) {
    if (P.stride == 3)
        configure_block_km<T, UPPER, 3, true>(P, sms);
    else if (P.stride == 4)
        configure_block_km<T, UPPER, 4, true>(P, sms);
    else if (P.stride == kLaneEntries)
        configure_block_km<T, UPPER, kLaneEntries, true>(P, sms);
    else
        configure_block_km<T, UPPER, kLaneEntries, false>(P, sms);
}

template <class T, bool UPPER, int KM, bool FIXED>
static void launch_block_km(const BlockPack& P, cudaStream_t s, T* in, const double* scale, T* out, unsigned* counter,
                            int* status, const int* gate, int step) {
    if (P.cl) {
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = cluster_launch_config(P, P.grid, P.smem, s, attr);
        GB_CUDA_CHECK(cudaLaunchKernelEx(&cfg, sptrsv_block_cluster_kernel<T, UPPER, KM, FIXED>, P.view<T>(), in, scale, out,
                                         counter, status, gate, step));
        return;
    }
    sptrsv_block_kernel<T, UPPER, KM, FIXED><<<std::min(P.grid, P.nblk), P.threads, P.smem, s>>>(P.view<T>(), in, scale, out,
                                                                                        counter, status, gate, step);
}

template <class T, bool UPPER>
static void launch_block(const BlockPack& P, cudaStream_t s, T* in, const double* scale, T* out, unsigned* counter,
                         int* status, const int* gate, int step) {
    if (P.nblk == 0) return;
    if (P.stride == 3)
        launch_block_km<T, UPPER, 3, true>(P, s, in, scale, out, counter, status, gate, step);
    else if (P.stride == 4)
        launch_block_km<T, UPPER, 4, true>(P, s, in, scale, out, counter, status, gate, step);
    else if (P.stride == kLaneEntries)
        launch_block_km<T, UPPER, kLaneEntries, true>(P, s, in, scale, out, counter, status, gate, step);
    else
        launch_block_km<T, UPPER, kLaneEntries, false>(P, s, in, scale, out, counter, status, gate, step);
}

template <class T>
static void fill_sentinel(T* p, long long n, cudaStream_t s, int sms) {
    if (n <= 0) return;
    const int threads = 256;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>(ceil_div<long long>(n, threads), 8LL * sms)));
    fill_sentinel_kernel<T><<<grid, threads, 0, s>>>(n, p);
    GB_CUDA_CHECK(cudaGetLastError());
}

// ---- structured-grid line-pipeline sweeps (line_sweep.cuh) ----------------------
// Grid shape of a factor pattern that is a full 7-point (3-D) or 5-point (2-D) stencil
// in natural order: strict-lower columns of row r = i + nx j + nx ny k exactly
// {r - nx ny (k > 0), r - nx (j > 0), r - 1 (i > 0)} and strict-upper columns exactly
// {r + 1 (i < nx - 1), r + nx (j < ny - 1), r + nx ny (k < nz - 1)}; a 2-D grid is
// ny = 1 with the line offset as the plane offset.  Returns false otherwise.
static bool detect_grid(int n, const int* rp, const int* ci, const std::vector<int>& diag, int& nx, int& ny,
                        int& nz) {
    if (n < 64) return false;
    // distinct strict-lower offsets (at most three)
    int offs[4];
    int no = 0;
    for (int r = 0; r < n && no <= 3; ++r)
        for (int p = rp[r]; p < diag[r] && no <= 3; ++p) {
            const int o = r - ci[p];
            bool seen = false;
            for (int t = 0; t < no; ++t) seen = seen || offs[t] == o;
            if (!seen) offs[no++] = o;
        }
    if (no < 2 || no > 3) return false;
    std::sort(offs, offs + no);
    if (offs[0] != 1) return false;
    const int P = offs[no - 1];
    nx = offs[1];
    if (nx < 2 || P % nx != 0 || n % P != 0) return false;
    ny = no == 3 ? P / nx : 1;
    if (no == 3 && ny < 2) return false;
    nz = n / P;
    if (nz < 2) return false;
    for (int r = 0; r < n; ++r) {
        const int i = r % nx;
        const int j = (r / nx) % ny;
        const int k = r / P;
        int want[3], nw = 0;
        if (k > 0) want[nw++] = r - P;
        if (no == 3 && j > 0) want[nw++] = r - nx;
        if (i > 0) want[nw++] = r - 1;
        if (diag[r] - rp[r] != nw) return false;
        for (int t = 0; t < nw; ++t)
            if (ci[rp[r] + t] != want[t]) return false;
        nw = 0;
        if (i < nx - 1) want[nw++] = r + 1;
        if (no == 3 && j < ny - 1) want[nw++] = r + nx;
        if (k < nz - 1) want[nw++] = r + P;
        if (rp[r + 1] - diag[r] - 1 != nw) return false;
        for (int t = 0; t < nw; ++t)
            if (ci[diag[r] + 1 + t] != want[t]) return false;
    }
    return true;
}

// Block geometry of the line-pipeline sweeps: lanes of a warp along y (wy, and
// wz = 32 / wy along z; a 2-D grid, ny = 1, has wy = 1) and warps of a CTA along y and z
// (by, bz).  Requested values (0 = automatic) are clamped to what the grid allows.
static LineGeom line_geometry(int nx, int ny, int nz, int wy_req, int by_req, int bz_req) {
    LineGeom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    // lanes along y: 8 (default) or the requested 1 / 4; a 2-D grid has 1
    int wy = 1;
    if (ny > 1) {
        wy = wy_req > 0 ? wy_req : (ny > 4 ? 8 : 4);
        if (wy != 1 && wy != 4 && wy != 8) wy = 8;
    }
    g.wy = wy;
    g.wz = 32 / wy;
    const int wly = ceil_div(ny, g.wy), wlz = ceil_div(nz, g.wz);  // warps along y / z
    int by = ny > 1 ? (by_req > 0 ? by_req : 2) : 1;
    // (2-D: one warp per CTA, so that the forward sweep's block-by-block rescale of the
    // Krylov vector is spread over as many CTAs as there are warps)
    int bz = bz_req > 0 ? bz_req : (ny > 1 ? 2 : 1);
    by = std::max(1, std::min(by, wly));
    bz = std::max(1, std::min(bz, wlz));
    if (ny > 1) {  // the halo warp holds one line of each incoming face per lane
        by = std::min(by, std::max(1, 32 / g.wy));
        bz = std::min(bz, std::max(1, 32 / g.wz));
    }
    while (by * bz > kLineMaxWarps) (bz > by ? bz : by) /= 2;
    g.by = by;
    g.bz = bz;
    g.nby = ceil_div(wly, by);
    g.nbz = ceil_div(wlz, bz);
    g.nblk = g.nby * g.nbz;
    g.steps = nx + g.wy + g.wz - 2;
    return g;
}

// Tickets of the block grid in dependency order: anti-diagonals iy + iz ascending (the
// same in the sweep coordinates of L and U); with clusters of cl blocks along z, the
// tickets are clusters (iy, izc), along the anti-diagonals of the cluster grid.
static std::vector<int> line_block_order(const LineGeom& g) {
    const int nz_units = g.cl > 0 ? g.nbzc : g.nbz;
    std::vector<int> o;
    o.reserve(static_cast<size_t>(g.nby) * nz_units);
    for (int d = 0; d < g.nby + nz_units - 1; ++d)
        for (int iz = 0; iz < nz_units; ++iz) {
            const int iy = d - iz;
            if (iy >= 0 && iy < g.nby) o.push_back(iy + g.nby * iz);
        }
    return o;
}

static cudaLaunchConfig_t line_cluster_config(int grid, int threads, size_t smem, int cl, cudaStream_t s,
                                              cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    cfg.blockDim = dim3(static_cast<unsigned>(threads));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cl);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// Raises the kernels' shared-memory limit, sizes the grid and allocates the packed
// operands of value type T; false when a CTA cannot be resident.  With G.g.cl > 0 the
// cluster variant is sized (clusters of cl CTAs along z); `try_cluster` (first type
// configured) decides G.g.cl: with `max_cluster` 1, clusters of 16, else 8, where the grid
// has at least two blocks along z and such a cluster can be scheduled; with 2 .. 16,
// clusters of at most that many CTAs; with 0, none.
template <class T>
static bool configure_line(LinePack& G, const DeviceInfo& dev, bool try_cluster, int max_cluster) {
    const size_t smem = std::max(static_cast<size_t>(line_smem_bytes<T>(G.g)), static_cast<size_t>(G.smem_floor));
    if (smem + 1024 > static_cast<size_t>(dev.smem_optin)) return false;
    if (try_cluster) {
        G.g.cl = 0;
        G.g.nbzc = 0;
        // clusters of 16 (non-portable) where they can be scheduled, else of 8
        const int wants[2] = {max_cluster == 1 ? 16 : max_cluster, max_cluster == 1 ? 8 : 0};
        for (int want : wants) {
            if (want < 2 || G.g.nbz < 2 || G.g.cl > 0) break;
            const int cl = std::min(want, G.g.nbz);
            const int nbzc = ceil_div(G.g.nbz, cl);
            int ok = 1;
            int nclusters = 1 << 30;
            for (bool upper : {false, true}) {
                const void* kern = upper ? reinterpret_cast<const void*>(sptrsv_line_cluster_kernel<T, true>)
                                         : reinterpret_cast<const void*>(sptrsv_line_cluster_kernel<T, false>);
                GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
                if (cl > 8) GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
                cudaLaunchAttribute attr[1];
                cudaLaunchConfig_t cfg = line_cluster_config(G.g.nby * nbzc * cl, G.threads, smem, cl, nullptr, attr);
                int nc = 0;
                if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) != cudaSuccess) {
                    cudaGetLastError();
                    nc = 0;
                }
                if (nc < 1) ok = 0;
                nclusters = std::min(nclusters, nc);
            }
            if (ok) {
                G.g.cl = cl;
                G.g.nbzc = nbzc;
                G.grid = std::min(nclusters, G.g.nby * nbzc) * cl;
            }
        }
    }
    if (G.g.cl > 0) {
        for (bool upper : {false, true}) {
            const void* kern = upper ? reinterpret_cast<const void*>(sptrsv_line_cluster_kernel<T, true>)
                                     : reinterpret_cast<const void*>(sptrsv_line_cluster_kernel<T, false>);
            GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
            if (G.g.cl > 8) GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        }
    } else {
        int per_sm = 0;
        for (bool upper : {false, true}) {
            const void* kern = upper ? reinterpret_cast<const void*>(sptrsv_line_kernel<T, true>)
                                     : reinterpret_cast<const void*>(sptrsv_line_kernel<T, false>);
            GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
            int r = 0;
            GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, G.threads, smem));
            if (r < 1) return false;
            per_sm = per_sm == 0 ? r : std::min(per_sm, r);
        }
        G.grid = std::min(G.g.nblk, per_sm * dev.sms);
    }
    const size_t len = static_cast<size_t>(G.g.slots()) * 4;
    if constexpr (sizeof(T) == 8) {
        G.l64.reserve(len);
        G.u64.reserve(len);
    } else {
        G.l32.reserve(len);
        G.u32.reserve(len);
    }
    return true;
}

// Packs the factor values into the operand streams of type T.
template <class T>
static void pack_line(LinePack& G, const int* rp, const int* diag, const double* lu, cudaStream_t s, int sms) {
    const long long slots = G.g.slots();
    const int threads = 256;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>(ceil_div<long long>(slots, threads), 8LL * sms)));
    T* l = sizeof(T) == 8 ? reinterpret_cast<T*>(G.l64.get()) : reinterpret_cast<T*>(G.l32.get());
    T* u = sizeof(T) == 8 ? reinterpret_cast<T*>(G.u64.get()) : reinterpret_cast<T*>(G.u32.get());
    line_pack_kernel<T, false><<<grid, threads, 0, s>>>(G.g, rp, diag, lu, l);
    line_pack_kernel<T, true><<<grid, threads, 0, s>>>(G.g, rp, diag, lu, u);
    GB_CUDA_CHECK(cudaGetLastError());
}

template <class T, bool UPPER>
static void launch_line(const LinePack& G, cudaStream_t s, T* in, const double* scale, T* out, unsigned* counter,
                        int* status, const int* gate, int step) {
    const size_t smem = std::max(static_cast<size_t>(line_smem_bytes<T>(G.g)), static_cast<size_t>(G.smem_floor));
    if (G.g.cl > 0) {
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = line_cluster_config(G.grid, G.threads, smem, G.g.cl, s, attr);
        GB_CUDA_CHECK(cudaLaunchKernelEx(&cfg, sptrsv_line_cluster_kernel<T, UPPER>, G.view<T>(UPPER), in, scale, out,
                                         counter, status, gate, step));
    } else {
        sptrsv_line_kernel<T, UPPER><<<G.grid, G.threads, smem, s>>>(G.view<T>(UPPER), in, scale, out, counter,
                                                                      status, gate, step);
    }
    GB_CUDA_CHECK(cudaGetLastError());
}

}  // namespace gb300

namespace lljbash {

using namespace gb300;

// Automatic choice of the line-pipeline sweeps (structured-grid factors): each sweep of
// each value type is timed (CUDA events, second of two runs, right-hand side of ones, the
// factors just computed) with the line kernel and with the block-local / level-ordered
// kernel, and the line kernel is kept where it is faster by more than 2 %.  Both give
// the same results; only the time differs.
template <class T>
static int tune_line_sweeps(IluSolver::Impl& im, int& use, T* b, T* y, T* x, cudaStream_t s) {
    const int n = im.n;
    const int threads = 256;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>(ceil_div<long long>(n, threads), 8LL * im.dev.sms)));
    line_fill_kernel<T><<<grid, threads, 0, s>>>(n, b, T(1));
    cudaEvent_t e0, e1;
    GB_CUDA_CHECK(cudaEventCreate(&e0));
    GB_CUDA_CHECK(cudaEventCreate(&e1));
    int launches = 1;
    float best[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [sweep][0: other, 1: line]
    for (int sweep = 0; sweep < 2; ++sweep)
        for (int cand = 0; cand < 2; ++cand) {
            use = cand ? (sweep ? 2 : 1) : 0;
            for (int rep = 0; rep < 2; ++rep) {
                if (sweep == 0) {
                    fill_sentinel(y, n, s, im.dev.sms);
                    GB_CUDA_CHECK(cudaEventRecord(e0, s));
                    im.launch_lower<T>(s, b, nullptr, y, nullptr, 0);
                } else {
                    fill_sentinel(x, n, s, im.dev.sms);
                    GB_CUDA_CHECK(cudaEventRecord(e0, s));
                    im.launch_upper<T>(s, y, x, nullptr, 0);
                }
                GB_CUDA_CHECK(cudaEventRecord(e1, s));
                GB_CUDA_CHECK(cudaEventSynchronize(e1));
                GB_CUDA_CHECK(cudaEventElapsedTime(&best[sweep][cand], e0, e1));
                launches += 2;
            }
        }
    GB_CUDA_CHECK(cudaEventDestroy(e0));
    GB_CUDA_CHECK(cudaEventDestroy(e1));
    // the line kernel only where it is clearly faster (2 %): a near tie keeps the other
    // schedule, so that timing noise does not flip the choice between runs
    use = (best[0][1] < 0.98f * best[0][0] ? 1 : 0) | (best[1][1] < 0.98f * best[1][0] ? 2 : 0);
    return launches;
}

static void tune_line(IluSolver::Impl& im, cudaStream_t s) {
    const size_t nv = static_cast<size_t>(std::max(im.n, 1));
    if (im.grid64) im.launches += tune_line_sweeps<double>(im, im.line_use64, im.sb64.get(), im.sy64.get(), im.sx64.get(), s);
    if (im.grid32) {
        DeviceBuffer<float> b32, x32;
        b32.reserve(nv);
        x32.reserve(nv);
        im.launches += tune_line_sweeps<float>(im, im.line_use32, b32.get(), im.sy32.get(), x32.get(), s);
        // the FP32 forward-sweep vector is back at the sentinel for its next user
        fill_sentinel(im.sy32.get(), static_cast<long long>(nv), s, im.dev.sms);
        GB_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    fill_sentinel(im.sy64.get(), static_cast<long long>(nv), s, im.dev.sms);
    im.line_tuned = true;
    im.check_status(s);
}

IluSolver::Impl::~Impl() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

template <class T>
void IluSolver::Impl::launch_lower(cudaStream_t s, T* b, const double* scale, T* y, const int* gate, int step) const {
    if (levelsync) {
        launch_levelsync<T, false>(LS, grid_levelsync, s, b, scale, y, counters.get() + 4, status.get(), gate, step);
        return;
    }
    if ((sizeof(T) == 8 ? line_use64 : line_use32) & 1) {
        launch_line<T, false>(GP, s, b, scale, y, counters.get() + 1, status.get(), gate, step);
        return;
    }
    if (sizeof(T) == 8 ? blk64 : blk32) {
        launch_block<T, false>(sizeof(T) == 8 ? LB64 : LB32, s, b, scale, y, counters.get() + 1, status.get(), gate,
                               step);
        return;
    }
    if (L.ntask == 0) return;
    launch_level_lower<T>(L, grid_solve, solve_threads, s, b, scale, y, counters.get() + 1, status.get(), gate, step);
}

template <class T>
void IluSolver::Impl::launch_upper(cudaStream_t s, T* y, T* x, const int* gate, int step) const {
    if (levelsync) {
        launch_levelsync<T, true>(US, grid_levelsync, s, y, nullptr, x, counters.get() + 4, status.get(), gate, step);
        return;
    }
    if ((sizeof(T) == 8 ? line_use64 : line_use32) & 2) {
        launch_line<T, true>(GP, s, y, nullptr, x, counters.get() + 2, status.get(), gate, step);
        return;
    }
    if (sizeof(T) == 8 ? blk64 : blk32) {
        launch_block<T, true>(sizeof(T) == 8 ? UB64 : UB32, s, y, nullptr, x, counters.get() + 2, status.get(), gate,
                              step);
        return;
    }
    if (U.ntask == 0) return;
    launch_level_upper<T>(U, grid_solve, solve_threads, s, y, x, counters.get() + 2, status.get(), gate, step);
}

template <class T>
const void* IluSolver::Impl::subst_key() const {
    if (levelsync) return LS.cols.get();
    if (const int bits = sizeof(T) == 8 ? line_use64 : line_use32; bits != 0)  // the schedule is part of the key
        return (sizeof(T) == 8 ? reinterpret_cast<const char*>(GP.l64.get()) : reinterpret_cast<const char*>(GP.l32.get())) + bits;
    if (sizeof(T) == 8 ? blk64 : blk32) return (sizeof(T) == 8 ? LB64 : LB32).codes.get();
    return L.cols.get();
}

template const void* IluSolver::Impl::subst_key<double>() const;
template const void* IluSolver::Impl::subst_key<float>() const;
template void IluSolver::Impl::launch_lower<double>(cudaStream_t, double*, const double*, double*, const int*, int) const;
template void IluSolver::Impl::launch_lower<float>(cudaStream_t, float*, const double*, float*, const int*, int) const;
template void IluSolver::Impl::launch_upper<double>(cudaStream_t, double*, double*, const int*, int) const;
template void IluSolver::Impl::launch_upper<float>(cudaStream_t, float*, float*, const int*, int) const;

void IluSolver::Impl::push_wait_limit() {
    if (!status.get()) return;
    GB_CUDA_CHECK(cudaMemcpyAsync(status.get() + kStatusWaitLimitUs, &wait_limit_us, sizeof(int),
                                  cudaMemcpyHostToDevice, stream));
    GB_CUDA_CHECK(cudaStreamSynchronize(stream));
}

void IluSolver::Impl::check_status(cudaStream_t s) {
    int h[kStatusWords];
    GB_CUDA_CHECK(cudaMemcpyAsync(h, status.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (h[kStatusTimeout] != 0) {
        const int zero = 0;
        GB_CUDA_CHECK(cudaMemcpy(status.get() + kStatusTimeout, &zero, sizeof(int), cudaMemcpyHostToDevice));
        // a kernel that gave up may leave its ticket counters or grid-barrier words set
        GB_CUDA_CHECK(cudaMemset(counters.get(), 0, sizeof(unsigned) * 8));
        throw std::runtime_error("dependency wait timed out on the device");
    }
}

IluSolver::Impl* IluSolver::impl_ensure() {
    if (!impl_) impl_ = new Impl;
    return impl_;
}

IluSolver::~IluSolver() {
    delete impl_;
    impl_ = nullptr;
    DestroyCsrMatrix(&aMatrix_);
}

void IluSolver::SetupMatrix() {
    const int n = aMatrix_.size;
    if (n < 0 || aMatrix_.row_ptr == nullptr) throw std::runtime_error("matrix not set");
    const int* rp = aMatrix_.row_ptr;
    const int* ci = aMatrix_.col_idx;
    validate_csr(n, rp, ci, "ILU matrix", aMatrix_.max_nnz > 0 ? aMatrix_.max_nnz : -1);
    Analysis an;
    diagonal_pointers(n, rp, ci, an.diag);  // throws "missing diag"
    const DagView gl{rp, ci, an.diag.data(), true};
    const DagView gu{rp, ci, an.diag.data(), false};
    elimination_tree(n, gl, an.etree_l);
    elimination_tree(n, gu, an.etree_u);
    an.nlev_l = level_sets(n, gl, an.depth_l, an.order_l, an.lptr_l);
    an.nlev_u = level_sets(n, gu, an.depth_u, an.order_u, an.lptr_u);

    Impl& im = *impl_ensure();
    im.dev = current_device();
    if (!im.stream) GB_CUDA_CHECK(cudaStreamCreateWithFlags(&im.stream, cudaStreamNonBlocking));
    if (!im.ev0) {
        GB_CUDA_CHECK(cudaEventCreate(&im.ev0));
        GB_CUDA_CHECK(cudaEventCreate(&im.ev1));
    }
    cudaStream_t s = im.stream;
    im.n = n;
    im.nnz = rp[n];
    im.an = std::move(an);
    im.factorized = false;
    im.rp.upload(rp, static_cast<size_t>(n) + 1, s);
    im.ci.upload(ci, static_cast<size_t>(im.nnz), s);
    im.diag.upload(im.an.diag.data(), static_cast<size_t>(n), s);
    im.order_l.upload(im.an.order_l.data(), static_cast<size_t>(n), s);
    std::vector<int> tree_order;  // the factorisation's ticket order when ticket_order == 1
    im.sub_parts = 0;
    im.sub_rows = 0;
    if (im.ticket_order == 1 && n > 0) {
        // the reference's subtree schedule (one worker per SM): the workers' subtree rows
        // interleaved round-robin (rows of different subtrees are independent), then the
        // queue rows; a topological order, as every ticket order must be
        const TreeScheduleResult ts =
            tree_schedule(n, gl, std::max(1, im.dev.sms), 1, 1.0, RowWeights{rp, im.an.diag.data(), 0, 1});
        std::vector<int> ord;
        ord.reserve(static_cast<size_t>(n));
        const int np = ts.nproc;
        int longest = 0;
        for (int w = 0; w < np; ++w)
            longest = std::max(longest, ts.part_ptr[static_cast<size_t>(w) + 1] - ts.part_ptr[static_cast<size_t>(w)]);
        for (int i = 0; i < longest; ++i)
            for (int w = 0; w < np; ++w)
                if (ts.part_ptr[static_cast<size_t>(w)] + i < ts.part_ptr[static_cast<size_t>(w) + 1])
                    ord.push_back(ts.partitions[static_cast<size_t>(ts.part_ptr[static_cast<size_t>(w)] + i)]);
        for (int k = ts.part_ptr[static_cast<size_t>(np)]; k < n; ++k) ord.push_back(ts.partitions[static_cast<size_t>(k)]);
        if (static_cast<int>(ord.size()) != n) throw std::runtime_error("tree schedule order is not a permutation");
        im.order_fact.upload(ord.data(), ord.size(), s);
        GB_CUDA_CHECK(cudaStreamSynchronize(s));  // ord must outlive the copy
        tree_order.swap(ord);
    }
    im.depth_l.upload(im.an.depth_l.data(), static_cast<size_t>(n), s);
    im.shift.reserve(static_cast<size_t>(std::max(n, 1)));
    im.prepass.ensure(im.dev.sms);
    im.lu.reserve(static_cast<size_t>(im.nnz));
    im.done.reserve(static_cast<size_t>(std::max(n, 1)));
    GB_CUDA_CHECK(cudaMemsetAsync(im.done.get(), 0, sizeof(int) * static_cast<size_t>(std::max(n, 1)), s));
    im.stamp = 0;
    im.counters.reserve(8);
    GB_CUDA_CHECK(cudaMemsetAsync(im.counters.get(), 0, sizeof(unsigned) * 8, s));
    im.status.reserve(kStatusWords);
    GB_CUDA_CHECK(cudaMemsetAsync(im.status.get(), 0, sizeof(int) * kStatusWords, s));
    im.push_wait_limit();
    ++im.setup_gen;
    // structured-grid line-pipeline sweeps: 7- / 5-point stencil factors in natural order
    // (automatic, grid_mode 0: when the other schedules are automatic too; 1: always)
    im.grid64 = im.grid32 = false;
    if (im.grid_mode == 1 || (im.grid_mode == 0 && im.block_rows == 0)) {
        int gx = 0, gy = 0, gz = 0;
        if (detect_grid(n, rp, ci, im.an.diag, gx, gy, gz)) {
            // the requested (or automatic) CTA shape, halved along its longer side until
            // the FP64 kernels' shared memory fits
            int by = im.grid_by, bz = im.grid_bz;
            for (int attempt = 0; attempt < 8; ++attempt) {
                im.GP.g = line_geometry(gx, gy, gz, im.grid_wy, by, bz);
                im.GP.threads = (im.GP.g.nw() + 1) * kWarp;  // compute warps + the halo warp
                // one CTA per SM on request: more than half of an SM's shared memory
                im.GP.smem_floor = im.grid_one_cta_per_sm
                                       ? std::min(im.dev.smem_per_sm / 2 + 1024, im.dev.smem_optin - 1024)
                                       : 0;
                im.grid64 = configure_line<double>(im.GP, im.dev, true, im.grid_cluster);
                if (im.grid64 || im.GP.g.nw() == 1) break;
                by = im.GP.g.by;
                bz = im.GP.g.bz;
                (bz >= by ? bz : by) = std::max(1, (bz >= by ? bz : by) / 2);
            }
            im.grid32 = configure_line<float>(im.GP, im.dev, false, 0);
            for (int f = 0; f < 2; ++f)
                for (int u = 0; u < 2; ++u) {
                    auto& buf = im.GP.tl[f][u];
                    buf.release();
                    if (im.sweep_timeline && (f == 0 ? im.grid64 : im.grid32)) {
                        const size_t len = static_cast<size_t>(im.GP.g.nblk) * kLineTimeline;
                        buf.reserve(len);
                        GB_CUDA_CHECK(cudaMemsetAsync(buf.get(), 0, len * sizeof(unsigned long long), s));
                    }
                }
            const std::vector<int> order = line_block_order(im.GP.g);
            im.GP.order.upload(order.data(), order.size(), s);
            GB_CUDA_CHECK(cudaStreamSynchronize(s));  // `order` must outlive the copy
        }
    }
    // forced (grid_mode 1): every sweep of a configured type; automatic: timed against the
    // other schedules at the first Factorize (tune_line_sweeps)
    const bool line_forced = im.grid_mode == 1;
    im.line_use64 = line_forced && im.grid64 ? 3 : 0;
    im.line_use32 = line_forced && im.grid32 ? 3 : 0;
    im.line_tuned = line_forced || !(im.grid64 || im.grid32);
    const bool grid_both = line_forced && im.grid64 && im.grid32;
    im.blk64 = im.blk32 = false;
    if (im.block_rows >= 0 && !grid_both) {
        // block-local schedule: an explicit block size, or (0) the one the cost model
        // picks per value type; a type whose block does not fit in shared memory, or for
        // which the model prefers the level-ordered kernel, keeps the level kernel
        const size_t budget = static_cast<size_t>(std::max(0, im.dev.smem_optin - 1024));
        for (int elem : {8, 4}) {
            // candidates in order: the model's ranking, or an explicit block size with
            // clusters first (block + halo must fit and a cluster be schedulable)
            std::vector<BlockChoice> cand;
            if (im.block_rows > 0) {
                cand = {{im.block_rows, kBlockClusterBig, 0.0}, {im.block_rows, kBlockCluster, 0.0}, {im.block_rows, 0, 0.0}};
            } else {
                cand = choose_block_schedules(n, rp, ci, im.an.diag, im.an.nlev_l, elem, budget,
                                              static_cast<size_t>(im.dev.smem_per_sm), im.dev.sms);
            }
            BlockPack& lb = elem == 8 ? im.LB64 : im.LB32;
            BlockPack& ub = elem == 8 ? im.UB64 : im.UB32;
            bool ok = false;
            for (const BlockChoice& ch : cand) {
                const int B = ch.rows;
                const int cl = ch.cl;
                if (cl > 0 && n <= B) continue;  // a single block has no handoffs
                build_block_pack(n, rp, ci, im.an.diag, true, B, elem, budget, cl, lb, s);
                build_block_pack(n, rp, ci, im.an.diag, false, B, elem, budget, cl, ub, s);
                if (!(lb.fits && ub.fits)) continue;
                if (elem == 8) {
                    configure_block<double, false>(lb, im.dev.sms);
                    configure_block<double, true>(ub, im.dev.sms);
                } else {
                    configure_block<float, false>(lb, im.dev.sms);
                    configure_block<float, true>(ub, im.dev.sms);
                }
                if (lb.grid > 0 && ub.grid > 0) {
                    ok = true;
                    break;
                }
            }
            if (!ok) continue;
            (elem == 8 ? im.blk64 : im.blk32) = true;
        }
    }
    im.levelsync = im.block_rows == -2 && !grid_both;
    if (im.levelsync) {
        build_levelsync_pack(n, rp, ci, im.an.diag, im.an.order_l, im.an.lptr_l, im.an.nlev_l, true, im.LS, s);
        build_levelsync_pack(n, rp, ci, im.an.diag, im.an.order_u, im.an.lptr_u, im.an.nlev_u, false, im.US, s);
        // cooperative launch: every CTA resident (the grid barrier waits for all of them)
        int per_sm = 0;
        for (auto kern : {sptrsv_levelsync_kernel<double, false>, sptrsv_levelsync_kernel<double, true>}) {
            int r = 0;
            GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, kSolveWarps * kWarp, 0));
            per_sm = per_sm == 0 ? r : std::min(per_sm, r);
        }
        for (auto kern : {sptrsv_levelsync_kernel<float, false>, sptrsv_levelsync_kernel<float, true>}) {
            int r = 0;
            GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, kSolveWarps * kWarp, 0));
            per_sm = std::min(per_sm, r);
        }
        if (per_sm < 1) throw std::runtime_error("level-synchronous kernel cannot be resident");
        im.grid_levelsync = std::min(per_sm, 2) * im.dev.sms;
    }
    im.level_packs = !((im.blk64 || (line_forced && im.grid64)) && (im.blk32 || (line_forced && im.grid32)));
    if (im.level_packs) {
        int kl = 0, ku = 0;
        for (int r = 0; r < n; ++r) {
            kl = std::max(kl, im.an.diag[r] - rp[r]);
            ku = std::max(ku, rp[r + 1] - im.an.diag[r] - 1);
        }
        build_level_pack(n, rp, ci, im.an.diag, im.an.order_l, true, row_lanes_for(kl, im.row_lanes), im.L, s);
        build_level_pack(n, rp, ci, im.an.diag, im.an.order_u, false, row_lanes_for(ku, im.row_lanes), im.U, s);
    }
    const size_t nv = static_cast<size_t>(std::max(n, 1));
    im.sb64.reserve(nv);
    im.sy64.reserve(nv);
    im.sx64.reserve(nv);
    im.sy32.reserve(nv);
    fill_sentinel(im.sy64.get(), static_cast<long long>(nv), s, im.dev.sms);
    fill_sentinel(im.sy32.get(), static_cast<long long>(nv), s, im.dev.sms);
    // Factorisation kernel: warp per row (automatic), or lane per row for short rows when
    // requested
    im.fact_lane = false;
    if (im.factor_kernel == 2 && im.ticket_order != 2 && n > 0)
        im.fact_lane = build_lane_factor(n, rp, ci, im.an.diag,
                                         im.ticket_order == 1 ? tree_order : im.an.order_l, im, s);
    // Factorisation launch: rows staged in shared memory up to the longest row where a
    // warp's share fits (fewer warps per block for long rows), a wider register window
    // of the next pivot row when pivot rows are long.
    {
        int maxlen = 0, maxup = 0;
        for (int r = 0; r < n; ++r) {
            maxlen = std::max(maxlen, rp[r + 1] - rp[r]);
            maxup = std::max(maxup, rp[r + 1] - im.an.diag[r] - 1);
        }
        // per warp: cap staged entries plus a column -> position table of hcap slots
        auto hcap_of = [](int c) {
            int h = 64;
            while (h < 2 * c) h <<= 1;
            return h;
        };
        auto warp_bytes = [&](int c) { return static_cast<long long>(c) * kFactEntryBytes + 8ll * hcap_of(c); };
        int cap = std::max(kFactCap, ceil_div(maxlen, kWarp) * kWarp);
        while (cap > kFactCap && warp_bytes(cap) > kFactSmemMax) cap -= kWarp;  // longer rows: global memory
        int warps = kFactWarps;
        while (warps > 1 && warps * warp_bytes(cap) > kFactSmemMax) --warps;
        im.fact_cap = cap;
        im.fact_hcap = hcap_of(cap);
        im.fact_warps = warps;
        im.fact_pre = maxup > 2 * kWarp ? 8 : 2;
        im.fact_smem = static_cast<size_t>(warps * warp_bytes(cap));
        auto kern = im.fact_pre == 8 ? ilu_factor_kernel<8> : ilu_factor_kernel<2>;
        GB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(im.fact_smem)));
        int per_sm = 0;
        GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * kWarp, im.fact_smem));
        im.grid_fact = std::max(1, per_sm) * im.dev.sms;
    }
    if (im.ticket_order == 2 && n > 0) {
        // subtree partitions, one CTA each (ilu_factor_subtree_kernel): the reference's
        // subtree scheduler with one worker per SM (fewer for small matrices: about 256
        // rows per worker; with more workers than SMs its subtree division leaves the large
        // matrices measured here without partitions), each run by a CTA of up to
        // kSubtreeWarps warps; each partition's rows grouped by level depth; the remaining
        // (separator) rows by tickets in level order (any topological order is
        // deadlock-free, level order keeps the most rows ready)
        const int workers = std::max(1, std::min(im.dev.sms, n / 256));
        const TreeScheduleResult ts =
            tree_schedule(n, gl, workers, 1, 1.0, RowWeights{rp, im.an.diag.data(), 0, 1});
        const int np = ts.nproc;
        std::vector<int> part_ptr(1, 0), grp_ptr(1, 0), rows;
        rows.reserve(static_cast<size_t>(n));
        for (int w = 0; w < np; ++w) {
            const int a0 = ts.part_ptr[static_cast<size_t>(w)], a1 = ts.part_ptr[static_cast<size_t>(w) + 1];
            if (a1 <= a0) continue;
            std::vector<int> pr(ts.partitions.begin() + a0, ts.partitions.begin() + a1);
            std::stable_sort(pr.begin(), pr.end(), [&](int x, int y) { return im.an.depth_l[x] < im.an.depth_l[y]; });
            for (size_t k = 0; k < pr.size(); ++k) {
                if (k > 0 && im.an.depth_l[pr[k]] != im.an.depth_l[pr[k - 1]]) grp_ptr.push_back(static_cast<int>(rows.size()));
                rows.push_back(pr[k]);
            }
            grp_ptr.push_back(static_cast<int>(rows.size()));
            part_ptr.push_back(static_cast<int>(grp_ptr.size()) - 1);
        }
        im.sub_parts = static_cast<int>(part_ptr.size()) - 1;
        im.sub_rows = static_cast<int>(rows.size());
        {
            // every pivot of a partition row lies in the same partition (whole subtrees of
            // the elimination tree): the kernel waits for no other CTA
            std::vector<int> owner(static_cast<size_t>(n), -1);
            for (int pp = 0; pp < im.sub_parts; ++pp)
                for (int q = grp_ptr[static_cast<size_t>(part_ptr[static_cast<size_t>(pp)])];
                     q < grp_ptr[static_cast<size_t>(part_ptr[static_cast<size_t>(pp) + 1])]; ++q)
                    owner[static_cast<size_t>(rows[static_cast<size_t>(q)])] = pp;
            for (int j = 0; j < n; ++j) {
                if (owner[static_cast<size_t>(j)] < 0) continue;
                for (int t = rp[j]; t < im.an.diag[static_cast<size_t>(j)]; ++t)
                    if (owner[static_cast<size_t>(ci[t])] != owner[static_cast<size_t>(j)])
                        throw std::runtime_error("subtree partition is not closed under the row's pivots");
            }
        }
        std::vector<int> queue(ts.partitions.begin() + ts.part_ptr[static_cast<size_t>(np)], ts.partitions.end());
        std::stable_sort(queue.begin(), queue.end(), [&](int x, int y) { return im.an.depth_l[x] < im.an.depth_l[y]; });
        if (im.sub_rows + static_cast<int>(queue.size()) != n)
            throw std::runtime_error("tree schedule partitions do not cover the rows");
        im.sub_part_ptr.upload(part_ptr.data(), part_ptr.size(), s);
        im.sub_grp_ptr.upload(grp_ptr.data(), grp_ptr.size(), s);
        im.sub_rows_d.upload(rows.data(), std::max<size_t>(rows.size(), 1), s);
        im.order_fact.upload(queue.data(), std::max<size_t>(queue.size(), 1), s);
        im.sub_queue = static_cast<int>(queue.size());
        GB_CUDA_CHECK(cudaStreamSynchronize(s));  // host vectors must outlive the copies
        auto sk = im.fact_pre == 8 ? ilu_factor_subtree_kernel<8> : ilu_factor_subtree_kernel<2>;
        const size_t per_warp = im.fact_smem / static_cast<size_t>(im.fact_warps);
        im.sub_warps = std::max(1, std::min<int>(kSubtreeWarps, static_cast<int>(kFactSmemMax / per_warp)));
        im.sub_smem = per_warp * static_cast<size_t>(im.sub_warps);
        GB_CUDA_CHECK(cudaFuncSetAttribute(sk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(im.sub_smem)));
    }
    // Level-ordered kernels: warps draw tasks in level order and spin on the rows they
    // depend on.  Rows of one lane poll in rounds and want many warps ahead (1,216 warps
    // best on the 128^3 7-point factor, ~64 levels ahead on the 256^2 5-point one); lane
    // groups want about 10 levels ahead (27-point factors on 64^3: 300-400 warps, ILU(1)
    // sweeps 1.0 ms against 1.34 ms at 1,216); rows too long for a lane group spin in
    // blocking waits, and warps far ahead of the critical path then slow its L2
    // handoffs.  Automatic: that many levels' worth of warps, spread over the SMs.
    {
        const int levels = std::max(1, std::max(im.an.nlev_l, im.an.nlev_u));
        const int tasks = std::max(im.L.ntask, im.U.ntask);
        const int cap = im.dev.sms * kSolveWarps;
        const bool long_rows = n > 0 && (im.nnz - n) > 2ll * kLaneEntries * n &&  // mean entries per triangle
                               (im.L.group == 1 || im.U.group == 1);
        const bool groups = im.L.group > 1 || im.U.group > 1;
        const double ahead = long_rows ? kSolveLevelsAheadLong : (groups ? kSolveLevelsAheadGroup : kSolveLevelsAhead);
        int warps = im.solve_warps > 0 ? im.solve_warps
                                       : static_cast<int>(std::ceil(ahead * static_cast<double>(tasks) / levels));
        warps = std::max(1, std::min(cap, warps));
        const int per_cta = std::max(1, std::min(kSolveWarps, ceil_div(warps, im.dev.sms)));
        im.solve_threads = per_cta * kWarp;
        im.grid_solve = std::max(1, ceil_div(warps, per_cta));
    }
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
}

bool IluSolver::Factorize() { return FactorizeFrom(aMatrix_.value, false); }

bool IluSolver::FactorizeDevice(const double* d_values) { return FactorizeFrom(d_values, true); }

bool IluSolver::FactorizeFrom(const double* values, bool on_device) {
    if (!impl_ || impl_->n != aMatrix_.size) throw std::runtime_error("SetupMatrix() must be called first");
    Impl& im = *impl_;
    cudaStream_t s = im.stream;
    const int n = im.n;
    // One numeric factorisation of `values` with an optional diagonal shift; returns the
    // status words.  With the learned model the shift comes from the fused pre-pass.
    auto factor_once = [&](int shift_kind) {  // 0 none, 1 explicit, 2 learned
        if (im.nnz > 0)
            GB_CUDA_CHECK(cudaMemcpyAsync(im.lu.get(), values, sizeof(double) * static_cast<size_t>(im.nnz),
                                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        int init[kStatusWords] = {0, 0, INT_MAX, im.wait_limit_us};
        GB_CUDA_CHECK(cudaMemcpyAsync(im.status.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
        if (++im.stamp == INT_MAX) {
            im.stamp = 1;
            GB_CUDA_CHECK(cudaMemsetAsync(im.done.get(), 0, sizeof(int) * static_cast<size_t>(std::max(n, 1)), s));
        }
        GB_CUDA_CHECK(cudaEventRecord(im.ev0, s));
        if (n > 0) {
            const double* shift = nullptr;
            if (shift_kind == 2) {
                im.prepass.run(s, im.dev.sms, n, im.rp.get(), im.ci.get(), im.lu.get(), im.diag.get(), im.depth_l.get(),
                               im.an.nlev_l, im.mlp.get(), im.min_shift, im.shift.get(), nullptr, nullptr);
                im.launches += 2;
                shift = im.shift.get();
            } else if (shift_kind == 1) {
                shift = im.shift.get();
            }
            if (im.fact_lane) {
                fill_sentinel(im.lf_pub.get(), im.lf_pub_len, s, im.dev.sms);
                LaneFactor F;
                F.n = n;
                F.ntask = im.lf_ntask;
                F.rows = im.lf_rows.get();
                F.rp = im.rp.get();
                F.ci = im.ci.get();
                F.diag = im.diag.get();
                F.pub_off = im.lf_pub_off.get();
                F.upd_ptr = im.lf_upd_ptr.get();
                F.upd = im.lf_upd.get();
                ilu_factor_lane_kernel<<<im.grid_lane_fact, kLaneFactWarps * kWarp, 0, s>>>(
                    F, im.lu.get(), shift, im.lf_pub.get(), im.counters.get(), im.status.get());
                GB_CUDA_CHECK(cudaGetLastError());
                im.launches += 2;
            }
            auto kern = im.fact_pre == 8 ? ilu_factor_kernel<8> : ilu_factor_kernel<2>;
            if (!im.fact_lane && im.ticket_order == 2) {
                // subtree partitions first (one CTA each, no waits), then the separator rows
                if (im.sub_parts > 0) {
                    auto sk = im.fact_pre == 8 ? ilu_factor_subtree_kernel<8> : ilu_factor_subtree_kernel<2>;
                    sk<<<im.sub_parts, im.sub_warps * kWarp, im.sub_smem, s>>>(
                        im.sub_part_ptr.get(), im.sub_grp_ptr.get(), im.sub_rows_d.get(), im.rp.get(), im.ci.get(),
                        im.diag.get(), im.lu.get(), shift, im.done.get(), im.stamp, im.status.get(), im.fact_cap,
                        im.fact_hcap);
                    im.launches += 1;
                }
                if (im.sub_queue > 0) {
                    kern<<<im.grid_fact, im.fact_warps * kWarp, im.fact_smem, s>>>(
                        im.sub_queue, im.rp.get(), im.ci.get(), im.diag.get(), im.order_fact.get(), im.lu.get(), shift,
                        im.done.get(), im.stamp, im.counters.get(), im.status.get(), im.fact_cap, im.fact_hcap);
                    im.launches += 1;
                }
            } else if (!im.fact_lane) {
                kern<<<im.grid_fact, im.fact_warps * kWarp, im.fact_smem, s>>>(
                    n, im.rp.get(), im.ci.get(), im.diag.get(),
                    im.ticket_order == 1 ? im.order_fact.get() : im.order_l.get(), im.lu.get(), shift, im.done.get(),
                    im.stamp, im.counters.get(), im.status.get(), im.fact_cap, im.fact_hcap);
                im.launches += 1;
            }
            GB_CUDA_CHECK(cudaGetLastError());
            if (im.blk64) {
                gather_block(im.LB64, true, im.lu.get(), s, im.dev.sms);
                gather_block(im.UB64, false, im.lu.get(), s, im.dev.sms);
                im.launches += 2;
            }
            if (im.blk32) {
                gather_block(im.LB32, true, im.lu.get(), s, im.dev.sms);
                gather_block(im.UB32, false, im.lu.get(), s, im.dev.sms);
                im.launches += 2;
            }
            if (im.level_packs) {
                gather_level_pack(im.L, true, im.lu.get(), s, im.dev.sms);
                gather_level_pack(im.U, false, im.lu.get(), s, im.dev.sms);
                im.launches += 6;
            }
            if (im.levelsync) {
                gather_level_pack(im.LS, true, im.lu.get(), s, im.dev.sms);
                gather_level_pack(im.US, false, im.lu.get(), s, im.dev.sms);
                im.launches += 6;
            }
            if (im.grid64) {
                pack_line<double>(im.GP, im.rp.get(), im.diag.get(), im.lu.get(), s, im.dev.sms);
                im.launches += 2;
            }
            if (im.grid32) {
                pack_line<float>(im.GP, im.rp.get(), im.diag.get(), im.lu.get(), s, im.dev.sms);
                im.launches += 2;
            }
        }
        GB_CUDA_CHECK(cudaEventRecord(im.ev1, s));
        std::array<int, kStatusWords> h{};
        GB_CUDA_CHECK(cudaMemcpyAsync(h.data(), im.status.get(), sizeof(int) * kStatusWords, cudaMemcpyDeviceToHost, s));
        GB_CUDA_CHECK(cudaStreamSynchronize(s));
        float ms = 0.f;
        GB_CUDA_CHECK(cudaEventElapsedTime(&ms, im.ev0, im.ev1));
        im.last_factor_ms += ms;
        if (h[kStatusTimeout] != 0) {
            im.factorized = false;
            throw std::runtime_error("dependency wait timed out on the device");
        }
        return h;
    };
    im.last_factor_ms = 0.f;
    const int kind = im.model_active ? 2 : (im.shift_active ? 1 : 0);
    auto h = factor_once(kind);
    im.shift_applied = kind != 0;
    if (kind == 2 && h[kStatusBreakdowns] != 0) {
        // learned shift met a zero / non-finite pivot: plain ILU is the fallback
        h = factor_once(0);
        im.shift_applied = false;
    }
    if (!im.line_tuned) tune_line(im, s);
    if (!on_device && im.copy_back && im.nnz > 0) {
        GB_CUDA_CHECK(cudaMemcpyAsync(aMatrix_.value, im.lu.get(), sizeof(double) * static_cast<size_t>(im.nnz),
                                      cudaMemcpyDeviceToHost, s));
        GB_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    im.last_breakdowns = h[kStatusBreakdowns];
    im.first_breakdown = h[kStatusBreakdowns] ? h[kStatusFirstBreakdown] : -1;
    im.factorized = true;
    return im.last_breakdowns == 0;
}

void IluSolver::SetShiftModel(const float* params, int nparams, float min_shift) {
    Impl& im = *impl_ensure();
    if (params == nullptr || nparams == 0) {
        im.model_active = false;
        return;
    }
    if (nparams != kMlpParams) throw std::runtime_error("shift model must have 369 parameters");
    if (!im.stream) throw std::runtime_error("SetupMatrix() must be called first");
    im.mlp.upload(params, static_cast<size_t>(kMlpParams), im.stream);
    GB_CUDA_CHECK(cudaStreamSynchronize(im.stream));
    im.min_shift = min_shift;
    im.model_active = true;
}

void IluSolver::Substitute(const double* b, double* x) {
    if (!impl_ || !impl_->factorized) throw std::runtime_error("Factorize() must be called first");
    Impl& im = *impl_;
    cudaStream_t s = im.stream;
    const int n = im.n;
    if (n == 0) return;
    GB_CUDA_CHECK(cudaMemcpyAsync(im.sb64.get(), b, sizeof(double) * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
    fill_sentinel(im.sx64.get(), n, s, im.dev.sms);
    fill_sentinel(im.sy64.get(), n, s, im.dev.sms);
    im.launch_lower<double>(s, im.sb64.get(), nullptr, im.sy64.get(), nullptr, 0);
    im.launch_upper<double>(s, im.sy64.get(), im.sx64.get(), nullptr, 0);
    GB_CUDA_CHECK(cudaGetLastError());
    GB_CUDA_CHECK(cudaMemcpyAsync(x, im.sx64.get(), sizeof(double) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, s));
    im.check_status(s);
}

}  // namespace lljbash

// ---------------------------------------------------------------------------------
// Allocation-free substitution.
//
// Some callers cannot allocate device memory at the moment they need a preconditioner
// application: an application that reserves all device memory up front for its own
// pool (cudaMalloc then fails), or one that must not let a library call cudaMalloc /
// cudaFree because those may synchronise the whole device in the middle of its
// pipelined work.  IluSolver::SubstituteDeviceNoAlloc serves them: the intermediate
// vector of the forward sweep and the kernels' ticket counters and status words live
// in one statically sized device array of this file (g_noalloc_scratch, 16 MiB + 256 B,
// reserved on every GPU that loads the library until the process exits), so the call
// itself allocates nothing.  Its limit is kNoAllocMaxRows rows.
//
// The array's host-side name is only a stand-in: host code obtains its device address
// with cudaGetSymbolAddress, once per device, the first time the entry point runs on
// that device (with that device current).  That first call should therefore come
// before any stream capture.  All calls share the array and it keeps the previous
// call's contents, so every call re-initialises what must start at zero or at the
// sentinel; calls whose GPU work overlaps (different streams, threads or solvers at
// the same time) race on it.
// ---------------------------------------------------------------------------------
namespace gb300 {

constexpr long long kNoAllocMaxRows = 1ll << 21;
constexpr size_t kNoAllocScratchBytes = static_cast<size_t>(kNoAllocMaxRows) * sizeof(double) + 256;
// layout: [0, 8 * kNoAllocMaxRows) forward-sweep vector; then 4 ticket counters
// (unsigned) and kStatusWords status ints.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
std::vector<void*> g_noalloc_addr;  // per device ordinal, nullptr until set up

void* noalloc_scratch_address(int device) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (device >= static_cast<int>(g_noalloc_addr.size())) g_noalloc_addr.resize(static_cast<size_t>(device) + 1, nullptr);
    if (g_noalloc_addr[device] == nullptr) {
        void* ptr = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (err != cudaSuccess || ptr == nullptr) {
            throw std::runtime_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") +
                                     cudaGetErrorString(err));
        }
        g_noalloc_addr[device] = ptr;
    }
    return g_noalloc_addr[device];
}
}  // namespace

}  // namespace gb300

namespace lljbash {

void IluSolver::SubstituteDeviceNoAlloc(const double* d_b, double* d_x) {
    using namespace gb300;
    if (!impl_ || !impl_->factorized) throw std::runtime_error("Factorize() must be called first");
    Impl& im = *impl_;
    const int n = im.n;
    if (n > kNoAllocMaxRows)
        throw std::runtime_error("SubstituteDeviceNoAlloc supports at most 2097152 rows (static scratch limit)");
    if (n == 0) return;
    // The scratch address and the solver's stream must belong to the same GPU: the
    // address is resolved with the solver's device current, and a call made while
    // another device is current is refused instead of mixing the two.
    int device = 0;
    GB_CUDA_CHECK(cudaGetDevice(&device));
    if (device != im.dev.device)
        throw std::runtime_error("SubstituteDeviceNoAlloc: the current device (" + std::to_string(device) +
                                 ") is not the device the solver was set up on (" + std::to_string(im.dev.device) +
                                 ")");
    unsigned char* base = static_cast<unsigned char*>(noalloc_scratch_address(im.dev.device));
    double* y = reinterpret_cast<double*>(base);
    unsigned* counters = reinterpret_cast<unsigned*>(base + kNoAllocMaxRows * sizeof(double));
    int* status = reinterpret_cast<int*>(counters + 4);
    cudaStream_t s = im.stream;
    // what must start at zero (counters, status) and at the sentinel (y, x)
    GB_CUDA_CHECK(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned) + kStatusWords * sizeof(int), s));
    GB_CUDA_CHECK(cudaMemcpyAsync(status + kStatusWaitLimitUs, &im.wait_limit_us, sizeof(int), cudaMemcpyHostToDevice, s));
    fill_sentinel(y, n, s, im.dev.sms);
    fill_sentinel(d_x, n, s, im.dev.sms);
    double* b = const_cast<double*>(d_b);  // read only: no scale is passed to the forward sweep
    // each sweep on the schedule the solver uses for it (line-pipeline, block-local or
    // level-ordered; a level-synchronous solver's level packs give the same results)
    if (im.line_use64 & 1)
        launch_line<double, false>(im.GP, s, b, nullptr, y, counters + 1, status, nullptr, 0);
    else if (im.blk64)
        launch_block<double, false>(im.LB64, s, b, nullptr, y, counters + 1, status, nullptr, 0);
    else if (im.L.ntask > 0)
        launch_level_lower<double>(im.L, im.grid_solve, im.solve_threads, s, b, nullptr, y, counters + 1, status,
                                   nullptr, 0);
    if (im.line_use64 & 2)
        launch_line<double, true>(im.GP, s, y, nullptr, d_x, counters + 2, status, nullptr, 0);
    else if (im.blk64)
        launch_block<double, true>(im.UB64, s, y, nullptr, d_x, counters + 2, status, nullptr, 0);
    else if (im.U.ntask > 0)
        launch_level_upper<double>(im.U, im.grid_solve, im.solve_threads, s, y, d_x, counters + 2, status, nullptr, 0);
    GB_CUDA_CHECK(cudaGetLastError());
    int h[kStatusWords];
    GB_CUDA_CHECK(cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (h[kStatusTimeout] != 0) throw std::runtime_error("dependency wait timed out on the device");
}

}  // namespace lljbash
