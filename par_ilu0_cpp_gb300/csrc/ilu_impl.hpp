// Internal state of lljbash::IluSolver (shared by the ILU and GMRES translation units).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "device_util.hpp"
#include "factor_lane.cuh"
#include "line_sweep.cuh"
#include "ilu_kernels.cuh"
#include "ilu_solver.hpp"
#include "mlp_impl.hpp"

namespace gb300 {

// One packed triangular factor in the level-ordered warp layout (see PackedTri):
// schedule arrays plus packed values in FP64 and FP32.
struct LevelPack {
    int ntask = 0;
    int group = 1;  // lanes per row
    long long slots = 0;
    DeviceBuffer<int> rows, off, len, cols, src, dsrc;
    DeviceBuffer<double> v64, d64;
    DeviceBuffer<float> v32, d32;
    // level-synchronous packs only: tasks of level l are [ltask[l], ltask[l + 1])
    DeviceBuffer<int> ltask;
    int nlev = 0;

    template <class T>
    PackedTri<T> view() const;
};

template <>
inline PackedTri<double> LevelPack::view<double>() const {
    PackedTri<double> p;
    p.ntask = ntask;
    p.rows = rows.get();
    p.off = off.get();
    p.len = len.get();
    p.cols = cols.get();
    p.vals = v64.get();
    p.dvals = d64.get();
    return p;
}
template <>
inline PackedTri<float> LevelPack::view<float>() const {
    PackedTri<float> p;
    p.ntask = ntask;
    p.rows = rows.get();
    p.off = off.get();
    p.len = len.get();
    p.cols = cols.get();
    p.vals = v32.get();
    p.dvals = d32.get();
    return p;
}

// One packed triangular factor in the block-local layout (see BlockTri) for one value
// type (`elem` = sizeof(T)): the row partition, the per-block task lists and the packed
// values.  `fits`: the largest block's solution fits in shared memory.
struct BlockPack {
    int elem = 0;
    int nblk = 0;
    int block_rows = 0;   // rows per block (the last block may be shorter)
    int ntask = 0;
    int kmax = 0;         // most entries of a row
    int stride = 0;       // entries per lane of every task (3, 4, 8: the kernel's registers; 0: off / len)
    long long slots = 0;
    int threads = 0;      // CTA size
    int cl = 0;           // cluster size of the cluster variant (0: plain variant)
    int halo = 0;         // halo rows per CTA (cluster variant)
    int grid = 0;         // CTAs to launch: resident CTAs (plain) or resident clusters x cl
    size_t smem = 0;      // dynamic shared memory of the kernel
    bool fits = false;
    DeviceBuffer<int> blk_row, blk_task, rows, off, len, codes, src, dsrc, exps;
    DeviceBuffer<double> v64, d64;
    DeviceBuffer<float> v32, d32;

    template <class T>
    BlockTri<T> view() const {
        BlockTri<T> p;
        p.nblk = nblk;
        p.ntask = ntask;
        p.slots = slots;
        p.block_rows = block_rows;
        p.halo = halo;
        p.cl = cl;
        p.exps = exps.get();
        p.blk_row = blk_row.get();
        p.blk_task = blk_task.get();
        p.rows = rows.get();
        p.off = off.get();
        p.len = len.get();
        p.codes = codes.get();
        if constexpr (sizeof(T) == 8) {
            p.vals = v64.get();
            p.dvals = d64.get();
        } else {
            p.vals = v32.get();
            p.dvals = d32.get();
        }
        return p;
    }
};

// Structured-grid factor (line-pipeline sweeps, line_sweep.cuh): block geometry, ticket
// order and the packed operand streams of L and U per value type (rebuilt from the factor
// values after every factorisation).
struct LinePack {
    LineGeom g;
    int threads = 0;  // CTA size: nw warps
    int grid = 0;     // CTAs launched
    int smem_floor = 0;  // dynamic shared memory requested at least (bytes; one CTA per SM)
    DeviceBuffer<int> order;        // [nblk] block of each ticket
    DeviceBuffer<double> l64, u64;  // [4 slots]
    DeviceBuffer<float> l32, u32;
    // per-block timelines [fp32][upper] of the last sweep of each kind (allocated only
    // with the timeline option on)
    DeviceBuffer<unsigned long long> tl[2][2];

    template <class T>
    LineTri<T> view(bool upper) const {
        LineTri<T> p;
        p.g = g;
        p.order = order.get();
        p.tl = tl[sizeof(T) == 4 ? 1 : 0][upper ? 1 : 0].get();
        if constexpr (sizeof(T) == 8) {
            p.coef = upper ? u64.get() : l64.get();
        } else {
            p.coef = upper ? u32.get() : l32.get();
        }
        return p;
    }
};

// Host-side results of the pattern analysis (integer output identical to the
// reference's; see analysis.hpp).
struct Analysis {
    std::vector<int> diag;
    std::vector<int> etree_l, etree_u;
    std::vector<int> depth_l, depth_u;
    std::vector<int> order_l, order_u;
    std::vector<int> lptr_l, lptr_u;
    int nlev_l = 0, nlev_u = 0;
};

}  // namespace gb300

namespace lljbash {

struct IluSolver::Impl {
    gb300::DeviceInfo dev;
    cudaStream_t stream = nullptr;
    int n = 0;
    long long nnz = 0;
    gb300::Analysis an;

    gb300::DeviceBuffer<int> rp, ci, diag, order_l;
    gb300::DeviceBuffer<int> order_fact;  // ticket order of the factorisation (ticket_order = 1)
    int ticket_order = 0;  // factorisation tickets: 0 level order, 1 the subtree scheduler's order,
                           // 2 subtree partitions one CTA each, then the separator rows by tickets
    gb300::DeviceBuffer<int> sub_part_ptr, sub_grp_ptr, sub_rows_d;  // ticket_order 2: partitions
    int sub_parts = 0, sub_rows = 0, sub_queue = 0;
    int sub_warps = 0;      // warps per subtree CTA
    size_t sub_smem = 0;    // its dynamic shared memory
    // lane-per-row factorisation (factor_lane.cuh) for factors with short rows
    int factor_kernel = 0;  // 0 automatic, 1 warp per row, 2 lane per row (when the rows qualify)
    bool fact_lane = false;
    gb300::DeviceBuffer<int> lf_rows, lf_pub_off, lf_upd_ptr;
    gb300::DeviceBuffer<int2> lf_upd;
    gb300::DeviceBuffer<double> lf_pub;
    long long lf_pub_len = 0;
    int lf_ntask = 0, grid_lane_fact = 0;
    gb300::DeviceBuffer<double> lu;
    gb300::DeviceBuffer<double> shift;      // per-row diagonal shift (learned), optional
    gb300::DeviceBuffer<int> done;          // per-row ready stamps of the factorisation
    gb300::DeviceBuffer<unsigned> counters;  // ticket counters [0] fact, [1] L, [2] U
    gb300::DeviceBuffer<int> status;         // StatusWord array
    gb300::LevelPack L, U;     // level-ordered warp layout (default)
    // block-local layout per value type (used when blk64 / blk32 is set)
    gb300::BlockPack LB64, UB64, LB32, UB32;
    bool blk64 = false, blk32 = false;
    bool level_packs = false;  // L and U (level-ordered warp layout) are built
    // level-synchronous schedule (block_rows == -2): level-aligned packs, cooperative grid
    gb300::LevelPack LS, US;
    bool levelsync = false;
    int grid_levelsync = 0;
    // structured-grid line-pipeline sweeps (line_sweep.cuh) per value type, when the
    // factor is a 7- or 5-point stencil in natural order and grid_mode allows it
    gb300::LinePack GP;
    bool grid64 = false, grid32 = false;
    int grid_mode = 0;  // 1 or 0 (automatic): on when the pattern qualifies; -1: off
    int grid_wy = 0;    // requested lanes of a warp along y (0 automatic)
    int grid_by = 0;    // requested warps of a CTA along y (0 automatic)
    int grid_bz = 0;    // requested warps of a CTA along z (0 automatic)
    int grid_cluster = 1;  // 1: clusters along z of 16, else 8 CTAs; 2 .. 16: at most that many; 0: none
    bool sweep_timeline = false;  // record per-block timelines of the line-pipeline sweeps
    bool grid_one_cta_per_sm = false;  // line-pipeline CTAs request enough shared memory to be alone on an SM
    // line-pipeline sweeps in use per value type (bit 0: forward, bit 1: backward); in
    // automatic mode chosen at the first Factorize after SetupMatrix by timing each sweep
    // against the block-local / level-ordered kernel
    int line_use64 = 0, line_use32 = 0;
    bool line_tuned = true;
    unsigned setup_gen = 0;    // incremented by every SetupMatrix
    gb300::DeviceBuffer<double> sb64, sy64, sx64;  // Substitute() work vectors
    gb300::DeviceBuffer<float> sy32;               // FP32 forward-sweep intermediate

    int stamp = 0;
    bool factorized = false;
    bool copy_back = true;       // copy the factors into GetMatrix()->value after Factorize
    bool shift_active = false;   // add `shift` to the diagonal in the next Factorize
    // learned shift: MLP parameters on the device, the fused feature/inference pre-pass
    bool model_active = false;
    float min_shift = 0.f;
    gb300::DeviceBuffer<float> mlp;
    gb300::DeviceBuffer<int> depth_l;  // level depth of every row (MLP feature)
    gb300::ShiftPrepass prepass;
    bool shift_applied = false;        // the last Factorize used a (learned or explicit) shift
    int last_breakdowns = 0;
    int first_breakdown = -1;
    float last_factor_ms = 0.f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int grid_fact = 0;
    // factorisation launch: staged entries per warp, warps per block, pivot-row register
    // window per lane, dynamic shared memory per block
    int fact_cap = 0, fact_hcap = 0, fact_warps = 0, fact_pre = 2;
    size_t fact_smem = 0;
    // level-ordered substitution launch: grid_solve CTAs of solve_threads threads
    int grid_solve = 0, solve_threads = 0;
    int solve_warps = 0;  // requested warps for the level-ordered kernels (0 = automatic)
    int row_lanes = 0;    // requested lanes per row of the level-ordered kernels (0 = automatic)
    int wait_limit_us = 0;  // device wait limit in microseconds (0 = kWaitLimitUsDefault)
    int block_rows = 0;  // rows per substitution block (0 = automatic, -1 = level-ordered kernel,
                         // -2 = level-synchronous kernel)
    long long launches = 0;  // kernels launched by Factorize / Substitute

    ~Impl();

    // Device-side substitution pieces, used by GMRES (gated) and by Substitute().
    // lower: y = L^{-1}(scale * b) (b rescaled in place when scale != null);
    // upper: x = U^{-1} y (y reset to the sentinel).
    template <class T>
    void launch_lower(cudaStream_t s, T* b, const double* scale, T* y, const int* gate, int step) const;
    template <class T>
    void launch_upper(cudaStream_t s, T* y, T* x, const int* gate, int step) const;
    // Identifies the device data the substitution launches of type T read (CUDA graph key).
    template <class T>
    const void* subst_key() const;
    // Throws when a dependency wait timed out since the last call.
    void check_status(cudaStream_t s);
    // Writes wait_limit_us into the device status words (when they exist).
    void push_wait_limit();
};

}  // namespace lljbash
