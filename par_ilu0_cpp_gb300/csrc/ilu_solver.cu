// lljbash::IluSolver on GB300: host analysis of the pattern (bit-exact with the
// reference), sync-free ILU factorisation and sync-free triangular substitution on the
// device.  Replaces src/ilu_solver.cpp (SetupMatrix :225-373, Factorize :616-671,
// Substitute :736-831).
#include <cuda_runtime.h>

#include <algorithm>
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

namespace gb300 {

// Host construction of a packed factor from a schedule `order` (rows in level order).
// lower: entries [rp[r], diag[r]) ascending; upper: entries (diag[r], rp[r+1])
// descending plus the diagonal position.
static void build_level_pack(int n, const int* rp, const int* ci, const std::vector<int>& diag,
                       const std::vector<int>& order, bool lower, LevelPack& P, cudaStream_t s) {
    const int ntask = ceil_div(n, kWarp);
    std::vector<int> rows(static_cast<size_t>(ntask) * kWarp, -1);
    std::vector<int> off(ntask), len(ntask);
    std::vector<int> dsrc(lower ? 0 : static_cast<size_t>(ntask) * kWarp, -1);
    long long slots = 0;
    for (int t = 0; t < ntask; ++t) {
        int k = 0;
        for (int l = 0; l < kWarp; ++l) {
            const int q = t * kWarp + l;
            if (q >= n) break;
            const int r = order[q];
            rows[q] = r;
            const int cnt = lower ? diag[r] - rp[r] : rp[r + 1] - diag[r] - 1;
            k = std::max(k, cnt);
            if (!lower) dsrc[q] = diag[r];
        }
        off[t] = static_cast<int>(slots);
        len[t] = k;
        slots += static_cast<long long>(k) * kWarp;
        if (slots > INT_MAX) throw std::runtime_error("triangular factor too large for 32-bit slot offsets");
    }
    std::vector<int> cols(static_cast<size_t>(slots), -1), src(static_cast<size_t>(slots), -1);
    for (int t = 0; t < ntask; ++t) {
        for (int l = 0; l < kWarp; ++l) {
            const int q = t * kWarp + l;
            if (q >= n) break;
            const int r = order[q];
            int k = 0;
            if (lower) {
                for (int p = rp[r]; p < diag[r]; ++p, ++k) {
                    const size_t sidx = static_cast<size_t>(off[t]) + static_cast<size_t>(k) * kWarp + l;
                    cols[sidx] = ci[p];
                    src[sidx] = p;
                }
            } else {
                for (int p = rp[r + 1] - 1; p > diag[r]; --p, ++k) {
                    const size_t sidx = static_cast<size_t>(off[t]) + static_cast<size_t>(k) * kWarp + l;
                    cols[sidx] = ci[p];
                    src[sidx] = p;
                }
            }
        }
    }
    P.ntask = ntask;
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

// Host construction of a block-pipelined packed factor (see BlockTri).
// lower: entries [rp[r], diag[r]) ascending; upper: entries (diag[r], rp[r+1])
// descending plus the diagonal position.
static void build_pack(int n, const int* rp, const int* ci, const std::vector<int>& diag, bool lower,
                       int block_rows, TriPack& P, cudaStream_t s) {
    const int S = std::max(1, std::min(block_rows, std::max(n, 1)));
    const int nblk = n > 0 ? ceil_div(n, S) : 0;
    std::vector<int> blk_row(static_cast<size_t>(nblk) + 1), blk_lvl(static_cast<size_t>(nblk) + 1, 0);
    std::vector<int> lvl_task(1, 0), rows, off, len, dsrc;
    std::vector<int> depth(static_cast<size_t>(S)), cnt, ord;
    auto ebeg = [&](int r) { return lower ? rp[r] : diag[r] + 1; };
    auto eend = [&](int r) { return lower ? diag[r] : rp[r + 1]; };
    long long slots = 0;
    // pass 1: levels, tasks, lengths
    std::vector<std::vector<int>> blk_order(static_cast<size_t>(nblk));
    for (int c = 0; c < nblk; ++c) {
        const int lo = c * S;
        const int hi = std::min(n, lo + S);
        blk_row[c] = lo;
        int nlev = 0;
        for (int s2 = 0; s2 < hi - lo; ++s2) {
            const int r = lower ? lo + s2 : hi - 1 - s2;
            int d = 0;
            for (int p = ebeg(r); p < eend(r); ++p) {
                const int col = ci[p];
                if (col >= lo && col < hi) d = std::max(d, depth[col - lo] + 1);
            }
            depth[r - lo] = d;
            nlev = std::max(nlev, d + 1);
        }
        cnt.assign(static_cast<size_t>(nlev) + 1, 0);
        for (int r = lo; r < hi; ++r) ++cnt[depth[r - lo] + 1];
        for (int l = 0; l < nlev; ++l) cnt[l + 1] += cnt[l];
        ord.assign(static_cast<size_t>(hi - lo), 0);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int r = lo; r < hi; ++r) ord[fill[depth[r - lo]]++] = r;
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
                off.push_back(static_cast<int>(slots));
                len.push_back(K);
                slots += static_cast<long long>(K) * kWarp;
                if (slots > INT_MAX) throw std::runtime_error("triangular factor too large for 32-bit slot offsets");
            }
            lvl_task.push_back(static_cast<int>(off.size()));
        }
        blk_lvl[c + 1] = blk_lvl[c] + nlev;
    }
    blk_row[nblk] = n;
    const int ntask = static_cast<int>(off.size());
    // pass 2: entry codes and gather sources
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
    P.levels = blk_lvl[nblk];
    P.slots = slots;
    P.smem64 = sizeof(double) * static_cast<size_t>(S);
    P.smem32 = sizeof(float) * static_cast<size_t>(S);
    P.blk_row.upload(blk_row.data(), blk_row.size(), s);
    P.blk_lvl.upload(blk_lvl.data(), blk_lvl.size(), s);
    P.lvl_task.upload(lvl_task.data(), lvl_task.size(), s);
    P.rows.upload(rows.data(), rows.size(), s);
    P.off.upload(off.data(), off.size(), s);
    P.len.upload(len.data(), len.size(), s);
    P.codes.upload(codes.data(), codes.size(), s);
    P.src.upload(src.data(), src.size(), s);
    if (!lower) P.dsrc.upload(dsrc.data(), dsrc.size(), s);
    P.v64.reserve(static_cast<size_t>(slots));
    P.v32.reserve(static_cast<size_t>(slots));
    if (!lower) {
        P.d64.reserve(rows.size());
        P.d32.reserve(rows.size());
    }
    // host vectors must outlive the asynchronous copies
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
}

static void gather_pack(const TriPack& P, bool lower, const double* lu, cudaStream_t s, int sms) {
    const int threads = 256;
    auto grid_for = [&](long long count) {
        long long g = ceil_div<long long>(count, threads);
        return static_cast<int>(std::max<long long>(1, std::min<long long>(g, 8LL * sms)));
    };
    if (P.slots > 0) {
        pack_gather_kernel<double><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v64.get());
        pack_gather_kernel<float><<<grid_for(P.slots), threads, 0, s>>>(P.slots, P.src.get(), lu, P.v32.get());
    }
    if (!lower && P.ntask > 0) {
        const long long nd = static_cast<long long>(P.ntask) * kWarp;
        pack_gather_kernel<double><<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d64.get());
        pack_gather_recip_kernel<<<grid_for(nd), threads, 0, s>>>(nd, P.dsrc.get(), lu, P.d32.get());
    }
    GB_CUDA_CHECK(cudaGetLastError());
}

// Raises the dynamic shared-memory limit of both substitution kernels of type T to
// `smem` bytes; returns the persistent grid (CTAs resident at that footprint).
template <class T>
static int configure_block_kernels(size_t smem, int sms) {
    const int bytes = static_cast<int>(std::max<size_t>(smem, 16));
    GB_CUDA_CHECK(cudaFuncSetAttribute(sptrsv_block_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    GB_CUDA_CHECK(cudaFuncSetAttribute(sptrsv_block_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    int per_sm = 0;
    GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sptrsv_block_kernel<T, false>, kSolveThreads,
                                                               static_cast<size_t>(bytes)));
    return std::max(1, per_sm) * sms;
}

template <class T>
static void fill_sentinel(T* p, long long n, cudaStream_t s, int sms) {
    if (n <= 0) return;
    const int threads = 256;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>(ceil_div<long long>(n, threads), 8LL * sms)));
    fill_sentinel_kernel<T><<<grid, threads, 0, s>>>(n, p);
    GB_CUDA_CHECK(cudaGetLastError());
}

}  // namespace gb300

namespace lljbash {

using namespace gb300;

IluSolver::Impl::~Impl() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

template <class T>
void IluSolver::Impl::launch_lower(cudaStream_t s, T* b, const double* scale, T* y, const int* gate, int step) const {
    if (block_mode) {
        if (LB.nblk == 0) return;
        const int grid = sizeof(T) == 8 ? grid_block64 : grid_block32;
        const size_t smem = sizeof(T) == 8 ? LB.smem64 : LB.smem32;
        sptrsv_block_kernel<T, false><<<std::min(grid, LB.nblk), kSolveThreads, smem, s>>>(
            LB.view<T>(), b, scale, y, counters.get() + 1, status.get(), gate, step);
        return;
    }
    if (L.ntask == 0) return;
    sptrsv_lower_kernel<T><<<grid_solve, kSolveThreads, 0, s>>>(L.view<T>(), b, scale, y, counters.get() + 1,
                                                                status.get(), gate, step);
}

template <class T>
void IluSolver::Impl::launch_upper(cudaStream_t s, T* y, T* x, const int* gate, int step) const {
    if (block_mode) {
        if (UB.nblk == 0) return;
        const int grid = sizeof(T) == 8 ? grid_block64 : grid_block32;
        const size_t smem = sizeof(T) == 8 ? UB.smem64 : UB.smem32;
        sptrsv_block_kernel<T, true><<<std::min(grid, UB.nblk), kSolveThreads, smem, s>>>(
            UB.view<T>(), y, nullptr, x, counters.get() + 2, status.get(), gate, step);
        return;
    }
    if (U.ntask == 0) return;
    sptrsv_upper_kernel<T><<<grid_solve, kSolveThreads, 0, s>>>(U.view<T>(), y, x, counters.get() + 2, status.get(),
                                                                gate, step);
}

template void IluSolver::Impl::launch_lower<double>(cudaStream_t, double*, const double*, double*, const int*, int) const;
template void IluSolver::Impl::launch_lower<float>(cudaStream_t, float*, const double*, float*, const int*, int) const;
template void IluSolver::Impl::launch_upper<double>(cudaStream_t, double*, double*, const int*, int) const;
template void IluSolver::Impl::launch_upper<float>(cudaStream_t, float*, float*, const int*, int) const;

void IluSolver::Impl::check_status(cudaStream_t s) {
    int h[kStatusWords];
    GB_CUDA_CHECK(cudaMemcpyAsync(h, status.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (h[kStatusTimeout] != 0) {
        const int zero = 0;
        GB_CUDA_CHECK(cudaMemcpy(status.get() + kStatusTimeout, &zero, sizeof(int), cudaMemcpyHostToDevice));
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
    im.block_mode = im.block_rows > 0;
    if (im.block_mode) {
        build_pack(n, rp, ci, im.an.diag, true, im.block_rows, im.LB, s);
        build_pack(n, rp, ci, im.an.diag, false, im.block_rows, im.UB, s);
    } else {
        build_level_pack(n, rp, ci, im.an.diag, im.an.order_l, true, im.L, s);
        build_level_pack(n, rp, ci, im.an.diag, im.an.order_u, false, im.U, s);
    }
    const size_t nv = static_cast<size_t>(std::max(n, 1));
    im.sb64.reserve(nv);
    im.sy64.reserve(nv);
    im.sx64.reserve(nv);
    im.sy32.reserve(nv);
    fill_sentinel(im.sy64.get(), static_cast<long long>(nv), s, im.dev.sms);
    fill_sentinel(im.sy32.get(), static_cast<long long>(nv), s, im.dev.sms);
    im.grid_fact = persistent_grid(ilu_factor_kernel, kFactWarps * kWarp, im.dev.sms);
    // One CTA of the level-ordered kernel per SM: fewer spinning warps contend less for
    // L2 and the ready values propagate faster (measured: 1/SM beats full occupancy by
    // 1.8x on the 128^3 7-point factor).
    im.grid_solve = im.dev.sms;
    if (im.block_mode) {
        im.grid_block64 = configure_block_kernels<double>(std::max(im.LB.smem64, im.UB.smem64), im.dev.sms);
        im.grid_block32 = configure_block_kernels<float>(std::max(im.LB.smem32, im.UB.smem32), im.dev.sms);
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
        int init[kStatusWords] = {0, 0, INT_MAX, 0};
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
            ilu_factor_kernel<<<im.grid_fact, kFactWarps * kWarp, 0, s>>>(
                n, im.rp.get(), im.ci.get(), im.diag.get(), im.order_l.get(), im.lu.get(), shift, im.done.get(),
                im.stamp, im.counters.get(), im.status.get());
            GB_CUDA_CHECK(cudaGetLastError());
            if (im.block_mode) {
                gather_pack(im.LB, true, im.lu.get(), s, im.dev.sms);
                gather_pack(im.UB, false, im.lu.get(), s, im.dev.sms);
            } else {
                gather_level_pack(im.L, true, im.lu.get(), s, im.dev.sms);
                gather_level_pack(im.U, false, im.lu.get(), s, im.dev.sms);
            }
            im.launches += 7;
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
    int device = 0;
    GB_CUDA_CHECK(cudaGetDevice(&device));
    unsigned char* base = static_cast<unsigned char*>(noalloc_scratch_address(device));
    double* y = reinterpret_cast<double*>(base);
    unsigned* counters = reinterpret_cast<unsigned*>(base + kNoAllocMaxRows * sizeof(double));
    int* status = reinterpret_cast<int*>(counters + 4);
    cudaStream_t s = im.stream;
    // what must start at zero (counters, status) and at the sentinel (y, x)
    GB_CUDA_CHECK(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned) + kStatusWords * sizeof(int), s));
    fill_sentinel(y, n, s, im.dev.sms);
    fill_sentinel(d_x, n, s, im.dev.sms);
    double* b = const_cast<double*>(d_b);  // read only: no scale is passed to the forward sweep
    if (im.block_mode) {
        if (im.LB.nblk > 0) {
            sptrsv_block_kernel<double, false><<<std::min(im.grid_block64, im.LB.nblk), kSolveThreads, im.LB.smem64, s>>>(
                im.LB.view<double>(), b, nullptr, y, counters + 1, status, nullptr, 0);
            sptrsv_block_kernel<double, true><<<std::min(im.grid_block64, im.UB.nblk), kSolveThreads, im.UB.smem64, s>>>(
                im.UB.view<double>(), y, nullptr, d_x, counters + 2, status, nullptr, 0);
        }
    } else if (im.L.ntask > 0) {
        sptrsv_lower_kernel<double><<<im.grid_solve, kSolveThreads, 0, s>>>(im.L.view<double>(), b, nullptr, y,
                                                                            counters + 1, status, nullptr, 0);
        sptrsv_upper_kernel<double><<<im.grid_solve, kSolveThreads, 0, s>>>(im.U.view<double>(), y, d_x, counters + 2,
                                                                            status, nullptr, 0);
    }
    GB_CUDA_CHECK(cudaGetLastError());
    int h[kStatusWords];
    GB_CUDA_CHECK(cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (h[kStatusTimeout] != 0) throw std::runtime_error("dependency wait timed out on the device");
}

}  // namespace lljbash
