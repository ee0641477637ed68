// C ABI: the reference's LLJBASH_* wrappers (src_c/ilu_solver_c.cpp, src_c/gmres_c.cpp)
// plus the GB300 extensions of par_ilu0_gb300.h.
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "analysis.hpp"
#include "tree_schedule.hpp"
#include "batched_impl.hpp"
#include "gmres.hpp"
#include "gmres_c.h"
#include "gmres_impl.hpp"
#include "ilu_impl.hpp"
#include "ilu_solver.hpp"
#include "ilu_solver_c.h"
#include "mlp.cuh"
#include "mlp_impl.hpp"
#include "par_ilu0_gb300.h"

using lljbash::IluSolver;
using lljbash::PreconditionedGmres;

namespace {

thread_local std::string g_last_error;

int fail(const std::exception& e) {
    g_last_error = e.what();
    return std::string(e.what()) == "missing diag" ? -2 : -1;
}

IluSolver* ilu(IluSolverHdl h) { return static_cast<IluSolver*>(h); }
PreconditionedGmres* gm(GmresHdl h) { return static_cast<PreconditionedGmres*>(h); }

}  // namespace

extern "C" {

const char* LLJBASH_Gb300LastError(void) { return g_last_error.c_str(); }

IluSolverHdl IluSolverCreate(int nthreads) {
    auto* h = new IluSolver;
    h->SetThreads(nthreads);
    return h;
}

void IluSolverDestroy(IluSolverHdl hdl) { delete ilu(hdl); }

CsrMatrix* IluSolverGetMatrix(IluSolverHdl hdl) { return ilu(hdl)->GetMatrix(); }

int IluSolverSetup(IluSolverHdl hdl) {
    try {
        ilu(hdl)->SetupMatrix();
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int IluSolverFactorize(IluSolverHdl hdl) {
    try {
        ilu(hdl)->Factorize();
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

GmresHdl GmresCreate(void) { return new PreconditionedGmres; }

void GmresDestroy(GmresHdl hdl) { delete gm(hdl); }

GmresParameters* GmresGetParameters(GmresHdl hdl) { return &gm(hdl)->param(); }

const GmresStat* GmresGetStat(GmresHdl hdl) { return &gm(hdl)->stat(); }

void GmresSetPreconditioner(GmresHdl hdl, IluSolverHdl ilu_hdl) { gm(hdl)->SetIluPreconditioner(ilu(ilu_hdl)); }

bool GmresSolve(GmresHdl hdl, const CsrMatrix* mat, double* rhs, double* sol, int* iter) {
    try {
        auto ret = gm(hdl)->Solve(mat, rhs, sol);
        if (iter) *iter = ret.second;
        return ret.first;
    } catch (const std::exception& e) {
        fail(e);
        if (iter) *iter = 0;
        return false;
    }
}

int LLJBASH_IluSolverSubstitute(IluSolverHdl hdl, const double* b, double* x) {
    try {
        ilu(hdl)->Substitute(b, x);
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_IluSolverSubstituteDeviceNoAlloc(IluSolverHdl hdl, const double* d_b, double* d_x) {
    try {
        ilu(hdl)->SubstituteDeviceNoAlloc(d_b, d_x);
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_IluSolverFactorizeDevice(IluSolverHdl hdl, const double* d_values) {
    try {
        ilu(hdl)->FactorizeDevice(d_values);
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

bool LLJBASH_GmresSolveDevice(GmresHdl hdl, int n, const int* d_row_ptr, const int* d_col_idx, const double* d_values,
                              const double* d_rhs, double* d_sol, int* iter) {
    try {
        auto ret = gm(hdl)->SolveDevice(n, d_row_ptr, d_col_idx, d_values, d_rhs, d_sol);
        if (iter) *iter = ret.second;
        return ret.first;
    } catch (const std::exception& e) {
        fail(e);
        if (iter) *iter = 0;
        return false;
    }
}

int LLJBASH_IluSolverSetOption(IluSolverHdl hdl, int option, double value) {
    try {
        IluSolver* s = ilu(hdl);
        if (!s->impl()) s->impl_ensure();
        switch (option) {
            case LLJBASH_ILU_OPT_COPY_BACK:
                s->impl()->copy_back = value != 0.0;
                return 0;
            case LLJBASH_ILU_OPT_SOLVE_WARPS:
                if (value < 0 || value > 1e6) throw std::runtime_error("solve warps must be 0 (automatic) or a warp count");
                s->impl()->solve_warps = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_ROW_LANES: {
                const int v = static_cast<int>(value);
                if (value != v || (v != 0 && (v & (v - 1)) != 0) || v < 0 || v > 32)
                    throw std::runtime_error("row lanes must be 0 (automatic), 1, 2, 4, 8, 16 or 32");
                s->impl()->row_lanes = v;
                return 0;
            }
            case LLJBASH_ILU_OPT_WAIT_LIMIT_US:
                if (value < 0 || value > 2147483647.0 || value != static_cast<int>(value))
                    throw std::runtime_error("wait limit must be 0 (default) or a number of microseconds");
                s->impl()->wait_limit_us = static_cast<int>(value);
                s->impl()->push_wait_limit();
                return 0;
            case LLJBASH_ILU_OPT_BLOCK_ROWS:
                if (value < -2 || value > 1e8) throw std::runtime_error("block rows must be -2, -1, 0 or a row count");
                s->impl()->block_rows = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_FACTOR_KERNEL:
                if (value != 0 && value != 1 && value != 2) throw std::runtime_error("factor kernel must be 0, 1 or 2");
                s->impl()->factor_kernel = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_TICKET_ORDER:
                if (value != 0 && value != 1 && value != 2) throw std::runtime_error("ticket order must be 0, 1 or 2");
                s->impl()->ticket_order = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_GRID:
                if (value != -1 && value != 0 && value != 1) throw std::runtime_error("grid sweeps must be -1, 0 or 1");
                s->impl()->grid_mode = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_GRID_WARP_Y:
                if (value != 0 && value != 1 && value != 4 && value != 8)
                    throw std::runtime_error("grid lanes of a warp along y must be 0 (automatic), 1, 4 or 8");
                s->impl()->grid_wy = static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_GRID_CTA_Y:
            case LLJBASH_ILU_OPT_GRID_CTA_Z:
                if (value < 0 || value > 8 || value != static_cast<int>(value))
                    throw std::runtime_error("grid warps of a CTA must be 0 (automatic) or 1 .. 8");
                (option == LLJBASH_ILU_OPT_GRID_CTA_Y ? s->impl()->grid_by : s->impl()->grid_bz) =
                    static_cast<int>(value);
                return 0;
            case LLJBASH_ILU_OPT_GRID_ONE_CTA_PER_SM:
                if (value != 0 && value != 1) throw std::runtime_error("one CTA per SM must be 0 or 1");
                s->impl()->grid_one_cta_per_sm = value != 0;
                return 0;
            case LLJBASH_ILU_OPT_SWEEP_TIMELINE:
                if (value != 0 && value != 1) throw std::runtime_error("sweep timeline must be 0 or 1");
                s->impl()->sweep_timeline = value != 0;
                return 0;
            case LLJBASH_ILU_OPT_GRID_CLUSTER:
                if (value < 0 || value > 16 || value != static_cast<int>(value))
                    throw std::runtime_error("grid clusters must be 0 (none), 1 (automatic) or 2 .. 16 CTAs");
                s->impl()->grid_cluster = static_cast<int>(value);
                return 0;
            default:
                g_last_error = "unknown ILU option";
                return -1;
        }
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int LLJBASH_IluSolverSetShift(IluSolverHdl hdl, const double* shift) {
    try {
        IluSolver* s = ilu(hdl);
        if (!s->impl() || s->impl()->n != s->GetMatrix()->size) throw std::runtime_error("SetupMatrix() must be called first");
        auto* im = s->impl();
        if (!shift) {
            im->shift_active = false;
            return 0;
        }
        im->shift.upload(shift, static_cast<size_t>(im->n), im->stream);
        GB_CUDA_CHECK(cudaStreamSynchronize(im->stream));
        im->shift_active = true;
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_IluSolverSetShiftModel(IluSolverHdl hdl, const float* params, int nparams, double min_shift) {
    try {
        ilu(hdl)->SetShiftModel(params, nparams, static_cast<float>(min_shift));
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_ShiftModelNumParams(void) { return gb300::kMlpParams; }

int LLJBASH_ShiftFeatures(int n, const int* row_ptr, const int* col_idx, const double* values, const int* depth,
                          int nlev, float* X, const float* params, float* y) {
    try {
        gb300::shift_features_host(n, row_ptr, col_idx, values, depth, nlev, X, params, y);
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

LLJBASH_ShiftTrainerHdl LLJBASH_ShiftTrainerCreate(unsigned seed) {
    try {
        return new gb300::ShiftTrainer(seed);
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}

void LLJBASH_ShiftTrainerDestroy(LLJBASH_ShiftTrainerHdl tr) { delete static_cast<gb300::ShiftTrainer*>(tr); }

#define GB_TRY(stmt)                       \
    try {                                  \
        stmt;                              \
    } catch (const std::exception& e) {    \
        return fail(e);                    \
    }                                      \
    return 0

int LLJBASH_ShiftTrainerSetData(LLJBASH_ShiftTrainerHdl tr, const float* X, const float* targets, int n) {
    GB_TRY(static_cast<gb300::ShiftTrainer*>(tr)->set_data(X, targets, n));
}

int LLJBASH_ShiftTrainerSetParams(LLJBASH_ShiftTrainerHdl tr, const float* params) {
    GB_TRY(static_cast<gb300::ShiftTrainer*>(tr)->set_params(params));
}

int LLJBASH_ShiftTrainerGetParams(LLJBASH_ShiftTrainerHdl tr, float* params) {
    GB_TRY(static_cast<gb300::ShiftTrainer*>(tr)->get_params(params));
}

int LLJBASH_ShiftTrainerStep(LLJBASH_ShiftTrainerHdl tr, const int* idx, int batch, float lr, double* loss) {
    GB_TRY({
        const double l = static_cast<gb300::ShiftTrainer*>(tr)->run(idx, batch, lr, true, nullptr);
        if (loss) *loss = l;
    });
}

int LLJBASH_ShiftTrainerGradient(LLJBASH_ShiftTrainerHdl tr, float* grad, double* loss) {
    GB_TRY({
        const double l = static_cast<gb300::ShiftTrainer*>(tr)->run(nullptr, 0, 0.f, false, grad);
        if (loss) *loss = l;
    });
}

int LLJBASH_ShiftTrainerPredict(LLJBASH_ShiftTrainerHdl tr, float* y) {
    GB_TRY(static_cast<gb300::ShiftTrainer*>(tr)->predict(y));
}

LLJBASH_BatchHdl LLJBASH_BatchCreate(int nsys, const int* n, const int* row_ptr, const int* col_idx,
                                     const double* values, int nrhs, int restart, double rtol, int maxit) {
    try {
        return new gb300::BatchSolver(nsys, n, row_ptr, col_idx, values, nrhs, restart, rtol, maxit);
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}

LLJBASH_BatchHdl LLJBASH_BatchCreateEx(int nsys, const int* n, const int* row_ptr, const int* col_idx,
                                       const double* values, const double* factor_values, int nrhs, int restart,
                                       double rtol, int maxit) {
    try {
        return new gb300::BatchSolver(nsys, n, row_ptr, col_idx, values, nrhs, restart, rtol, maxit, factor_values);
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}

void LLJBASH_BatchDestroy(LLJBASH_BatchHdl hdl) { delete static_cast<gb300::BatchSolver*>(hdl); }

int LLJBASH_BatchSetShiftModel(LLJBASH_BatchHdl hdl, const float* params, int nparams, double min_shift) {
    GB_TRY({
        if (params && nparams != gb300::kMlpParams) throw std::runtime_error("shift model must have 369 parameters");
        static_cast<gb300::BatchSolver*>(hdl)->set_model(params, static_cast<float>(min_shift));
    });
}

int LLJBASH_BatchAutotune(LLJBASH_BatchHdl hdl, int* ctas_per_sm, int* largest_first) {
    GB_TRY({
        auto* b = static_cast<gb300::BatchSolver*>(hdl);
        b->autotune();
        if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm();
        if (largest_first) *largest_first = b->largest_first() ? 1 : 0;
    });
}

int LLJBASH_BatchGetShape(LLJBASH_BatchHdl hdl, int* ctas_per_sm, int* largest_first, int* rhs_per_cta) {
    GB_TRY({
        const auto* b = static_cast<gb300::BatchSolver*>(hdl);
        if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm();
        if (largest_first) *largest_first = b->largest_first() ? 1 : 0;
        if (rhs_per_cta) *rhs_per_cta = b->rhs_per_cta();
    });
}

int LLJBASH_BatchSetShape(LLJBASH_BatchHdl hdl, int ctas_per_sm, int largest_first, int rhs_per_cta) {
    GB_TRY({ static_cast<gb300::BatchSolver*>(hdl)->set_shape(ctas_per_sm, largest_first != 0, rhs_per_cta); });
}

int LLJBASH_BatchGetTrials(LLJBASH_BatchHdl hdl, int cap, int* ctas_per_sm, int* largest_first, int* rhs_per_cta,
                           double* ms) {
    const auto& t = static_cast<gb300::BatchSolver*>(hdl)->trials();
    const int k = static_cast<int>(t.size());
    for (int i = 0; i < k && i < cap; ++i) {
        if (ctas_per_sm) ctas_per_sm[i] = t[i].ctas_per_sm;
        if (largest_first) largest_first[i] = t[i].largest_first;
        if (rhs_per_cta) rhs_per_cta[i] = t[i].rhs_per_cta;
        if (ms) ms[i] = t[i].ms;
    }
    return k;
}

int LLJBASH_BatchSolve(LLJBASH_BatchHdl hdl, const double* rhs, double* x, int* iters, double* resid, int* converged,
                       double* ms) {
    GB_TRY({
        const float t = static_cast<gb300::BatchSolver*>(hdl)->solve(rhs, x, iters, resid, converged);
        if (ms) *ms = t;
    });
}

int LLJBASH_IluSolverGetInfo(IluSolverHdl hdl, LLJBASH_IluInfo* info) {
    IluSolver* s = ilu(hdl);
    if (!info) return -1;
    std::memset(info, 0, sizeof(*info));
    const auto* im = s->impl();
    if (!im) {
        g_last_error = "SetupMatrix() has not been called";
        return -1;
    }
    info->n = im->n;
    info->nnz = static_cast<int>(im->nnz);
    info->levels_lower = im->an.nlev_l;
    info->levels_upper = im->an.nlev_u;
    info->breakdowns = im->last_breakdowns;
    info->first_breakdown = im->first_breakdown;
    info->factor_ms = im->last_factor_ms;
    info->kernel_launches = im->launches;
    info->shift_applied = im->shift_applied ? 1 : 0;
    info->block_rows_fp64 = im->blk64 ? im->LB64.block_rows : 0;
    info->block_rows_fp32 = im->blk32 ? im->LB32.block_rows : 0;
    info->block_cluster_fp64 = im->blk64 ? im->LB64.cl : 0;
    info->block_cluster_fp32 = im->blk32 ? im->LB32.cl : 0;
    info->row_lanes_lower = im->level_packs ? im->L.group : 0;
    info->row_lanes_upper = im->level_packs ? im->U.group : 0;
    info->factor_lane = im->fact_lane ? 1 : 0;
    info->factor_subtree_parts = im->ticket_order == 2 ? im->sub_parts : 0;
    info->factor_subtree_rows = im->ticket_order == 2 ? im->sub_rows : 0;
    info->grid_fp64 = im->line_use64;
    info->grid_fp32 = im->line_use32;
    if (im->grid64 || im->grid32) {
        info->grid_nx = im->GP.g.nx;
        info->grid_ny = im->GP.g.ny;
        info->grid_nz = im->GP.g.nz;
        info->grid_warp_y = im->GP.g.wy;
        info->grid_warp_z = im->GP.g.wz;
        info->grid_cta_y = im->GP.g.by;
        info->grid_cta_z = im->GP.g.bz;
        info->grid_blocks = im->GP.g.nblk;
        info->grid_cluster = im->GP.g.cl;
    }
    return 0;
}

int LLJBASH_IluSolverGetSweepTimeline(IluSolverHdl hdl, int upper, int fp32, unsigned long long* out, int cap) {
    try {
        const auto* im = ilu(hdl)->impl();
        if (!im) throw std::runtime_error("SetupMatrix() has not been called");
        const auto& buf = im->GP.tl[fp32 ? 1 : 0][upper ? 1 : 0];
        if (buf.get() == nullptr)
            throw std::runtime_error(
                "no sweep timeline: set LLJBASH_ILU_OPT_SWEEP_TIMELINE before IluSolverSetup (line-pipeline sweeps of "
                "structured factors only)");
        const int nblk = im->GP.g.nblk;
        const size_t len = static_cast<size_t>(nblk) * gb300::kLineTimeline;
        if (out != nullptr) {
            if (cap < 0 || static_cast<size_t>(cap) < len) throw std::runtime_error("timeline buffer too small");
            // the solver's device for the wait and the copy, the caller's current device
            // back afterwards (also when either fails)
            struct CurrentDevice {
                int prev = 0;
                explicit CurrentDevice(int d) {
                    GB_CUDA_CHECK(cudaGetDevice(&prev));
                    GB_CUDA_CHECK(cudaSetDevice(d));
                }
                ~CurrentDevice() { cudaSetDevice(prev); }
            } current(im->dev.device);
            GB_CUDA_CHECK(cudaDeviceSynchronize());
            GB_CUDA_CHECK(cudaMemcpy(out, buf.get(), len * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        }
        return nblk;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int LLJBASH_Gb300TreeSchedule(int n, const int* row_ptr, const int* col_idx, int upper, int nproc, int granularity,
                              double relax, int* part_ptr, int* partitions, int* task_queue, int* ntasks,
                              int* subtree_size, int* subtree_weight) {
    try {
        gb300::validate_csr(n, row_ptr, col_idx, "pattern");
        if (granularity < 1) throw std::runtime_error("tree schedule granularity must be at least 1");
        std::vector<int> diag;
        gb300::diagonal_pointers(n, row_ptr, col_idx, diag);
        const gb300::DagView g{row_ptr, col_idx, diag.data(), upper == 0};
        const gb300::RowWeights w = upper ? gb300::RowWeights{diag.data(), row_ptr + 1, 0, 0}
                                          : gb300::RowWeights{row_ptr, diag.data(), 0, 1};
        const gb300::TreeScheduleResult r = gb300::tree_schedule(n, g, nproc, granularity, relax, w);
        auto put = [](int* dst, const std::vector<int>& v) {
            if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(int));
        };
        put(part_ptr, r.part_ptr);
        put(partitions, r.partitions);
        put(task_queue, r.task_queue);
        put(subtree_size, r.subtree_size);
        put(subtree_weight, r.subtree_weight);
        if (ntasks) *ntasks = r.ntasks;
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_IluSolverGetAnalysis(IluSolverHdl hdl, int* diag, int* etree_lower, int* etree_upper, int* depth_lower,
                                 int* depth_upper) {
    const auto* im = ilu(hdl)->impl();
    if (!im) {
        g_last_error = "SetupMatrix() has not been called";
        return -1;
    }
    const size_t n = static_cast<size_t>(im->n);
    auto put = [n](int* dst, const std::vector<int>& v) {
        if (dst && n) std::memcpy(dst, v.data(), n * sizeof(int));
    };
    put(diag, im->an.diag);
    put(etree_lower, im->an.etree_l);
    put(etree_upper, im->an.etree_u);
    put(depth_lower, im->an.depth_l);
    put(depth_upper, im->an.depth_u);
    return 0;
}

int LLJBASH_Gb300AnalyzePattern(int n, const int* row_ptr, const int* col_idx, int* diag, int* etree_lower,
                                int* etree_upper, int* depth_lower, int* depth_upper, int* nlevels) {
    try {
        gb300::validate_csr(n, row_ptr, col_idx, "pattern");
        gb300::Analysis an;
        gb300::diagonal_pointers(n, row_ptr, col_idx, an.diag);
        const gb300::DagView gl{row_ptr, col_idx, an.diag.data(), true};
        const gb300::DagView gu{row_ptr, col_idx, an.diag.data(), false};
        gb300::elimination_tree(n, gl, an.etree_l);
        gb300::elimination_tree(n, gu, an.etree_u);
        an.nlev_l = gb300::level_sets(n, gl, an.depth_l, an.order_l, an.lptr_l);
        an.nlev_u = gb300::level_sets(n, gu, an.depth_u, an.order_u, an.lptr_u);
        const size_t sz = static_cast<size_t>(n);
        auto put = [sz](int* dst, const std::vector<int>& v) {
            if (dst && sz) std::memcpy(dst, v.data(), sz * sizeof(int));
        };
        put(diag, an.diag);
        put(etree_lower, an.etree_l);
        put(etree_upper, an.etree_u);
        put(depth_lower, an.depth_l);
        put(depth_upper, an.depth_u);
        if (nlevels) {
            nlevels[0] = an.nlev_l;
            nlevels[1] = an.nlev_u;
        }
    } catch (const std::exception& e) {
        return fail(e);
    }
    return 0;
}

int LLJBASH_GmresSetOption(GmresHdl hdl, int option, double value) {
    try {
        PreconditionedGmres* g = gm(hdl);
        if (!g->impl()) g->impl_ensure();
        auto* im = g->impl();
        switch (option) {
            case LLJBASH_GMRES_OPT_MODE:
                if (value != 0.0 && value != 1.0) throw std::runtime_error("mode must be 0 or 1");
                im->mode = static_cast<int>(value);
                return 0;
            case LLJBASH_GMRES_OPT_TAU:
                if (!(value > 0.0 && value < 1.0)) throw std::runtime_error("tau must be in (0, 1)");
                im->tau = value;
                return 0;
            case LLJBASH_GMRES_OPT_USE_GRAPH:
                im->use_graph = value != 0.0;
                return 0;
            case LLJBASH_GMRES_OPT_PROFILE:
                im->profile = value != 0.0;
                return 0;
            case LLJBASH_GMRES_OPT_KEEP_MATRIX:
                im->keep_matrix = value != 0.0;
                return 0;
            case LLJBASH_GMRES_OPT_VERIFY:
                im->verify = value != 0.0;
                return 0;
            default:
                g_last_error = "unknown GMRES option";
                return -1;
        }
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int LLJBASH_GmresGetReport(GmresHdl hdl, LLJBASH_GmresReport* report) {
    auto* im = gm(hdl)->impl();
    if (!report) return -1;
    std::memset(report, 0, sizeof(*report));
    if (!im) {
        report->residual = -1;
        return 0;
    }
    report->mode = im->report.mode;
    report->iterations = im->report.iterations;
    report->cycles = im->report.cycles;
    report->converged = im->report.converged;
    report->residual = im->report.residual;
    report->solve_ms = im->report.solve_ms;
    report->kernel_launches = im->launches;
    return 0;
}

int LLJBASH_GmresGetKernelTimes(GmresHdl hdl, double* ms, long long* launches, int nkinds) {
    auto* im = gm(hdl)->impl();
    for (int k = 0; k < nkinds; ++k) {
        if (ms) ms[k] = (im && k < gb300::kKKinds) ? im->kernel_ms[k] : 0.0;
        if (launches) launches[k] = (im && k < gb300::kKKinds) ? im->kernel_launches[k] : 0;
    }
    return 0;
}

int LLJBASH_GmresResetKernelTimes(GmresHdl hdl) {
    auto* im = gm(hdl)->impl();
    if (im) {
        for (int k = 0; k < gb300::kKKinds; ++k) {
            im->kernel_ms[k] = 0.0;
            im->kernel_launches[k] = 0;
        }
    }
    return 0;
}

}  // extern "C"
