/*
 * Oracle test infrastructure only: never linked into, or called by, the product
 * library.  Compiled together with the reference's own, unmodified sources
 * (src/csr_matrix.cpp, src/iluk.cpp, src/ilu_solver.cpp, src/gmres.cpp,
 * src_c/ilu_solver_c.cpp, src_c/gmres_c.cpp) into oracle/_ref/libref.so by
 * oracle/build_ref.sh, so that tests and the fixture generator can run the
 * reference itself through ctypes.
 *
 * Everything here is a thin plain-pointer wrapper around reference entry points:
 *   IlukSymbolic                 src/iluk.cpp:5-54
 *   IluSolver::SetupMatrix       src/ilu_solver.cpp:225-373
 *   IluSolver::Factorize         src/ilu_solver.cpp:616-671
 *   IluSolver::Substitute        src/ilu_solver.cpp:736-831
 *   PreconditionedGmres::Solve   src/gmres.cpp:138-288
 *   build_etree_parent           src/subtree.hpp:35-68
 *   Levelization::levelize       src/subtree.hpp:524-551
 * The one restated piece is the diagonal-pointer scan (src/ilu_solver.cpp:276-289),
 * which lives in the private IluSolver::Ext and is three lines long.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "csr_matrix.h"
#include "gmres.hpp"
#include "ilu_solver.hpp"
#include "iluk.h"
#include "subtree.hpp"

using namespace lljbash;

namespace {
CsrMatrix g_last_f;  // result of the last ref_iluk_symbolic call
std::vector<int> g_last_nzmap;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void load_matrix(CsrMatrix* m, int n, const int* rp, const int* ci, const double* val) {
    const int nnz = rp[n];
    SetupCsrMatrix(m, n, nnz);
    std::copy_n(rp, n + 1, m->row_ptr);
    std::copy_n(ci, nnz, m->col_idx);
    if (val) {
        std::copy_n(val, nnz, m->value);
    } else {
        std::fill_n(m->value, nnz, 0.0);
    }
}
}  // namespace

extern "C" {

/* IlukSymbolic on A; keeps F and nzmap for ref_iluk_fetch; returns nnz(F). */
int ref_iluk_symbolic(int n, const int* rp, const int* ci, const double* val, int lof) {
    CsrMatrix a;
    load_matrix(&a, n, rp, ci, val);
    DestroyCsrMatrix(&g_last_f);
    g_last_f = CsrMatrix();
    g_last_nzmap.assign(static_cast<size_t>(rp[n]), -1);
    int knnz = IlukSymbolic(&a, lof, &g_last_f, g_last_nzmap.data());
    DestroyCsrMatrix(&a);
    return knnz;
}

/* Copies the last F (row_ptr[n+1], col_idx[knnz], value[knnz]) and nzmap[nnz(A)].
 * F's fill entries are left uninitialised by the reference (SetupCsrMatrix does not
 * zero them); they are written as 0 here, as test/benchmark.cpp:116 does before use. */
void ref_iluk_fetch(int* f_rp, int* f_ci, double* f_val, int* nzmap) {
    const int n = g_last_f.size;
    const int knnz = g_last_f.row_ptr[n];
    std::copy_n(g_last_f.row_ptr, n + 1, f_rp);
    std::copy_n(g_last_f.col_idx, knnz, f_ci);
    if (f_val) {
        std::fill_n(f_val, knnz, 0.0);
        for (size_t i = 0; i < g_last_nzmap.size(); ++i) f_val[g_last_nzmap[i]] = g_last_f.value[g_last_nzmap[i]];
    }
    if (nzmap) std::copy(g_last_nzmap.begin(), g_last_nzmap.end(), nzmap);
}

/* diag_ptr[i] = first position in row i with col >= i (src/ilu_solver.cpp:276-289). */
void ref_diag_ptr(int n, const int* rp, const int* ci, int* diag) {
    for (int i = 0; i < n; ++i) {
        for (int ji = rp[i]; ji < rp[i + 1]; ++ji) {
            if (ci[ji] >= i) {
                diag[i] = ji;
                break;
            }
        }
    }
}

/* Liu elimination tree of the L-DAG (lower != 0) or of the reversed U-DAG, exactly as
 * SetupMatrix hands them to tree_schedule (src/ilu_solver.cpp:321, :339). Roots get n. */
void ref_etree(int n, const int* rp, const int* ci, const int* diag, int lower, int* parent) {
    std::vector<int> stripped(static_cast<size_t>(n), 0);
    std::vector<int> root(static_cast<size_t>(n) + 1);
    if (lower) {
        build_etree_parent(n, 0, n, 1, ConstBiasArray<int>(const_cast<int*>(rp)), diag, ci, stripped.data(),
                           parent, root.data());
    } else {
        build_etree_parent(n, n - 1, -1, -1, ConstBiasArray<int>(const_cast<int*>(diag), 1), rp + 1, ci,
                           stripped.data(), parent, root.data());
    }
}

/* Level depth of every row in the L-DAG (lower != 0) or reversed U-DAG
 * (Levelization::levelize).  Returns the number of levels. */
int ref_levels(int n, const int* rp, const int* ci, const int* diag, int lower, int* depth) {
    Levelization lv;
    if (lower) {
        lv.levelize(0, n, 1, ConstBiasArray<int>(const_cast<int*>(rp)), diag, ci);
    } else {
        lv.levelize(n - 1, -1, -1, ConstBiasArray<int>(const_cast<int*>(diag), 1), rp + 1, ci);
    }
    for (int l = 0; l < lv.nlevels; ++l) {
        for (int k = lv.lset_ptr[l]; k < lv.lset_ptr[l + 1]; ++k) depth[lv.lset[k]] = l;
    }
    return lv.nlevels;
}

/* In-place ILU on the given pattern (SetupMatrix + Factorize). times[0..1] = setup, factorize (s). */
void ref_factorize(int n, const int* rp, const int* ci, double* val, int nthreads, double* times) {
    IluSolver s;
    s.SetThreads(nthreads);
    load_matrix(s.GetMatrix(), n, rp, ci, val);
    double t0 = now_s();
    s.SetupMatrix();
    double t1 = now_s();
    s.Factorize();
    double t2 = now_s();
    std::copy_n(s.GetMatrix()->value, rp[n], val);
    if (times) {
        times[0] = t1 - t0;
        times[1] = t2 - t1;
    }
}

/* x = U^{-1} L^{-1} b with already-factorised LU values (SetupMatrix + Substitute). */
void ref_substitute(int n, const int* rp, const int* ci, const double* lu, const double* b, double* x,
                    int nthreads, int reps, double* seconds) {
    IluSolver s;
    s.SetThreads(nthreads);
    load_matrix(s.GetMatrix(), n, rp, ci, lu);
    s.SetupMatrix();
    double t0 = now_s();
    for (int r = 0; r < std::max(reps, 1); ++r) s.Substitute(b, x);
    double t1 = now_s();
    if (seconds) *seconds = (t1 - t0) / std::max(reps, 1);
}

/* The test/benchmark.cpp:89-131 sequence: IlukSymbolic(A, lof) -> zero F, scatter A
 * through nzmap -> SetupMatrix -> Factorize -> PreconditionedGmres::Solve(A, rhs, x).
 * x is in/out (initial guess).  tol is the reference's ABSOLUTE residual tolerance.
 * times[0..3] = symbolic, setup, factorize, gmres (s); stat[0..1] = mv, precon time.
 * Returns the reference's success flag; *iters receives its iteration count. */
int ref_ilu_gmres(int n, const int* rp, const int* ci, const double* val, int lof, const double* rhs,
                  double* x, double tol, int restart, int maxit, int nthreads, int* iters, double* times,
                  double* stat) {
    CsrMatrix a;
    load_matrix(&a, n, rp, ci, val);
    IluSolver ilu;
    ilu.SetThreads(nthreads);
    PreconditionedGmres gmres;
    gmres.SetIluPreconditioner(&ilu);
    gmres.param().tolerance = tol;
    gmres.param().krylov_subspace_dimension = restart;
    gmres.param().max_iterations = maxit;
    const int nnz = rp[n];
    std::vector<int> nzmap(static_cast<size_t>(nnz));
    double t0 = now_s();
    int knnz = IlukSymbolic(&a, lof, ilu.GetMatrix(), nzmap.data());
    double t1 = now_s();
    std::memset(ilu.GetMatrix()->value, 0, sizeof(double) * static_cast<size_t>(knnz));
    for (int i = 0; i < nnz; ++i) ilu.GetMatrix()->value[nzmap[i]] = a.value[i];
    ilu.SetupMatrix();
    double t2 = now_s();
    ilu.Factorize();
    double t3 = now_s();
    std::vector<double> b(rhs, rhs + n);
    auto ret = gmres.Solve(&a, b.data(), x);
    double t4 = now_s();
    if (iters) *iters = ret.second;
    if (times) {
        times[0] = t1 - t0;
        times[1] = t2 - t1;
        times[2] = t3 - t2;
        times[3] = t4 - t3;
    }
    if (stat) {
        stat[0] = gmres.stat().total_mv_time;
        stat[1] = gmres.stat().total_precon_time;
    }
    DestroyCsrMatrix(&a);
    return ret.first ? 1 : 0;
}

/* y = A x through the reference's CsrMatVec (src/csr_matrix.cpp:163-171). */
void ref_csr_matvec(int n, const int* rp, const int* ci, const double* val, const double* x, double* y) {
    CsrMatrix a;
    a.size = n;
    a.max_nnz = rp[n];
    a.row_ptr = const_cast<int*>(rp);
    a.col_idx = const_cast<int*>(ci);
    a.value = const_cast<double*>(val);
    CsrMatVec(&a, x, y);
}

/* ---- timing session: the test/benchmark.cpp:104-170 repetition loop ----------------
 * ref_session_create: IlukSymbolic(A, lof) and the first SetupMatrix, as the benchmark's
 * first repetition; ref_session_set_threads: SetThreads + SetupMatrix again (the
 * reference's subtree schedule depends on the thread count); ref_session_step: one
 * repetition without setup (scatter A into F, Factorize, x = 0, Solve), the two timed
 * parts returned in times[0..1] (s) measured with steady_clock. */
struct RefSession {
    CsrMatrix a;
    IluSolver ilu;
    PreconditionedGmres gmres;
    std::vector<int> nzmap;
    int n = 0, nnz = 0, knnz = 0;
};

static void session_scatter(RefSession* s) {
    CsrMatrix* f = s->ilu.GetMatrix();
    std::memset(f->value, 0, sizeof(double) * static_cast<size_t>(s->knnz));
    for (int i = 0; i < s->nnz; ++i) f->value[s->nzmap[i]] = s->a.value[i];
}

void* ref_session_create(int n, const int* rp, const int* ci, const double* val, int lof, int restart, int maxit,
                         double tol, int nthreads, double* times) {
    auto* s = new RefSession;
    load_matrix(&s->a, n, rp, ci, val);
    s->n = n;
    s->nnz = rp[n];
    s->nzmap.assign(static_cast<size_t>(s->nnz), -1);
    s->ilu.SetThreads(nthreads);
    s->gmres.SetIluPreconditioner(&s->ilu);
    s->gmres.param().tolerance = tol;
    s->gmres.param().krylov_subspace_dimension = restart;
    s->gmres.param().max_iterations = maxit;
    double t0 = now_s();
    s->knnz = IlukSymbolic(&s->a, lof, s->ilu.GetMatrix(), s->nzmap.data());
    double t1 = now_s();
    session_scatter(s);
    s->ilu.SetupMatrix();
    double t2 = now_s();
    if (times) {
        times[0] = t1 - t0;
        times[1] = t2 - t1;
    }
    return s;
}

double ref_session_set_threads(void* hdl, int nthreads) {
    auto* s = static_cast<RefSession*>(hdl);
    s->ilu.SetThreads(nthreads);
    session_scatter(s);
    double t0 = now_s();
    s->ilu.SetupMatrix();
    return now_s() - t0;
}

int ref_session_step(void* hdl, const double* rhs, double* x, int* iters, double* times) {
    auto* s = static_cast<RefSession*>(hdl);
    std::vector<double> b(rhs, rhs + s->n);
    session_scatter(s);
    double t0 = now_s();
    s->ilu.Factorize();
    double t1 = now_s();
    std::fill_n(x, s->n, 0.0);
    double t2 = now_s();
    auto ret = s->gmres.Solve(&s->a, b.data(), x);
    double t3 = now_s();
    if (iters) *iters = ret.second;
    if (times) {
        times[0] = t1 - t0;
        times[1] = t3 - t2;
    }
    return ret.first ? 1 : 0;
}

void ref_session_destroy(void* hdl) {
    auto* s = static_cast<RefSession*>(hdl);
    DestroyCsrMatrix(&s->a);
    delete s;
}

/* ---- one system of a batch of independent systems: IlukSymbolic + SetupMatrix, one
 * Factorize, then for each of nrhs right-hand sides (rhs / x: nrhs vectors of n) a
 * GMRES solve from x0 = 0 to the reference's absolute criterion rtol * ||b_r||_2, all on
 * the calling thread with nthreads OpenMP threads (SetupMatrix sets the calling thread's
 * OpenMP thread count).  times[0] symbolic + setup, times[1] Factorize, times[2] all
 * solves (s, steady_clock); iters[r] per right-hand side.  Returns the number of
 * converged right-hand sides. */
int ref_solve_system(int n, const int* rp, const int* ci, const double* val, int lof, int restart, int maxit,
                     double rtol, int nthreads, int nrhs, const double* rhs, double* x, int* iters, double* times) {
    double t[2] = {0.0, 0.0};
    auto* s = static_cast<RefSession*>(ref_session_create(n, rp, ci, val, lof, restart, maxit, 0.0, nthreads, t));
    double t0 = now_s();
    s->ilu.Factorize();
    double t1 = now_s();
    int converged = 0;
    std::vector<double> b(static_cast<size_t>(n));
    for (int r = 0; r < nrhs; ++r) {
        const double* br = rhs + static_cast<size_t>(r) * n;
        double nb = 0.0;
        for (int i = 0; i < n; ++i) nb += br[i] * br[i];
        s->gmres.param().tolerance = rtol * std::sqrt(nb);
        std::copy_n(br, n, b.data());
        double* xr = x + static_cast<size_t>(r) * n;
        std::fill_n(xr, n, 0.0);
        auto ret = s->gmres.Solve(&s->a, b.data(), xr);
        if (iters) iters[r] = ret.second;
        converged += ret.first ? 1 : 0;
    }
    double t2 = now_s();
    if (times) {
        times[0] = t[0] + t[1];
        times[1] = t1 - t0;
        times[2] = t2 - t1;
    }
    ref_session_destroy(s);
    return converged;
}

/* ---- subtree scheduler (src/subtree.hpp tree_schedule) ------------------------------
 * The reference's tree_schedule on the L-DAG (lower != 0, load weights diag - row_ptr + 1
 * as its factorisation / forward substitution) or the reverse U-DAG (weights
 * row_ptr[v+1] - diag[v], as its backward substitution), no row stripping.  Outputs
 * part_ptr[nproc + 2], partitions[n], task_queue[ntasks + 1] (granularity > 1) and the
 * subtree sizes / weights [n + 1] from its own init_subtree.  Returns ntasks. */
struct RefNnzBalancer {
    using weight_t = int;
    const int* begin;
    const int* end;
    int base;
    int granu;
    weight_t weight_in_subtree(int i) const { return end[i] - begin[i] + base; }
    weight_t weight_in_queue(int i) const { return end[i] - begin[i] + base; }
    int queue_granularity() const { return granu; }
};

int ref_tree_schedule(int n, const int* rp, const int* ci, const int* diag, int lower, int nproc, int granularity,
                      double relax, int* part_ptr, int* partitions, int* task_queue, int* subtree_size,
                      int* subtree_weight) {
    int* tq = nullptr;
    int ntasks = 0;
    if (lower) {
        RefNnzBalancer lb{rp, diag, 1, granularity};
        ntasks = tree_schedule(nproc, 0, n, 1, ConstBiasArray<int>(const_cast<int*>(rp)), diag, ci, part_ptr, partitions,
                               tq, lb, relax, -1.0);
    } else {
        RefNnzBalancer lb{diag, rp + 1, 0, granularity};
        ntasks = tree_schedule(nproc, n - 1, -1, -1, ConstBiasArray<int>(const_cast<int*>(diag), 1), rp + 1, ci, part_ptr,
                               partitions, tq, lb, relax, -1.0);
    }
    if (tq != nullptr) {
        if (task_queue) std::copy_n(tq, ntasks + 1, task_queue);
        delete[] tq;
    }
    // subtree sizes and weights exactly as partition_subtree computes them
    std::vector<int> stripped(static_cast<size_t>(n), 0), parent(static_cast<size_t>(n)), root(static_cast<size_t>(n) + 1);
    std::vector<int> size(static_cast<size_t>(n) + 1), weight(static_cast<size_t>(n) + 1);
    const int vb = lower ? 0 : n - 1, ve = lower ? n : -1, vd = lower ? 1 : -1;
    if (lower) {
        build_etree_parent(n, vb, ve, vd, ConstBiasArray<int>(const_cast<int*>(rp)), diag, ci, stripped.data(),
                           parent.data(), root.data());
    } else {
        build_etree_parent(n, vb, ve, vd, ConstBiasArray<int>(const_cast<int*>(diag), 1), rp + 1, ci, stripped.data(),
                           parent.data(), root.data());
    }
    RefNnzBalancer lb = lower ? RefNnzBalancer{rp, diag, 1, granularity} : RefNnzBalancer{diag, rp + 1, 0, granularity};
    for (int v = vb; v != ve; v += vd) {
        weight[static_cast<size_t>(v)] = lb.weight_in_subtree(v);
        size[static_cast<size_t>(v)] = 1;
    }
    weight[static_cast<size_t>(n)] = 0;
    size[static_cast<size_t>(n)] = 0;
    init_subtree(vb, ve, vd, stripped.data(), parent.data(), size.data(), weight.data());
    if (subtree_size) std::copy(size.begin(), size.end(), subtree_size);
    if (subtree_weight) std::copy(weight.begin(), weight.end(), subtree_weight);
    return ntasks;
}

}  // extern "C"
