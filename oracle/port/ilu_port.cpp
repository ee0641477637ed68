/*
 * ORACLE — test infrastructure only.  Never linked into or called by the product
 * library (par_ilu0_cpp_gb300/csrc).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it, as the checker / CPU baseline.
 *
 * A plain C++ restatement of the reference's ILU(k) + GMRES path, written from the
 * reference's algorithm (not its code), with the same per-entry operation order:
 *
 *   port_iluk_symbolic   IlukSymbolic, src/iluk.cpp:5-54 (ordered map per row,
 *                        first-found level kept via try_emplace, :22-27)
 *   port_diag_ptr        diag_ptr scan, src/ilu_solver.cpp:276-289
 *   port_etree           Liu etree with path compression, src/subtree.hpp:35-68
 *   port_levels          Levelization::levelize, src/subtree.hpp:524-551
 *   port_factorize       up-looking row ILU, src/ilu_solver.cpp:553-589; nthreads>1
 *                        runs the reference's ticketed queue with per-row ready
 *                        flags (src/ilu_solver.cpp:394-443, Wait policy :516-521)
 *   port_substitute      serial L then U sweeps, src/ilu_solver.cpp:779-796
 *   port_gmres           restarted right-preconditioned GMRES(m) with modified
 *                        Gram-Schmidt and Givens rotations, src/gmres.cpp:138-288
 *   port_csr_matvec      CsrMatVec, src/csr_matrix.cpp:163-171
 *
 * Parity of this restatement is pinned against the reference itself (compiled from
 * its own sources by oracle/build_ref.sh) through the fixtures in tests/golden/.
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

std::vector<int> g_f_rp, g_f_ci, g_nzmap;
std::vector<double> g_f_val;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

/* Row j of the up-looking ILU (src/ilu_solver.cpp:553-589), dense scatter row `w`. */
inline void ilu_row(int j, const int* rp, const int* ci, const int* diag, double* a, double* w) {
    for (int p = rp[j]; p < rp[j + 1]; ++p) w[ci[p]] = a[p];
    for (int p = rp[j]; p < diag[j]; ++p) {
        const int k = ci[p];
        w[k] /= a[diag[k]];
        const double l = w[k];
        for (int q = diag[k] + 1; q < rp[k + 1]; ++q) w[ci[q]] -= a[q] * l;
    }
    for (int p = rp[j]; p < rp[j + 1]; ++p) a[p] = w[ci[p]];
}

int num_threads(int req) {
#ifdef _OPENMP
    return req > 0 ? req : omp_get_max_threads();
#else
    (void)req;
    return 1;
#endif
}

}  // namespace

extern "C" {

/* Level-of-fill symbolic pattern; returns nnz(F); fetch with port_iluk_fetch. */
int port_iluk_symbolic(int n, const int* rp, const int* ci, int lof) {
    std::vector<std::map<int, int>> rows(static_cast<size_t>(n));
    long long knnz = 0;
    for (int i = 0; i < n; ++i) {
        auto& row = rows[i];
        for (int p = rp[i]; p < rp[i + 1]; ++p) row[ci[p]] = 0;
        for (auto it = row.begin(); it != row.end(); ++it) {
            const int k = it->first;
            if (k >= i) break;
            const int lev_ik = it->second;
            if (lev_ik >= lof) continue;
            const auto& rk = rows[k];
            for (auto jt = rk.find(k); jt != rk.end(); ++jt) {
                const int lev = lev_ik + jt->second + 1;
                if (lev <= lof) row.try_emplace(jt->first, lev);  // first level found is kept
            }
        }
        knnz += static_cast<long long>(row.size());
    }
    g_f_rp.assign(static_cast<size_t>(n) + 1, 0);
    g_f_ci.assign(static_cast<size_t>(knnz), 0);
    g_nzmap.assign(static_cast<size_t>(rp[n]), -1);
    int pos = 0, apos = 0;
    for (int i = 0; i < n; ++i) {
        g_f_rp[i] = pos;
        for (const auto& e : rows[i]) {
            g_f_ci[pos] = e.first;
            if (e.second == 0) g_nzmap[apos++] = pos;
            ++pos;
        }
    }
    g_f_rp[n] = pos;
    return static_cast<int>(knnz);
}

/* F pattern, nzmap (A position -> F position), and F values (A scattered, fill = 0). */
void port_iluk_fetch(const double* a_val, int* f_rp, int* f_ci, double* f_val, int* nzmap) {
    const int n = static_cast<int>(g_f_rp.size()) - 1;
    std::copy(g_f_rp.begin(), g_f_rp.end(), f_rp);
    std::copy(g_f_ci.begin(), g_f_ci.end(), f_ci);
    if (nzmap) std::copy(g_nzmap.begin(), g_nzmap.end(), nzmap);
    if (f_val) {
        std::fill_n(f_val, g_f_rp[n], 0.0);
        for (size_t p = 0; p < g_nzmap.size(); ++p) f_val[g_nzmap[p]] = a_val ? a_val[p] : 0.0;
    }
}

void port_diag_ptr(int n, const int* rp, const int* ci, int* diag) {
    for (int i = 0; i < n; ++i) {
        diag[i] = -1;
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            if (ci[p] >= i) {
                diag[i] = p;
                break;
            }
        }
    }
}

/* Liu's elimination tree.  lower != 0: vertices 0..n-1 ascending, edges = strict-lower
 * part of each row.  lower == 0: vertices n-1..0 descending, edges = strict-upper part.
 * parent[v] = n for roots. */
void port_etree(int n, const int* rp, const int* ci, const int* diag, int lower, int* parent) {
    std::vector<int> anc(static_cast<size_t>(n), n);
    for (int v = 0; v < n; ++v) parent[v] = n;
    for (int s = 0; s < n; ++s) {
        const int j = lower ? s : n - 1 - s;
        const int b = lower ? rp[j] : diag[j] + 1;
        const int e = lower ? diag[j] : rp[j + 1];
        for (int p = b; p < e; ++p) {
            int i = ci[p];
            while (anc[i] != n) {  // climb to the current root, compressing the path onto j
                const int next = anc[i];
                anc[i] = j;
                i = next;
            }
            if (i != j) {
                anc[i] = j;
                parent[i] = j;
            }
        }
    }
}

/* depth[v] = 1 + max depth over v's dependencies (0 for sources); returns #levels. */
int port_levels(int n, const int* rp, const int* ci, const int* diag, int lower, int* depth) {
    int nlev = 0;
    for (int s = 0; s < n; ++s) {
        const int j = lower ? s : n - 1 - s;
        const int b = lower ? rp[j] : diag[j] + 1;
        const int e = lower ? diag[j] : rp[j + 1];
        int d = 0;
        for (int p = b; p < e; ++p) d = std::max(d, depth[ci[p]] + 1);
        depth[j] = d;
        nlev = std::max(nlev, d + 1);
    }
    return nlev;
}

/* In-place ILU on the CSR pattern.  nthreads == 1: plain row loop.  nthreads > 1: rows
 * handed out in ascending order from an atomic ticket; a row spins on the ready flag of
 * each row it reads (the reference's queue schedule).  Returns seconds spent. */
double port_factorize(int n, const int* rp, const int* ci, double* a, int nthreads) {
    std::vector<int> diag(static_cast<size_t>(n));
    port_diag_ptr(n, rp, ci, diag.data());
    const int nt = num_threads(nthreads);
    const double t0 = now_s();
    if (nt <= 1) {
        std::vector<double> w(static_cast<size_t>(n));
        for (int j = 0; j < n; ++j) ilu_row(j, rp, ci, diag.data(), a, w.data());
        return now_s() - t0;
    }
    std::unique_ptr<std::atomic<int>[]> done(new std::atomic<int>[n]);
    for (int j = 0; j < n; ++j) done[j].store(0, std::memory_order_relaxed);
    std::atomic<int> ticket(0);
#pragma omp parallel num_threads(nt)
    {
        std::vector<double> w(static_cast<size_t>(n));
        while (true) {
            const int j = ticket.fetch_add(1, std::memory_order_relaxed);
            if (j >= n) break;
            for (int p = rp[j]; p < diag[j]; ++p) {
                while (!done[ci[p]].load(std::memory_order_acquire)) {
                }
            }
            ilu_row(j, rp, ci, diag.data(), a, w.data());
            done[j].store(1, std::memory_order_release);
        }
    }
    return now_s() - t0;
}

/* x = U^{-1} L^{-1} b (unit L), serial sweeps in the reference's entry order. */
void port_substitute(int n, const int* rp, const int* ci, const double* lu, const double* b, double* x) {
    std::vector<int> diag(static_cast<size_t>(n));
    port_diag_ptr(n, rp, ci, diag.data());
    if (b != x) std::copy_n(b, n, x);
    for (int i = 0; i < n; ++i) {
        double xi = x[i];
        for (int p = rp[i]; p < diag[i]; ++p) xi -= x[ci[p]] * lu[p];
        x[i] = xi;
    }
    for (int i = n - 1; i >= 0; --i) {
        double xi = x[i];
        for (int p = rp[i + 1] - 1; p > diag[i]; --p) xi -= x[ci[p]] * lu[p];
        x[i] = xi / lu[diag[i]];
    }
}

void port_csr_matvec(int n, const int* rp, const int* ci, const double* val, const double* x, double* y) {
    for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (int p = rp[r]; p < rp[r + 1]; ++p) s += val[p] * x[ci[p]];
        y[r] = s;
    }
}

/* Restarted right-preconditioned GMRES(m) (src/gmres.cpp:138-288), ILU(0/k) factors `lu`
 * on pattern (f_rp, f_ci) as the preconditioner, A = (rp, ci, val).  tol is absolute.
 * nthreads > 1 parallelises the SpMV and vector kernels (sums then change order).
 * Returns 1 on the reference's success flag, 0 otherwise; *iters = its. */
int port_gmres(int n, const int* rp, const int* ci, const double* val, const int* f_rp, const int* f_ci,
               const double* lu, const double* rhs, double* sol, double tol, int im, int maxits, int nthreads,
               int* iters, double* precon_seconds) {
    const int nt = num_threads(nthreads);
    const int im1 = im + 1;
    constexpr double epsmac = 1e-16;
    const double eps1 = tol;
    std::vector<double> vv(static_cast<size_t>(im1) * n), z(static_cast<size_t>(im) * n),
        hh(static_cast<size_t>(im1) * (im + 3));
    double* c = hh.data() + static_cast<size_t>(im1) * im;
    double* s = c + im1;
    double* rs = s + im1;
    std::vector<int> fdiag(static_cast<size_t>(n));
    port_diag_ptr(n, f_rp, f_ci, fdiag.data());
    double tprec = 0.0;

    auto spmv = [&](const double* x, double* y, double alpha, double beta) {
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int r = 0; r < n; ++r) {
            double acc = 0.0;
            for (int p = rp[r]; p < rp[r + 1]; ++p) acc += val[p] * x[ci[p]];
            y[r] = beta == 0.0 ? alpha * acc : alpha * acc + beta * y[r];
        }
    };
    auto dot = [&](const double* x, const double* y) {
        double acc = 0.0;
#pragma omp parallel for num_threads(nt) reduction(+ : acc) schedule(static)
        for (int r = 0; r < n; ++r) acc += x[r] * y[r];
        return acc;
    };
    auto axpy = [&](double a, const double* x, double* y) {
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int r = 0; r < n; ++r) y[r] += a * x[r];
    };
    auto scal = [&](double a, double* x) {
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int r = 0; r < n; ++r) x[r] *= a;
    };
    auto precon = [&](const double* b, double* x) {
        const double t0 = now_s();
        std::copy_n(b, n, x);
        for (int i = 0; i < n; ++i) {
            double xi = x[i];
            for (int p = f_rp[i]; p < fdiag[i]; ++p) xi -= x[f_ci[p]] * lu[p];
            x[i] = xi;
        }
        for (int i = n - 1; i >= 0; --i) {
            double xi = x[i];
            for (int p = f_rp[i + 1] - 1; p > fdiag[i]; --p) xi -= x[f_ci[p]] * lu[p];
            x[i] = xi / lu[fdiag[i]];
        }
        tprec += now_s() - t0;
    };

    int its = 0;
    int ptih = 0;
    bool ok = true;
    while (its < maxits) {
        std::copy_n(rhs, n, vv.data());
        spmv(sol, vv.data(), -1.0, 1.0);
        double beta = std::sqrt(dot(vv.data(), vv.data()));
        if (beta <= tol) break;
        scal(1.0 / beta, vv.data());
        rs[0] = beta;
        int i = -1;
        bool nan = false;
        while ((i < im - 1) && (beta > eps1) && (its++ < maxits)) {
            ++i;
            const int i1 = i + 1;
            double* vi = vv.data() + static_cast<size_t>(i) * n;
            double* w = vv.data() + static_cast<size_t>(i1) * n;
            double* zi = z.data() + static_cast<size_t>(i) * n;
            precon(vi, zi);
            spmv(zi, w, 1.0, 0.0);
            ptih = i * im1;
            for (int j = 0; j <= i; ++j) {
                const double t = dot(vv.data() + static_cast<size_t>(j) * n, w);
                hh[ptih + j] = t;
                axpy(-t, vv.data() + static_cast<size_t>(j) * n, w);
            }
            double t = std::sqrt(dot(w, w));
            hh[ptih + i1] = t;
            if (t <= epsmac) break;
            scal(1.0 / t, w);
            for (int k = 1; k <= i; ++k) {
                const int k1 = k - 1;
                const double tt = hh[ptih + k1];
                hh[ptih + k1] = c[k1] * tt + s[k1] * hh[ptih + k];
                hh[ptih + k] = -s[k1] * tt + c[k1] * hh[ptih + k];
            }
            double gam = std::sqrt(hh[ptih + i] * hh[ptih + i] + hh[ptih + i1] * hh[ptih + i1]);
            if (gam == 0.0) gam = epsmac;
            c[i] = hh[ptih + i] / gam;
            s[i] = hh[ptih + i1] / gam;
            rs[i1] = -s[i] * rs[i];
            rs[i] = c[i] * rs[i];
            hh[ptih + i] = c[i] * hh[ptih + i] + s[i] * hh[ptih + i1];
            beta = std::fabs(rs[i1]);
            if (std::isnan(beta)) {
                nan = true;
                break;
            }
        }
        if (nan) {
            ok = false;
            break;
        }
        rs[i] = rs[i] / hh[ptih + i];
        for (int ii = i - 1; ii >= 0; --ii) {
            double t = rs[ii];
            for (int j = ii + 1; j <= i; ++j) t -= hh[static_cast<size_t>(j) * im1 + ii] * rs[j];
            rs[ii] = t / hh[static_cast<size_t>(ii) * im1 + ii];
        }
        for (int j = 0; j <= i; ++j) axpy(rs[j], z.data() + static_cast<size_t>(j) * n, sol);
        if (beta <= eps1) break;
        if (its > maxits) {
            ok = false;
            break;
        }
    }
    if (iters) *iters = its;
    if (precon_seconds) *precon_seconds = tprec;
    return ok ? 1 : 0;
}

}  // extern "C"
