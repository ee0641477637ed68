// par-ilu0-benchmark: the command-line benchmark of the library, with the options and the
// summary of the reference's test/benchmark.cpp:17-32, 89-215:
//
//   par-ilu0-benchmark -m A.mtx [-k LOF] [--amd | --nd] [-e EPS] [-i MAXIT] [-r RESTART]
//                      [-t THREADS] [-n REP] [-w[N] | --warmup[=N]] [--onlyfact | --onlysubs]
//                      [--mixed]
//
// It reads a 1-based MatrixMarket file (ReadCsrMatrixMM1), optionally reorders it with a
// fill-reducing ordering (rows and columns permuted by the inverse permutation, each
// row's columns sorted), takes rhs = A * ones, builds the ILU(k) pattern (IlukSymbolic)
// and runs `rep` repetitions of factorisation + GMRES from x = 0 (or the factorisation
// alone, or one substitution alone) after `warmup` untimed ones, SetupMatrix in the first
// warm-up and in the first timed repetition, as the reference does.  Times are wall-clock
// seconds (std::chrono::steady_clock).
// --mixed (no counterpart in the reference) runs the FP32 Krylov cycles inside FP64
// iterative refinement.  -t is accepted and ignored (the work runs on the GPU).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <tuple>
#include <vector>

#include "csr_matrix.h"
#include "gmres.hpp"
#include "ilu_solver.hpp"
#include "iluk.h"
#include "par_ilu0_gb300.h"

using namespace lljbash;

namespace {

struct Options {
    std::string mat;
    int lof = 0;
    bool amd = false, nd = false;
    double eps = 1e-8;
    int maxit = 1000;
    int restart = 60;
    int threads = 1;
    int rep = 1;
    int warmup = 0;
    bool onlyfact = false, onlysubs = false, mixed = false;
};

void usage(const char* prog) {
    std::printf(
        "benchmark for ILU(k) GMRES on the GPU\n"
        "Usage:\n  %s -m FILE [options]\n\n"
        "  -m, --mat FILE       coefficient matrix file (MatrixMarket, 1-based)\n"
        "  -k, --lof K          ILU(k) level of fill (default 0)\n"
        "      --amd            approximate minimum degree reordering\n"
        "      --nd             nested dissection reordering\n"
        "  -e, --eps EPS        GMRES tolerance (default 1e-8)\n"
        "  -i, --maxit N        GMRES max iterations (default 1000)\n"
        "  -r, --restart M      GMRES restart iterations (default 60)\n"
        "  -t, --threads N      number of threads (accepted, unused on the GPU)\n"
        "  -n, --rep N          number of repeats (default 1)\n"
        "  -w, --warmup[=N]     include warmups (default 1 when given)\n"
        "      --onlyfact       only test factorization\n"
        "      --onlysubs       only test substitution\n"
        "      --mixed          FP32 Krylov cycles in FP64 iterative refinement\n"
        "  -h, --help           print usage\n",
        prog);
}

bool parse(int argc, char** argv, Options& o) {
    auto value = [&](int& i, const std::string& a, std::size_t eq) -> std::string {
        if (eq != std::string::npos) return a.substr(eq + 1);
        if (i + 1 >= argc) {
            std::fprintf(stderr, "option %s needs a value\n", a.c_str());
            std::exit(1);
        }
        return argv[++i];
    };
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        const std::size_t eq = a.rfind("--", 0) == 0 ? a.find('=') : std::string::npos;
        const std::string name = eq == std::string::npos ? a : a.substr(0, eq);
        if (name == "-h" || name == "--help") {
            usage(argv[0]);
            std::exit(0);
        } else if (name == "-m" || name == "--mat") {
            o.mat = value(i, a, eq);
        } else if (name == "-k" || name == "--lof") {
            o.lof = std::atoi(value(i, a, eq).c_str());
        } else if (name == "--amd") {
            o.amd = true;
        } else if (name == "--nd") {
            o.nd = true;
        } else if (name == "-e" || name == "--eps") {
            o.eps = std::atof(value(i, a, eq).c_str());
        } else if (name == "-i" || name == "--maxit") {
            o.maxit = std::atoi(value(i, a, eq).c_str());
        } else if (name == "-r" || name == "--restart") {
            o.restart = std::atoi(value(i, a, eq).c_str());
        } else if (name == "-t" || name == "--threads") {
            o.threads = std::atoi(value(i, a, eq).c_str());
        } else if (name == "-n" || name == "--rep") {
            o.rep = std::atoi(value(i, a, eq).c_str());
        } else if (name == "--warmup") {
            o.warmup = eq == std::string::npos ? 1 : std::atoi(a.substr(eq + 1).c_str());
        } else if (a.rfind("-w", 0) == 0) {
            o.warmup = a.size() > 2 ? std::atoi(a.c_str() + 2) : 1;
        } else if (name == "--onlyfact") {
            o.onlyfact = true;
        } else if (name == "--onlysubs") {
            o.onlysubs = true;
        } else if (name == "--mixed") {
            o.mixed = true;
        } else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return false;
        }
    }
    if (o.mat.empty()) {
        std::fprintf(stderr, "no matrix file (-m)\n");
        return false;
    }
    return true;
}

// Symmetric permutation B = P A P^T with B(ip[i], ip[j]) = A(i, j); each row's columns
// sorted ascending (ties cannot occur: a permutation maps distinct columns apart).
void permute(CsrMatrix* a, const std::vector<int>& ip) {
    const int n = a->size;
    std::vector<int> rp(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) rp[static_cast<size_t>(ip[i]) + 1] = a->row_ptr[i + 1] - a->row_ptr[i];
    for (int i = 0; i < n; ++i) rp[static_cast<size_t>(i) + 1] += rp[static_cast<size_t>(i)];
    std::vector<std::pair<int, double>> row;
    std::vector<int> ci(static_cast<size_t>(rp[n]));
    std::vector<double> va(static_cast<size_t>(rp[n]));
    for (int i = 0; i < n; ++i) {
        row.clear();
        for (int p = a->row_ptr[i]; p < a->row_ptr[i + 1]; ++p) row.emplace_back(ip[a->col_idx[p]], a->value[p]);
        std::sort(row.begin(), row.end());
        int q = rp[ip[i]];
        for (const auto& e : row) {
            ci[static_cast<size_t>(q)] = e.first;
            va[static_cast<size_t>(q++)] = e.second;
        }
    }
    std::copy(rp.begin(), rp.end(), a->row_ptr);
    std::copy(ci.begin(), ci.end(), a->col_idx);
    std::copy(va.begin(), va.end(), a->value);
}

}  // namespace

int main(int argc, char* argv[]) {
    Options o;
    if (!parse(argc, argv, o)) {
        usage(argv[0]);
        return 1;
    }
    CsrMatrix csr = CSR_MATRIX_DEFAULT;
    ReadCsrMatrixMM1(&csr, o.mat.c_str());
    const int n = csr.size;
    const int nnz = GetCsrNonzeros(&csr);

    if (o.amd || o.nd) {
        std::vector<int> p(static_cast<size_t>(n)), ip(static_cast<size_t>(n));
        // the reference's return conventions: AMD 0 on success, ND 1 on success
        const int rc = o.amd ? CsrAmdOrder(&csr, p.data(), ip.data()) : CsrNdOrder(&csr, p.data(), ip.data());
        if (rc != (o.amd ? 0 : 1)) {
            std::fprintf(stderr, "%s ordering failed (%d)\n", o.amd ? "AMD" : "ND", rc);
            return 1;
        }
        permute(&csr, ip);
    }

    std::vector<double> rhs(static_cast<size_t>(n)), sol(static_cast<size_t>(n), 1.0), x(static_cast<size_t>(n));
    CsrMatVec(&csr, sol.data(), rhs.data());

    IluSolver ilu;
    CsrMatrix* csr_ilu = ilu.GetMatrix();
    PreconditionedGmres gmres;
    gmres.SetIluPreconditioner(&ilu);
    gmres.param().tolerance = o.eps;
    gmres.param().max_iterations = o.maxit;
    gmres.param().krylov_subspace_dimension = o.restart;
    if (o.mixed) LLJBASH_GmresSetOption(static_cast<GmresHdl>(&gmres), LLJBASH_GMRES_OPT_MODE, 1);
    ilu.SetThreads(o.threads);

    std::vector<int> nzmap(static_cast<size_t>(nnz));
    const int knnz = IlukSymbolic(&csr, o.lof, csr_ilu, nzmap.data());
    std::printf("knnz: %d\n", knnz);

    double setup_time = 0.0, fact_time = 0.0, gmres_time = 0.0;
    auto timed = [](const std::function<void()>& f, double& acc) {
        const auto t0 = std::chrono::steady_clock::now();
        f();
        acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    };
    auto scatter_values = [&]() {
        std::memset(csr_ilu->value, 0, sizeof(double) * static_cast<size_t>(knnz));
        for (int i = 0; i < nnz; ++i) csr_ilu->value[nzmap[static_cast<size_t>(i)]] = csr.value[i];
    };
    int status = 0;
    auto run = [&](bool setup) {
        if (o.onlysubs) {
            if (setup) {
                scatter_values();
                timed([&] { ilu.SetupMatrix(); }, setup_time);
                ilu.Factorize();
            }
            timed([&] { ilu.Substitute(rhs.data(), x.data()); }, gmres.stat().total_precon_time);
            return;
        }
        scatter_values();
        if (setup) timed([&] { ilu.SetupMatrix(); }, setup_time);
        timed([&] { ilu.Factorize(); }, fact_time);
        if (o.onlyfact) return;
        std::fill(x.begin(), x.end(), 0.0);
        std::pair<bool, int> ret;
        timed([&] { ret = gmres.Solve(&csr, rhs.data(), x.data()); }, gmres_time);
        if (!ret.first) {
            std::puts("GMRES error");
            status = 2;
        }
        std::printf("iter: %d\n", ret.second);
    };

    try {
        // as the reference: SetupMatrix in the first warm-up and again in the first timed
        // repetition; the three timers restart after the warm-ups, the GMRES statistics
        // keep accumulating
        for (int i = 0; i < o.warmup; ++i) run(i == 0);
        setup_time = fact_time = gmres_time = 0.0;
        for (int i = 0; i < o.rep; ++i) run(i == 0);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }

    double max_err = 0.0;
    for (int i = 0; i < n; ++i) max_err = std::max(max_err, std::fabs(x[static_cast<size_t>(i)] - sol[static_cast<size_t>(i)]));
    std::printf("max_err: %g\n", max_err);

    const int rep = std::max(o.rep, 1);
    std::puts("\nSummary:");
    std::printf("n:                          %d\n", n);
    std::printf("nnz:                        %d\n", nnz);
    std::printf("k:                          %d\n", o.lof);
    std::printf("nnz(F)/nnz(A):              %f\n", static_cast<double>(knnz) / nnz);
    std::printf("gmres tolerance:            %g\n", gmres.param().tolerance);
    std::printf("gmres max iterations:       %d\n", gmres.param().max_iterations);
    std::printf("gmres restart iterations:   %d\n", gmres.param().krylov_subspace_dimension);
    std::printf("threads:                    %d\n", o.threads);
    std::printf("reps:                       %d\n", rep);
    std::printf("precision:                  %s\n", o.mixed ? "mixed (FP32 cycles, FP64 refinement)" : "FP64");
    std::printf("setup time (s):             %g\n", setup_time);
    std::printf("total factorize time (s):   %g\n", fact_time);
    std::printf("total gmres time (s):       %g\n", gmres_time);
    std::printf("total mv time (s):          %g\n", gmres.stat().total_mv_time);
    std::printf("total precon time (s):      %g\n", gmres.stat().total_precon_time);
    std::printf("average factorize time (s): %g\n", fact_time / rep);
    std::printf("average precon time (s):    %g\n", gmres.stat().total_precon_time / rep);
    std::printf("average gmres time (s):     %g\n", gmres_time / rep);
    DestroyCsrMatrix(&csr);
    return status;
}
