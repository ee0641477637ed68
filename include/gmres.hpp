/*
 * lljbash::PreconditionedGmres — restarted right-preconditioned GMRES(m) on the GPU.
 * Source-compatible with the reference's include/gmres.hpp:9-22.  The Krylov cycle
 * (SpMV, ILU substitution, CGS2 orthogonalisation, Givens/Hessenberg least squares)
 * runs entirely on the device; rhs and sol are host arrays.
 */
#pragma once

#include <utility>

#include "gmres_param.h"
#include "ilu_solver.hpp"

namespace lljbash {

class PreconditionedGmres {
public:
    PreconditionedGmres() = default;
    PreconditionedGmres(const PreconditionedGmres&) = delete;
    PreconditionedGmres& operator=(const PreconditionedGmres&) = delete;
    ~PreconditionedGmres();

    GmresParameters& param() { return param_; }
    GmresStat& stat() { return stat_; }

    /* Uses the solver's factors (on the device) as the right preconditioner.  Without
     * a preconditioner GMRES runs unpreconditioned. */
    void SetIluPreconditioner(IluSolver* ilu_solver) { ilu_ = ilu_solver; }

    /* Solves mat * sol = rhs from the initial guess in sol.  Returns the reference's
     * (success, iterations) pair with its semantics (src/gmres.cpp:138-288):
     * iterations count Arnoldi steps over all restarts; success is false on NaN or when
     * the iteration count passes max_iterations. */
    std::pair<bool, int> Solve(const CsrMatrix* mat, double* rhs, double* sol);

    /* GB300 extension: the same solve on arrays already in device memory (CSR of A with
     * n rows, rhs, and sol holding the initial guess; sol is overwritten).  The arrays
     * must be ready when the call is made (work that produced them synchronised). */
    std::pair<bool, int> SolveDevice(int n, const int* d_row_ptr, const int* d_col_idx, const double* d_values,
                                     const double* d_rhs, double* d_sol);

    struct Impl;
    Impl* impl() { return impl_; }
    Impl* impl_ensure();
    IluSolver* preconditioner() const { return ilu_; }

private:
    GmresParameters param_;
    GmresStat stat_;
    IluSolver* ilu_ = nullptr;
    Impl* impl_ = nullptr;
};

}  // namespace lljbash
