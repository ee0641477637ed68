/*
 * lljbash::IluSolver — GB300 ILU(k) factorisation and triangular substitution.
 * Source-compatible with the reference's include/ilu_solver.hpp:8-30: same class,
 * same public members and meaning.  The factors are computed on the GPU and, by
 * default, copied back into GetMatrix()->value after Factorize() (the reference
 * factorises that array in place, src/ilu_solver.cpp:616-671).
 */
#pragma once

#include <string>

#include "csr_matrix.h"

namespace lljbash {

class IluSolver {
public:
    IluSolver() = default;
    IluSolver(const IluSolver&) = delete;
    IluSolver& operator=(const IluSolver&) = delete;

    ~IluSolver();
    const CsrMatrix& GetILUMatrix() const { return aMatrix_; }
    CsrMatrix* GetMatrix() { return &aMatrix_; }

    /* Accepted for compatibility; the GPU path does not use host threads. */
    void SetThreads(int threads) { threads_ = threads; }

    /* Analysis of GetMatrix()'s pattern (diagonal pointers, elimination trees, level
     * sets, GPU schedules) and upload of the pattern.  Throws std::runtime_error("missing
     * diag") when a row has no diagonal entry. */
    void SetupMatrix();
    /* Numeric ILU of GetMatrix()'s values on the pattern; returns false on a zero or
     * non-finite pivot (the factors are still written, as the reference does). */
    bool Factorize();
    /* x = U^{-1} L^{-1} b on host arrays of length n (b == x allowed). */
    void Substitute(const double* b, double* x);

    /* GB300 extension: Factorize() with the matrix values (GetMatrix()'s pattern) taken
     * from device memory; the factors stay on the device (GetMatrix()->value is left
     * untouched). */
    bool FactorizeDevice(const double* d_values);

    /* GB300 extension: learned diagonal shift.  With a model set (369 FP32 MLP
     * parameters), every factorisation first runs the fused feature + MLP pre-pass and
     * factorises A + diag(shift); a zero or non-finite pivot makes it fall back to plain
     * ILU.  Rows whose predicted relative shift is below min_shift get none.  nullptr
     * removes the model. */
    void SetShiftModel(const float* params, int nparams, float min_shift);

    /* GB300 extension: Substitute() on device arrays (d_b read, d_x written, n entries)
     * that allocates nothing: its intermediate vector and counters live in a static
     * device array of the library (at most 2,097,152 rows).  The first call on a device
     * resolves that array's address and should come before any stream capture; calls
     * that overlap on the GPU share the array and race. */
    void SubstituteDeviceNoAlloc(const double* d_b, double* d_x);

    /* Implementation state (device buffers, schedules); opaque to users. */
    struct Impl;
    Impl* impl() { return impl_; }
    const Impl* impl() const { return impl_; }
    Impl* impl_ensure();
    int threads() const { return threads_; }

private:
    bool FactorizeFrom(const double* values, bool on_device);
    int threads_ = 0;
    CsrMatrix aMatrix_;
    Impl* impl_ = nullptr;
};

}  // namespace lljbash
