/*
 * Oracle test infrastructure only (never linked into the product library).
 *
 * A minimal stand-in for the parts of Intel MKL that the reference solver calls,
 * so that the reference's own sources (src/ilu_solver.cpp, src/gmres.cpp,
 * src/csr_matrix.cpp, src/iluk.cpp) compile unmodified in this container, where
 * MKL is not installed.  Every routine is a plain loop restating the BLAS /
 * sparse-BLAS definition; MKL's own blocking is not reproduced.  Sums are taken in
 * index order, except in the timing build (SHIM_THREADED_BLAS), where long vectors are
 * split over the OpenMP threads as MKL's threaded BLAS-1 does.
 *
 * Call sites in the reference:
 *   cblas_dcopy/ddot/daxpy/dnrm2/dscal : src/gmres.cpp:181,185,191,220,223,226,233,275
 *   cblas_dcopy                         : src/ilu_solver.cpp:776, src/csr_matrix.cpp:41,46
 *   cblas_daxpy/idamax                  : test/benchmark.cpp:185-186
 *   mkl_sparse_d_create_csr / mv        : src/gmres.cpp:172,183,212
 *   mkl_malloc / mkl_free               : src/csr_matrix.cpp:13-23, src/gmres.cpp:150-152
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdlib>

typedef int MKL_INT;

inline void* mkl_malloc(std::size_t size, int alignment) {
    void* p = nullptr;
    std::size_t a = alignment < 16 ? 16 : static_cast<std::size_t>(alignment);
    std::size_t s = (size + a - 1) / a * a;
    if (s == 0) s = a;
    if (posix_memalign(&p, a, s) != 0) return nullptr;
    return p;
}
inline void mkl_free(void* p) { std::free(p); }
inline void MKL_Free_Buffers() {}

/* SHIM_THREADED_BLAS (the CPU timing build): long unit-stride vectors are split over the
 * OpenMP threads, as MKL's threaded BLAS-1 does; the sums then follow the threads'
 * partition instead of index order.  Without it every routine is a serial loop. */
#ifdef SHIM_THREADED_BLAS
#define SHIM_PAR(n, inc1, inc2) ((n) >= 32768 && (inc1) == 1 && (inc2) == 1)
#define SHIM_OMP_FOR _Pragma("omp parallel for schedule(static) if(par)")
#define SHIM_OMP_SUM _Pragma("omp parallel for schedule(static) reduction(+ : s) if(par)")
#else
#define SHIM_PAR(n, inc1, inc2) false
#define SHIM_OMP_FOR
#define SHIM_OMP_SUM
#endif

inline void cblas_dcopy(MKL_INT n, const double* x, MKL_INT incx, double* y, MKL_INT incy) {
    const bool par = SHIM_PAR(n, incx, incy);
    (void)par;
    SHIM_OMP_FOR
    for (MKL_INT i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}
inline double cblas_ddot(MKL_INT n, const double* x, MKL_INT incx, const double* y, MKL_INT incy) {
    const bool par = SHIM_PAR(n, incx, incy);
    (void)par;
    double s = 0.0;
    SHIM_OMP_SUM
    for (MKL_INT i = 0; i < n; ++i) s += x[i * incx] * y[i * incy];
    return s;
}
inline void cblas_daxpy(MKL_INT n, double a, const double* x, MKL_INT incx, double* y, MKL_INT incy) {
    const bool par = SHIM_PAR(n, incx, incy);
    (void)par;
    SHIM_OMP_FOR
    for (MKL_INT i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}
inline double cblas_dnrm2(MKL_INT n, const double* x, MKL_INT incx) {
    const bool par = SHIM_PAR(n, incx, 1);
    (void)par;
    double s = 0.0;
    SHIM_OMP_SUM
    for (MKL_INT i = 0; i < n; ++i) s += x[i * incx] * x[i * incx];
    return std::sqrt(s);
}
inline void cblas_dscal(MKL_INT n, double a, double* x, MKL_INT incx) {
    const bool par = SHIM_PAR(n, incx, 1);
    (void)par;
    SHIM_OMP_FOR
    for (MKL_INT i = 0; i < n; ++i) x[i * incx] *= a;
}
/* 1-based index of the first entry of largest magnitude (BLAS i?amax). */
inline MKL_INT cblas_idamax(MKL_INT n, const double* x, MKL_INT incx) {
    if (n <= 0) return 0;
    MKL_INT best = 0;
    double bv = std::fabs(x[0]);
    for (MKL_INT i = 1; i < n; ++i) {
        double v = std::fabs(x[i * incx]);
        if (v > bv) { bv = v; best = i; }
    }
    return best + 1;
}

/* ---- sparse BLAS (inspector-executor) subset ---- */
typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_SUPPORTED = 6 } sparse_status_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_TRIANGULAR = 23 } sparse_matrix_type_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41, SPARSE_FILL_MODE_FULL = 42 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;

struct matrix_descr {
    sparse_matrix_type_t type;
    sparse_fill_mode_t mode;
    sparse_diag_type_t diag;
};

struct shim_sparse_csr {
    MKL_INT rows, cols;
    const MKL_INT* rows_start;
    const MKL_INT* rows_end;
    const MKL_INT* col_indx;
    const double* values;
};
typedef shim_sparse_csr* sparse_matrix_t;

inline sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t* A, sparse_index_base_t /*base*/,
                                               MKL_INT rows, MKL_INT cols, MKL_INT* rows_start,
                                               MKL_INT* rows_end, MKL_INT* col_indx, double* values) {
    *A = new shim_sparse_csr{rows, cols, rows_start, rows_end, col_indx, values};
    return SPARSE_STATUS_SUCCESS;
}
inline sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
    delete A;
    return SPARSE_STATUS_SUCCESS;
}
/* y = alpha * A * x + beta * y, each row summed in column order. */
inline sparse_status_t mkl_sparse_d_mv(sparse_operation_t op, double alpha, const sparse_matrix_t A,
                                       matrix_descr /*descr*/, const double* x, double beta, double* y) {
    if (op != SPARSE_OPERATION_NON_TRANSPOSE) return SPARSE_STATUS_NOT_SUPPORTED;
#pragma omp parallel for schedule(static)
    for (MKL_INT r = 0; r < A->rows; ++r) {
        double s = 0.0;
        for (MKL_INT k = A->rows_start[r]; k < A->rows_end[r]; ++k) s += A->values[k] * x[A->col_indx[k]];
        y[r] = (beta == 0.0) ? alpha * s : alpha * s + beta * y[r];
    }
    return SPARSE_STATUS_SUCCESS;
}
