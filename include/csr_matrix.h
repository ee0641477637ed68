/*
 * Host CSR container and its utilities.  Same struct layout, names and signatures as
 * the reference's include/csr_matrix.h:9-49 (0-based CSR, int32 indices, float64
 * values).  Arrays are owned by the struct and managed only through these functions.
 */
#pragma once

#include "lljbash_decl.h"

#ifdef __cplusplus
extern "C" {
#endif

/* replaces include/csr_matrix.h:10-16 */
#define CsrMatrix LLJBASH_DECL(CsrMatrix)
struct CsrMatrix {
    int size LLJBASH_DEFAULT_VALUE(-1);
    int max_nnz LLJBASH_DEFAULT_VALUE(0);
    int* row_ptr LLJBASH_DEFAULT_VALUE(LLJBASH_NULL);
    int* col_idx LLJBASH_DEFAULT_VALUE(LLJBASH_NULL);
    double* value LLJBASH_DEFAULT_VALUE(LLJBASH_NULL);
};
LLJBASH_STRUCT_TYPEDEF(CsrMatrix);

/* replaces include/csr_matrix.h:19-20 (src/csr_matrix.cpp:25) */
#define CSR_MATRIX_DEFAULT LLJBASH_DECL(CSR_MATRIX_DEFAULT)
extern const CsrMatrix CSR_MATRIX_DEFAULT;

/* (Re)allocates row_ptr[size+1], col_idx[max_nnz], value[max_nnz], 64-byte aligned and
 * page-locked when a CUDA device is present; contents are not initialised.
 * replaces include/csr_matrix.h:22-23 (src/csr_matrix.cpp:27-33) */
#define SetupCsrMatrix LLJBASH_DECL(SetupCsrMatrix)
void SetupCsrMatrix(CsrMatrix* mat, int size, int max_nnz);

/* replaces include/csr_matrix.h:25-26 (src/csr_matrix.cpp:35-42) */
#define CopyCsrMatrix LLJBASH_DECL(CopyCsrMatrix)
void CopyCsrMatrix(CsrMatrix* dst, const CsrMatrix* src);

/* replaces include/csr_matrix.h:28-29 (src/csr_matrix.cpp:44-47) */
#define CopyCsrMatrixValues LLJBASH_DECL(CopyCsrMatrixValues)
void CopyCsrMatrixValues(CsrMatrix* dst, const CsrMatrix* src);

/* replaces include/csr_matrix.h:31-32 (src/csr_matrix.cpp:49-51) */
#define DestroyCsrMatrix LLJBASH_DECL(DestroyCsrMatrix)
void DestroyCsrMatrix(CsrMatrix* mat);

/* replaces include/csr_matrix.h:34-37 */
#define GetCsrNonzeros LLJBASH_DECL(GetCsrNonzeros)
static inline int GetCsrNonzeros(const CsrMatrix* mat) {
    return mat->row_ptr[mat->size];
}

/* Reads a 1-based coordinate MatrixMarket file, permutes rows by a maximum matching so
 * every diagonal entry has |a_ii| > 1e-12, sorts columns.  Exits the process on a
 * malformed file, as the reference does.  replaces include/csr_matrix.h:39-40
 * (src/csr_matrix.cpp:53-159) */
#define ReadCsrMatrixMM1 LLJBASH_DECL(ReadCsrMatrixMM1)
void ReadCsrMatrixMM1(CsrMatrix* mat, const char* filename);

/* sol = mat * vec on the host.  replaces include/csr_matrix.h:42-43
 * (src/csr_matrix.cpp:163-171) */
#define CsrMatVec LLJBASH_DECL(CsrMatVec)
void CsrMatVec(const CsrMatrix* mat, const double* vec, double* sol);

/* Fill-reducing orderings of the pattern of A + A^T: p[k] = the row placed k-th, ip (may
 * be NULL) its inverse.  The reference delegates them to SuiteSparse AMD / CHOLMOD nested
 * dissection (src/csr_matrix.cpp:173-225); this library computes its own (approximate
 * minimum degree on the quotient graph; recursive bisection at breadth-first level
 * separators), so the permutations differ from SuiteSparse's.  Return values are the
 * reference's: CsrAmdOrder 0 on success, -1 on failure; CsrNdOrder 1 on success, 0 on
 * failure.  replaces include/csr_matrix.h:45-49 */
#define CsrAmdOrder LLJBASH_DECL(CsrAmdOrder)
int CsrAmdOrder(const CsrMatrix* mat, int* p, int* ip);

#define CsrNdOrder LLJBASH_DECL(CsrNdOrder)
int CsrNdOrder(const CsrMatrix* mat, int* p, int* ip);

#ifdef __cplusplus
}
#endif
