/*
 * Symbolic ILU(k).  replaces include/iluk.h:10-15 (src/iluk.cpp:5-54).
 */
#pragma once

#include "csr_matrix.h"
#include "lljbash_decl.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Level-of-fill pattern F of A (rows of A column-sorted, no duplicates).
 * lof: level of fill.  F is (re)allocated with SetupCsrMatrix; its level-0 entries
 * receive A's values, fill entries are set to 0.  nzmap[nnz(A)] (optional output):
 * f->value[nzmap[i]] corresponds to a->value[i].  Returns nnz(F).
 * The integer output (F's row_ptr/col_idx and nzmap) is identical to the reference's,
 * including its rule that an entry keeps the first level found for it. */
#define IlukSymbolic LLJBASH_DECL(IlukSymbolic)
int IlukSymbolic(const CsrMatrix* a, int lof, CsrMatrix* f, int* nzmap);

#ifdef __cplusplus
}
#endif
