/*
 * Oracle test infrastructure only.  Stub of SuiteSparse AMD so that the
 * reference's src/csr_matrix.cpp compiles; CsrAmdOrder (src/csr_matrix.cpp:173-195)
 * is off the ILU/GMRES path and this stub always reports failure.
 */
#pragma once

#define AMD_OK 0
#define AMD_OUT_OF_MEMORY (-1)
#define AMD_INVALID (-2)

inline int amd_order(int n, const int*, const int*, int* p, double*, double*) {
    for (int i = 0; i < n; ++i) p[i] = i;
    return AMD_INVALID;
}
