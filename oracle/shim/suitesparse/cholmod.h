/*
 * Oracle test infrastructure only.  Stub of SuiteSparse CHOLMOD so that the
 * reference's src/csr_matrix.cpp compiles; CsrNdOrder (src/csr_matrix.cpp:197-225)
 * is off the ILU/GMRES path and this stub reports failure (identity order).
 */
#pragma once

#include <cstdlib>

#define CHOLMOD_OK 0
#define CHOLMOD_INVALID (-4)
#define CHOLMOD_PATTERN 0

struct cholmod_common {
    int status;
};
struct cholmod_sparse {
    void* p;
    void* i;
    int stype;
};

inline int cholmod_start(cholmod_common* c) { c->status = CHOLMOD_OK; return 1; }
inline int cholmod_finish(cholmod_common*) { return 1; }
inline cholmod_sparse* cholmod_spzeros(std::size_t n, std::size_t, std::size_t nnz, int, cholmod_common*) {
    cholmod_sparse* s = new cholmod_sparse;
    s->p = std::calloc(n + 1, sizeof(int));
    s->i = std::calloc(nnz ? nnz : 1, sizeof(int));
    s->stype = 0;
    return s;
}
inline int cholmod_free_sparse(cholmod_sparse** s, cholmod_common*) {
    if (s && *s) {
        std::free((*s)->p);
        std::free((*s)->i);
        delete *s;
        *s = nullptr;
    }
    return 1;
}
inline long cholmod_nested_dissection(cholmod_sparse*, int*, std::size_t, int* perm, int*, int*,
                                      cholmod_common* c) {
    (void)perm;
    c->status = CHOLMOD_INVALID;
    return -1;
}
