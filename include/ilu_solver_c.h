/*
 * C ABI of the ILU solver.  Same names, signatures and return codes as the
 * reference's include_c/ilu_solver_c.h:15-31 (src_c/ilu_solver_c.cpp:6-50).
 */
#pragma once

#ifndef __cplusplus
#include <stdbool.h>
#else
#include <cstdbool>
#endif

#include "csr_matrix.h"

#ifdef __cplusplus
extern "C" {
#endif

#define IluSolverHdl LLJBASH_DECL(IluSolverHdl)
typedef void* IluSolverHdl;

/* nthreads is accepted for compatibility (GPU build). */
#define IluSolverCreate LLJBASH_DECL(IluSolverCreate)
IluSolverHdl IluSolverCreate(int nthreads);

#define IluSolverDestroy LLJBASH_DECL(IluSolverDestroy)
void IluSolverDestroy(IluSolverHdl hdl);

#define IluSolverGetMatrix LLJBASH_DECL(IluSolverGetMatrix)
CsrMatrix* IluSolverGetMatrix(IluSolverHdl hdl);

/* 0 on success, -2 if a row has no diagonal entry, -1 on any other error. */
#define IluSolverSetup LLJBASH_DECL(IluSolverSetup)
int IluSolverSetup(IluSolverHdl hdl);

/* 0 on success, -2 "missing diag", -1 on any other error (e.g. a device error or a
 * dependency wait that timed out). */
#define IluSolverFactorize LLJBASH_DECL(IluSolverFactorize)
int IluSolverFactorize(IluSolverHdl hdl);

#ifdef __cplusplus
}
#endif
