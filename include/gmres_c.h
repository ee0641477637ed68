/*
 * C ABI of the GMRES solver.  Same names and signatures as the reference's
 * include_c/gmres_c.h:10-29 (src_c/gmres_c.cpp:6-33).
 */
#pragma once

#include "gmres_param.h"
#include "ilu_solver_c.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GmresHdl LLJBASH_DECL(GmresHdl)
typedef void* GmresHdl;

#define GmresCreate LLJBASH_DECL(GmresCreate)
GmresHdl GmresCreate(void);

#define GmresDestroy LLJBASH_DECL(GmresDestroy)
void GmresDestroy(GmresHdl hdl);

#define GmresGetParameters LLJBASH_DECL(GmresGetParameters)
GmresParameters* GmresGetParameters(GmresHdl hdl);

#define GmresGetStat LLJBASH_DECL(GmresGetStat)
const GmresStat* GmresGetStat(GmresHdl hdl);

#define GmresSetPreconditioner LLJBASH_DECL(GmresSetPreconditioner)
void GmresSetPreconditioner(GmresHdl hdl, IluSolverHdl ilu);

/* Returns the reference's success flag; *iter (if non-null) receives the iteration
 * count.  rhs and sol are host arrays of length mat->size; sol holds the initial guess
 * on entry. */
#define GmresSolve LLJBASH_DECL(GmresSolve)
bool GmresSolve(GmresHdl hdl, const CsrMatrix* mat, double* rhs, double* sol, int* iter);

#ifdef __cplusplus
}
#endif
