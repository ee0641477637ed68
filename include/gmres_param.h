/*
 * GMRES parameters and statistics.  Byte-identical layouts to the reference's
 * include/gmres_param.h:10-24.
 */
#pragma once

#include "lljbash_decl.h"

#ifdef __cplusplus
extern "C" {
#endif

/* tolerance is an ABSOLUTE bound on ||b - A x||_2 (src/gmres.cpp:186,199,278). */
#define GmresParameters LLJBASH_DECL(GmresParameters)
struct GmresParameters {
    double tolerance LLJBASH_DEFAULT_VALUE(1e-8);
    int krylov_subspace_dimension LLJBASH_DEFAULT_VALUE(60);
    int max_iterations LLJBASH_DEFAULT_VALUE(200);
};
LLJBASH_STRUCT_TYPEDEF(GmresParameters);

/* Accumulated seconds.  total_mv_time / total_precon_time are filled from CUDA events
 * around the SpMV / preconditioner kernels when kernel timing is enabled
 * (LLJBASH_GmresSetOption, par_ilu0_gb300.h); total_fgmr_time accumulates the wall
 * time of Solve; total_init_time the matrix upload/preparation time. */
#define GmresStat LLJBASH_DECL(GmresStat)
struct GmresStat {
    double total_init_time LLJBASH_DEFAULT_VALUE(0.0);
    double total_fgmr_time LLJBASH_DEFAULT_VALUE(0.0);
    double total_mv_time LLJBASH_DEFAULT_VALUE(0.0);
    double total_precon_time LLJBASH_DEFAULT_VALUE(0.0);
};
LLJBASH_STRUCT_TYPEDEF(GmresStat);

#ifdef __cplusplus
}
#endif
