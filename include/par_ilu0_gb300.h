/*
 * GB300 extensions of the ILU/GMRES C ABI.  Everything here is additive: the entry
 * points of ilu_solver_c.h / gmres_c.h keep the reference's behaviour, and these add
 * what the reference does not expose (a C-level substitution, precision modes, the
 * learned diagonal shift, the batched solver, analysis results and timings).
 * Return codes: 0 success, -1 failure (message via LLJBASH_Gb300LastError), -2 a row
 * without diagonal entry.
 */
#pragma once

#include "gmres_c.h"
#include "ilu_solver_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Message of the last failure reported by an entry point of this library in the
 * calling thread ("" when none). */
const char* LLJBASH_Gb300LastError(void);

/* x = U^{-1} L^{-1} b with the factors of the last IluSolverFactorize (host arrays of
 * length n, b == x allowed).  No counterpart in the reference's C ABI: it replaces the
 * C++-only lljbash::IluSolver::Substitute (include/ilu_solver.hpp:20,
 * src/ilu_solver.cpp:736-831). */
int LLJBASH_IluSolverSubstitute(IluSolverHdl hdl, const double* b, double* x);

/* IluSolverFactorize with the values of GetMatrix()'s pattern read from device memory
 * (d_values: nnz doubles, ready when called).  The factors stay on the device.  No
 * counterpart in the reference (its data never leaves the host). */
int LLJBASH_IluSolverFactorizeDevice(IluSolverHdl hdl, const double* d_values);

/* GmresSolve on device-resident operands: the CSR arrays of A (n rows), rhs and sol
 * (initial guess in, solution out) in device memory, ready when called.  Same return
 * convention as GmresSolve.  No counterpart in the reference. */
bool LLJBASH_GmresSolveDevice(GmresHdl hdl, int n, const int* d_row_ptr, const int* d_col_idx, const double* d_values,
                              const double* d_rhs, double* d_sol, int* iter);

/* x = U^{-1} L^{-1} b on device arrays (d_b: n doubles read, d_x: n doubles written),
 * allocating nothing.  No counterpart in the reference.  For callers that cannot call
 * cudaMalloc when they apply the preconditioner: an application that reserved all
 * device memory for its own pool, or one that must not let a library call
 * cudaMalloc / cudaFree (which may synchronise the device) inside its pipelined work.
 * The forward-sweep vector and the kernels' counters live in one static device array
 * of the library, so n is limited to 2,097,152 rows (larger n returns -1).  The first
 * call on a device resolves that array's address (cudaGetSymbolAddress) and should be
 * made before any stream capture.  Every call shares the array; calls whose GPU work
 * overlaps race on it.  The work runs on the solver's own stream (created non-blocking,
 * so it is not ordered after the legacy default stream): d_b must be complete when the
 * call is made (synchronise the stream that produced it first), and the call blocks
 * until d_x is written.  The device that is current must be the one the solver was set
 * up on (another one returns -1).  Same return codes as the other entry points. */
int LLJBASH_IluSolverSubstituteDeviceNoAlloc(IluSolverHdl hdl, const double* d_b, double* d_x);

/* ILU solver options. */
enum {
    /* 1 (default): copy the factors into GetMatrix()->value after Factorize, as the
     * reference's in-place factorisation leaves them; 0: keep them on the device only. */
    LLJBASH_ILU_OPT_COPY_BACK = 1,
    /* substitution schedule, taking effect at the next IluSolverSetup (results are the
     * same for every schedule):
     *   > 0: contiguous blocks of that many rows, block-local kernel (each CTA keeps a
     *        block's solution in shared memory; dependencies inside a block are handed
     *        over in shared memory); a value type (FP64 / FP32) whose block does not fit
     *        in shared memory keeps the level-ordered kernel;
     *   0:   automatic (default): per value type, block-local with multiples of the
     *        matrix's plane size when a cost model expects it to beat the level-ordered
     *        kernel (factors with at most 8 entries per row and triangle), else the
     *        level-ordered kernel; LLJBASH_IluInfo reports the choice;
     *   -1:  the level-ordered sync-free kernel;
     *   -2:  level-synchronous (the reference's USE_LEVEL variant): the rows of each level
     *        solved by the whole grid without waits, a grid barrier between levels
     *        (cooperative launch), for both value types. */
    LLJBASH_ILU_OPT_BLOCK_ROWS = 2,
    /* warps of the level-ordered substitution kernels (0 = automatic: about 48 levels'
     * worth of tasks, 4 levels' worth when a triangle has rows too long for a lane group
     * and its rows average more than 8 entries; at most 8 per SM).  Takes effect at the
     * next IluSolverSetup. */
    LLJBASH_ILU_OPT_SOLVE_WARPS = 3,
    /* lanes per row of the level-ordered substitution kernels (results are the same for
     * every value):
     *   0:  automatic (default): per triangle, one lane while rows have at most 8
     *       entries, else the smallest group of 2, 4, .. 32 lanes holding the longest
     *       row in 8 entries per lane; one lane (blocking waits) past 256 entries;
     *   1:  one lane per row;
     *   2, 4, 8, 16, 32: at least that many lanes per row (rows of up to 256 entries).
     * Takes effect at the next IluSolverSetup. */
    LLJBASH_ILU_OPT_ROW_LANES = 4,
    /* limit of one device-side dependency wait, in microseconds of device time (0 =
     * default, 4 s).  A wait that reaches it gives up: the call that launched it returns
     * -1 ("dependency wait timed out on the device") and the solver stays usable.  Takes
     * effect at the next launch. */
    LLJBASH_ILU_OPT_WAIT_LIMIT_US = 5,
    /* structured-grid line-pipeline sweeps (results are the same as with every other
     * schedule): for factors that are a full 7-point (3-D) or 5-point (2-D) stencil in
     * natural order, a lane walks one grid line in registers, the other two neighbours
     * arrive by warp shuffles (lanes skewed by one step each), shared memory between the
     * warps of a CTA and L2 between CTAs.  1: both sweeps of both precisions when the
     * pattern qualifies, whatever LLJBASH_ILU_OPT_BLOCK_ROWS says; 0 (default, automatic):
     * when the pattern qualifies and LLJBASH_ILU_OPT_BLOCK_ROWS is automatic (0), each
     * sweep of each precision is timed at the first Factorize against the block-local /
     * level-ordered kernel and the faster kept (LLJBASH_IluInfo grid_fp64 / grid_fp32);
     * -1: off.  Takes effect at the next IluSolverSetup. */
    LLJBASH_ILU_OPT_GRID = 6,
    /* shape of the line-pipeline sweeps (0 = automatic), next IluSolverSetup: lanes of a
     * warp along y (1, 4, 8; the rest along z; 2-D grids use 1), warps of a CTA along y
     * and along z (at most 8 warps in all). */
    LLJBASH_ILU_OPT_GRID_WARP_Y = 7,
    LLJBASH_ILU_OPT_GRID_CTA_Y = 8,
    LLJBASH_ILU_OPT_GRID_CTA_Z = 9,
    /* order in which the factorisation kernel's warps take rows (results are the same
     * for every order): 0 (default) level order (the reference's Levelization); 1 the
     * reference's subtree scheduler (src/subtree.hpp tree_schedule, one worker per SM):
     * the workers' independent subtrees interleaved row by row, then the remaining
     * (separator) rows in elimination-tree post order; 2 the same partitions, each
     * factorised by one CTA level by level without waiting on other CTAs, then the
     * separator rows by tickets (LLJBASH_IluInfo factor_subtree_parts / _rows).  Next
     * IluSolverSetup. */
    LLJBASH_ILU_OPT_TICKET_ORDER = 11,
    /* factorisation kernel (results are the same for every choice): 0 (default,
     * automatic) and 1: one warp per row; 2: one lane per row when no row has more than
     * 16 entries (each finished row publishes u_kk and its upper entries, rows waiting for
     * it poll exactly those values), else one warp per row.  Next IluSolverSetup. */
    LLJBASH_ILU_OPT_FACTOR_KERNEL = 12,
    /* line-pipeline sweeps in thread-block clusters of 8 CTAs along z, the handoffs inside
     * a cluster through distributed shared memory: 1 (default) clusters of 16 CTAs, else
     * of 8, where such clusters can be scheduled; 2 .. 16 clusters of at most that many
     * CTAs; 0 never.  Results are the same.  Next IluSolverSetup. */
    LLJBASH_ILU_OPT_GRID_CLUSTER = 13,
    /* 1: record a per-block timeline of every line-pipeline sweep (read with
     * LLJBASH_IluSolverGetSweepTimeline); 0 (default) off.  Next IluSolverSetup. */
    LLJBASH_ILU_OPT_SWEEP_TIMELINE = 14,
    /* 1: line-pipeline CTAs request more than half of an SM's shared memory, so that no
     * two share an SM; 0 (default) their own size.  Results are the same.  Next
     * IluSolverSetup. */
    LLJBASH_ILU_OPT_GRID_ONE_CTA_PER_SM = 15
};
int LLJBASH_IluSolverSetOption(IluSolverHdl hdl, int option, double value);

/* Per-row diagonal shift added to a_ii before the next factorisations (host array of
 * length n; NULL removes it).  The learned-shift path sets it from the MLP. */
int LLJBASH_IluSolverSetShift(IluSolverHdl hdl, const double* shift);

/* Learned diagonal shift (no counterpart in the reference).  params: the 369 FP32
 * parameters of the 4-16-16-1 MLP (layout in csrc/mlp.cuh), NULL to remove the model.
 * Every later factorisation runs the fused feature + MLP pre-pass and factorises
 * A + diag(shift); a zero / non-finite pivot falls back to plain ILU (reported by
 * LLJBASH_IluInfo.shift_applied).  Rows with predicted relative shift < min_shift get
 * none. */
int LLJBASH_IluSolverSetShiftModel(IluSolverHdl hdl, const float* params, int nparams, double min_shift);

/* Number of MLP parameters (369). */
int LLJBASH_ShiftModelNumParams(void);

/* Per-row MLP features X[n][4] of a host CSR matrix (rows column-sorted, diagonal
 * present), computed on the device; depth: level depth per row (NULL = 0) of nlev
 * levels.  With params, y[n] receives the MLP outputs (relative shifts). */
int LLJBASH_ShiftFeatures(int n, const int* row_ptr, const int* col_idx, const double* values, const int* depth,
                          int nlev, float* X, const float* params, float* y);

/* GPU trainer of the shift MLP (hand-written forward / backward / Adam kernels). */
typedef void* LLJBASH_ShiftTrainerHdl;
LLJBASH_ShiftTrainerHdl LLJBASH_ShiftTrainerCreate(unsigned seed);
void LLJBASH_ShiftTrainerDestroy(LLJBASH_ShiftTrainerHdl tr);
int LLJBASH_ShiftTrainerSetData(LLJBASH_ShiftTrainerHdl tr, const float* X, const float* targets, int n);
int LLJBASH_ShiftTrainerSetParams(LLJBASH_ShiftTrainerHdl tr, const float* params);
int LLJBASH_ShiftTrainerGetParams(LLJBASH_ShiftTrainerHdl tr, float* params);
/* One Adam step on the samples idx[0..batch) (host array); *loss = mean squared error. */
int LLJBASH_ShiftTrainerStep(LLJBASH_ShiftTrainerHdl tr, const int* idx, int batch, float lr, double* loss);
/* Mean-squared-error loss and its gradient over the whole data set (no update). */
int LLJBASH_ShiftTrainerGradient(LLJBASH_ShiftTrainerHdl tr, float* grad, double* loss);
/* MLP outputs for the whole data set. */
int LLJBASH_ShiftTrainerPredict(LLJBASH_ShiftTrainerHdl tr, float* y);

typedef struct LLJBASH_IluInfo {
    int n;
    int nnz;
    int levels_lower;     /* level sets of the lower dependency DAG */
    int levels_upper;     /* level sets of the reversed upper DAG */
    int breakdowns;       /* zero / non-finite pivots in the last Factorize */
    int first_breakdown;  /* smallest such row, -1 if none */
    double factor_ms;     /* device time of the last Factorize (factorisation + packing) */
    long long kernel_launches; /* kernels launched by this solver so far */
    int shift_applied;    /* the last Factorize used a diagonal shift (learned or explicit) */
    int block_rows_fp64;  /* substitution schedule of the FP64 sweeps: rows per block of the
                           * block-local kernel, 0 = level-ordered kernel */
    int block_rows_fp32;  /* the same for the FP32 (mixed-precision) sweeps */
    int block_cluster_fp64; /* CTAs per thread-block cluster of the block-local FP64 sweeps
                             * (boundary rows handed over in distributed shared memory),
                             * 0 = no clusters */
    int block_cluster_fp32; /* the same for the FP32 sweeps */
    int row_lanes_lower;  /* lanes per row of the level-ordered lower / upper sweeps */
    int row_lanes_upper;
    int factor_lane;      /* 1: the factorisation runs one lane per row (else one warp per row) */
    int grid_fp64;        /* FP64 / FP32 sweeps on the line-pipeline schedule: bit 0 the
                           * forward, bit 1 the backward sweep */
    int grid_fp32;
    int grid_nx, grid_ny, grid_nz;  /* its grid (2-D: grid_ny = 1) */
    int grid_warp_y;      /* lanes of a warp along y and z */
    int grid_warp_z;
    int grid_cta_y;       /* warps of a CTA along y and z */
    int grid_cta_z;
    int grid_blocks;      /* CTA-sized blocks of grid lines */
    int grid_cluster;     /* CTAs per thread-block cluster of the line-pipeline sweeps, 0: none */
    int factor_subtree_parts; /* ticket order 2: subtree partitions (one CTA each) and their rows */
    int factor_subtree_rows;
} LLJBASH_IluInfo;
int LLJBASH_IluSolverGetInfo(IluSolverHdl hdl, LLJBASH_IluInfo* info);

/* Per-block timeline of the last line-pipeline sweep of one kind (upper: 0 forward /
 * 1 backward; fp32: 0 FP64 / 1 FP32), recorded with LLJBASH_ILU_OPT_SWEEP_TIMELINE on:
 * 12 values per block (sweep coordinates, block iy + nby iz): [0] compute start
 * (%globaltimer ns), [1] SM id, [2 + w] end of compute warp w, [2 + warps] end of the
 * block's halo warp, the rest 0.  Waits for the device, copies nblocks * 12 values into
 * `out` (capacity `cap`; NULL only queries) and returns nblocks; -1 when no timeline
 * was recorded.  A diagnostic: no counterpart in the reference. */
int LLJBASH_IluSolverGetSweepTimeline(IluSolverHdl hdl, int upper, int fp32, unsigned long long* out, int cap);

/* Integer results of SetupMatrix's analysis (each array of length n, any may be NULL):
 * diagonal positions, Liu elimination-tree parents of the lower DAG and of the
 * reversed upper DAG (roots = n), and level depths of both DAGs.  Identical to the
 * reference's (src/ilu_solver.cpp:276-289, src/subtree.hpp:35-68, :524-551). */
int LLJBASH_IluSolverGetAnalysis(IluSolverHdl hdl, int* diag, int* etree_lower, int* etree_upper, int* depth_lower,
                                 int* depth_upper);

/* Host-only form of SetupMatrix's analysis for a CSR pattern (rows column-sorted):
 * the same five arrays as LLJBASH_IluSolverGetAnalysis plus the level counts.  Touches
 * no device.  Returns -2 when a row has no diagonal entry. */
int LLJBASH_Gb300AnalyzePattern(int n, const int* row_ptr, const int* col_idx, int* diag, int* etree_lower,
                                int* etree_upper, int* depth_lower, int* depth_upper, int* nlevels /* [2] */);

/* The reference's subtree scheduler (src/subtree.hpp:103-475 tree_schedule, no row
 * stripping), restated on the host with identical integer output, for the L-DAG
 * (upper = 0; row weights diag - row_ptr + 1, as the reference's factorisation and forward
 * substitution) or the reverse U-DAG (upper = 1; weights row_ptr[v+1] - diag[v]).
 * Outputs (any may be NULL): part_ptr[nproc + 2], partitions[n] (workers' subtree rows,
 * then the queue rows), task_queue[*ntasks + 1] (granularity > 1: queue tasks in
 * priority order; at most n + 1 entries), the elimination-tree subtree sizes and
 * weights [n + 1] (index n: the virtual root).  Host only; touches no device. */
int LLJBASH_Gb300TreeSchedule(int n, const int* row_ptr, const int* col_idx, int upper, int nproc, int granularity,
                              double relax, int* part_ptr, int* partitions, int* task_queue, int* ntasks,
                              int* subtree_size, int* subtree_weight);

/* Batched persistent solver (no counterpart in the reference): nsys independent
 * systems of uneven size, nrhs right-hand sides each, solved in ONE persistent kernel
 * launch — ILU(0) with FP32 factors (optionally with the learned shift) and GMRES(restart)
 * in FP32 cycles inside FP64 refinement to ||b - A x||_2 <= rtol ||b||_2 (FP64).
 * row_ptr: the systems' row pointers one after the other (n[s] + 1 entries each);
 * col_idx / values: their entries (columns local to each system).  rhs / x: for every
 * system in order, nrhs vectors of n[s] doubles. */
typedef void* LLJBASH_BatchHdl;
LLJBASH_BatchHdl LLJBASH_BatchCreate(int nsys, const int* n, const int* row_ptr, const int* col_idx,
                                     const double* values, int nrhs, int restart, double rtol, int maxit);
/* As LLJBASH_BatchCreate, with separate values to factorise (same layout as values,
 * e.g. A plus a diagonal shift); GMRES iterates on values. */
LLJBASH_BatchHdl LLJBASH_BatchCreateEx(int nsys, const int* n, const int* row_ptr, const int* col_idx,
                                       const double* values, const double* factor_values, int nrhs, int restart,
                                       double rtol, int maxit);
void LLJBASH_BatchDestroy(LLJBASH_BatchHdl hdl);
int LLJBASH_BatchSetShiftModel(LLJBASH_BatchHdl hdl, const float* params, int nparams, double min_shift);
/* Picks the launch shape by timing a sample of the batch (up to two systems per SM,
 * largest first, right-hand sides b = A x for a pseudo-random x, at most 40 iterations
 * each): right-hand sides per solve item (1, 4 or 16: a CTA of 512 threads handles
 * 512 / G rows of G right-hand sides per round, loading each coefficient once for the G)
 * x CTAs per SM (1, 2).  Returns the chosen CTAs per SM and order; right-hand sides and
 * solutions held from a previous solve are overwritten. */
int LLJBASH_BatchAutotune(LLJBASH_BatchHdl hdl, int* ctas_per_sm, int* largest_first);
/* The launch shape in use (after LLJBASH_BatchAutotune or LLJBASH_BatchSetShape). */
int LLJBASH_BatchGetShape(LLJBASH_BatchHdl hdl, int* ctas_per_sm, int* largest_first, int* rhs_per_cta);
int LLJBASH_BatchSetShape(LLJBASH_BatchHdl hdl, int ctas_per_sm, int largest_first, int rhs_per_cta);
/* The autotuner's trials (up to cap of them copied): shape and device time in ms.
 * Returns the number of trials. */
int LLJBASH_BatchGetTrials(LLJBASH_BatchHdl hdl, int cap, int* ctas_per_sm, int* largest_first, int* rhs_per_cta,
                           double* ms);
/* iters / resid / converged: nsys * nrhs entries (any may be NULL); *ms: device time of
 * the launch. */
int LLJBASH_BatchSolve(LLJBASH_BatchHdl hdl, const double* rhs, double* x, int* iters, double* resid, int* converged,
                       double* ms);

/* GMRES options. */
enum {
    LLJBASH_GMRES_OPT_MODE = 1,        /* 0 plain FP64 (default), 1 FP32 cycles in FP64 refinement */
    LLJBASH_GMRES_OPT_TAU = 2,         /* mixed mode: residual reduction per FP32 cycle (default 1e-6) */
    LLJBASH_GMRES_OPT_USE_GRAPH = 3,   /* 1 (default): replay each restart cycle as a CUDA graph */
    LLJBASH_GMRES_OPT_PROFILE = 4,     /* 1: time every kernel with CUDA events (no graph) */
    LLJBASH_GMRES_OPT_KEEP_MATRIX = 5, /* 1: reuse the device copy of A from the previous Solve */
    LLJBASH_GMRES_OPT_VERIFY = 6       /* 1 (default): compute the FP64 true residual at exit */
};
int LLJBASH_GmresSetOption(GmresHdl hdl, int option, double value);

typedef struct LLJBASH_GmresReport {
    int mode;
    int iterations;
    int cycles;
    int converged;    /* FP64 true residual <= tolerance at exit */
    double residual;  /* ||b - A x||_2 at exit, FP64 (-1 if not computed) */
    double solve_ms;  /* device time of the cycles */
    long long kernel_launches; /* kernels launched by this solver so far (graph nodes included) */
} LLJBASH_GmresReport;
int LLJBASH_GmresGetReport(GmresHdl hdl, LLJBASH_GmresReport* report);

/* Kernel categories: 0 residual, 1 forward substitution, 2 backward substitution,
 * 3 SpMV, 4 CGS dot, 5 CGS axpy+dot, 6 CGS axpy+norm, 7 solution update.  Filled in
 * profiling mode; accumulated until reset. */
#define LLJBASH_GMRES_KERNEL_KINDS 8
int LLJBASH_GmresGetKernelTimes(GmresHdl hdl, double* ms, long long* launches, int nkinds);
int LLJBASH_GmresResetKernelTimes(GmresHdl hdl);

#ifdef __cplusplus
}
#endif
