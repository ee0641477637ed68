// Batched persistent ILU(0) + GMRES(m): many independent sparse systems of uneven size,
// each with several right-hand sides, in ONE persistent kernel launch.
//
// Work items, drawn from a ticket counter by whole CTAs: first one factorisation item per
// system, then one solve item per (system, group of G right-hand sides).  A solve item waits for its
// system's ready flag, which the factorising CTA (holding a smaller ticket, hence
// running) publishes with release semantics; the wait is bounded.
//
// A CTA owns its item completely:
//  * factorisation: A's values (+ the learned diagonal shift, computed in the same CTA
//    by the fused feature / MLP pre-pass) are eliminated level by level of the lower
//    dependency DAG (rows of one level in parallel, one thread per row, the reference's
//    up-looking order per entry, FP64), then stored as FP32 factors + FP32 1/u_ii;
//  * solve: GMRES(m) in FP32 cycles with FP64 iterative refinement (every cycle starts
//    from the FP64 residual b - A x and adds its FP32 correction to the FP64 x; only the
//    FP64 residual can end the solve) for G right-hand sides in lockstep (vectors
//    interleaved [row][G], one thread per row and right-hand side), level-synchronous
//    triangular solves within the CTA, CGS2 with block reductions, Givens and least
//    squares on one thread per right-hand side.
#pragma once

#include "common.cuh"
#include "mlp.cuh"

namespace gb300 {

constexpr int kBatchThreads = 512;
constexpr int kBatchWarps = kBatchThreads / kWarp;
constexpr int kBatchMaxM = 64;
constexpr int kBatchMaxG = 16;  // right-hand sides per solve item

struct BatchDesc {
    int nsys = 0, nrhs = 0, m = 0, maxit = 0;
    double rtol = 1e-8, tau = 1e-6;
    // per system
    const int* n = nullptr;
    const long long* rp_off = nullptr;   // into rp (n_s + 1 entries each)
    const long long* nnz_off = nullptr;  // into ci / values
    const long long* row_off = nullptr;  // into per-row arrays
    const long long* lvl_off = nullptr;  // into lptrL / lptrU (nlev + 1 entries each)
    const int* nlevL = nullptr;
    const int* nlevU = nullptr;
    const long long* rhs_off = nullptr;  // into rhs / x (nrhs * n_s entries each)
    const int* sys_of_slot = nullptr;    // processing order of the systems
    // concatenated arrays (local indices inside each system)
    const int* rp = nullptr;
    const int* ci = nullptr;
    const double* a64 = nullptr;
    const double* f64 = nullptr;  // values to factorise (A's values when null)
    float* a32 = nullptr;
    double* lu64 = nullptr;
    float* lu32 = nullptr;
    const int* diag = nullptr;
    const int* ordL = nullptr;
    const int* ordU = nullptr;
    const int* lptrL = nullptr;
    const int* lptrU = nullptr;
    const int* depth = nullptr;
    float* dinv = nullptr;
    // learned shift (optional)
    const float* mlp = nullptr;
    float min_shift = 0.f;
    // input / output
    const double* rhs = nullptr;
    double* x = nullptr;
    int* iters = nullptr;
    double* resid = nullptr;
    int* converged = nullptr;
    int* shifted = nullptr;  // per system: the learned shift was applied
    int* ready = nullptr;
    int epoch = 1;
    unsigned* ticket = nullptr;
    int* status = nullptr;
    // per-CTA workspace
    float* V = nullptr;
    float* Z = nullptr;
    double* xw = nullptr;
    double* rw = nullptr;
    double* H = nullptr;  // per CTA and right-hand side: Hessenberg columns [m][kBatchMaxM + 1]
    long long ws = 0;  // padded vector length
};

}  // namespace gb300
