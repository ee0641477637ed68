// Host analysis of an ILU pattern: diagonal pointers, Liu elimination trees and level
// sets of the lower (L) and reversed upper (U) dependency DAGs.  Integer output is
// identical to the reference's (src/ilu_solver.cpp:276-289, src/subtree.hpp:35-68,
// src/subtree.hpp:524-551).
#pragma once

#include <algorithm>
#include <climits>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace gb300 {

// Structural check of a CSR matrix handed in by a caller, run on the host before any of
// it reaches a kernel (an index outside its range would make a kernel read or write
// outside its buffers): n >= 0, row_ptr[0] == 0, row_ptr non-decreasing and, when
// `capacity` >= 0, row_ptr[n] <= capacity (the entries the arrays hold); every column
// index in [0, n) and the columns of each row strictly ascending.  Throws
// std::runtime_error naming `what` and the first offending row.  Matrices of more than
// 2^20 entries are checked by several host threads.
inline void validate_csr(int n, const int* rp, const int* ci, const char* what, long long capacity = -1) {
    const std::string tag = std::string("invalid CSR matrix (") + what + "): ";
    if (n < 0) throw std::runtime_error(tag + "negative size " + std::to_string(n));
    if (n == 0) return;
    if (rp == nullptr) throw std::runtime_error(tag + "row_ptr is NULL");
    if (rp[0] != 0) throw std::runtime_error(tag + "row_ptr[0] = " + std::to_string(rp[0]) + ", expected 0");
    for (int i = 0; i < n; ++i)
        if (rp[i + 1] < rp[i])
            throw std::runtime_error(tag + "row_ptr decreases at row " + std::to_string(i) + " (" +
                                     std::to_string(rp[i]) + " -> " + std::to_string(rp[i + 1]) + ")");
    const long long nnz = rp[n];
    if (capacity >= 0 && nnz > capacity)
        throw std::runtime_error(tag + "row_ptr[n] = " + std::to_string(nnz) + " exceeds the " +
                                 std::to_string(capacity) + " entries the matrix holds");
    if (nnz > 0 && ci == nullptr) throw std::runtime_error(tag + "col_idx is NULL");
    // first offending row of [r0, r1) (INT_MAX: none); kind 1 out of range, 2 not ascending
    auto scan = [&](int r0, int r1, int& bad, int& kind) {
        bad = INT_MAX;
        kind = 0;
        for (int i = r0; i < r1; ++i) {
            int prev = -1;
            for (int p = rp[i]; p < rp[i + 1]; ++p) {
                const int c = ci[p];
                if (c < 0 || c >= n) {
                    bad = i;
                    kind = 1;
                    return;
                }
                if (c <= prev) {
                    bad = i;
                    kind = 2;
                    return;
                }
                prev = c;
            }
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = static_cast<int>(std::min<long long>({static_cast<long long>(hw), 16ll, 1 + (nnz >> 20)}));
    std::vector<int> bad(static_cast<size_t>(nt)), kind(static_cast<size_t>(nt));
    if (nt == 1) {
        scan(0, n, bad[0], kind[0]);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) {
            const int r0 = static_cast<int>(static_cast<long long>(n) * t / nt);
            const int r1 = static_cast<int>(static_cast<long long>(n) * (t + 1) / nt);
            pool.emplace_back([&, t, r0, r1] { scan(r0, r1, bad[t], kind[t]); });
        }
        for (auto& th : pool) th.join();
    }
    for (int t = 0; t < nt; ++t) {
        if (bad[t] == INT_MAX) continue;
        const int i = bad[t];
        if (kind[t] == 1)
            throw std::runtime_error(tag + "row " + std::to_string(i) + " has a column index outside [0, " +
                                     std::to_string(n) + ")");
        throw std::runtime_error(tag + "the column indices of row " + std::to_string(i) +
                                 " are not strictly ascending");
    }
}

// diag[i] = first position p in row i with col_idx[p] >= i.  Throws "missing diag" when
// that position does not hold column i.
inline void diagonal_pointers(int n, const int* rp, const int* ci, std::vector<int>& diag) {
    diag.assign(static_cast<size_t>(n), -1);
    bool missing = false;
    for (int i = 0; i < n; ++i) {
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            if (ci[p] >= i) {
                diag[i] = p;
                break;
            }
        }
        if (diag[i] < 0 || ci[diag[i]] != i) missing = true;
    }
    if (missing) throw std::runtime_error("missing diag");
}

// Dependencies of row j: lower DAG = strict-lower entries [rp[j], diag[j]); upper DAG =
// strict-upper entries (diag[j], rp[j+1]) with vertices visited n-1 .. 0.
struct DagView {
    const int* rp;
    const int* ci;
    const int* diag;
    bool lower;
    int begin(int j) const { return lower ? rp[j] : diag[j] + 1; }
    int end(int j) const { return lower ? diag[j] : rp[j + 1]; }
};

// Liu's elimination tree with path compression; roots get parent n.
inline void elimination_tree(int n, const DagView& g, std::vector<int>& parent) {
    parent.assign(static_cast<size_t>(n), n);
    std::vector<int> anc(static_cast<size_t>(n), n);
    for (int s = 0; s < n; ++s) {
        const int j = g.lower ? s : n - 1 - s;
        for (int p = g.begin(j); p < g.end(j); ++p) {
            int i = g.ci[p];
            while (anc[i] != n) {
                const int up = anc[i];
                anc[i] = j;
                i = up;
            }
            if (i != j) {
                anc[i] = j;
                parent[i] = j;
            }
        }
    }
}

// depth[j] = 1 + max depth of j's dependencies (0 for rows without any).  Also returns
// the rows grouped by level, ascending row index inside a level (the reference's lset).
inline int level_sets(int n, const DagView& g, std::vector<int>& depth, std::vector<int>& order,
                      std::vector<int>& level_ptr) {
    depth.assign(static_cast<size_t>(n), 0);
    int nlev = 0;
    for (int s = 0; s < n; ++s) {
        const int j = g.lower ? s : n - 1 - s;
        int d = 0;
        for (int p = g.begin(j); p < g.end(j); ++p) d = std::max(d, depth[g.ci[p]] + 1);
        depth[j] = d;
        nlev = std::max(nlev, d + 1);
    }
    level_ptr.assign(static_cast<size_t>(nlev) + 1, 0);
    for (int j = 0; j < n; ++j) ++level_ptr[depth[j] + 1];
    for (int l = 0; l < nlev; ++l) level_ptr[l + 1] += level_ptr[l];
    order.assign(static_cast<size_t>(n), 0);
    std::vector<int> fill(level_ptr.begin(), level_ptr.end() - 1);
    for (int j = 0; j < n; ++j) order[fill[depth[j]]++] = j;
    return nlev;
}

}  // namespace gb300
