// Host analysis of an ILU pattern: diagonal pointers, Liu elimination trees and level
// sets of the lower (L) and reversed upper (U) dependency DAGs.  Integer output is
// identical to the reference's (src/ilu_solver.cpp:276-289, src/subtree.hpp:35-68,
// src/subtree.hpp:524-551).
#pragma once

#include <algorithm>
#include <stdexcept>
#include <vector>

namespace gb300 {

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
