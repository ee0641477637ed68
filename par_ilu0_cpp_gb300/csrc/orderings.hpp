// Fill-reducing orderings of a sparse symmetric pattern (the graph of A + A^T without
// its diagonal), the project's own implementations behind CsrAmdOrder / CsrNdOrder (the
// reference calls SuiteSparse AMD and CHOLMOD's nested dissection, src/csr_matrix.cpp:
// 173-225, which this library does not ship; their orderings are not reproduced bit for
// bit):
//
// * minimum_degree_order: approximate minimum degree on the quotient graph (Amestoy,
//   Davis & Duff, 1996): each step eliminates a variable of least approximate external
//   degree, forms the new element from its variable neighbours and the variables of the
//   elements it absorbs, prunes the neighbours' lists, bounds their external degrees by
//   the AMD formula (|A_i| + |L_p \ i| + sum over other elements of |L_e \ L_p|), and
//   merges indistinguishable variables (same variable and element neighbours, found by
//   hashing) into supervariables that are eliminated together;
// * nested_dissection_order: recursive bisection; a part is split at the middle level
//   of a breadth-first level structure rooted at a pseudo-peripheral vertex, the two
//   sides are ordered first (recursively), the separator last; parts of at most
//   kNdLeaf vertices are ordered by minimum_degree_order.
//
// Both return perm with perm[k] = the vertex eliminated k-th.
#pragma once

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

namespace gb300 {

// Adjacency of the symmetrised pattern without self loops (CSR: xadj, adj).
inline void symmetric_graph(int n, const int* rp, const int* ci, std::vector<int>& xadj, std::vector<int>& adj) {
    std::vector<int> cnt(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i)
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            const int j = ci[p];
            if (j == i) continue;
            ++cnt[static_cast<size_t>(i) + 1];
            ++cnt[static_cast<size_t>(j) + 1];
        }
    for (int i = 0; i < n; ++i) cnt[static_cast<size_t>(i) + 1] += cnt[static_cast<size_t>(i)];
    std::vector<int> tmp(static_cast<size_t>(cnt[static_cast<size_t>(n)]));
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < n; ++i)
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            const int j = ci[p];
            if (j == i) continue;
            tmp[static_cast<size_t>(fill[static_cast<size_t>(i)]++)] = j;
            tmp[static_cast<size_t>(fill[static_cast<size_t>(j)]++)] = i;
        }
    // sort and deduplicate every list (A and A^T may both hold an edge)
    xadj.assign(static_cast<size_t>(n) + 1, 0);
    adj.clear();
    adj.reserve(tmp.size());
    for (int i = 0; i < n; ++i) {
        auto b = tmp.begin() + cnt[static_cast<size_t>(i)];
        auto e = tmp.begin() + cnt[static_cast<size_t>(i) + 1];
        std::sort(b, e);
        const auto last = std::unique(b, e);
        adj.insert(adj.end(), b, last);
        xadj[static_cast<size_t>(i) + 1] = static_cast<int>(adj.size());
    }
}

// Approximate minimum degree ordering of the graph (xadj, adj) of n vertices.
inline std::vector<int> minimum_degree_order(int n, const std::vector<int>& xadj, const std::vector<int>& adj) {
    std::vector<int> order;
    order.reserve(static_cast<size_t>(n));
    if (n == 0) return order;
    enum : unsigned char { kVar = 0, kElem = 1, kDead = 2 };  // dead: absorbed element or merged variable
    std::vector<unsigned char> kind(static_cast<size_t>(n), kVar);
    std::vector<int> nv(static_cast<size_t>(n), 1);            // supervariable sizes
    std::vector<int> next_member(static_cast<size_t>(n), -1);  // members of a supervariable
    std::vector<int> last_member(static_cast<size_t>(n));
    std::iota(last_member.begin(), last_member.end(), 0);
    std::vector<std::vector<int>> A(static_cast<size_t>(n)), E(static_cast<size_t>(n)), L(static_cast<size_t>(n));
    std::vector<int> deg(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        A[static_cast<size_t>(i)].assign(adj.begin() + xadj[static_cast<size_t>(i)], adj.begin() + xadj[static_cast<size_t>(i) + 1]);
        deg[static_cast<size_t>(i)] = static_cast<int>(A[static_cast<size_t>(i)].size());
    }
    // degree buckets (doubly linked lists)
    std::vector<int> head(static_cast<size_t>(n) + 1, -1), nxt(static_cast<size_t>(n), -1), prv(static_cast<size_t>(n), -1);
    int mindeg = n;
    auto bucket_insert = [&](int i) {
        const int d = std::min(deg[static_cast<size_t>(i)], n);
        nxt[static_cast<size_t>(i)] = head[static_cast<size_t>(d)];
        prv[static_cast<size_t>(i)] = -1;
        if (head[static_cast<size_t>(d)] >= 0) prv[static_cast<size_t>(head[static_cast<size_t>(d)])] = i;
        head[static_cast<size_t>(d)] = i;
        mindeg = std::min(mindeg, d);
    };
    auto bucket_remove = [&](int i) {
        const int d = std::min(deg[static_cast<size_t>(i)], n);
        if (prv[static_cast<size_t>(i)] >= 0) {
            nxt[static_cast<size_t>(prv[static_cast<size_t>(i)])] = nxt[static_cast<size_t>(i)];
        } else {
            head[static_cast<size_t>(d)] = nxt[static_cast<size_t>(i)];
        }
        if (nxt[static_cast<size_t>(i)] >= 0) prv[static_cast<size_t>(nxt[static_cast<size_t>(i)])] = prv[static_cast<size_t>(i)];
    };
    for (int i = n - 1; i >= 0; --i) bucket_insert(i);
    std::vector<int> mark(static_cast<size_t>(n), -1);  // stamp: member of the current L_p
    std::vector<int> wext(static_cast<size_t>(n), -1);  // |L_e \ L_p| (weighted), valid when wstamp[e] == step
    std::vector<int> wstamp(static_cast<size_t>(n), -1);
    std::vector<uint64_t> hash(static_cast<size_t>(n));
    int eliminated = 0;
    for (int step = 0; eliminated < n; ++step) {
        while (head[static_cast<size_t>(mindeg)] < 0) ++mindeg;
        const int p = head[static_cast<size_t>(mindeg)];
        bucket_remove(p);
        // the new element: p's variable neighbours and the variables of its elements
        std::vector<int>& Lp = L[static_cast<size_t>(p)];
        Lp.clear();
        mark[static_cast<size_t>(p)] = step;
        for (int j : A[static_cast<size_t>(p)])
            if (kind[static_cast<size_t>(j)] == kVar && mark[static_cast<size_t>(j)] != step) {
                mark[static_cast<size_t>(j)] = step;
                Lp.push_back(j);
            }
        for (int e : E[static_cast<size_t>(p)]) {
            if (kind[static_cast<size_t>(e)] != kElem) continue;
            for (int j : L[static_cast<size_t>(e)])
                if (kind[static_cast<size_t>(j)] == kVar && mark[static_cast<size_t>(j)] != step) {
                    mark[static_cast<size_t>(j)] = step;
                    Lp.push_back(j);
                }
            kind[static_cast<size_t>(e)] = kDead;  // absorbed into p
            std::vector<int>().swap(L[static_cast<size_t>(e)]);
        }
        kind[static_cast<size_t>(p)] = kElem;
        std::vector<int>().swap(A[static_cast<size_t>(p)]);
        std::vector<int>().swap(E[static_cast<size_t>(p)]);
        for (int m = p; m >= 0; m = next_member[static_cast<size_t>(m)]) order.push_back(m);
        eliminated += nv[static_cast<size_t>(p)];
        int lp_w = 0;
        for (int v : Lp) lp_w += nv[static_cast<size_t>(v)];
        // |L_e \ L_p| for the other elements next to L_p
        for (int v : Lp) {
            bucket_remove(v);
            for (int e : E[static_cast<size_t>(v)]) {
                if (kind[static_cast<size_t>(e)] != kElem || e == p) continue;
                if (wstamp[static_cast<size_t>(e)] != step) {
                    int w = 0;
                    for (int j : L[static_cast<size_t>(e)])
                        if (kind[static_cast<size_t>(j)] == kVar) w += nv[static_cast<size_t>(j)];
                    wext[static_cast<size_t>(e)] = w;
                    wstamp[static_cast<size_t>(e)] = step;
                }
                wext[static_cast<size_t>(e)] -= nv[static_cast<size_t>(v)];
            }
        }
        // prune the neighbours' lists, add element p, bound their external degrees
        for (int v : Lp) {
            std::vector<int>& Ev = E[static_cast<size_t>(v)];
            int ext = 0;
            size_t w = 0;
            for (int e : Ev) {
                if (kind[static_cast<size_t>(e)] != kElem || e == p) continue;
                if (wstamp[static_cast<size_t>(e)] == step && wext[static_cast<size_t>(e)] <= 0) {
                    kind[static_cast<size_t>(e)] = kDead;  // L_e inside L_p: absorbed as well
                    std::vector<int>().swap(L[static_cast<size_t>(e)]);
                    continue;
                }
                ext += wstamp[static_cast<size_t>(e)] == step ? wext[static_cast<size_t>(e)] : 0;
                Ev[w++] = e;
            }
            Ev.resize(w);
            Ev.push_back(p);
            std::vector<int>& Av = A[static_cast<size_t>(v)];
            w = 0;
            int aw = 0;
            for (int j : Av) {
                if (kind[static_cast<size_t>(j)] != kVar || mark[static_cast<size_t>(j)] == step) continue;  // covered by element p
                Av[w++] = j;
                aw += nv[static_cast<size_t>(j)];
            }
            Av.resize(w);
            const int bound = aw + (lp_w - nv[static_cast<size_t>(v)]) + ext;
            deg[static_cast<size_t>(v)] = std::max(0, std::min({n - eliminated - nv[static_cast<size_t>(v)], bound}));
        }
        // supervariables: variables of L_p with the same element and variable neighbours
        for (int v : Lp) {
            uint64_t h = 1469598103934665603ull;
            std::vector<int>& Ev = E[static_cast<size_t>(v)];
            std::vector<int>& Av = A[static_cast<size_t>(v)];
            std::sort(Ev.begin(), Ev.end());
            std::sort(Av.begin(), Av.end());
            for (int e : Ev) h = (h ^ static_cast<uint64_t>(e) * 2654435761ull) * 1099511628211ull;
            h ^= 0x9e3779b97f4a7c15ull;
            for (int j : Av) h = (h ^ static_cast<uint64_t>(j) * 2246822519ull) * 1099511628211ull;
            hash[static_cast<size_t>(v)] = h;
        }
        std::vector<int> byhash(Lp);
        std::sort(byhash.begin(), byhash.end(), [&](int a, int b) {
            return hash[static_cast<size_t>(a)] < hash[static_cast<size_t>(b)] || (hash[static_cast<size_t>(a)] == hash[static_cast<size_t>(b)] && a < b);
        });
        for (size_t a = 0; a < byhash.size(); ++a) {
            const int u = byhash[a];
            if (kind[static_cast<size_t>(u)] != kVar) continue;
            for (size_t b = a + 1; b < byhash.size() && hash[static_cast<size_t>(byhash[b])] == hash[static_cast<size_t>(u)]; ++b) {
                const int v = byhash[b];
                if (kind[static_cast<size_t>(v)] != kVar) continue;
                // v and u must also see each other only through shared elements
                if (E[static_cast<size_t>(u)] != E[static_cast<size_t>(v)] || A[static_cast<size_t>(u)] != A[static_cast<size_t>(v)]) continue;
                const int merged = nv[static_cast<size_t>(v)];
                nv[static_cast<size_t>(u)] += merged;
                deg[static_cast<size_t>(u)] = std::max(0, deg[static_cast<size_t>(u)] - merged);  // v is no longer external to u
                next_member[static_cast<size_t>(last_member[static_cast<size_t>(u)])] = v;
                last_member[static_cast<size_t>(u)] = last_member[static_cast<size_t>(v)];
                kind[static_cast<size_t>(v)] = kDead;
                nv[static_cast<size_t>(v)] = 0;
                std::vector<int>().swap(A[static_cast<size_t>(v)]);
                std::vector<int>().swap(E[static_cast<size_t>(v)]);
            }
        }
        for (int v : Lp)
            if (kind[static_cast<size_t>(v)] == kVar) {
                deg[static_cast<size_t>(v)] = std::max(0, std::min(deg[static_cast<size_t>(v)], n - eliminated - nv[static_cast<size_t>(v)]));
                bucket_insert(v);
            }
        // element p keeps only its live variables
        size_t w = 0;
        for (int v : Lp)
            if (kind[static_cast<size_t>(v)] == kVar) Lp[w++] = v;
        Lp.resize(w);
        if (Lp.empty()) kind[static_cast<size_t>(p)] = kDead;
        mindeg = 0;
    }
    return order;
}

constexpr int kNdLeaf = 64;

// Nested dissection ordering of the graph (xadj, adj) of n vertices.
inline std::vector<int> nested_dissection_order(int n, const std::vector<int>& xadj, const std::vector<int>& adj) {
    std::vector<int> order(static_cast<size_t>(n));
    std::vector<int> where(static_cast<size_t>(n), 0);  // part id of a vertex while it is being split
    std::vector<int> level(static_cast<size_t>(n), -1);
    std::vector<int> local(static_cast<size_t>(n), -1);
    int next_part = 1;
    // stack of (part id, vertices, first position in `order` for its block)
    struct Job {
        int id;
        std::vector<int> verts;
        int pos;
    };
    std::vector<Job> stack;
    {
        Job root{0, std::vector<int>(static_cast<size_t>(n)), 0};
        std::iota(root.verts.begin(), root.verts.end(), 0);
        stack.push_back(std::move(root));
    }
    auto bfs = [&](int id, int src, std::vector<int>& q) {  // level structure inside part `id`
        q.clear();
        q.push_back(src);
        level[static_cast<size_t>(src)] = 0;
        for (size_t h = 0; h < q.size(); ++h) {
            const int v = q[h];
            for (int k = xadj[static_cast<size_t>(v)]; k < xadj[static_cast<size_t>(v) + 1]; ++k) {
                const int u = adj[static_cast<size_t>(k)];
                if (where[static_cast<size_t>(u)] == id && level[static_cast<size_t>(u)] < 0) {
                    level[static_cast<size_t>(u)] = level[static_cast<size_t>(v)] + 1;
                    q.push_back(u);
                }
            }
        }
    };
    std::vector<int> q, q2;
    while (!stack.empty()) {
        Job job = std::move(stack.back());
        stack.pop_back();
        const int m = static_cast<int>(job.verts.size());
        if (m == 0) continue;
        if (m <= kNdLeaf) {
            // leaf: minimum degree on the induced subgraph
            for (int i = 0; i < m; ++i) local[static_cast<size_t>(job.verts[static_cast<size_t>(i)])] = i;
            std::vector<int> sx(static_cast<size_t>(m) + 1, 0), sa;
            for (int i = 0; i < m; ++i) {
                const int v = job.verts[static_cast<size_t>(i)];
                for (int k = xadj[static_cast<size_t>(v)]; k < xadj[static_cast<size_t>(v) + 1]; ++k) {
                    const int u = adj[static_cast<size_t>(k)];
                    if (where[static_cast<size_t>(u)] == job.id) sa.push_back(local[static_cast<size_t>(u)]);
                }
                sx[static_cast<size_t>(i) + 1] = static_cast<int>(sa.size());
            }
            const std::vector<int> lo = minimum_degree_order(m, sx, sa);
            for (int i = 0; i < m; ++i) order[static_cast<size_t>(job.pos + i)] = job.verts[static_cast<size_t>(lo[static_cast<size_t>(i)])];
            for (int v : job.verts) where[static_cast<size_t>(v)] = -1;
            continue;
        }
        // a connected component of the part (from its first unvisited vertex)
        for (int v : job.verts) level[static_cast<size_t>(v)] = -1;
        bfs(job.id, job.verts[0], q);
        if (static_cast<int>(q.size()) < m) {
            // several components: split off this one, the rest stays a part of its own
            const int idA = next_part++, idB = next_part++;
            std::vector<int> comp(q), rest;
            for (int v : comp) where[static_cast<size_t>(v)] = idA;
            for (int v : job.verts)
                if (where[static_cast<size_t>(v)] == job.id) {
                    where[static_cast<size_t>(v)] = idB;
                    rest.push_back(v);
                }
            stack.push_back(Job{idB, std::move(rest), job.pos + static_cast<int>(comp.size())});
            stack.push_back(Job{idA, std::move(comp), job.pos});
            continue;
        }
        // pseudo-peripheral vertex: restart from the last vertex of the deepest level
        // while the level structure gets deeper
        int src = q.back(), depth = level[static_cast<size_t>(q.back())];
        for (int it = 0; it < 4; ++it) {
            for (int v : job.verts) level[static_cast<size_t>(v)] = -1;
            bfs(job.id, src, q2);
            const int d2 = level[static_cast<size_t>(q2.back())];
            if (d2 <= depth) break;
            depth = d2;
            src = q2.back();
            q.swap(q2);
        }
        for (int v : job.verts) level[static_cast<size_t>(v)] = -1;
        bfs(job.id, src, q);
        depth = level[static_cast<size_t>(q.back())];
        if (depth < 2) {  // no separating level: order by minimum degree as a leaf would
            // force the leaf path by splitting into chunks of at most kNdLeaf vertices
            // (a near-clique: every order fills it completely)
            for (int i = 0; i < m; i += kNdLeaf) {
                const int id = next_part++;
                std::vector<int> chunk(job.verts.begin() + i, job.verts.begin() + std::min(m, i + kNdLeaf));
                for (int v : chunk) where[static_cast<size_t>(v)] = id;
                stack.push_back(Job{id, std::move(chunk), job.pos + i});
            }
            continue;
        }
        // separator: the level at which half of the vertices lie below
        std::vector<int> count(static_cast<size_t>(depth) + 1, 0);
        for (int v : q) ++count[static_cast<size_t>(level[static_cast<size_t>(v)])];
        // (sep <= depth - 1: both sides non-empty, so every part shrinks)
        int sep = 1, below = count[0];
        while (sep < depth - 1 && below + count[static_cast<size_t>(sep)] <= m / 2) {
            below += count[static_cast<size_t>(sep)];
            ++sep;
        }
        std::vector<int> partA, partB, S;
        for (int v : q) {
            const int l = level[static_cast<size_t>(v)];
            (l < sep ? partA : (l == sep ? S : partB)).push_back(v);
        }
        // thin the separator: a separator vertex with no neighbour beyond it joins A
        {
            std::vector<int> keep;
            for (int v : S) {
                bool touches_b = false;
                for (int k = xadj[static_cast<size_t>(v)]; k < xadj[static_cast<size_t>(v) + 1] && !touches_b; ++k) {
                    const int u = adj[static_cast<size_t>(k)];
                    touches_b = where[static_cast<size_t>(u)] == job.id && level[static_cast<size_t>(u)] == sep + 1;
                }
                (touches_b ? keep : partA).push_back(v);
            }
            S.swap(keep);
        }
        const int idA = next_part++, idB = next_part++;
        for (int v : partA) where[static_cast<size_t>(v)] = idA;
        for (int v : partB) where[static_cast<size_t>(v)] = idB;
        for (int v : S) where[static_cast<size_t>(v)] = -1;
        const int nA = static_cast<int>(partA.size()), nB = static_cast<int>(partB.size());
        for (int i = 0; i < static_cast<int>(S.size()); ++i) order[static_cast<size_t>(job.pos + nA + nB + i)] = S[static_cast<size_t>(i)];
        stack.push_back(Job{idB, std::move(partB), job.pos + nA});
        stack.push_back(Job{idA, std::move(partA), job.pos});
    }
    return order;
}

}  // namespace gb300
