// Host restatement of the reference's subtree scheduler (src/subtree.hpp:35-475,
// 598-688, src/heap.hpp): for a dependency DAG of n rows (the L-DAG in ascending order,
// or the U-DAG in descending order) and nproc workers it computes the elimination tree,
// every subtree's size and weight, a division of the tree into independent subtrees for
// the workers (largest first, long chains shortened), their assignment (largest subtree to
// the least-loaded worker), the workers' row lists in post order, and — for the rows left
// over, the separator part — the task queue: rows aggregated into supernodes of up to
// `granularity` etree-consecutive rows, ordered by a weighted critical-path priority.
// The integer output is identical to the reference's for the same inputs (tested against
// the reference build); the steps are the reference's, in code of this project, because
// the output is part of the parity contract.
//
// Uses on the GPU: the subtree sizes and weights are reported with the analysis, and the
// schedule's row order (workers' partitions, then the queue) is a ticket order of the
// factorisation kernel (LLJBASH_ILU_OPT_TICKET_ORDER).  Row stripping (the reference's
// strip_ratio > 0 variant, whose stripped range is filled from its level sets) is not
// restated.
#pragma once

#include <algorithm>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <utility>
#include <vector>

#include "analysis.hpp"

namespace gb300 {

constexpr int kEtreeEmpty = -1;

// Indexed binary heap (the reference's lljbash::Heap): entries are known by an index
// (their position in the caller's array), ordered by `cmp` (< 0: first) with ties broken
// by the smaller index.  pop() retires the top's index and gives it to the entry holding
// the highest index, mirroring the caller moving its last element into the freed slot.
template <class Cmp>
class IndexedHeap {
public:
    explicit IndexedHeap(Cmp cmp) : cmp_(cmp), key_(1), idx_(1) {}
    void push(int key) {
        ++size_;
        key_.push_back(key);
        idx_.push_back(size_ - 1);
        loc_.push_back(size_);
        up(size_);
    }
    void pop() {
        const int i = loc_[static_cast<size_t>(size_ - 1)];
        idx_[static_cast<size_t>(i)] = idx_[1];
        loc_[static_cast<size_t>(idx_[static_cast<size_t>(i)])] = i;
        idx_[1] = idx_[static_cast<size_t>(size_)];
        loc_[static_cast<size_t>(idx_[1])] = 1;
        key_[1] = key_[static_cast<size_t>(size_)];
        --size_;
        key_.pop_back();
        idx_.pop_back();
        loc_.pop_back();
        down(1);
    }
    void modify(int index, int key) {
        const int i = loc_[static_cast<size_t>(index)];
        const bool decrease = cmp_(key, key_[static_cast<size_t>(i)]) < 0;
        key_[static_cast<size_t>(i)] = key;
        if (decrease) {
            up(i);
        } else {
            down(i);
        }
    }
    int top_index() const { return idx_[1]; }

private:
    bool before(int i, int j) const {
        const int c = cmp_(key_[static_cast<size_t>(i)], key_[static_cast<size_t>(j)]);
        return c < 0 || (c == 0 && idx_[static_cast<size_t>(i)] < idx_[static_cast<size_t>(j)]);
    }
    void swap_slots(int i, int j) {
        std::swap(key_[static_cast<size_t>(i)], key_[static_cast<size_t>(j)]);
        std::swap(idx_[static_cast<size_t>(i)], idx_[static_cast<size_t>(j)]);
        loc_[static_cast<size_t>(idx_[static_cast<size_t>(i)])] = i;
        loc_[static_cast<size_t>(idx_[static_cast<size_t>(j)])] = j;
    }
    void up(int i) {
        while (i > 1 && before(i, i / 2)) {
            swap_slots(i, i / 2);
            i /= 2;
        }
    }
    void down(int i) {
        while (2 * i <= size_) {
            int j = 2 * i;
            if (j + 1 <= size_ && before(j + 1, j)) ++j;
            if (!before(j, i)) break;
            swap_slots(i, j);
            i = j;
        }
    }
    Cmp cmp_;
    int size_ = 0;
    std::vector<int> key_, idx_, loc_;
};

struct TreeScheduleResult {
    int nproc = 0;
    std::vector<int> parent;          // [n] etree parent (roots: n)
    std::vector<int> subtree_size;    // [n + 1] rows of each vertex's subtree (index n: the virtual root)
    std::vector<int> subtree_weight;  // [n + 1] summed row weights of each subtree
    std::vector<int> part_ptr;        // [nproc + 2]: worker w owns partitions[part_ptr[w], part_ptr[w+1])
    std::vector<int> partitions;      // [n] rows: workers' subtrees, then the queue part
    std::vector<int> task_queue;      // [ntasks + 1] (granularity > 1): queue tasks' ranges in partitions
    int ntasks = 0;
};

// weight(v) of a row: row_end(v) - row_begin(v) + base (the reference's NNZLoadBalancer).
struct RowWeights {
    const int* begin;
    const int* end;
    int bias_begin;  // begin[v] + bias_begin
    int base;
    int operator()(int v) const { return end[v] - (begin[v] + bias_begin) + base; }
};

inline TreeScheduleResult tree_schedule(int n, const DagView& g, int nproc, int granularity, double relax,
                                        const RowWeights& weight) {
    if (nproc < 1) throw std::runtime_error("tree schedule needs at least one worker");
    TreeScheduleResult out;
    out.nproc = nproc;
    const bool asc = g.lower;
    const int vb = asc ? 0 : n - 1, ve = asc ? n : -1, vd = asc ? 1 : -1;
    // elimination tree with path compression (src/subtree.hpp:35-68)
    std::vector<int> parent(static_cast<size_t>(n)), root(static_cast<size_t>(n) + 1);
    for (int v = vb; v != ve; v += vd) parent[static_cast<size_t>(v)] = root[static_cast<size_t>(v)] = n;
    for (int j = vb; j != ve; j += vd) {
        for (int k = g.begin(j); k < g.end(j); ++k) {
            int i = g.ci[k];
            while (root[static_cast<size_t>(i)] != n) {
                const int t = root[static_cast<size_t>(i)];
                root[static_cast<size_t>(i)] = j;
                i = t;
            }
            if (i != j) {
                root[static_cast<size_t>(i)] = j;
                parent[static_cast<size_t>(i)] = j;
            }
        }
    }
    // first child / next sibling (src/subtree.hpp:70-86)
    std::vector<int> child(static_cast<size_t>(n) + 1, kEtreeEmpty), sibling(static_cast<size_t>(n) + 1, kEtreeEmpty);
    for (int v = n - 1; v >= 0; --v) {
        const int p = parent[static_cast<size_t>(v)];
        sibling[static_cast<size_t>(v)] = child[static_cast<size_t>(p)];
        child[static_cast<size_t>(p)] = v;
    }
    // subtree sizes and weights (src/subtree.hpp:88-101)
    std::vector<int> size(static_cast<size_t>(n) + 1), wt(static_cast<size_t>(n) + 1);
    for (int v = vb; v != ve; v += vd) {
        wt[static_cast<size_t>(v)] = weight(v);
        size[static_cast<size_t>(v)] = 1;
    }
    wt[static_cast<size_t>(n)] = 0;
    size[static_cast<size_t>(n)] = 0;
    for (int v = vb; v != ve; v += vd) {
        const int p = parent[static_cast<size_t>(v)];
        wt[static_cast<size_t>(p)] += wt[static_cast<size_t>(v)];
        size[static_cast<size_t>(p)] += size[static_cast<size_t>(v)];
    }
    // division into independent subtrees (src/subtree.hpp:103-227)
    std::vector<int> sub(static_cast<size_t>(std::max(n, 1)));
    int nsub = 0;
    if (nproc > 1) {
        int ngen = 1, ichain = n, top = 0;
        int max_w = wt[static_cast<size_t>(n)], sum_w = wt[static_cast<size_t>(n)];
        sub[0] = n;
        auto cmp = [&wt](int a, int b) {
            return wt[static_cast<size_t>(a)] > wt[static_cast<size_t>(b)] ? -1 : (wt[static_cast<size_t>(a)] < wt[static_cast<size_t>(b)] ? 1 : 0);
        };
        IndexedHeap<decltype(cmp)> heap(cmp);
        heap.push(sub[0]);
        while (ngen > 0 && max_w * nproc * relax > sum_w) {
            int t = sub[static_cast<size_t>(top)], f = child[static_cast<size_t>(t)];
            while (f != kEtreeEmpty && sibling[static_cast<size_t>(f)] == kEtreeEmpty) {
                t = f;
                f = child[static_cast<size_t>(t)];
            }
            if (f == kEtreeEmpty) {  // an unbranched chain: set aside
                sub[static_cast<size_t>(--ichain)] = sub[static_cast<size_t>(top)];
                sub[static_cast<size_t>(top)] = sub[static_cast<size_t>(--ngen)];
                heap.pop();
            } else {
                sum_w -= wt[static_cast<size_t>(sub[static_cast<size_t>(top)])];
                int ch = child[static_cast<size_t>(t)];
                sub[static_cast<size_t>(top)] = ch;
                heap.modify(top, ch);
                sum_w += wt[static_cast<size_t>(ch)];
                while (sibling[static_cast<size_t>(ch)] >= 0) {
                    ch = sibling[static_cast<size_t>(ch)];
                    sub[static_cast<size_t>(ngen++)] = ch;
                    heap.push(ch);
                    sum_w += wt[static_cast<size_t>(ch)];
                }
            }
            if (ngen > 0) {
                top = heap.top_index();
                max_w = wt[static_cast<size_t>(sub[static_cast<size_t>(top)])];
            }
        }
        if (ngen > 0) {
            std::swap(sub[static_cast<size_t>(ngen - 1)], sub[static_cast<size_t>(top)]);
            std::sort(sub.begin(), sub.begin() + (ngen - 1),
                      [&wt](int x, int y) { return wt[static_cast<size_t>(x)] < wt[static_cast<size_t>(y)]; });
        }
        nsub = static_cast<int>(std::copy(sub.begin() + ichain, sub.begin() + n, sub.begin() + ngen) - sub.begin());
        while (nsub >= nproc && wt[static_cast<size_t>(sub[static_cast<size_t>(nsub - 1)])] * nproc * relax > sum_w) {
            const int last = sub[static_cast<size_t>(nsub - 1)];
            int ch = child[static_cast<size_t>(last)];
            int second = wt[static_cast<size_t>(sub[static_cast<size_t>(nsub - 2)])];
            int th = static_cast<int>(sum_w / relax / nproc);
            th = second < th ? second : th;
            sum_w -= wt[static_cast<size_t>(last)];
            while (ch != kEtreeEmpty && wt[static_cast<size_t>(ch)] > th) ch = child[static_cast<size_t>(ch)];
            if (ch == kEtreeEmpty) {
                --nsub;
            } else {
                const int nw = wt[static_cast<size_t>(ch)];
                sum_w += nw;
                int pos = nsub - 2;
                for (; pos >= 0 && wt[static_cast<size_t>(sub[static_cast<size_t>(pos)])] > nw; --pos)
                    sub[static_cast<size_t>(pos + 1)] = sub[static_cast<size_t>(pos)];
                sub[static_cast<size_t>(pos + 1)] = ch;
            }
        }
        if (nsub < nproc) nsub = 0;  // fall back to the queue
    }
    // assignment: largest subtree first to the least-loaded worker (src/subtree.hpp:229-266)
    std::vector<int> assign(static_cast<size_t>(n), kEtreeEmpty);
    std::vector<int> load(static_cast<size_t>(nproc), 0);
    out.part_ptr.assign(static_cast<size_t>(nproc) + 2, 0);
    for (int i = nsub - 1; i >= 0; --i) {
        const int t = sub[static_cast<size_t>(i)];
        int best = 0, m = std::numeric_limits<int>::max();
        for (int w = 0; w < nproc; ++w)
            if (m > load[static_cast<size_t>(w)]) {
                m = load[static_cast<size_t>(w)];
                best = w;
            }
        assign[static_cast<size_t>(t)] = best;
        load[static_cast<size_t>(best)] += wt[static_cast<size_t>(t)];
        out.part_ptr[static_cast<size_t>(best)] += size[static_cast<size_t>(t)];
    }
    for (int i = 0, pre = 0; i <= nproc; ++i) {
        const int tmp = out.part_ptr[static_cast<size_t>(i)];
        out.part_ptr[static_cast<size_t>(i)] = pre;
        pre += tmp;
    }
    out.part_ptr[static_cast<size_t>(nproc) + 1] += out.part_ptr[static_cast<size_t>(nproc)];
    // partitions in post order (src/subtree.hpp:268-361): first the rows outside every
    // subtree (the queue part), then each subtree into its worker's range
    std::vector<int>& part = out.partitions;
    part.assign(static_cast<size_t>(n), 0);
    {
        auto next_free = [&](int c) {
            while (c != kEtreeEmpty && assign[static_cast<size_t>(c)] != kEtreeEmpty) c = sibling[static_cast<size_t>(c)];
            return c;
        };
        for (int k = out.part_ptr[static_cast<size_t>(nproc) + 1], cur = n; k < n;) {
            for (int f = next_free(child[static_cast<size_t>(cur)]); f != kEtreeEmpty; f = next_free(child[static_cast<size_t>(cur)]))
                cur = f;
            part[static_cast<size_t>(k++)] = cur;
            int nx;
            for (nx = next_free(sibling[static_cast<size_t>(cur)]); nx == kEtreeEmpty && k < n;
                 nx = next_free(sibling[static_cast<size_t>(cur)])) {
                cur = parent[static_cast<size_t>(cur)];
                part[static_cast<size_t>(k++)] = cur;
            }
            cur = nx;
        }
        std::vector<int> fill(out.part_ptr.begin(), out.part_ptr.begin() + nproc);
        for (int i = 0; i < nsub; ++i) {
            const int t = sub[static_cast<size_t>(nsub - 1 - i)];
            const int w = assign[static_cast<size_t>(t)];
            int k = fill[static_cast<size_t>(w)];
            const int end = k + size[static_cast<size_t>(t)];
            fill[static_cast<size_t>(w)] = end;
            for (int cur = t; k < end;) {
                for (int f = child[static_cast<size_t>(cur)]; f != kEtreeEmpty; f = child[static_cast<size_t>(f)]) cur = f;
                part[static_cast<size_t>(k++)] = cur;
                int nx;
                for (nx = sibling[static_cast<size_t>(cur)]; nx == kEtreeEmpty && k < end; nx = sibling[static_cast<size_t>(cur)]) {
                    cur = parent[static_cast<size_t>(cur)];
                    part[static_cast<size_t>(k++)] = cur;
                }
                cur = nx;
            }
        }
    }
    // each worker's rows (and the empty stripped range) sorted in processing order
    for (int i = 0; i < nproc + 1; ++i) {
        auto b = part.begin() + out.part_ptr[static_cast<size_t>(i)];
        auto e = part.begin() + out.part_ptr[static_cast<size_t>(i) + 1];
        if (asc) {
            std::sort(b, e);
        } else {
            std::sort(b, e, std::greater<int>());
        }
    }
    out.parent = parent;
    out.subtree_size = size;
    out.subtree_weight = wt;
    if (granularity == 1) return out;
    // queue: supernodes of etree-consecutive rows in post order (src/subtree.hpp:363-403)
    const int qbegin = out.part_ptr[static_cast<size_t>(nproc)];
    std::vector<int> etree(parent), col2sup(static_cast<size_t>(n)), sup2col(static_cast<size_t>(n) + 1);
    {
        std::vector<int>& inv = sup2col;
        std::vector<int>& tmp = col2sup;
        for (int j = qbegin; j < n; ++j) {
            const int p = part[static_cast<size_t>(j)];
            tmp[static_cast<size_t>(j)] = etree[static_cast<size_t>(p)];
            inv[static_cast<size_t>(p)] = j;
        }
        inv[static_cast<size_t>(n)] = n;
        for (int j = qbegin; j < n; ++j) etree[static_cast<size_t>(j)] = inv[static_cast<size_t>(tmp[static_cast<size_t>(j)])];
    }
    std::fill(col2sup.begin(), col2sup.end(), kEtreeEmpty);
    int nsuper = 0;
    sup2col[0] = qbegin;
    for (int j = qbegin; j < n;) {
        int par = etree[static_cast<size_t>(j)];
        const int first = j;
        while (par != n && par - first < granularity) {
            j = par;
            par = etree[static_cast<size_t>(j)];
        }
        ++j;
        for (int k = first; k < j; ++k) col2sup[static_cast<size_t>(part[static_cast<size_t>(k)])] = nsuper;
        sup2col[static_cast<size_t>(++nsuper)] = j;
    }
    // weighted critical-path priority (src/subtree.hpp:405-440)
    std::vector<int> swt(static_cast<size_t>(nsuper)), level(static_cast<size_t>(nsuper));
    for (int i = 0; i < nsuper; ++i) {
        int l = 0;
        for (int j = sup2col[static_cast<size_t>(i)]; j < sup2col[static_cast<size_t>(i) + 1]; ++j) l += weight(j);
        swt[static_cast<size_t>(i)] = l;
        level[static_cast<size_t>(i)] = nsuper - l;
    }
    for (int i = nsuper - 1; i >= 0; --i) {
        const int l = level[static_cast<size_t>(i)];
        for (int v = sup2col[static_cast<size_t>(i)]; v < sup2col[static_cast<size_t>(i) + 1]; ++v) {
            const int j = part[static_cast<size_t>(v)];
            for (int k = g.begin(j); k < g.end(j); ++k) {
                const int ii = col2sup[static_cast<size_t>(g.ci[k])];
                if (ii != kEtreeEmpty && ii != i) {
                    const int ll = l - swt[static_cast<size_t>(ii)];
                    if (level[static_cast<size_t>(ii)] > ll) level[static_cast<size_t>(ii)] = ll;
                }
            }
        }
    }
    std::vector<int> perm(static_cast<size_t>(nsuper));
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(),
              [&level](int x, int y) { return level[static_cast<size_t>(x)] < level[static_cast<size_t>(y)]; });
    // queue tasks in priority order (src/subtree.hpp:442-453)
    out.task_queue.assign(static_cast<size_t>(nsuper) + 1, 0);
    std::vector<int> tmp(part);
    int t = qbegin;
    for (int i = 0; i < nsuper; ++i) {
        const int s = perm[static_cast<size_t>(i)];
        out.task_queue[static_cast<size_t>(i)] = t;
        for (int v = sup2col[static_cast<size_t>(s)]; v < sup2col[static_cast<size_t>(s) + 1]; ++v)
            tmp[static_cast<size_t>(t++)] = part[static_cast<size_t>(v)];
    }
    out.task_queue[static_cast<size_t>(nsuper)] = n;
    std::copy(tmp.begin() + qbegin, tmp.end(), part.begin() + qbegin);
    out.ntasks = nsuper;
    return out;
}

}  // namespace gb300
