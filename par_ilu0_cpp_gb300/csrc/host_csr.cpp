// Host-side CSR utilities of the drop-in library: the CsrMatrix lifecycle, CsrMatVec,
// the MatrixMarket reader, the (unsupported) fill-reducing orderings and the symbolic
// ILU(k) pattern.  Replaces the reference's src/csr_matrix.cpp and src/iluk.cpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <queue>
#include <unordered_map>
#include <utility>
#include <vector>

#include "analysis.hpp"
#include "csr_matrix.h"
#include "iluk.h"
#include "orderings.hpp"

namespace {

// Arrays handed out by SetupCsrMatrix are page-locked (cudaMallocHost) when a CUDA
// device is usable, so that host<->device copies of matrices run at full link speed;
// otherwise 64-byte aligned heap memory.  The registry records which allocator owns
// each pointer so that the matching free is used.
std::mutex g_alloc_mu;
std::unordered_map<void*, bool> g_pinned;  // pointer -> allocated by cudaMallocHost
int g_cuda_usable = -1;

bool cuda_usable() {
    if (g_cuda_usable < 0) {
        int count = 0;
        g_cuda_usable = (cudaGetDeviceCount(&count) == cudaSuccess && count > 0) ? 1 : 0;
        if (!g_cuda_usable) cudaGetLastError();
    }
    return g_cuda_usable == 1;
}

void* host_alloc(size_t bytes) {
    if (bytes == 0) return nullptr;
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    void* p = nullptr;
    if (bytes >= (1u << 16) && cuda_usable() && cudaMallocHost(&p, bytes) == cudaSuccess) {
        g_pinned[p] = true;
        return p;
    }
    cudaGetLastError();
    size_t rounded = (bytes + 63) / 64 * 64;
    if (posix_memalign(&p, 64, rounded) != 0) return nullptr;
    g_pinned[p] = false;
    return p;
}

void host_free(void* p) {
    if (!p) return;
    bool pinned = false;
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        auto it = g_pinned.find(p);
        if (it != g_pinned.end()) {
            pinned = it->second;
            g_pinned.erase(it);
        }
    }
    if (pinned) {
        cudaFreeHost(p);
    } else {
        std::free(p);
    }
}

template <class T>
void realloc_array(T*& arr, long long count) {
    host_free(arr);
    arr = count > 0 ? static_cast<T*>(host_alloc(sizeof(T) * static_cast<size_t>(count))) : nullptr;
}

}  // namespace

// Fill-reducing orderings (orderings.hpp) of the pattern of A + A^T: p[k] = the row
// eliminated k-th, ip its inverse.  Return values as the reference's wrappers
// (src/csr_matrix.cpp:173-225): AMD 0 on success and -1 on failure, ND 1 on success and
// 0 on failure.
namespace {
template <class F>
int run_ordering(const CsrMatrix* mat, int* p, int* ip, F order_fn) {
    if (mat == nullptr || mat->size < 0 || p == nullptr || (mat->size > 0 && mat->row_ptr == nullptr)) return -1;
    const int n = mat->size;
    try {
        gb300::validate_csr(n, mat->row_ptr, mat->col_idx, "ordering input");
        std::vector<int> xadj, adj;
        gb300::symmetric_graph(n, mat->row_ptr, mat->col_idx, xadj, adj);
        const std::vector<int> order = order_fn(n, xadj, adj);
        if (static_cast<int>(order.size()) != n) return -1;
        std::copy(order.begin(), order.end(), p);
        if (ip)
            for (int i = 0; i < n; ++i) ip[p[i]] = i;
    } catch (const std::exception&) {
        return -1;
    }
    return 0;
}
}  // namespace

extern "C" {

const CsrMatrix CSR_MATRIX_DEFAULT{};

void SetupCsrMatrix(CsrMatrix* mat, int size, int max_nnz) {
    mat->size = size;
    mat->max_nnz = max_nnz;
    realloc_array(mat->row_ptr, static_cast<long long>(size) + 1);
    realloc_array(mat->col_idx, max_nnz);
    realloc_array(mat->value, max_nnz);
}

void CopyCsrMatrix(CsrMatrix* dst, const CsrMatrix* src) {
    const int n = src->size;
    const int nnz = GetCsrNonzeros(src);
    SetupCsrMatrix(dst, n, nnz);
    std::memcpy(dst->row_ptr, src->row_ptr, sizeof(int) * (static_cast<size_t>(n) + 1));
    std::memcpy(dst->col_idx, src->col_idx, sizeof(int) * static_cast<size_t>(nnz));
    std::memcpy(dst->value, src->value, sizeof(double) * static_cast<size_t>(nnz));
}

void CopyCsrMatrixValues(CsrMatrix* dst, const CsrMatrix* src) {
    const int nnz = GetCsrNonzeros(src);
    std::memcpy(dst->value, src->value, sizeof(double) * static_cast<size_t>(nnz));
}

void DestroyCsrMatrix(CsrMatrix* mat) { SetupCsrMatrix(mat, -1, 0); }

void CsrMatVec(const CsrMatrix* mat, const double* vec, double* sol) {
    for (int r = 0; r < mat->size; ++r) {
        double s = 0.0;
        for (int p = mat->row_ptr[r]; p < mat->row_ptr[r + 1]; ++p) s += mat->value[p] * vec[mat->col_idx[p]];
        sol[r] = s;
    }
}

// MatrixMarket reader (reference behaviour: src/csr_matrix.cpp:53-159).  Each row is
// sorted by value (descending), rows without a usable diagonal are matched to a column
// by augmenting paths (depth-first, first usable entry first, |a| > 1e-12), rows are
// permuted so that row i holds the entries of the row matched to column i, and each
// row is sorted by column.  Malformed input ends the process, as in the reference.
void ReadCsrMatrixMM1(CsrMatrix* mat, const char* filename) {
    constexpr double kMinDiag = 1e-12;
    std::FILE* fin = std::fopen(filename, "r");
    if (!fin) {
        std::fprintf(stderr, "cannot open file %s\n", filename);
        std::exit(-1);
    }
    char buf[256];
    bool header = true;
    int n = -1, nnz = 0, seen = 0;
    std::vector<std::vector<std::pair<int, double>>> rows;
    std::vector<int> match;  // match[col] = row
    while ((header || seen < nnz) && std::fgets(buf, sizeof(buf), fin)) {
        if (buf[0] == '%') continue;
        if (header) {
            int m = -1;
            if (std::sscanf(buf, "%d%d%d", &n, &m, &nnz) != 3) continue;
            if (m > n) n = m;
            SetupCsrMatrix(mat, n, nnz + n);
            rows.assign(static_cast<size_t>(n), {});
            match.assign(static_cast<size_t>(n), -1);
            header = false;
        } else {
            int i = 0, j = 0;
            double a = 0.0;
            if (std::sscanf(buf, "%d%d%lf", &i, &j, &a) != 3) continue;
            rows[i - 1].emplace_back(j - 1, a);
            if (i == j && std::fabs(a) > kMinDiag) match[i - 1] = i - 1;
            ++seen;
        }
    }
    std::fclose(fin);
    if (seen != nnz) {
        std::puts("nnz number error");
        std::exit(-1);
    }
    for (auto& r : rows) {
        std::sort(r.begin(), r.end(), [](const std::pair<int, double>& x, const std::pair<int, double>& y) {
            return x.second > y.second;
        });
    }
    // Augmenting paths for the rows left unmatched by their own diagonal.  Iterative
    // depth-first search with the same visiting order as a recursive one.
    const std::vector<int> initial(match);
    std::vector<int> visited(static_cast<size_t>(n));
    struct Frame {
        int row;
        size_t next;
    };
    std::vector<Frame> stack;
    std::vector<int> via;  // column taken at each stack level
    for (int i = 0; i < n; ++i) {
        if (initial[i] != -1) continue;
        std::fill(visited.begin(), visited.end(), 0);
        stack.assign(1, Frame{i, 0});
        via.clear();
        bool found = false;
        while (!stack.empty() && !found) {
            Frame& fr = stack.back();
            const auto& r = rows[fr.row];
            bool descended = false;
            while (fr.next < r.size()) {
                const int j = r[fr.next].first;
                const double a = r[fr.next].second;
                ++fr.next;
                if (std::fabs(a) > kMinDiag && !visited[j]) {
                    visited[j] = 1;
                    if (match[j] == -1) {
                        // augment along the stack: level d's row takes column via[d]
                        via.push_back(j);
                        for (size_t d = 0; d < stack.size(); ++d) match[via[d]] = stack[d].row;
                        found = true;
                    } else {
                        via.push_back(j);
                        stack.push_back(Frame{match[j], 0});
                        descended = true;
                    }
                    break;
                }
            }
            if (found) break;
            if (!descended) {
                stack.pop_back();
                if (!via.empty()) via.pop_back();
            }
        }
        if (!found) {
            std::puts("error while matching");
            std::exit(-1);
        }
    }
    int pos = 0;
    for (int i = 0; i < n; ++i) {
        auto& r = rows[match[i]];
        std::sort(r.begin(), r.end());
        mat->row_ptr[i] = pos;
        bool diag = false;
        for (const auto& e : r) {
            mat->col_idx[pos] = e.first;
            mat->value[pos] = e.second;
            ++pos;
            if (e.first == i && std::fabs(e.second) > kMinDiag) diag = true;
        }
        if (!diag) {
            std::puts("error: missing diag");
            std::exit(-1);
        }
    }
    mat->row_ptr[n] = pos;
}

int CsrAmdOrder(const CsrMatrix* mat, int* p, int* ip) {
    return run_ordering(mat, p, ip, gb300::minimum_degree_order);
}

int CsrNdOrder(const CsrMatrix* mat, int* p, int* ip) {
    return run_ordering(mat, p, ip, gb300::nested_dissection_order) == 0 ? 1 : 0;
}

// Symbolic ILU(k) (reference behaviour: src/iluk.cpp:5-54).  Row i starts from A's
// columns at level 0; pivots k < i are taken in ascending column order, including
// fill columns created earlier in the same row; a pivot whose own level is >= lof is
// skipped; for a pivot k every entry (j, lev_kj) of row k from its diagonal onward
// proposes level lev_ik + lev_kj + 1, and an absent column is added when that level is
// <= lof.  A column keeps the first level proposed for it.  Pivots are drawn from a
// min-heap (new fill columns are always larger than the current pivot, so the heap
// order equals the ascending scan), membership is a per-row stamp array, and each
// finished row is stored column-sorted.
int IlukSymbolic(const CsrMatrix* a, int lof, CsrMatrix* f, int* nzmap) {
    const int n = a->size;
    const int nnz = GetCsrNonzeros(a);
    std::vector<long long> frp(static_cast<size_t>(n) + 1, 0);
    std::vector<int> fcol;
    std::vector<int> flev;
    fcol.reserve(static_cast<size_t>(nnz) * (lof > 0 ? 2 : 1));
    flev.reserve(fcol.capacity());
    std::vector<int> stamp(static_cast<size_t>(n), -1);
    std::vector<int> lev(static_cast<size_t>(n), 0);
    std::vector<int> cols;
    std::priority_queue<int, std::vector<int>, std::greater<int>> pivots;
    for (int i = 0; i < n; ++i) {
        cols.clear();
        for (int p = a->row_ptr[i]; p < a->row_ptr[i + 1]; ++p) {
            const int c = a->col_idx[p];
            if (stamp[c] != i) {
                stamp[c] = i;
                lev[c] = 0;
                cols.push_back(c);
                if (c < i) pivots.push(c);
            }
        }
        while (!pivots.empty()) {
            const int k = pivots.top();
            pivots.pop();
            const int lev_ik = lev[k];
            if (lev_ik >= lof) continue;
            const int* kb = fcol.data() + frp[k];
            const int* ke = fcol.data() + frp[k + 1];
            const int* kd = std::lower_bound(kb, ke, k);
            if (kd == ke || *kd != k) continue;
            const int* lk = flev.data() + (kd - fcol.data());
            for (const int* q = kd; q < ke; ++q, ++lk) {
                const int j = *q;
                const int l = lev_ik + *lk + 1;
                if (l <= lof && stamp[j] != i) {
                    stamp[j] = i;
                    lev[j] = l;
                    cols.push_back(j);
                    if (j < i) pivots.push(j);
                }
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int c : cols) {
            fcol.push_back(c);
            flev.push_back(lev[c]);
        }
        frp[i + 1] = static_cast<long long>(fcol.size());
    }
    const long long knnz = frp[n];
    if (knnz > 0x7fffffffLL) {
        std::puts("error: ILU(k) pattern exceeds 2^31 entries");
        return -1;
    }
    SetupCsrMatrix(f, n, static_cast<int>(knnz));
    int apos = 0;
    for (int i = 0; i < n; ++i) {
        f->row_ptr[i] = static_cast<int>(frp[i]);
        for (long long p = frp[i]; p < frp[i + 1]; ++p) {
            f->col_idx[p] = fcol[p];
            if (flev[p] == 0) {
                // level-0 entries take A's values in order (A's rows column-sorted)
                f->value[p] = apos < nnz ? a->value[apos] : 0.0;
                if (nzmap && apos < nnz) nzmap[apos] = static_cast<int>(p);
                ++apos;
            } else {
                f->value[p] = 0.0;
            }
        }
    }
    f->row_ptr[n] = static_cast<int>(knnz);
    if (apos != nnz) {
        std::puts("error");
        return -1;
    }
    return static_cast<int>(knnz);
}

}  // extern "C"
