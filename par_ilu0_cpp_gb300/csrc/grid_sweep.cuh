// Structured-grid triangular substitution ("wavefront lanes").
//
// For factors whose strict-lower part couples row r = i + nx j + nx ny k only to rows
// r - 1 (i > 0), r - nx (j > 0) and r - nx ny (k > 0) — a 7-point (3-D) or 5-point
// (2-D, ny = 1) stencil in natural order, ILU(0) — and whose strict-upper part is the
// mirror image, the sweeps run on a fixed schedule instead of level sets:
//
// * a lane owns E consecutive i of one z-line (i, j, *) and walks it in k, so the
//   z-dependency (i, j, k -/+ 1) is the lane's own previous result (registers);
// * lane l works on k = s - l at step s, so the x-dependency of its first element,
//   computed by lane l - 1 one step earlier, arrives by a warp shuffle; the i-chunks of
//   32 E lanes form nic warps per line, lane 0 / 31 taking the x-neighbour from the
//   neighbouring chunk's warp 31 steps ahead (shared memory);
// * the warp of line j takes the y-dependency from the warp of line j - 1 at the same
//   step, through a small ring in shared memory.
//
// A CTA solves one tile: up to jb lines (nic warps each) over the planes [k0, k1).
// Tiles are taken by tickets in dependency order (diagonals over the tile grid); a tile
// reads the values it needs from its predecessor tiles (line j0 - 1 and plane k0 - 1)
// in global memory, polled while they hold the sentinel.  No co-residency is assumed:
// every wait is for a smaller ticket (another tile) or, inside the CTA, for an event of
// smaller rank (step + 33 chunk + line), and every wait is bounded (WaitBudget).
//
// Vectors are in the sweep layout (GridLayout): position ((w nz + k + l) 32 + l) E + e
// for element i = 32 E c + E l + e of line j, warp-line w = j nic + c.  At each step a
// warp's 32 lanes touch one contiguous row of 32 E entries, so every load and store of
// the sweep is coalesced; the solver gathers the right-hand side into this layout and
// scatters the solution back (grid_gather_kernel / grid_scatter_kernel).
//
// Each row's operations are those of the reference's substitute_row_L / _U
// (src/ilu_solver.cpp:687-696, 719-729): the z term, then the y term, then the x term
// (ascending columns for L; descending for U), then the division by u_ii (FP64) or the
// product with the rounded reciprocal (FP32, as the other FP32 kernels).  A missing
// neighbour at the grid's boundary contributes fma(-0, 0, acc) == acc exactly, so
// results are bit-identical to the level-ordered and block-local kernels.
#pragma once

#include "common.cuh"
#include "ilu_kernels.cuh"

namespace gb300 {

constexpr int kGridRingY = 8;    // steps of a warp's outputs kept for the next line's warp
constexpr int kGridRingX = 64;   // steps of a warp's edge-lane outputs kept for the next chunk's warp
constexpr int kGridMaxWarps = 32;

struct GridLayout {
    int nx = 0, ny = 0, nz = 0;
    int E = 1;      // elements per lane (consecutive i)
    int nic = 1;    // warps per line: ceil(nx / (32 E))
    long long len = 0;  // layout length: (ny nic nz + 31) 32 E
    __host__ __device__ long long pos(int i, int j, int k) const {
        const int c = i / (32 * E);
        const int r = i - c * 32 * E;
        const int l = r / E;
        const int e = r - l * E;
        const long long w = static_cast<long long>(j) * nic + c;
        return ((w * nz + k + l) * 32 + l) * E + e;
    }
};

template <class T>
struct GridTri {
    GridLayout g;
    int jb = 1, kc = 1;   // tile: lines, planes
    int ntile = 0;
    const int2* tiles = nullptr;  // [ntile] (tile line index, tile plane index) in ticket order
    const T* cz = nullptr;  // coefficient of the z neighbour (r -/+ nx ny), 0 where absent
    const T* cy = nullptr;  // of the y neighbour (r -/+ nx)
    const T* cx = nullptr;  // of the x neighbour (r -/+ 1)
    const T* d = nullptr;   // upper only: u_ii (FP64) or RN(1 / u_ii) (FP32)
};

// Coalesced E-wide load / store of a lane's elements (E consecutive entries).
template <class T, int E>
__device__ __forceinline__ void grid_load(const T* p, T (&v)[E]) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = p[e];
}
template <class T, int E>
__device__ __forceinline__ void grid_store_relaxed(T* p, const T (&v)[E], int nvalid) {
#pragma unroll
    for (int e = 0; e < E; ++e)
        if (e < nvalid) st_relaxed(p + e, v[e]);
}

__device__ __forceinline__ int ld_volatile_int(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Waits until the shared progress word *p reaches `target` (bounded); `cache` holds the
// last value seen so that a producer far ahead costs no load.  Returns false on timeout.
__device__ __forceinline__ bool grid_wait_progress(const int* p, int target, int& cache, int* status) {
    if (cache >= target) return true;
    cache = ld_volatile_int(p);
    if (cache >= target) {
        __threadfence_block();
        return true;
    }
    WaitBudget wb;
    while (!wb.expired(status)) {
        cache = ld_volatile_int(p);
        if (cache >= target) {
            __threadfence_block();
            return true;
        }
    }
    atomicExch(status + kStatusTimeout, 1);
    return false;
}

// One lane's solve of its E elements at one step.  lower: e ascending, x-neighbour of
// element 0 = xin (the element before it); upper: e descending, x-neighbour of element
// E - 1 = xin.  Elements e >= nvalid lie beyond the grid (i >= nx) and are set to 0, so
// that a valid element next to them sees an exact zero neighbour.
template <class T, bool UPPER, int E>
__device__ __forceinline__ void grid_row_ops(const T (&b)[E], const T (&cz)[E], const T (&cy)[E], const T (&cx)[E],
                                             const T (&d)[E], const T (&z)[E], const T (&y)[E], T xin, int nvalid,
                                             T (&x)[E]) {
    if constexpr (!UPPER) {
        T xl = xin;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            T acc = b[e];
            acc = fma(-cz[e], z[e], acc);
            acc = fma(-cy[e], y[e], acc);
            acc = fma(-cx[e], xl, acc);
            x[e] = e < nvalid ? Sentinel<T>::canon(acc) : T(0);
            xl = x[e];
        }
    } else {
        T xr = xin;
#pragma unroll
        for (int e = E - 1; e >= 0; --e) {
            T acc = b[e];
            acc = fma(-cz[e], z[e], acc);
            acc = fma(-cy[e], y[e], acc);
            acc = fma(-cx[e], xr, acc);
            // FP64: the reference's division; FP32 (mixed path): d holds 1 / u_ii
            const T r = sizeof(T) == 8 ? acc / d[e] : acc * d[e];
            x[e] = e < nvalid ? Sentinel<T>::canon(r) : T(0);
            xr = x[e];
        }
    }
}

// The operands of one step of a lane (right-hand side and coefficients), loaded
// kGridPrefetch<T> steps before use (FP64 steps are longer, and two steps of FP64
// operands already take the registers of four FP32 ones).
template <class T>
constexpr int kGridPrefetch = sizeof(T) == 8 ? 2 : 4;

template <class T, int E>
struct GridOps {
    T b[E], cz[E], cy[E], cx[E], d[E];
};

template <class T, bool UPPER, int E>
__device__ __forceinline__ void grid_load_ops(const GridTri<T>& P, const T* in, long long p, bool ok, GridOps<T, E>& o) {
    if (ok) {
        grid_load<T, E>(in + p, o.b);
        grid_load<T, E>(P.cz + p, o.cz);
        grid_load<T, E>(P.cy + p, o.cy);
        grid_load<T, E>(P.cx + p, o.cx);
        if constexpr (UPPER) grid_load<T, E>(P.d + p, o.d);
    }
    if constexpr (!UPPER) {
#pragma unroll
        for (int e = 0; e < E; ++e) o.d[e] = T(1);
    }
}

// Solves one tile.  Shared memory: yring [nw][kGridRingY][32 E], xring [nw][kGridRingX],
// prog [nw] (steps completed per warp, reset to 0 by the caller before the tile).
template <class T, bool UPPER, int E>
__device__ __forceinline__ void grid_tile(const GridTri<T>& P, int jt, int kt, const T* in, T* out, T* yring,
                                          T* xring, int* prog, int* status) {
    const GridLayout& G = P.g;
    const int lane = threadIdx.x & 31;
    const int wi = threadIdx.x >> 5;
    const int nic = G.nic;
    const int cp = wi % nic;  // i-chunk in processing order
    const int jl = wi / nic;  // line in processing order
    const int j0 = jt * P.jb;
    const int j1 = min(G.ny, j0 + P.jb);
    const int k0 = kt * P.kc;
    const int k1 = min(G.nz, k0 + P.kc);
    const int j = UPPER ? j1 - 1 - jl : j0 + jl;
    if (UPPER ? j < j0 : j >= j1) return;  // no line for this warp in a short tile
    const int c = UPPER ? nic - 1 - cp : cp;  // i-chunk in grid coordinates
    const int i0 = c * 32 * E + lane * E;     // first element of the lane
    const int nvalid = max(0, min(E, G.nx - i0));
    const int Q = (k1 - k0) + 31;
    constexpr long long kRow = 32LL * E;
    const long long w = static_cast<long long>(j) * nic + c;
    const long long ystep = static_cast<long long>(nic) * G.nz * kRow;  // position offset of the next line
    const bool y_local = jl > 0;
    const bool y_global = !y_local && (UPPER ? j + 1 < G.ny : j > 0);
    const bool z_global = UPPER ? k1 < G.nz : k0 > 0;
    const bool has_ycons = UPPER ? (j - 1 >= j0) : (j + 1 < j1);
    const bool has_xprod = cp > 0;
    const bool has_xcons = cp + 1 < nic;
    const bool right_edge = UPPER && i0 + nvalid >= G.nx;  // upper: no x-neighbour beyond the grid
    const int edge_lane = UPPER ? 31 : 0;  // lane taking the x-neighbour from the previous chunk's warp
    const int give_lane = UPPER ? 0 : 31;  // lane whose value the next chunk's warp takes
    T* my_yring = yring + static_cast<size_t>(wi) * kGridRingY * kRow;
    const T* prod_yring = yring + static_cast<size_t>(wi - nic) * kGridRingY * kRow;
    T* my_xring = xring + static_cast<size_t>(wi) * kGridRingX;
    const T* prod_xring = xring + static_cast<size_t>(wi - 1) * kGridRingX;
    auto step_of = [&](int q) { return UPPER ? (k1 - 1 + 31) - q : k0 + q; };
    auto pos_of = [&](int s) { return ((w * G.nz + s) * 32 + lane) * E; };
    auto active = [&](int s) { return nvalid > 0 && s - lane >= k0 && s - lane < k1; };
    // stream the warp's rows of the tile into L2 (contiguous: rows w nz + [k0, k1 + 31))
    {
        const long long r0 = ((w * G.nz + k0) * 32) * E;
        const long long bytes = static_cast<long long>(Q) * kRow * static_cast<long long>(sizeof(T));
        prefetch_l2_range(in + r0, bytes & ~15ll, lane);
        prefetch_l2_range(P.cz + r0, bytes & ~15ll, lane);
        prefetch_l2_range(P.cy + r0, bytes & ~15ll, lane);
        prefetch_l2_range(P.cx + r0, bytes & ~15ll, lane);
        if (UPPER) prefetch_l2_range(P.d + r0, bytes & ~15ll, lane);
    }
    int cache_y = 0, cache_x = 0, cache_yc = 0, cache_xc = 0;
    T z[E];
#pragma unroll
    for (int e = 0; e < E; ++e) z[e] = T(0);
    T edge_prev = T(0);  // this lane's x-neighbour-facing value of the previous step
    GridOps<T, E> ops[kGridPrefetch<T>];
#pragma unroll
    for (int u = 0; u < kGridPrefetch<T>; ++u) {
        const int s = step_of(u);
        grid_load_ops<T, UPPER, E>(P, in, pos_of(s), u < Q && active(s), ops[u]);
    }
    bool failed = false;
    for (int q = 0; q < Q && !failed; ++q) {
        const int s = step_of(q);
        const int k = s - lane;
        const bool act = active(s);
        const long long p0 = pos_of(s);
        const GridOps<T, E> cur = ops[0];
#pragma unroll
        for (int u = 0; u + 1 < kGridPrefetch<T>; ++u) ops[u] = ops[u + 1];
        {
            const int qn = q + kGridPrefetch<T>;
            const int sn = step_of(qn);
            grid_load_ops<T, UPPER, E>(P, in, pos_of(sn), qn < Q && active(sn), ops[kGridPrefetch<T> - 1]);
        }
        // x-neighbour: the adjacent lane's value of the previous step
        T xin = UPPER ? __shfl_down_sync(0xffffffffu, edge_prev, 1) : __shfl_up_sync(0xffffffffu, edge_prev, 1);
        if (lane == edge_lane) {
            xin = T(0);
            if (has_xprod && act) {
                if (!grid_wait_progress(prog + wi - 1, q + 32, cache_x, status)) failed = true;
                xin = prod_xring[(q + 31) % kGridRingX];
            }
        }
        if (right_edge) xin = T(0);
        T y[E];
#pragma unroll
        for (int e = 0; e < E; ++e) y[e] = T(0);
        if (y_local) {
            if (!grid_wait_progress(prog + wi - nic, q + 1, cache_y, status)) failed = true;
            if (act) {
                const T* src = prod_yring + static_cast<size_t>(q % kGridRingY) * kRow + lane * E;
#pragma unroll
                for (int e = 0; e < E; ++e) y[e] = src[e];
            }
        } else if (y_global && act) {
            const T* src = out + (UPPER ? p0 + ystep : p0 - ystep);
#pragma unroll
            for (int e = 0; e < E; ++e)
                if (e < nvalid) y[e] = wait_value(src + e, status);
        }
        T x[E];
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = T(0);
        if (act) {
            if (z_global && k == (UPPER ? k1 - 1 : k0)) {
                const T* src = out + (UPPER ? p0 + kRow : p0 - kRow);
#pragma unroll
                for (int e = 0; e < E; ++e)
                    if (e < nvalid) z[e] = wait_value(src + e, status);
            }
            grid_row_ops<T, UPPER, E>(cur.b, cur.cz, cur.cy, cur.cx, cur.d, z, y, xin, nvalid, x);
            grid_store_relaxed<T, E>(out + p0, x, nvalid);
#pragma unroll
            for (int e = 0; e < E; ++e) z[e] = x[e];
            edge_prev = UPPER ? x[0] : x[E - 1];
        }
        // hand the step's results to the next line's and the next chunk's warps
        if (has_ycons) {
            if (!grid_wait_progress(prog + wi + nic, q - kGridRingY + 1, cache_yc, status)) failed = true;
            T* dst = my_yring + static_cast<size_t>(q % kGridRingY) * kRow + lane * E;
#pragma unroll
            for (int e = 0; e < E; ++e) dst[e] = x[e];
        }
        if (has_xcons) {
            if (!grid_wait_progress(prog + wi + 1, q - kGridRingX - 30, cache_xc, status)) failed = true;
            if (lane == give_lane) my_xring[q % kGridRingX] = edge_prev;
        }
        failed = __any_sync(0xffffffffu, failed);
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            *reinterpret_cast<volatile int*>(prog + wi) = failed ? (1 << 30) : q + 1;
        }
    }
}

// Forward (UPPER = false): out = L^{-1} in; backward (UPPER = true): out = U^{-1} in.
// in / out in the sweep layout; out holds the sentinel at every position on entry.
// Dynamic shared memory: nw (kGridRingY 32 E + kGridRingX) sizeof(T) + nw ints.
template <class T, bool UPPER, int E>
__global__ void __launch_bounds__(kGridMaxWarps * kWarp, 1)
    sptrsv_grid_kernel(GridTri<T> P, const T* in, T* out, unsigned* counter, int* status, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char grid_smem[];
    const int nw = blockDim.x >> 5;
    T* yring = reinterpret_cast<T*>(grid_smem);
    T* xring = yring + static_cast<size_t>(nw) * kGridRingY * 32 * E;
    int* prog = reinterpret_cast<int*>(xring + static_cast<size_t>(nw) * kGridRingX);
    __shared__ int s_ticket;
    for (int t = draw_block_ticket(counter, P.ntile, &s_ticket); t < P.ntile;
         t = draw_block_ticket(counter, P.ntile, &s_ticket)) {
        const int2 tile = P.tiles[t];
        if (threadIdx.x < nw) prog[threadIdx.x] = 0;
        __syncthreads();
        grid_tile<T, UPPER, E>(P, tile.x, tile.y, in, out, yring, xring, prog, status);
    }
}

// Natural order -> sweep layout: lay[pos[r]] = in[r] (* scale, which is also written
// back to in[r]: GMRES normalises its Krylov vector in this pass); reset[pos[r]] = the
// sentinel (the forward sweep's output).  One thread per natural row.
template <class T>
__global__ void grid_gather_kernel(int n, const long long* __restrict__ pos, T* in, const double* scale, T* lay,
                                   T* reset, const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    const bool scaled = scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<long long>(gridDim.x) * blockDim.x) {
        T v = in[r];
        if (scaled) {
            v = v * sc;
            in[r] = v;
        }
        const long long p = pos[r];
        lay[p] = v;
        if (reset) reset[p] = Sentinel<T>::value();
    }
}

// Sweep layout -> natural order: out[r] = lay[pos[r]], and lay[pos[r]] reset to the
// sentinel (the backward sweep's output, for the next application).
template <class T>
__global__ void grid_scatter_kernel(int n, const long long* __restrict__ pos, T* lay, T* out, const int* gate,
                                    int step) {
    if (gate_closed(gate, step)) return;
    for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p = pos[r];
        out[r] = lay[p];
        lay[p] = Sentinel<T>::value();
    }
}

// Coefficient gather of a structured factor: dst[p] = lu[src[p]] (0 where src < 0);
// recip: dst[p] = RN(1 / lu[src[p]]) computed in FP64 (FP32 upper diagonal).
template <class T>
__global__ void grid_coef_kernel(long long len, const int* __restrict__ src, const double* __restrict__ lu, T* dst,
                                 bool recip) {
    for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < len;
         p += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int s = src[p];
        double v = s >= 0 ? lu[s] : 0.0;
        if (recip && s >= 0) v = 1.0 / v;
        dst[p] = static_cast<T>(v);
    }
}

}  // namespace gb300
