// Structured-grid triangular substitution: the line pipeline.
//
// For factors whose strict-lower part couples row r = X + nx (Y + ny Z) only to rows
// r - 1 (X > 0), r - nx (Y > 0) and r - nx ny (Z > 0) — a 7-point (3-D) or 5-point (2-D:
// ny = 1, the second offset taken as the plane offset) stencil in natural order, ILU(0) —
// and whose strict-upper part is the mirror image, every row depends on its three
// predecessors along x, y and z.  The sweeps then run on a fixed software pipeline
// instead of level sets:
//
// * in sweep coordinates (x', y', z') — the natural ones for L, mirrored for U — a lane
//   owns one grid line (y', z') and walks it in x', so the x-dependency is the lane's
//   own previous result, in a register;
// * a warp holds wy x wz lines (lane = zz wy + yy) and lane (yy, zz) works on
//   x' = s - (yy + zz) at step s: its y- and z-predecessors at the same x' were computed
//   by lanes (yy - 1, zz) and (yy, zz - 1) one step earlier and arrive by warp shuffles;
// * a CTA holds by x bz warps; a warp's first lanes along y / z take their predecessors
//   from the previous warp's face in shared memory ([nx][wz] / [nx][wy] values per
//   warp, written once per block, value-as-flag: reset to the sentinel with the block);
// * a block's first warps take them from the previous block through `out` in L2,
//   loaded PF steps ahead and polled only while they still hold the sentinel.
//
// The per-step work of a lane is one row: three FMAs (z, y, x terms in the reference's
// order) and, for U, the division by u_ii (FP64) or the product with the rounded
// reciprocal (FP32, as the other FP32 kernels).  The operands of each step (coefficients
// in a packed stream per warp, right-hand side) are loaded PF steps before use.  The
// critical path is nx + ny + nz steps plus the handoffs between warps and blocks,
// against one level per step for the level-set kernels.
//
// Blocks are taken from a ticket counter in dependency order (anti-diagonals of the block
// grid), so a block only waits for blocks of smaller tickets, whose CTAs are running or
// done; inside a block a warp only waits for warps of smaller index along y or z (all
// resident), whose faces never wait on their consumers.  Every wait is bounded.
//
// A missing neighbour at the grid's boundary has coefficient 0 and value 0, and
// fma(-0, 0, acc) == acc exactly, so the results are bit-identical to the level-ordered
// and block-local kernels (src/ilu_solver.cpp:687-696 for L, 719-729 for U).
#pragma once

#include "common.cuh"
#include "ilu_kernels.cuh"

namespace gb300 {

constexpr int kLineMaxWarps = 8;  // compute warps per CTA of the line kernels (plus one halo warp)

struct LineGeom {
    int nx = 0, ny = 0, nz = 0;
    int wy = 1, wz = 32;  // lanes of a warp along y / z (wy * wz == 32)
    int by = 1, bz = 1;   // warps of a CTA along y / z
    int nby = 1, nbz = 1; // blocks along y / z
    int steps = 0;        // steps of a warp: nx + wy + wz - 2
    int nblk = 0;         // nby * nbz
    int cl = 0;           // CTAs per thread-block cluster (consecutive blocks along z), 0: none
    int nbzc = 0;         // clusters along z: ceil(nbz / cl)
    __host__ __device__ int nw() const { return by * bz; }
    // Slot of lane `lane` of warp w of block b at step s in the packed operand stream.
    __host__ __device__ long long slot(int b, int w, int s, int lane) const {
        return ((static_cast<long long>(b) * nw() + w) * steps + s) * 32 + lane;
    }
    __host__ __device__ long long slots() const { return static_cast<long long>(nblk) * nw() * steps * 32; }
};

template <class T>
struct LineTri {
    LineGeom g;
    const int* order = nullptr;  // [nblk] block (iy + nby iz, sweep coordinates) of each ticket;
                                 // with clusters [nby nbzc]: cluster (iy + nby izc) of each ticket
    const T* coef = nullptr;     // [slots][4]: c_z, c_y, c_x, d (d: u_ii FP64 / RN(1 / u_ii) FP32; L: unused)
    unsigned long long* tl = nullptr;  // per-block timeline [nblk][kLineTimeline] (null: off)
};

// Timeline record of one block (nanoseconds of %globaltimer): [0] compute start (faces
// reset, after the CTA barrier), [1] SM id, [2 + w] end of compute warp w (w < nw), [2 +
// nw] end of the halo warp; unused entries 0.
constexpr int kLineTimeline = 12;

__device__ __forceinline__ unsigned sm_id() {
    unsigned r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}
template <class T>
__device__ __forceinline__ void line_stamp_start(const LineTri<T>& P, int blk) {
    if (P.tl != nullptr && threadIdx.x == 0) {
        unsigned long long* r = P.tl + static_cast<long long>(blk) * kLineTimeline;
        r[0] = global_ns();
        r[1] = sm_id();
    }
}
template <class T>
__device__ __forceinline__ void line_stamp_end(const LineTri<T>& P, int blk) {
    if (P.tl != nullptr && (threadIdx.x & 31) == 0)
        P.tl[static_cast<long long>(blk) * kLineTimeline + 2 + (threadIdx.x >> 5)] = global_ns();
}

// ---- asynchronous global -> shared copies (cp.async, per thread) ----
// src_bytes = 0 fills the destination with zeros without reading the source.
__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
                 "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_8(void* smem, const void* gmem, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
                 "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_4(void* smem, const void* gmem, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
                 "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Stores issued only where `on` holds, as predicated instructions (no branch).
__device__ __forceinline__ void st_relaxed_if(bool on, double* p, double v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.relaxed.gpu.global.f64 [%1], %2; }" ::"r"(static_cast<unsigned>(on)),
                 "l"(p), "d"(v));
}
__device__ __forceinline__ void st_relaxed_if(bool on, float* p, float v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.relaxed.gpu.global.f32 [%1], %2; }" ::"r"(static_cast<unsigned>(on)),
                 "l"(p), "f"(v));
}
__device__ __forceinline__ void st_global_if(bool on, double* p, double v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.global.f64 [%1], %2; }" ::"r"(static_cast<unsigned>(on)), "l"(p),
                 "d"(v));
}
__device__ __forceinline__ void st_global_if(bool on, float* p, float v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.global.f32 [%1], %2; }" ::"r"(static_cast<unsigned>(on)), "l"(p),
                 "f"(v));
}
__device__ __forceinline__ void st_shared_if(bool on, double* p, double v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.volatile.shared.f64 [%1], %2; }" ::"r"(static_cast<unsigned>(on)),
                 "r"(static_cast<unsigned>(__cvta_generic_to_shared(p))), "d"(v));
}
__device__ __forceinline__ void st_shared_if(bool on, float* p, float v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.volatile.shared.f32 [%1], %2; }" ::"r"(static_cast<unsigned>(on)),
                 "r"(static_cast<unsigned>(__cvta_generic_to_shared(p))), "f"(v));
}

__device__ __forceinline__ void st_cluster_if(bool on, unsigned addr, double v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.relaxed.cluster.shared::cluster.f64 [%1], %2; }" ::"r"(
                     static_cast<unsigned>(on)),
                 "r"(addr), "d"(v));
}
__device__ __forceinline__ void st_cluster_if(bool on, unsigned addr, float v) {
    asm volatile("{ .reg .pred q; setp.ne.u32 q, %0, 0; @q st.relaxed.cluster.shared::cluster.f32 [%1], %2; }" ::"r"(
                     static_cast<unsigned>(on)),
                 "r"(addr), "f"(v));
}

// Waits (bounded) until the shared-memory value *p is no longer the sentinel; after many
// polls it sleeps between polls (a warp waiting for a block far behind).
template <class T>
__device__ __noinline__ T line_wait_shared(const T* p, int* status) {
    T v = ld_volatile_shared(p);
    WaitBudget wb;
    int polls = 0;
    while (Sentinel<T>::is(v)) {
        if (wb.expired(status)) {
            atomicExch(status + kStatusTimeout, 1);
            return T(0);
        }
        if (++polls > 4096) __nanosleep(256);  // a long wait (a block far behind)
        v = ld_volatile_shared(p);
    }
    return v;
}

// Coefficients of one row in the packed stream (c_z, c_y, c_x, d).
template <class T>
struct alignas(4 * sizeof(T)) LineCoef {
    T cz, cy, cx, d;
};

// Steps of operands in flight per lane (cp.async ring in shared memory).
template <class T>
constexpr int kLineRing = sizeof(T) == 4 ? 16 : 8;

// Shared memory of a CTA: faces (consumer-indexed: slot w holds what warp w reads; faceY
// [nw][nx][wz] when ny > 1, faceZ [nw][nx][wy]), one word holding 0, then the operand
// rings [R][nw * 32] of coefficients and of right-hand side values.
__host__ __device__ inline long long line_face_slot_y(const LineGeom& g) {
    return g.ny > 1 ? static_cast<long long>(g.nx) * g.wz : 0;
}
__host__ __device__ inline long long line_face_slot_z(const LineGeom& g) { return static_cast<long long>(g.nx) * g.wy; }
template <class T>
__host__ __device__ inline long long line_face_len(const LineGeom& g) {
    return static_cast<long long>(g.nw()) * (line_face_slot_y(g) + line_face_slot_z(g));
}
template <class T>
__host__ __device__ inline long long line_ring_offset(const LineGeom& g) {
    return ((line_face_len<T>(g) + 1) * static_cast<long long>(sizeof(T)) + 15) & ~15ll;
}
template <class T>
__host__ __device__ inline long long line_smem_bytes(const LineGeom& g) {
    return line_ring_offset<T>(g) +
           static_cast<long long>(kLineRing<T>) * g.nw() * 32 * (static_cast<long long>(sizeof(LineCoef<T>)) + sizeof(T));
}

// One compute warp's share of block `blk`: wy x wz lines over nx + wy + wz - 2 steps.
// faceY / faceZ: slot w holds the y / z predecessors of warp w's first lanes along y / z,
// written by the previous warp of the CTA or by the halo warp (previous block), or zeros
// at the grid's boundary.
template <class T, bool UPPER>
__device__ __forceinline__ void line_warp(const LineTri<T>& P, int blk, T* in, bool scaled, T sc, T* out, T* faceY,
                                          T* faceZ, const T* zero_word, LineCoef<T>* cring, T* bring,
                                          unsigned fz_remote, int* status) {
    constexpr int R = kLineRing<T>;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int nx = P.g.nx, ny = P.g.ny, nz = P.g.nz;
    const int wy = P.g.wy, wz = P.g.wz, by = P.g.by, bz = P.g.bz;
    const int nw = by * bz;
    const int wyi = w % by, wzi = w / by;
    const int yy = lane % wy, zz = lane / wy;
    const int iy = blk % P.g.nby, iz = blk / P.g.nby;
    const int yq = (iy * by + wyi) * wy + yy;  // sweep coordinates of the lane's line
    const int zq = (iz * bz + wzi) * wz + zz;
    const bool line_ok = yq < ny && zq < nz;
    const int skew = yy + zz;
    const int steps = P.g.steps;
    const long long plane = static_cast<long long>(nx) * ny;
    const long long Y = UPPER ? ny - 1 - yq : yq;
    const long long Z = UPPER ? nz - 1 - zq : zq;
    const int sx = UPPER ? -1 : 1;
    T* const in0 = in + ((UPPER ? nx - 1 : 0) + nx * Y + plane * Z);  // natural row of x' = 0
    T* const out0 = out + ((UPPER ? nx - 1 : 0) + nx * Y + plane * Z);
    const bool y_edge = ny > 1 && yy == 0;
    const bool z_edge = zz == 0;
    const long long fsy = line_face_slot_y(P.g), fsz = line_face_slot_z(P.g);
    const T* fy = faceY + w * fsy + zz;  // stride wz per x'
    const T* fz = faceZ + w * fsz + yy;  // stride wy per x'
    T* const fy_out = (ny > 1 && yy == wy - 1 && wyi < by - 1) ? faceY + (w + 1) * fsy + zz : nullptr;
    T* const fz_out = (zz == wz - 1 && wzi < bz - 1) ? faceZ + (w + by) * fsz + yy : nullptr;
    // cluster variant: the last warps along z push into the next CTA of the cluster (its
    // warp (wyi, 0) slot), fz_remote being that CTA's faceZ in the cluster's shared window
    const unsigned fz_push = (fz_remote != 0u && zz == wz - 1 && wzi == bz - 1)
                                 ? fz_remote + static_cast<unsigned>((wyi * fsz + yy) * static_cast<long long>(sizeof(T)))
                                 : 0u;
    const LineCoef<T>* const cs = reinterpret_cast<const LineCoef<T>*>(P.coef) + P.g.slot(blk, w, 0, lane);
    LineCoef<T>* const cr = cring + w * 32 + lane;  // slot k at cr[k * nw * 32]
    T* const br = bring + w * 32 + lane;
    const int rs = nw * 32;

    // step t's operands into ring slot t % R (zeros where the lane has no row)
    const unsigned span = line_ok ? static_cast<unsigned>(nx) : 0u;  // active: (unsigned)(t - skew) < span
    auto issue = [&](int t) {
        const int xq = t - skew;
        const bool act = static_cast<unsigned>(xq) < span;
        const int k = t & (R - 1);
        const LineCoef<T>* c = act ? cs + static_cast<long long>(t) * 32 : cs;
        const T* bp = act ? in0 + static_cast<long long>(sx) * xq : in;
        if constexpr (sizeof(T) == 4) {
            cp_async_16(cr + k * rs, c, act ? 16 : 0);
            cp_async_4(br + k * rs, bp, act ? 4 : 0);
        } else {
            cp_async_16(cr + k * rs, c, act ? 16 : 0);
            cp_async_16(reinterpret_cast<char*>(cr + k * rs) + 16, reinterpret_cast<const char*>(c) + 16, act ? 16 : 0);
            cp_async_8(br + k * rs, bp, act ? 8 : 0);
        }
        cp_async_commit();
    };
#pragma unroll 1
    for (int t = 0; t < R - 1; ++t) issue(t);
    // face reads: edge lanes at x' (clamped: no read outside the face where the lane has no
    // row), the other lanes from a word that holds 0; each step's values are loaded one
    // step ahead, so that the check for a late predecessor is resolved off the chain
    const T* const fy_rd = y_edge ? fy : zero_word;
    const T* const fz_rd = z_edge ? fz : zero_word;
    const int fy_st = y_edge ? wz : 0, fz_st = z_edge ? wy : 0;
    auto face_at = [&](int t, const T* base, int st) -> const T* {
        const int xq = t - skew;
        return base + (static_cast<unsigned>(xq) < span ? xq : 0) * st;
    };
    T pfy = ld_volatile_shared(face_at(0, fy_rd, fy_st));
    T pfz = ld_volatile_shared(face_at(0, fz_rd, fz_st));
    T* out_p = out0 - static_cast<long long>(sx) * skew;  // row of step s: out_p (advanced by sx per step)
    T prev = T(0);  // the lane's result of the previous step (used only where it had a row)
#pragma unroll 2
    for (int s = 0; s < steps; ++s) {
        cp_async_wait<R - 2>();  // step s has landed
        const int k = s & (R - 1);
        const LineCoef<T> c = cr[k * rs];
        const T bv = br[k * rs];
        issue(s + R - 1);  // into the slot read one step ago
        const int xq = s - skew;
        const bool act = static_cast<unsigned>(xq) < span;
        T fyv = pfy, fzv = pfz;
        pfy = ld_volatile_shared(face_at(s + 1, fy_rd, fy_st));
        pfz = ld_volatile_shared(face_at(s + 1, fz_rd, fz_st));
        const bool late = act && (Sentinel<T>::is(fyv) || Sentinel<T>::is(fzv));
        const T sh_y = __shfl_up_sync(0xffffffffu, prev, 1);
        const T sh_z = __shfl_up_sync(0xffffffffu, prev, wy);
        const T xin = xq > 0 ? prev : T(0);
        const T a0 = scaled ? bv * sc : bv;
        auto row = [&](T fy_v, T fz_v) -> T {
            const T vy = y_edge ? fy_v : (ny > 1 ? sh_y : T(0));
            const T vz = z_edge ? fz_v : sh_z;
            T acc = fma(-c.cz, vz, a0);
            acc = fma(-c.cy, vy, acc);
            acc = fma(-c.cx, xin, acc);
            // FP64: the reference's division (lanes without a row divide by 1: no slow
            // path); FP32 (mixed path): d holds 1 / u_ii
            if constexpr (UPPER) acc = sizeof(T) == 8 ? acc / (act ? c.d : T(1)) : acc * c.d;
            return acc;
        };
        T r = row(fyv, fzv);
        if (__any_sync(0xffffffffu, late)) {  // a predecessor was not there yet: wait, redo
            const int xc = act ? xq : 0;
            if (late && Sentinel<T>::is(fyv)) fyv = line_wait_shared(fy_rd + xc * fy_st, status);
            if (late && Sentinel<T>::is(fzv)) fzv = line_wait_shared(fz_rd + xc * fz_st, status);
            r = row(fyv, fzv);
        }
        // the next step reads r directly (an active lane's shuffle partners and its own
        // previous step are active at the same x'); only the stored copies, which other
        // warps and blocks poll, are kept off the sentinel
        prev = r;
        const T rs_ = Sentinel<T>::canon(r);
        st_relaxed_if(act, out_p, rs_);
        out_p += sx;
        const int xc = act ? xq : 0;
        st_shared_if(act && fy_out != nullptr, fy_out + xc * wz, rs_);
        st_shared_if(act && fz_out != nullptr, fz_out + xc * wy, rs_);
        st_cluster_if(act && fz_push != 0u, fz_push + static_cast<unsigned>(xc * wy * static_cast<int>(sizeof(T))), rs_);
    }
    cp_async_wait<0>();
}

// The halo warp of block `blk`: copies the predecessors that the block's first warps
// along y and z read from the previous blocks (their last lines, in `out`) into the
// faces.  Lane e owns entry e of the y-face (the block's z-line e, at most 32) and entry
// e of the z-face (its y-line e, at most 32) and walks each in x' with its own cursor;
// each round loads the next kLineHalo positions of both (one L2 round trip) and retires,
// in order, those that no longer hold the sentinel.
constexpr int kLineHalo = 16;

template <class T>
struct HaloCursor {
    const T* src = nullptr;  // natural row of x' = 0 of the source line (null: no entry)
    T* dst = nullptr;        // face slot of x' = 0
    int stride = 0;          // face stride per x'
    int x = 0;               // next x' to copy
};

// Loads positions [x, x + kLineHalo) of a cursor (0 past the line's end or without entry).
template <class T, bool UPPER>
__device__ __forceinline__ void halo_load(const HaloCursor<T>& h, int nx, T (&v)[kLineHalo]) {
    constexpr long long sx = UPPER ? -1 : 1;
#pragma unroll
    for (int u = 0; u < kLineHalo; ++u)
        v[u] = (h.src != nullptr && h.x + u < nx) ? ld_relaxed_nb(h.src + sx * (h.x + u)) : T(0);
}

// Copies, in order, the loaded positions that no longer hold the sentinel; true when
// the cursor moved.
template <class T>
__device__ __forceinline__ bool halo_retire(HaloCursor<T>& h, int nx, const T (&v)[kLineHalo]) {
    if (h.src == nullptr || h.x >= nx) return false;
    int adv = 0;
    bool stop = false;
#pragma unroll
    for (int u = 0; u < kLineHalo; ++u) {
        stop = stop || h.x + u >= nx || Sentinel<T>::is(v[u]);
        st_shared_if(!stop, h.dst + static_cast<long long>(h.x + u) * h.stride, v[u]);
        adv += stop ? 0 : 1;
    }
    h.x += adv;
    return adv > 0;
}

template <class T, bool UPPER>
__device__ __forceinline__ void line_halo(const LineTri<T>& P, int blk, const T* out, T* faceY, T* faceZ,
                                          bool z_from_l2, int* status) {
    const int lane = threadIdx.x & 31;
    const int nx = P.g.nx, ny = P.g.ny, nz = P.g.nz;
    const int wy = P.g.wy, wz = P.g.wz, by = P.g.by, bz = P.g.bz;
    const int iy = blk % P.g.nby, iz = blk / P.g.nby;
    const long long plane = static_cast<long long>(nx) * ny;
    auto row0 = [&](int ys, int zs) {
        const long long Y = UPPER ? ny - 1 - ys : ys;
        const long long Z = UPPER ? nz - 1 - zs : zs;
        return (UPPER ? nx - 1 : 0) + nx * Y + plane * Z;
    };
    HaloCursor<T> hy, hz;
    if (ny > 1 && iy > 0 && lane < bz * wz) {  // line (y0 - 1, z) of block (iy - 1, iz)
        const int wzi = lane / wz, zz = lane % wz;
        const int zs = (iz * bz + wzi) * wz + zz;
        if (zs < nz) {
            hy.src = out + row0(iy * by * wy - 1, zs);
            hy.dst = faceY + (wzi * by) * line_face_slot_y(P.g) + zz;
            hy.stride = wz;
        }
    }
    if (z_from_l2 && iz > 0 && lane < by * wy) {  // line (y, z0 - 1) of block (iy, iz - 1)
        const int wyi = lane / wy, yy = lane % wy;
        const int ys = (iy * by + wyi) * wy + yy;
        if (ys < ny) {
            hz.src = out + row0(ys, iz * bz * wz - 1);
            hz.dst = faceZ + wyi * line_face_slot_z(P.g) + yy;
            hz.stride = wy;
        }
    }
    WaitBudget wb;
    while ((hy.src != nullptr && hy.x < nx) || (hz.src != nullptr && hz.x < nx)) {
        // both cursors' loads in flight together: one L2 round trip per round
        T vy[kLineHalo], vz[kLineHalo];
        halo_load<T, UPPER>(hy, nx, vy);
        halo_load<T, UPPER>(hz, nx, vz);
        const bool a = halo_retire<T>(hy, nx, vy);
        const bool b = halo_retire<T>(hz, nx, vz);
        if (!a && !b && wb.expired(status)) {
            atomicExch(status + kStatusTimeout, 1);
            // unblock the compute warps: the remaining entries become 0
            for (; hy.src != nullptr && hy.x < nx; ++hy.x) st_volatile_shared(hy.dst + static_cast<long long>(hy.x) * hy.stride, T(0));
            for (; hz.src != nullptr && hz.x < nx; ++hz.x) st_volatile_shared(hz.dst + static_cast<long long>(hz.x) * hz.stride, T(0));
            break;
        }
    }
}

// Resets a block's faces: the sentinel where a value will be written, 0 where the lines
// lie at the grid's boundary (slots of the first warps along y / z of the first blocks).
template <class T>
__device__ __forceinline__ void line_reset_faces(const LineGeom& g, int iy, int iz, T* faceY, T* zero_word) {
    const long long fsy = line_face_slot_y(g), fsz = line_face_slot_z(g);
    const long long fy_len = g.nw() * fsy;
    const long long face_len = line_face_len<T>(g);
    for (long long i = threadIdx.x; i < face_len; i += blockDim.x) {
        const bool zero = i < fy_len ? (iy == 0 && static_cast<int>(i / fsy) % g.by == 0)
                                     : (iz == 0 && static_cast<int>((i - fy_len) / fsz) / g.by == 0);
        faceY[i] = zero ? T(0) : Sentinel<T>::value();
    }
    if (threadIdx.x == 0) *zero_word = T(0);
}

// GMRES normalises its new Krylov vector in the forward sweep: once a compute warp is
// done with its lines (its own lanes are the only readers of their rows of `in`, and
// all their copies have landed), it rescales them in place, the same product b * scale
// its rows used.  Its y-lines of one plane z are one contiguous run of rows, walked by
// the whole warp, 16 bytes per access where the runs allow it (eight accesses in flight
// per lane).
template <class T>
__device__ __forceinline__ void line_rescale_warp(const LineGeom& g, int blk, T* in, T sc) {
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int wyi = w % g.by, wzi = w / g.by;
    const int iy = blk % g.nby, iz = blk / g.nby;
    const int y0 = (iy * g.by + wyi) * g.wy, y1 = min(g.ny, y0 + g.wy);
    const int z0 = (iz * g.bz + wzi) * g.wz, z1 = min(g.nz, z0 + g.wz);
    if (y0 >= y1 || z0 >= z1) return;
    const long long run = static_cast<long long>(g.nx) * (y1 - y0);
    const long long plane = static_cast<long long>(g.nx) * g.ny;
    T* const base = in + static_cast<long long>(g.nx) * y0 + plane * z0;
    constexpr int V = 16 / sizeof(T);  // rows per 16-byte access
    const bool vec = run % V == 0 && plane % V == 0 && (reinterpret_cast<unsigned long long>(base) & 15ull) == 0;
    if (vec) {
        const int rv = static_cast<int>(run / V);
        for (int zi = 0; zi < z1 - z0; ++zi) {
#pragma unroll 8
            for (int e = lane; e < rv; e += 32) {
                T* p = base + zi * plane + static_cast<long long>(e) * V;
                if constexpr (sizeof(T) == 4) {
                    float4 v = *reinterpret_cast<const float4*>(p);
                    v.x *= sc;
                    v.y *= sc;
                    v.z *= sc;
                    v.w *= sc;
                    *reinterpret_cast<float4*>(p) = v;
                } else {
                    double2 v = *reinterpret_cast<const double2*>(p);
                    v.x *= sc;
                    v.y *= sc;
                    *reinterpret_cast<double2*>(p) = v;
                }
            }
        }
    } else {
        for (int zi = 0; zi < z1 - z0; ++zi) {
            T* const q = base + zi * plane;
#pragma unroll 8
            for (long long e = lane; e < run; e += 32) q[e] = q[e] * sc;
        }
    }
}

// Forward (UPPER = false): out = L^{-1} (scale * in), in rescaled in place when `scale`
// is given (each compute warp's lines once that warp has solved them); backward (UPPER = true):
// out = U^{-1} in.  in / out in natural order; out holds the sentinel at every row on
// entry.  nw compute warps + 1 halo warp; dynamic shared memory line_smem_bytes.
template <class T, bool UPPER>
__global__ void __launch_bounds__((kLineMaxWarps + 1) * kWarp, 1)
    sptrsv_line_kernel(LineTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                       const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char line_smem[];
    const int nw = P.g.nw();
    const long long fsy = line_face_slot_y(P.g), fsz = line_face_slot_z(P.g);
    const long long fy_len = nw * fsy;
    const long long face_len = line_face_len<T>(P.g);
    T* faceY = reinterpret_cast<T*>(line_smem);
    T* faceZ = faceY + fy_len;
    T* zero_word = faceY + face_len;  // holds 0
    LineCoef<T>* cring = reinterpret_cast<LineCoef<T>*>(line_smem + line_ring_offset<T>(P.g));
    T* bring = reinterpret_cast<T*>(cring + static_cast<long long>(kLineRing<T>) * nw * 32);
    __shared__ int s_ticket;
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    const int w = threadIdx.x >> 5;
    for (int tk = draw_block_ticket(counter, P.g.nblk, &s_ticket); tk < P.g.nblk;
         tk = draw_block_ticket(counter, P.g.nblk, &s_ticket)) {
        const int blk = P.order[tk];
        const int iy = blk % P.g.nby, iz = blk / P.g.nby;
        line_reset_faces<T>(P.g, iy, iz, faceY, zero_word);
        // stream the warps' operands into L2 (the right-hand side was written by the
        // previous kernel and is there already)
        if (w < nw)
            prefetch_l2_range(P.coef + P.g.slot(blk, w, 0, 0) * 4,
                              static_cast<long long>(P.g.steps) * 128 * static_cast<long long>(sizeof(T)),
                              threadIdx.x & 31);
        __syncthreads();
        line_stamp_start(P, blk);
        if (w < nw)
            line_warp<T, UPPER>(P, blk, in, scaled, sc, out, faceY, faceZ, zero_word, cring, bring, 0u, status);
        else
            line_halo<T, UPPER>(P, blk, out, faceY, faceZ, true, status);
        line_stamp_end(P, blk);
        if (scaled && w < nw) line_rescale_warp<T>(P.g, blk, in, sc);
    }
}

// Cluster variant: launched with clusters of g.cl CTAs; the cluster of ticket q takes the
// blocks (iy, izc cl + rank) of cluster q (tickets along anti-diagonals of the cluster
// grid: a cluster only waits for clusters of smaller tickets, whose CTAs are running or
// done; the CTAs of one cluster are co-scheduled).  A CTA's last warps along z push
// their results into the next CTA's face in distributed shared memory, so only the first
// CTA of a cluster and the y-direction take their predecessors from L2 (halo warp).
template <class T, bool UPPER>
__global__ void __launch_bounds__((kLineMaxWarps + 1) * kWarp, 1)
    sptrsv_line_cluster_kernel(LineTri<T> P, T* in, const double* scale, T* out, unsigned* counter, int* status,
                               const int* gate, int step) {
    if (gate_closed(gate, step)) return;
    extern __shared__ __align__(16) unsigned char line_smem[];
    const int nw = P.g.nw();
    const long long fy_len = static_cast<long long>(nw) * line_face_slot_y(P.g);
    const long long face_len = line_face_len<T>(P.g);
    T* faceY = reinterpret_cast<T*>(line_smem);
    T* faceZ = faceY + fy_len;
    T* zero_word = faceY + face_len;
    LineCoef<T>* cring = reinterpret_cast<LineCoef<T>*>(line_smem + line_ring_offset<T>(P.g));
    T* bring = reinterpret_cast<T*>(cring + static_cast<long long>(kLineRing<T>) * nw * 32);
    __shared__ int s_ticket;
    const bool scaled = !UPPER && scale != nullptr;
    const T sc = scaled ? static_cast<T>(*scale) : T(1);
    const int w = threadIdx.x >> 5;
    const unsigned rank = cluster_rank_u32();
    const unsigned CL = cluster_size_u32();
    const int nq = P.g.nby * P.g.nbzc;
    const int nclusters = static_cast<int>(gridDim.x / CL);
    for (;;) {
        // the previous round is complete in every CTA of the cluster (no push in flight)
        // before the ticket and the faces are reset
        cluster_sync_all();
        if (rank == 0 && threadIdx.x == 0) {
            const int q = static_cast<int>(atomicAdd(counter, 1u));
            if (q == nq + nclusters - 1) atomicExch(counter, 0u);
            for (unsigned r = 0; r < CL; ++r) st_cluster(map_shared_rank(&s_ticket, r), q);
        }
        cluster_sync_all();
        const int q = *reinterpret_cast<volatile int*>(&s_ticket);
        if (q >= nq) break;
        const int cb = P.order[q];
        const int iy = cb % P.g.nby;
        const int iz = (cb / P.g.nby) * static_cast<int>(CL) + static_cast<int>(rank);
        const bool active = iz < P.g.nbz;
        const int blk = iy + P.g.nby * iz;
        if (active) {
            line_reset_faces<T>(P.g, iy, iz, faceY, zero_word);
            if (w < nw)
                prefetch_l2_range(P.coef + P.g.slot(blk, w, 0, 0) * 4,
                                  static_cast<long long>(P.g.steps) * 128 * static_cast<long long>(sizeof(T)),
                                  threadIdx.x & 31);
        }
        __syncthreads();
        // every face of the cluster is reset before any CTA pushes into it
        cluster_sync_all();
        if (active) {
            const bool push = rank + 1 < CL && iz + 1 < P.g.nbz;
            const unsigned remote = push ? map_shared_rank(faceZ, rank + 1) : 0u;
            line_stamp_start(P, blk);
            if (w < nw)
                line_warp<T, UPPER>(P, blk, in, scaled, sc, out, faceY, faceZ, zero_word, cring, bring, remote, status);
            else
                line_halo<T, UPPER>(P, blk, out, faceY, faceZ, rank == 0, status);
            line_stamp_end(P, blk);
            if (scaled && w < nw) line_rescale_warp<T>(P.g, blk, in, sc);
        }
        __syncthreads();
    }
}

// Packs the operand stream of a structured factor from its CSR values: one thread per
// slot.  L: c_z, c_y, c_x are the row's strict-lower entries (columns ascending:
// r - nx ny, r - nx, r - 1, each present only inside the grid), d = 0.  U: c_z, c_y, c_x
// are the strict-upper entries r + nx ny, r + nx, r + 1 (columns descending) and d = u_ii
// (FP64) or RN(1 / u_ii), computed in FP64 and rounded once (FP32, as the other FP32
// kernels).  Slots without a row hold zeros.
template <class T, bool UPPER>
__global__ void line_pack_kernel(LineGeom g, const int* __restrict__ rp, const int* __restrict__ diag,
                                 const double* __restrict__ lu, T* __restrict__ dst) {
    const long long total = g.slots();
    const int nw = g.nw();
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int lane = static_cast<int>(i & 31);
        long long t = i >> 5;
        const int s = static_cast<int>(t % g.steps);
        t /= g.steps;
        const int w = static_cast<int>(t % nw);
        const int b = static_cast<int>(t / nw);
        const int wyi = w % g.by, wzi = w / g.by;
        const int yy = lane % g.wy, zz = lane / g.wy;
        const int iy = b % g.nby, iz = b / g.nby;
        const int yq = (iy * g.by + wyi) * g.wy + yy;
        const int zq = (iz * g.bz + wzi) * g.wz + zz;
        const int xq = s - (yy + zz);
        double cz = 0.0, cy = 0.0, cx = 0.0, d = 0.0;
        if (yq < g.ny && zq < g.nz && xq >= 0 && xq < g.nx) {
            const int X = UPPER ? g.nx - 1 - xq : xq;
            const int Y = UPPER ? g.ny - 1 - yq : yq;
            const int Z = UPPER ? g.nz - 1 - zq : zq;
            const long long r = X + static_cast<long long>(g.nx) * (Y + static_cast<long long>(g.ny) * Z);
            if constexpr (!UPPER) {
                int p = rp[r];
                if (Z > 0) cz = lu[p++];
                if (Y > 0) cy = lu[p++];
                if (X > 0) cx = lu[p++];
            } else {
                int p = diag[r];
                d = lu[p++];
                if (X < g.nx - 1) cx = lu[p++];
                if (Y < g.ny - 1) cy = lu[p++];
                if (Z < g.nz - 1) cz = lu[p++];
                if (sizeof(T) == 4) d = 1.0 / d;
            }
        }
        T* o = dst + 4 * i;
        o[0] = static_cast<T>(cz);
        o[1] = static_cast<T>(cy);
        o[2] = static_cast<T>(cx);
        o[3] = static_cast<T>(d);
    }
}

template <class T>
__global__ void line_fill_kernel(long long n, T* p, T v) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        p[i] = v;
}

}  // namespace gb300
