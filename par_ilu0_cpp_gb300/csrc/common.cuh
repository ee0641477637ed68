// Shared device helpers: error checking, coherent loads/stores for the sync-free
// kernels, sentinel values used as "not yet computed" markers, warp reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace gb300 {

#define GB_CUDA_CHECK(expr)                                                                       \
    do {                                                                                          \
        cudaError_t gb_err_ = (expr);                                                             \
        if (gb_err_ != cudaSuccess) {                                                             \
            throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(gb_err_) + \
                                     " at " + __FILE__ + ":" + std::to_string(__LINE__));         \
        }                                                                                         \
    } while (0)

constexpr int kWarp = 32;

// Device status words (one int array per solver):
//   [0] a dependency wait gave up
//   [1] number of zero / non-finite pivots met in the last factorisation
//   [2] smallest row index with such a pivot (INT_MAX when none)
//   [3] wait limit in microseconds, written by the host (0: kWaitLimitUsDefault)
enum StatusWord {
    kStatusTimeout = 0,
    kStatusBreakdowns = 1,
    kStatusFirstBreakdown = 2,
    kStatusWaitLimitUs = 3,
    kStatusWords = 4
};

// A dependency wait gives up when the awaited value has not arrived within the wait
// limit (default 4 s of device time: every wait on the critical path of a correct
// computation ends far sooner), or after kPollLimit polls whatever the clock says.
constexpr int kWaitLimitUsDefault = 4000000;
constexpr long long kPollLimit = 1ll << 28;

// "Not yet written" markers for value-as-flag waits.  A computed value is never equal to
// them: results that are NaN are stored as the canonical quiet NaN instead.
template <class T>
struct Sentinel;
template <>
struct Sentinel<double> {
    static constexpr unsigned long long bits = 0xFFFFFFFFFFFFFFFFull;
    __device__ static double value() { return __longlong_as_double(static_cast<long long>(bits)); }
    __device__ static bool is(double v) {
        return static_cast<unsigned long long>(__double_as_longlong(v)) == bits;
    }
    __device__ static double canon(double v) { return v != v ? __longlong_as_double(0x7FF8000000000000ll) : v; }
};
template <>
struct Sentinel<float> {
    static constexpr unsigned int bits = 0xFFFFFFFFu;
    __device__ static float value() { return __uint_as_float(bits); }
    __device__ static bool is(float v) { return __float_as_uint(v) == bits; }
    __device__ static float canon(float v) { return v != v ? __uint_as_float(0x7FC00000u) : v; }
};

// Loads/stores that go to the point of coherence (L2) at GPU scope.
__device__ __forceinline__ double ld_relaxed(const double* p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ float ld_relaxed(const float* p) {
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
// The same loads without a compiler memory barrier: they may be scheduled around other
// memory accesses (prefetches whose result is checked for the sentinel before use).
__device__ __forceinline__ double ld_relaxed_nb(const double* p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_relaxed_nb(const float* p) {
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_relaxed(double* p, double v) {
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(float* p, float v) {
    asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_int(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bookkeeping of one bounded wait (or one bounded polling loop), called once per poll.
// expired() turns true once the wait limit has passed since the wait began (the clock
// is read every 64 polls), once another thread has given up (status checked every 1024
// polls), or after kPollLimit polls.  Every lane of a warp that polls in lockstep gets
// the same answer, so a warp leaves such a loop as a whole.
struct WaitBudget {
    unsigned long long t0 = 0;
    unsigned long long limit_ns = 0;
    long long polls = 0;

    __device__ __forceinline__ bool expired(const int* status) {
        ++polls;
        if ((polls & 63) != 0) return false;
        if (polls >= kPollLimit) return true;
        if ((polls & 1023) == 0 && ld_relaxed_int(status + kStatusTimeout) != 0) return true;
        const unsigned long long now = global_ns();
        if (t0 == 0) {
            const int us = status[kStatusWaitLimitUs];
            limit_ns = 1000ull * static_cast<unsigned long long>(us > 0 ? us : kWaitLimitUsDefault);
            t0 = now;
            return false;
        }
        return now - t0 > limit_ns;
    }
};

// Polls made back to back before a wait starts to sleep between polls: a dependency on
// the critical path is usually published within a few round trips, and a sleep (whose
// actual length is far above its nominal 32 ns) would delay its detection.
constexpr int kSpinBeforeSleep = 256;

// Waits until *p is no longer the sentinel; returns the value.  When the wait expires
// (WaitBudget) the timeout is recorded in status[kStatusTimeout] and 0 is returned.
template <class T>
__device__ __forceinline__ T wait_value(const T* p, int* status) {
    T v = ld_relaxed(p);
    if (!Sentinel<T>::is(v)) return v;
    WaitBudget wb;
    while (!wb.expired(status)) {
        if (wb.polls > kSpinBeforeSleep) __nanosleep(32);
        v = ld_relaxed(p);
        if (!Sentinel<T>::is(v)) return v;
    }
    atomicExch(status + kStatusTimeout, 1);
    return T(0);
}

// Waits until *flag == stamp (acquire).  Same give-up rules as wait_value.
__device__ __forceinline__ bool wait_flag(const int* flag, int stamp, int* status) {
    if (ld_acquire(flag) == stamp) return true;
    WaitBudget wb;
    while (!wb.expired(status)) {
        if (wb.polls > kSpinBeforeSleep) __nanosleep(32);
        if (ld_acquire(flag) == stamp) return true;
    }
    atomicExch(status + kStatusTimeout, 1);
    return false;
}

// L2 prefetch of a contiguous range (cp.async.bulk.prefetch): no destination, no
// completion to wait for.  `p` 16-byte aligned; the range is rounded to 16-byte pieces
// issued in chunks of at most 64 KB, split over the calling warp's lanes.
__device__ __forceinline__ void prefetch_l2_range(const void* p, long long bytes, int lane) {
    const unsigned long long a = reinterpret_cast<unsigned long long>(p);
    const long long n16 = bytes >> 4;
    constexpr long long kChunk16 = 4096;  // 64 KB
    for (long long c = static_cast<long long>(lane) * kChunk16; c < n16; c += 32 * kChunk16) {
        const unsigned sz = static_cast<unsigned>((n16 - c < kChunk16 ? n16 - c : kChunk16) << 4);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a + (static_cast<unsigned long long>(c) << 4)),
                     "r"(sz)
                     : "memory");
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class T>
__host__ __device__ constexpr T ceil_div(T a, T b) {
    return (a + b - 1) / b;
}

}  // namespace gb300
