/*
 * Oracle test infrastructure only.  Portable replacement for the reference's
 * include/tictoc.hpp, whose x86 cpuid/rdtsc inline assembly (include/tictoc.hpp:9-19)
 * does not build on aarch64 and whose fixed 2.4 GHz conversion (:26) is wrong on
 * other clocks.  Same names (Rdtsc/Tic/Toc), steady_clock nanoseconds underneath,
 * so Toc() returns seconds.
 */
#pragma once

#include <chrono>
#include <cstdint>

namespace lljbash {

inline uint64_t g_cycles;

inline uint64_t Rdtsc() {
    return static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
                                     std::chrono::steady_clock::now().time_since_epoch())
                                     .count());
}

inline void Tic() { g_cycles = Rdtsc(); }

inline double Toc(uint64_t tic = g_cycles) { return static_cast<double>(Rdtsc() - tic) * 1e-9; }

}  // namespace lljbash
