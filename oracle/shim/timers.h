/*
 * Stand-in for the reference's timers.h: TIME_COLD runs the kernel body and
 * records its wall time in ref_last_ms (the reference's 80 MB cache flush is
 * done by the caller, see ref_flush_cache in ref_bridge.cpp).
 * Test infrastructure only.
 */
#ifndef TT_ORACLE_SHIM_TIMERS_H
#define TT_ORACLE_SHIM_TIMERS_H
#include <chrono>
extern double ref_last_ms;
#define TIME_COLD(...) {                                                          \
    auto tt_t0_ = std::chrono::steady_clock::now();                              \
    __VA_ARGS__;                                                                  \
    ref_last_ms = std::chrono::duration<double, std::milli>(                     \
        std::chrono::steady_clock::now() - tt_t0_).count();                      \
  }
#endif
