// darwin_time.h -- forced-included when the reference's C++ benches are
// compiled on Linux in the client-compatibility test: they time with the
// Darwin call clock_gettime_nsec_np, which glibc lacks.
#pragma once
#include <cstdint>
#include <ctime>

static inline uint64_t clock_gettime_nsec_np(clockid_t clock) {
  timespec t{};
  clock_gettime(clock, &t);
  return uint64_t(t.tv_sec) * 1000000000ull + uint64_t(t.tv_nsec);
}
