// zgh_internal.hpp — shared helpers of the host layer: status checks that turn a failing zg_* call
// into an exception (there is no CPU fallback), lazy device initialisation, and the host Philox
// draw used where the host itself needs random numbers (vertex relabelling, seeds, estimate()
// calls made directly on the host).
#ifndef ZGH_INTERNAL_HPP
#define ZGH_INTERNAL_HPP

#include <stdint.h>

#include <stdexcept>
#include <string>

#include "../../../include/zgraph_gpu.h"

namespace zgh {

// Throws std::runtime_error carrying zg_last_error() when rc != ZG_OK.
void check(int rc, const char* what);
// zg_init on the device named by ZGRAPH_DEVICE (default 0), once per process.
void ensure_init();
// A fresh 64-bit seed: ZGRAPH_SEED when set (then deterministic per call count), else time-based.
uint64_t next_seed();

// Philox4x32-10 (Salmon et al., SC'11), counter (c0..c3), key (k0, k1); 64-bit output.
uint64_t philox64(uint64_t counter, uint32_t c2, uint32_t c3, uint64_t key);
// Uniform integer in [lo, hi] from a 64-bit word by multiply-high (hi - lo + 1 == 0: the word).
inline uint64_t map_range(uint64_t r, uint64_t lo, uint64_t hi) {
  uint64_t range = hi - lo + 1;
  if (range == 0) return r;
  return lo + (uint64_t)(((unsigned __int128)r * range) >> 64);
}

}  // namespace zgh

#endif
