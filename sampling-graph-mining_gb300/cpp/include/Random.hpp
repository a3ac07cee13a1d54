// Random.hpp — the estimators' random source.  On this platform every estimate the library
// returns is computed on the GPU from Philox counter streams; this host class only serves the
// host primitives (validation replay and direct estimate() calls).  In replay mode it returns the
// queued draws of a device trace and records whether the requested ranges matched.
#ifndef RANDOM_HPP
#define RANDOM_HPP

#include <stdint.h>

#include <deque>

class Random {
 public:
  Random();
  unsigned long long rand_int();
  unsigned long long rand_int(unsigned long long min, unsigned long long max);

  // replay of recorded draws (lo, hi, value)
  struct Draw {
    uint64_t lo, hi, val;
  };
  void replay(const Draw* draws, int n);
  void stop_replay();
  bool replaying() const { return replaying_; }
  uint64_t mismatches() const { return mismatches_; }
  uint64_t consumed() const { return consumed_; }
  size_t pending() const { return queue_.size(); }

 private:
  uint64_t seed_, counter_;
  bool replaying_;
  std::deque<Draw> queue_;
  uint64_t mismatches_, consumed_;
};

#endif
