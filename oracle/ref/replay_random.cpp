/*
 * Replacement for the reference's src/Random.cpp in the oracle build: Random::rand_int
 * (src/Random.cpp:7-14) returns replayed values instead of mt19937 draws, so per-sample
 * outcomes of the reference estimators can be compared bit for bit.  Test infrastructure.
 */
#include "Random.hpp"
#include "zgref_replay.hpp"

int zgref_num_cpus = 1;
ZgrefReplay zgref_replay;

unsigned long long Random::rand_int() { return zgref_replay.raw(); }

unsigned long long Random::rand_int(unsigned long long min, unsigned long long max) {
  return zgref_replay.range(min, max);
}
