/*
 * Replay state behind the oracle build's Random::rand_int (see replay_random.cpp).
 * Test infrastructure: it lets the reference's own estimate() bodies consume the draws the
 * GPU / the C oracle recorded, and checks that every requested range matches.
 */
#ifndef ZGREF_REPLAY_HPP
#define ZGREF_REPLAY_HPP

#include <stdint.h>
#include <deque>
#include <vector>

struct ZgrefDraw { uint64_t lo, hi, val; };

struct ZgrefReplay {
  /* Random::rand_int() (no range): the CSR shuffle's positions (src/Graph.cpp:225-230). */
  std::vector<uint64_t> raw_script;
  size_t raw_pos = 0;
  /* Random::rand_int(min, max): queued draws in consumption order. */
  std::deque<ZgrefDraw> q;
  uint64_t consumed = 0;
  uint64_t mismatches = 0; /* requested range differs from the recorded one */
  uint64_t overruns = 0;   /* a draw was requested beyond the queue */
  uint64_t raw_overruns = 0;

  /* Called when q runs dry; appends the next draws and returns false when there are none. */
  bool (*refill)(void*) = nullptr;
  void* refill_ctx = nullptr;

  void reset_counts() { consumed = mismatches = overruns = raw_overruns = 0; }
  uint64_t raw() {
    if (raw_pos < raw_script.size()) return raw_script[raw_pos++];
    ++raw_overruns;
    return 0;
  }
  uint64_t range(uint64_t lo, uint64_t hi) {
    if (q.empty() && refill) refill(refill_ctx);
    if (q.empty()) { ++overruns; return lo; }
    ZgrefDraw d = q.front();
    q.pop_front();
    ++consumed;
    if (d.lo != lo || d.hi != hi) ++mismatches;
    return d.val;
  }
};

extern ZgrefReplay zgref_replay;

/* Fisher-Yates positions that make the reference's shuffle (for e_i = n..2:
 * swap(a[e_i-1], a[rand_int() % e_i])) produce out[i] = in[perm[i]]. */
static inline std::vector<uint64_t> zgref_shuffle_script(const uint64_t* perm, uint64_t n) {
  std::vector<uint64_t> script;
  if (n < 2) return script;
  std::vector<uint64_t> pos_of(n), who(n);
  for (uint64_t i = 0; i < n; ++i) { pos_of[i] = i; who[i] = i; }
  script.reserve(n - 1);
  for (uint64_t e = n; e > 1; --e) {
    uint64_t want = perm ? perm[e - 1] : e - 1;
    uint64_t p = pos_of[want];
    script.push_back(p);
    uint64_t a = who[e - 1], b = who[p];
    who[e - 1] = b; who[p] = a;
    pos_of[b] = e - 1; pos_of[a] = p;
  }
  return script;
}

#endif
