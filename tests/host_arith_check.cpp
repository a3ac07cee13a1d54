// Host-side check of the arithmetic the sampling kernels share with the host (compiled by g++ from
// the library's own header): Philox with per-launch round keys, the 192-bit x 32-bit weight
// multiply, the packed edge record's fields and the fingerprint's range.  Prints one line per case
// for tests/test_host_arith.py, which recomputes every value with Python integers.
#include <stdio.h>

#include "zg_internal.cuh"

static uint64_t s_state = 0x9E3779B97F4A7C15ull;
static uint64_t next64() {  // splitmix64 stream for the inputs
  s_state += 0x9E3779B97F4A7C15ull;
  return zg_mix64(s_state);
}

int main() {
  // Philox: precomputed round keys give the block the on-the-fly key schedule gives
  for (int i = 0; i < 64; ++i) {
    const uint64_t seed = next64(), sample = next64();
    const uint32_t stream = (uint32_t)next64(), d = (uint32_t)next64() & 7;
    const ZgKeys K = zg_round_keys(seed);
    printf("philox %llu %llu %u %u %llu %llu\n", (unsigned long long)seed, (unsigned long long)sample, stream, d,
           (unsigned long long)zg_sample_word(seed, stream, sample, d),
           (unsigned long long)zg_sample_word_k(K, stream, sample, d));
  }
  // 192-bit x 32-bit products, with and without overflow
  for (int i = 0; i < 64; ++i) {
    ZgU192 a;
    a.l[0] = next64();
    a.l[1] = i < 32 ? next64() : 0;
    a.l[2] = i < 16 ? next64() : (i < 32 ? next64() >> 40 : 0);
    const uint32_t f = (uint32_t)next64();
    printf("mul %llu %llu %llu %u", (unsigned long long)a.l[0], (unsigned long long)a.l[1],
           (unsigned long long)a.l[2], f);
    const bool o = zg_u192_mul32(a, f);
    printf(" %llu %llu %llu %d\n", (unsigned long long)a.l[0], (unsigned long long)a.l[1],
           (unsigned long long)a.l[2], (int)o);
  }
  // packed records: fields at the widths a graph may choose (2V + S <= 64, S + 2P <= 64)
  const uint32_t widths[][3] = {{1, 1, 1}, {8, 4, 10}, {20, 16, 23}, {24, 16, 24}, {31, 2, 31}, {26, 12, 26}};
  for (const auto& w : widths) {
    const uint32_t vb = w[0], sb = w[1], pb = w[2];
    for (int i = 0; i < 16; ++i) {
      const uint64_t vm = (1ull << vb) - 1, sm = (1ull << sb) - 1, pm = (1ull << pb) - 1;
      const uint32_t src = (uint32_t)(next64() & vm), dst = (uint32_t)(next64() & vm);
      const uint32_t ss = (uint32_t)(next64() & sm), sd = (uint32_t)(next64() & sm);
      const uint32_t ps = (uint32_t)(next64() & pm), pd = (uint32_t)(next64() & pm);
      const uint64_t w0 = (uint64_t)src | ((uint64_t)dst << vb) | ((uint64_t)ss << (2 * vb));
      const uint64_t w1 = (uint64_t)sd | ((uint64_t)ps << sb) | ((uint64_t)pd << (sb + pb));
      uint32_t f[6];
      zg_unpack(vb, sb, pb, w0, w1, f[0], f[1], f[2], f[3], f[4], f[5]);
      printf("packed %u %u %u %u %u %u %u %u %u %u %u %u %u %u %u\n", vb, sb, pb, src, dst, ss, sd, ps, pd, f[0], f[1],
             f[2], f[3], f[4], f[5]);
    }
  }
  // fingerprints: 31 bits, never the empty entry's field
  uint32_t worst = 0;
  for (int i = 0; i < 1 << 16; ++i) {
    const uint32_t fp = zg_fingerprint(next64(), 0x5A4748415348ull);
    if (fp > worst) worst = fp;
  }
  printf("fingerprint_max %u\n", worst);
  return 0;
}
