// zg_sample_kernel.cuh — the production sampling kernel k_sample, shared by zg_sample.cu (the
// library's launches) and zg_touch.cu (the same kernel compiled with load counting, for the
// roofline's bytes per sample).
#pragma once

#include "zg_programs.cuh"

namespace {

constexpr int kBlock = 256;

// The 4-chain's sample loop with the warp's samples grouped by program.  FourChain.cpp draws one
// of three programs per sample, and their dependent-load chains differ in length (the second
// program adds a lower-bound search): a warp mixing them waits for its slowest lane at every step.
// Each warp draws the program of its next 32 samples (the same sample indices the plain loop gives
// its lanes), queues them per program in shared memory and runs a program's queue whenever it
// holds 32 samples (PAIRED: 64, two per lane with their load chains interleaved by
// prog_four_chain_n, which needs more registers), so every warp runs one program on all lanes;
// leftovers run at the end.
// Exact sums are unchanged (the same samples, integer sums); the variance term is summed per lane
// in another order.
template <int LAYOUT, bool PAIRED>
__device__ __forceinline__ void four_chain_grouped(const ZgDevGraph& g, uint64_t n, uint64_t first, uint64_t seed,
                                                   const ZgKeys& keys, uint32_t stream, uint32_t den, Acc& a,
                                                   AccSlots<kBlock>& sl) {
  __shared__ uint32_t queue[kBlock / 32][3][128];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t below = (1u << lane) - 1;
  const uint64_t base = (uint64_t)blockIdx.x * kBlock + warp * 32;
  const uint64_t stride = (uint64_t)gridDim.x * kBlock;
  uint32_t(*q)[128] = queue[warp];
  uint32_t c1 = 0, c2 = 0, c3 = 0;  // queued samples per program, the same on every lane
  for (uint32_t k = 0;; ++k) {
    const uint64_t i = base + (uint64_t)k * stride + lane;
    const bool valid = i < n;
    if (!__ballot_sync(0xffffffffu, valid)) break;
    const uint32_t sel = valid ? (uint32_t)zg_draw_map(zg_sample_word_k(keys, stream, first + i, 0), 1, 3) : 0u;
    const unsigned m1 = __ballot_sync(0xffffffffu, sel == 1), m2 = __ballot_sync(0xffffffffu, sel == 2),
                   m3 = __ballot_sync(0xffffffffu, sel == 3);
    // every count is below a run (<= 63) before this round, so a queue of 128 never overflows
    if (sel == 1) q[0][c1 + __popc(m1 & below)] = k * 32 + lane;
    if (sel == 2) q[1][c2 + __popc(m2 & below)] = k * 32 + lane;
    if (sel == 3) q[2][c3 + __popc(m3 & below)] = k * 32 + lane;
    c1 += __popc(m1);
    c2 += __popc(m2);
    c3 += __popc(m3);
    __syncwarp();
    constexpr uint32_t kRun = PAIRED ? 64u : 32u;
#pragma unroll 1
    for (;;) {  // run every queue that holds a full run
      const uint32_t p = c1 >= kRun ? 1u : c2 >= kRun ? 2u : c3 >= kRun ? 3u : 0u;
      if (!p) break;
      const uint32_t cp = p == 1 ? c1 : p == 2 ? c2 : c3;
      const uint32_t s0 = q[p - 1][cp - kRun + lane], s1 = PAIRED ? q[p - 1][cp - 32 + lane] : 0u;
      c1 -= p == 1 ? kRun : 0u;
      c2 -= p == 2 ? kRun : 0u;
      c3 -= p == 3 ? kRun : 0u;
      __syncwarp();  // read before the next round refills the queue
      const uint64_t si0 = base + (uint64_t)(s0 >> 5) * stride + (s0 & 31);
      if (PAIRED) {
        const uint64_t si1 = base + (uint64_t)(s1 >> 5) * stride + (s1 & 31);
        Ctx c[2] = {{seed, first + si0, stream, 0, nullptr, 0, 0, &keys},
                    {seed, first + si1, stream, 0, nullptr, 0, 0, &keys}};
        Res r[2];
        res_init(r[0]);
        res_init(r[1]);
        prog_four_chain_n<2>(g, c, r, p);
        acc_add_slots(a, sl, r[0], den);
        acc_add_slots(a, sl, r[1], den);
      } else {
        Ctx c{seed, first + si0, stream, 0, nullptr, 0, 0, &keys};
        Res r;
        res_init(r);
        prog_four_chain<false>(g, c, r, p);
        acc_add_slots(a, sl, r, den);
      }
    }
  }
  __syncwarp();
  // the leftovers: less than a run per program, one sample per lane at a time
#pragma unroll 1
  for (uint32_t p = 1; p <= 3; ++p) {
    const uint32_t cp = p == 1 ? c1 : p == 2 ? c2 : c3;
#pragma unroll 1
    for (uint32_t off = 0; off < cp; off += 32) {
      if (off + lane < cp) {
        const uint32_t slot = q[p - 1][off + lane];
        const uint64_t si = base + (uint64_t)(slot >> 5) * stride + (slot & 31);
        Ctx c{seed, first + si, stream, 0, nullptr, 0, 0, &keys};
        Res r;
        res_init(r);
        prog_four_chain<false>(g, c, r, p);
        acc_add_slots(a, sl, r, den);
      }
    }
  }
}

// Production kernels: one specialisation per program, per register budget (MINB resident blocks
// of 256 threads requested from the compiler; zg_tune picks the fastest per program) and per record
// layout (0 compact, 1 wide, 2 packed: the layout tests of the record accessors fold away; each
// layout gets its own registers).
template <int KIND, int MINB, int LAYOUT>
__device__ __forceinline__ void sample_loop(ZgDevGraph g, const ZgProgParams& pp, uint64_t n, uint64_t first,
                                            uint64_t seed, const ZgKeys& keys, uint32_t stream,
                                            ZgPartial* __restrict__ partials) {
  g.wide = LAYOUT == 1;
  g.packed = LAYOUT == 2;
  // Sums in shared-memory slots for the programs with long dependent chains (measured: 4-clique
  // and 4-chain faster); the triangle and 3-chain were faster with them in registers.
  constexpr bool kSlots = KIND != ZG_PROG_THREE_CHAIN && KIND != ZG_PROG_TRIANGLE;
  __shared__ AccSlots<kBlock> sl;
  ZG_TOUCH_BEGIN();
  Acc a;
  acc_init(a);
  if (kSlots) acc_slots_init(sl);
  if (KIND == ZG_PROG_FOUR_CHAIN) {
    // two samples in flight per lane where the register budget allows it (<= 3 resident blocks)
    four_chain_grouped<LAYOUT, (MINB <= 3)>(g, n, first, seed, keys, stream, pp.den_log2, a, sl);
    acc_from_slots(a, sl);
    block_reduce_store<kBlock>(a, &partials[blockIdx.x]);
    ZG_TOUCH_END();
    return;
  }
  uint64_t stride = (uint64_t)gridDim.x * kBlock;
  for (uint64_t i = blockIdx.x * (uint64_t)kBlock + threadIdx.x; i < n; i += stride) {
    Ctx c{seed, first + i, stream, 0, nullptr, 0, 0, &keys};
    Res r;
    res_init(r);
    if (KIND == ZG_PROG_TRIANGLE) prog_triangle<false>(g, c, r);
    else if (KIND == ZG_PROG_FOUR_CLIQUE) prog_four_clique<false>(g, c, r);
    else if (KIND == ZG_PROG_FOUR_CLIQUE_UNBIASED) prog_four_clique<false, true>(g, c, r);
    else if (KIND == ZG_PROG_THREE_CHAIN) prog_three_chain<false>(g, c, r);
    else if (KIND == ZG_PROG_FOUR_CHAIN) prog_four_chain<false>(g, c, r);
    else if (KIND == ZG_PROG_CHAIN) prog_chain<false>(g, (int)pp.param, c, r);
    else prog_pattern<false>(g, pp, c, r);
    if (kSlots)
      acc_add_slots(a, sl, r, pp.den_log2);
    else
      acc_add(a, r, pp.den_log2);
  }
  if (kSlots) acc_from_slots(a, sl);
  block_reduce_store<kBlock>(a, &partials[blockIdx.x]);
  ZG_TOUCH_END();
}


template <int KIND, int MINB, int LAYOUT>
__global__ void __launch_bounds__(kBlock, MINB)
    k_sample(ZgDevGraph g, ZgProgParams pp, uint64_t n, uint64_t first, uint64_t seed, const __grid_constant__ ZgKeys keys,
             uint32_t stream, ZgPartial* __restrict__ partials) {
  sample_loop<KIND, MINB, LAYOUT>(g, pp, n, first, seed, keys, stream, partials);
}

}  // namespace
