// zg_touch.cu — the bytes the production sampling kernel moves per sample, counted on the device.
//
// This translation unit compiles k_sample (zg_sample_kernel.cuh) a second time with ZG_TOUCH
// defined: every global load of the programs also adds the 32-byte sectors it spans to a per-thread
// count (a sector equal to the thread's previous load's last sector is not counted again), and
// each thread adds its count to one device total at the end.  The loads themselves, their order and
// the results are those of the production kernel.  sectors x 32 / samples is the kernel's bytes per
// sample: the numerator of its roofline (bytes per launch / launch time).  Whether a sector comes
// from L2 or HBM is not known here; ncu's dram__bytes gives that split.
#define ZG_TOUCH 1
#include "zg_sample_kernel.cuh"

ZgProgParams zg_prog_params(const zg_program* p);

int zg_get_variant(int kind, int* variant, int* min_blocks, int* grid);

namespace {

// The counting copy of k_sample under its own name (profiles tell the two apart).
template <int KIND, int MINB, int LAYOUT>
__global__ void __launch_bounds__(kBlock, MINB)
    k_sample_touch(ZgDevGraph g, ZgProgParams pp, uint64_t n, uint64_t first, uint64_t seed,
                   const __grid_constant__ ZgKeys keys, uint32_t stream, ZgPartial* __restrict__ partials) {
  sample_loop<KIND, MINB, LAYOUT>(g, pp, n, first, seed, keys, stream, partials);
}

typedef void (*TouchKernel)(ZgDevGraph, ZgProgParams, uint64_t, uint64_t, uint64_t, const ZgKeys, uint32_t,
                            ZgPartial*);

// Every program's loads are the same under every launch shape except the 4-chain's, whose shapes
// with at most 3 resident blocks interleave two samples per lane: that one follows the shape the
// production kernel uses.
template <int LAYOUT>
TouchKernel touch_kernel(int kind, bool paired) {
  switch (kind) {
    case ZG_PROG_TRIANGLE: return k_sample_touch<ZG_PROG_TRIANGLE, 4, LAYOUT>;
    case ZG_PROG_FOUR_CLIQUE: return k_sample_touch<ZG_PROG_FOUR_CLIQUE, 4, LAYOUT>;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return k_sample_touch<ZG_PROG_FOUR_CLIQUE_UNBIASED, 4, LAYOUT>;
    case ZG_PROG_THREE_CHAIN: return k_sample_touch<ZG_PROG_THREE_CHAIN, 4, LAYOUT>;
    case ZG_PROG_FOUR_CHAIN:
      return paired ? k_sample_touch<ZG_PROG_FOUR_CHAIN, 2, LAYOUT> : k_sample_touch<ZG_PROG_FOUR_CHAIN, 4, LAYOUT>;
    case ZG_PROG_CHAIN: return k_sample_touch<ZG_PROG_CHAIN, 4, LAYOUT>;
    default: return k_sample_touch<ZG_PROG_PATTERN, 4, LAYOUT>;
  }
}

}  // namespace

extern "C" int zg_touch_sectors(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                                uint64_t seed, uint32_t stream_id, void* cuda_stream, uint64_t* sectors) {
  if (!g || !p || !sectors) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_touch_sectors: null argument"), ZG_ERR_INVALID_ARG;
  if (n == 0 || n > (1ull << 32))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_touch_sectors: n must be in [1, 2^32]"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const int layout = g->wide ? 1 : g->packed ? 2 : 0;
  int mb = 4;
  if (p->kind == ZG_PROG_FOUR_CHAIN) {
    int rc = zg_get_variant(ZG_PROG_FOUR_CHAIN, nullptr, &mb, nullptr);
    if (rc) return rc;
  }
  const bool paired = mb <= 3;
  TouchKernel k = layout == 1   ? touch_kernel<1>(p->kind, paired)
                  : layout == 2 ? touch_kernel<2>(p->kind, paired)
                                : touch_kernel<0>(p->kind, paired);
  int per_sm = 0;
  ZG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBlock, 0));
  uint64_t need = (n + kBlock - 1) / kBlock;
  uint64_t grid = (uint64_t)(per_sm > 0 ? per_sm : 1) * zg_num_sms();
  if (grid > need) grid = need;
  ZgPartial* parts = nullptr;
  ZG_CUDA(cudaMalloc((void**)&parts, sizeof(ZgPartial) * grid));
  const unsigned long long zero = 0;
  unsigned long long total = 0;
  cudaError_t ce = cudaMemcpyToSymbolAsync(zg_touch_total, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s);
  if (ce == cudaSuccess) {
    k<<<(unsigned)grid, kBlock, 0, s>>>(g->d, zg_prog_params(p), n, first_sample, seed, zg_round_keys(seed), stream_id,
                                        parts);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyFromSymbolAsync(&total, zg_touch_total, sizeof(total), 0, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  cudaFree(parts);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_touch_sectors");
  *sectors = total;
  return ZG_OK;
}
