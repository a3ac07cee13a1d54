// zg_sample.cu — the sampling kernels and their host entry points on sm_103a.
//
// One estimator per thread on a persistent grid sized to the SM count, running one program of
// zg_programs.cuh; per-block partial sums (exact 32-bit digit lanes) are reduced by a
// single-block finalize kernel in a fixed order.  Also here: the debug kernel (per-sample traces),
// the grouped runs of the error-latency profile, the fused 3-motif kernel, the launch-shape
// variants and their autotuner, and the allocation-free entry point's launcher.
#include <algorithm>
#include <mutex>
#include <vector>

#include "zg_sample_kernel.cuh"

namespace {

template <bool DBG>
__device__ __forceinline__ void run_program(const ZgDevGraph& g, const ZgProgParams& pp, Ctx& c, Res& r) {
  switch (pp.kind) {
    case ZG_PROG_TRIANGLE: prog_triangle<DBG>(g, c, r); break;
    case ZG_PROG_FOUR_CLIQUE: prog_four_clique<DBG>(g, c, r); break;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: prog_four_clique<DBG, true>(g, c, r); break;
    case ZG_PROG_THREE_CHAIN: prog_three_chain<DBG>(g, c, r); break;
    case ZG_PROG_FOUR_CHAIN: prog_four_chain<DBG>(g, c, r); break;
    case ZG_PROG_CHAIN: prog_chain<DBG>(g, (int)pp.param, c, r); break;
    default: prog_pattern<DBG>(g, pp, c, r); break;
  }
}

__global__ void __launch_bounds__(kBlock) k_sample_debug(ZgDevGraph g, ZgProgParams pp, uint64_t n, uint64_t first,
                                                         uint64_t seed, uint32_t stream, ZgPartial* __restrict__ partials,
                                                         zg_sample_trace* __restrict__ traces) {
  Acc a;
  acc_init(a);
  uint64_t stride = (uint64_t)gridDim.x * kBlock;
  for (uint64_t i = blockIdx.x * (uint64_t)kBlock + threadIdx.x; i < n; i += stride) {
    zg_sample_trace* t = &traces[i];
    Ctx c{seed, first + i, stream, 0, t, 0};
    Res r;
    res_init(r);
    run_program<true>(g, pp, c, r);
    acc_add(a, r, pp.den_log2);
    t->ndraws = c.nd;
    t->hit = r.hit;
    t->fail = r.fail;
    t->shift = r.hit ? r.shift : 0;
    t->sectors = c.sectors;
    t->closures = c.closures;
    t->w = r.hit ? r.w : 0.0;
    t->num[0] = r.hit ? r.num.l[0] : 0;
    t->num[1] = r.hit ? r.num.l[1] : 0;
    t->num[2] = r.hit ? (r.ovf ? ~0ull : r.num.l[2]) : 0;
  }
  block_reduce_store<kBlock>(a, &partials[blockIdx.x]);
}

// ---- grouped runs for the error-latency profile ------------------------------------------
// Group gi = samples [first + gi*group, first + (gi+1)*group): the mean of estimate() summed in
// sample order in double and divided by the group size, which is what one-threaded
// calculate(group) returns (src/ZGraphInstance.cpp:273-292).
__global__ void __launch_bounds__(kBlock) k_groups(ZgDevGraph g, ZgProgParams pp, uint64_t n_groups, uint32_t group,
                                                   uint64_t first, uint64_t seed, uint32_t stream,
                                                   double* __restrict__ out) {
  for (uint64_t gi = blockIdx.x * (uint64_t)kBlock + threadIdx.x; gi < n_groups;
       gi += (uint64_t)gridDim.x * kBlock) {
    double acc = 0.0;
    for (uint32_t j = 0; j < group; ++j) {
      Ctx c{seed, first + gi * group + j, stream, 0, nullptr, 0};
      Res r;
      res_init(r);
      run_program<true>(g, pp, c, r);
      acc = __dadd_rn(acc, r.hit ? r.w : 0.0);
    }
    out[gi] = __ddiv_rn(acc, u2d(group));
  }
}

// ---- ThreeMotif: applications/ThreeMotif.cpp:48-121 with the sub-pattern cache ---------
template <bool DBG>
__global__ void __launch_bounds__(kBlock) k_three_motif(ZgDevGraph g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                                                        uint32_t stream_chain, uint32_t stream_tri,
                                                        ZgPartial* __restrict__ pc, ZgPartial* __restrict__ pt,
                                                        zg_sample_trace* __restrict__ tc,
                                                        zg_sample_trace* __restrict__ tt) {
  Acc ac, at;
  acc_init(ac);
  acc_init(at);
  uint64_t n = n_chain > n_tri ? n_chain : n_tri;
  uint64_t stride = (uint64_t)gridDim.x * kBlock;
  for (uint64_t i = blockIdx.x * (uint64_t)kBlock + threadIdx.x; i < n; i += stride) {
    if (i < n_chain) {
      // ThreeChainCountingInstance: keep the wedge; the triangle instance closes it (:54-62)
      Ctx c{seed, i, stream_chain, 0, DBG ? &tc[i] : nullptr, 0};
      uint32_t tri_sectors = 0;
      Res r;
      res_init(r);
      Res rt;
      res_init(rt);
      if (g.m == 0) {
        r.fail = true;
      } else {
        uint64_t e0 = c.draw(0, g.m - 1);
        uint4 q, qp;
        edge_rec(g, e0, q, qp);
        uint64_t S = (uint64_t)q.z + q.w;
        if (DBG) c.sectors += 1 + model_anchor(g, q.x) + model_anchor(g, q.y);
        if (S == 0) {
          r.fail = true;
        } else {
          if (DBG) c.sectors += 1;
          uint64_t r1 = c.draw(0, S - 1);
          const bool on_y = r1 >= q.z;
          if (on_y) r1 -= q.z;
          const uint32_t other = on_y ? q.x : q.y;
          res_mul(r, g.m);
          res_mul(r, S);
          r.hit = true;
          if (i < n_tri) {
            uint2 e1 = ZG_LDG(&g.adj_e[after_edge(g, q, qp, on_y) + (uint32_t)r1]);
            uint32_t a1 = 1 + (e1.x == q.x || e1.x == q.y);
            if (a1 == 2) r.shift = 1;
            rt.hit = a1 == 1 && edge_after(g, other, e1.x, e1.y + 1);
            if (DBG) tri_sectors = model_close(g, other, e1.x);
            rt.num = r.num;
            rt.shift = r.shift;
          }
          if (DBG) {
            double p = 1.0;
            p = dmul(p, ddiv(1.0, u2d(g.m)));
            p = dmul(p, ddiv(1.0, u2d(S)));
            r.w = ddiv(1.0, p);
            rt.w = rt.hit ? r.w : 0.0;
          }
        }
      }
      acc_add(ac, r, 1);
      if (DBG) {
        zg_sample_trace* t = &tc[i];
        t->ndraws = c.nd;
        t->hit = r.hit;
        t->fail = r.fail;
        t->shift = r.hit ? r.shift : 0;
        t->sectors = c.sectors;
        t->closures = c.closures;
        t->w = r.hit ? r.w : 0.0;
        t->num[0] = r.hit ? r.num.l[0] : 0;
        t->num[1] = r.hit ? r.num.l[1] : 0;
        t->num[2] = r.hit ? r.num.l[2] : 0;
      }
      if (i < n_tri) {
        acc_add(at, rt, 1);
        if (DBG) {
          zg_sample_trace* t = &tt[i];
          t->ndraws = 0;
          t->hit = rt.hit;
          t->fail = 0;
          t->shift = rt.hit ? rt.shift : 0;
          t->sectors = tri_sectors;
          t->closures = tri_sectors ? 1 : 0;
          t->w = rt.w;
          t->num[0] = rt.hit ? rt.num.l[0] : 0;
          t->num[1] = rt.hit ? rt.num.l[1] : 0;
          t->num[2] = rt.hit ? rt.num.l[2] : 0;
        }
      }
    } else {
      Ctx c{seed, i, stream_tri, 0, DBG ? &tt[i] : nullptr, 0};
      Res r;
      res_init(r);
      prog_triangle<DBG>(g, c, r);
      acc_add(at, r, 1);
      if (DBG) {
        zg_sample_trace* t = &tt[i];
        t->ndraws = c.nd;
        t->hit = r.hit;
        t->fail = r.fail;
        t->shift = r.hit ? r.shift : 0;
        t->sectors = c.sectors;
        t->closures = c.closures;
        t->w = r.hit ? r.w : 0.0;
        t->num[0] = r.hit ? r.num.l[0] : 0;
        t->num[1] = r.hit ? r.num.l[1] : 0;
        t->num[2] = r.hit ? r.num.l[2] : 0;
      }
    }
  }
  block_reduce_store<kBlock>(ac, &pc[blockIdx.x]);
  __syncthreads();
  block_reduce_store<kBlock>(at, &pt[blockIdx.x]);
}

// Single-block reduction of the per-block partials, fixed order.
__global__ void __launch_bounds__(kBlock) k_finalize(const ZgPartial* __restrict__ parts, int nparts,
                                                     ZgPartial* __restrict__ out) {
  unsigned long long v[12] = {0};
  double d0 = 0, d1 = 0;
  for (int b = threadIdx.x; b < nparts; b += kBlock) {
    const ZgPartial& p = parts[b];
    v[0] += p.samples;
    v[1] += p.hits;
    v[2] += p.fails;
    v[3] += p.overflow;
    for (int i = 0; i < 8; ++i) v[4 + i] += p.lane[i];
    d0 += p.sum_w4;
    d1 += p.sum_w2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    d0 += __shfl_xor_sync(0xffffffffu, d0, o);
    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
  }
  __shared__ unsigned long long sv[kBlock / 32][12];
  __shared__ double sd[kBlock / 32][2];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    for (int i = 0; i < 12; ++i) sv[warp][i] = v[i];
    sd[warp][0] = d0;
    sd[warp][1] = d1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t[12] = {0};
    double s0 = 0, s1 = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
      for (int i = 0; i < 12; ++i) t[i] += sv[w][i];
      s0 += sd[w][0];
      s1 += sd[w][1];
    }
    ZgPartial p;
    p.samples = t[0];
    p.hits = t[1];
    p.fails = t[2];
    p.overflow = t[3];
    for (int i = 0; i < 8; ++i) p.lane[i] = t[4 + i];
    p.sum_w4 = s0;
    p.sum_w2 = s1;
    *out = p;
  }
}

// ---- host side ------------------------------------------------------------------------
typedef unsigned __int128 u128;

// 320-bit value -> correctly rounded double of value / 2^den / n: q = floor(value * 2^128 / n)
// carries 128 fraction bits, the remainder is the sticky bit.
double exact_mean(const uint64_t s[5], uint32_t den, uint64_t n) {
  if (n == 0) return 0.0;
  uint64_t q[7];
  uint64_t x[7] = {0, 0, s[0], s[1], s[2], s[3], s[4]};
  u128 rem = 0;
  for (int i = 6; i >= 0; --i) {
    u128 cur = (rem << 64) | x[i];
    q[i] = (uint64_t)(cur / n);
    rem = cur % n;
  }
  den += 128;
  int top = -1;
  for (int i = 6; i >= 0 && top < 0; --i)
    if (q[i]) top = i * 64 + 63 - __builtin_clzll(q[i]);
  if (top < 0) return 0.0;  // below 2^-128 * 2^-den: no estimator weight is that small
  // take 64 bits from the top, sticky from everything below and the remainder
  auto bit = [&](int k) -> uint64_t { return k < 0 ? 0 : (q[k / 64] >> (k % 64)) & 1ull; };
  uint64_t mant = 0;
  for (int k = top; k > top - 64; --k) mant = (mant << 1) | bit(k);
  bool sticky = rem != 0;
  for (int k = top - 64; k >= 0 && !sticky; --k) sticky = bit(k);
  // round 64 -> 53 bits
  uint64_t keep = mant >> 11, low = mant & 0x7ff;
  int e = top - 63 + 11;
  if (low > 0x400 || (low == 0x400 && (sticky || (keep & 1)))) {
    keep++;
    if (keep == (1ull << 53)) {
      keep >>= 1;
      e++;
    }
  }
  return ldexp((double)keep, e - (int)den);
}

void partial_to_counters(const ZgPartial& p, uint32_t den, zg_counters* out) {
  memset(out, 0, sizeof(*out));
  out->samples = p.samples;
  out->hits = p.hits;
  out->fails = p.fails;
  out->overflow = p.overflow ? 1 : 0;
  out->den_log2 = den;
  u128 carry = 0;
  for (int i = 0; i < 5; ++i) {
    u128 acc = carry;
    // lanes are 32-bit digits: digit k has weight 2^(32k); limb i = digits 2i, 2i+1
    if (2 * i < 8) acc += (u128)p.lane[2 * i];
    if (2 * i + 1 < 8) acc += (u128)p.lane[2 * i + 1] << 32;
    out->sum_num[i] = (uint64_t)acc;
    carry = acc >> 64;
  }
  out->sum_w = exact_mean(out->sum_num, den, 1);  // the exact sum, rounded once
  out->sum_w2 = p.sum_w2;
  out->sum_w4 = p.sum_w4;
  out->estimate = exact_mean(out->sum_num, den, p.samples);
}

uint32_t den_for(const zg_program* p) {
  switch (p->kind) {
    case ZG_PROG_TRIANGLE: return 1;
    case ZG_PROG_FOUR_CLIQUE: return 2;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return 2;
    case ZG_PROG_THREE_CHAIN: return 1;
    case ZG_PROG_FOUR_CHAIN: return 2;
    case ZG_PROG_CHAIN: return p->param - 2;
    default: return p->pe - 1;
  }
}

ZgProgParams params_for(const zg_program* p) {
  ZgProgParams pp;
  pp.kind = p->kind;
  pp.param = p->param;
  pp.pv = p->pv;
  pp.pe = p->pe;
  pp.num_unique = p->num_unique;
  pp.masks = p->d_masks;
  pp.den_log2 = den_for(p);
  return pp;
}

template <typename K>
int grid_of(K kernel) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  return per_sm * zg_num_sms();
}

// Launch-shape variants: __launch_bounds__ min-blocks (register caps 255/128/80/64/48/40/32).
constexpr int kVariants = 7;
constexpr int kMinBlocks[kVariants] = {1, 2, 3, 4, 5, 6, 8};
typedef void (*SampleKernel)(ZgDevGraph, ZgProgParams, uint64_t, uint64_t, uint64_t, const ZgKeys, uint32_t,
                             ZgPartial*);

template <int KIND, int LAYOUT>
SampleKernel kernel_variant(int v) {
  switch (v) {
    case 0: return k_sample<KIND, 1, LAYOUT>;
    case 1: return k_sample<KIND, 2, LAYOUT>;
    case 2: return k_sample<KIND, 3, LAYOUT>;
    case 3: return k_sample<KIND, 4, LAYOUT>;
    case 4: return k_sample<KIND, 5, LAYOUT>;
    case 5: return k_sample<KIND, 6, LAYOUT>;
    default: return k_sample<KIND, 8, LAYOUT>;
  }
}

template <int LAYOUT>
SampleKernel kernel_for_layout(int kind, int v) {
  switch (kind) {
    case ZG_PROG_TRIANGLE: return kernel_variant<ZG_PROG_TRIANGLE, LAYOUT>(v);
    case ZG_PROG_FOUR_CLIQUE: return kernel_variant<ZG_PROG_FOUR_CLIQUE, LAYOUT>(v);
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return kernel_variant<ZG_PROG_FOUR_CLIQUE_UNBIASED, LAYOUT>(v);
    case ZG_PROG_THREE_CHAIN: return kernel_variant<ZG_PROG_THREE_CHAIN, LAYOUT>(v);
    case ZG_PROG_FOUR_CHAIN: return kernel_variant<ZG_PROG_FOUR_CHAIN, LAYOUT>(v);
    case ZG_PROG_CHAIN: return kernel_variant<ZG_PROG_CHAIN, LAYOUT>(v);
    default: return kernel_variant<ZG_PROG_PATTERN, LAYOUT>(v);
  }
}

SampleKernel kernel_for(int kind, int v, int layout) {
  return layout == 1 ? kernel_for_layout<1>(kind, v) : layout == 2 ? kernel_for_layout<2>(kind, v)
                                                                  : kernel_for_layout<0>(kind, v);
}

// The record layout a graph's sampling kernels are compiled for: 0 compact, 1 wide, 2 packed.
int rec_layout(const zg_graph* g) { return g->wide ? 1 : g->packed ? 2 : 0; }

// Per device: the variant each program kind uses and its occupancy grid.
constexpr int kMaxDev = 64;
std::mutex g_tune_mu;
int g_variant[kMaxDev][8];
int g_grid[kMaxDev][8][kVariants][3];
bool g_tune_init[kMaxDev];
// Defaults before tuning (register footprints measured with -Xptxas -v).
constexpr int kDefaultVariant[8] = {3, 3, 2, 3, 2, 3, 3, 3};

// The tuning tables hold kMaxDev devices.  Every entry point checks the current device first
// (check_device) and refuses one beyond the tables rather than give it another device's launch
// shapes; current_device() is only reached after that check.
int check_device() {
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return zg_check_cuda(e, "cudaGetDevice");
  if (d < 0 || d >= kMaxDev)
    return zg_set_error(ZG_ERR_INVALID_ARG, "device %d is beyond the %d devices the library tracks", d, kMaxDev),
           ZG_ERR_INVALID_ARG;
  return ZG_OK;
}

int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return (d >= 0 && d < kMaxDev) ? d : 0;
}

int kind_slot(int kind) { return (kind >= 0 && kind < 8) ? kind : ZG_PROG_PATTERN; }

int variant_for(int kind) {
  int d = current_device();
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (!g_tune_init[d]) {
    for (int k = 0; k < 8; ++k) g_variant[d][k] = kDefaultVariant[k];
    g_tune_init[d] = true;
  }
  return g_variant[d][kind_slot(kind)];
}

// Blocks per launch over the resident ones, per record layout (compact, wide, packed).  On
// wide-record graphs (read from HBM) SMs progress at different rates, and a grid of exactly the
// resident blocks gives each SM a fixed share: the launch waits for the slowest one.  With many
// times the resident blocks, each short, the block scheduler hands the remaining blocks to
// whichever SM frees up first and the last wave is short.  Measured on GB300, R-MAT 26, 4-clique
// per 2^30 samples: 134.1 ms (1x), 117.8 ms (6x), 112.5 ms (24x, as fast as the batch kernel's
// work queue); triangle per 2^28: 33.2, 29.3, 27.8 ms; Chung-Lu 42 M edges, the four programs
// per 2^26 each: 16.2 ms (1x), 14.5 ms (6x and 24x).  On near-L2 graphs (compact, packed records)
// the extra blocks cost more than they balance (R-MAT 20: 5.75 -> 5.86 ms at 6x), so those launch
// the resident blocks only.  Every grid stays within the no-allocation entry point's fixed
// scratch (ZG_NOALLOC_MAX_BLOCKS partials).
constexpr int kOversubscribe[3] = {1, 24, 1};

int grid_for_variant(int kind, int v, int layout) {
  int d = current_device();
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int& g = g_grid[d][kind_slot(kind)][v][layout];
  if (!g) g = std::min(grid_of(kernel_for(kind, v, layout)) * kOversubscribe[layout], (int)ZG_NOALLOC_MAX_BLOCKS);
  return g;
}

int grid_for_kind(int kind, int layout) { return grid_for_variant(kind, variant_for(kind), layout); }

int validate_run(const zg_graph* g, const zg_program* p) {
  if (!g || !p) return zg_set_error(ZG_ERR_INVALID_ARG, "null graph or program"), ZG_ERR_INVALID_ARG;
  return check_device();
}

int launch_variant(const zg_graph* g, const zg_program* p, int v, uint64_t n, uint64_t first, uint64_t seed,
                   uint32_t stream_id, cudaStream_t s, ZgPartial* parts, int grid) {
  ZgProgParams pp = params_for(p);
  SampleKernel k = kernel_for(p->kind, v, rec_layout(g));
  k<<<grid, kBlock, 0, s>>>(g->d, pp, n, first, seed, zg_round_keys(seed), stream_id, parts);
  return ZG_OK;
}

int launch_sample(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first, uint64_t seed,
                  uint32_t stream_id, cudaStream_t s, ZgPartial* parts, int grid) {
  return launch_variant(g, p, variant_for(p->kind), n, first, seed, stream_id, s, parts, grid);
}

}  // namespace

// Counters of a reduced partial, for other translation units.
void zg_partial_to_counters(const void* partial, uint32_t den, zg_counters* out) {
  partial_to_counters(*static_cast<const ZgPartial*>(partial), den, out);
}

// The exact mean of a 320-bit sum, for other translation units.
double zg_exact_mean_host(const uint64_t s[5], uint32_t den, uint64_t n) { return exact_mean(s, den, n); }

// Shared by the allocation-free entry points of other translation units (after zg_check_device).
int zg_sample_grid(int kind, int layout) { return grid_for_kind(kind, layout); }
int zg_check_device() { return check_device(); }

// A program's kernel parameters, for other translation units.
ZgProgParams zg_prog_params(const zg_program* p) { return params_for(p); }

// Per-group estimates (device array out[n_groups]) on stream s.
int zg_launch_groups(const zg_graph* g, const zg_program* p, uint64_t n_groups, uint32_t group, uint64_t first,
                     uint64_t seed, uint32_t stream_id, cudaStream_t s, double* out) {
  ZgProgParams pp = params_for(p);
  uint64_t blocks = (n_groups + kBlock - 1) / kBlock;
  int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)zg_num_sms() * 8));
  k_groups<<<grid, kBlock, 0, s>>>(g->d, pp, n_groups, group, first, seed, stream_id, out);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "grouped run");
  return ZG_OK;
}

// Enqueues the sampling and finalize kernels with caller-provided block scratch (grid blocks of
// ZgPartial) and result slot; allocates nothing.
int zg_launch_sample_with_scratch(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first, uint64_t seed,
                                  uint32_t stream_id, cudaStream_t s, ZgPartial* scratch, int grid, void* d_result) {
  launch_sample(g, p, n, first, seed, stream_id, s, scratch, grid);
  k_finalize<<<1, kBlock, 0, s>>>(scratch, grid, (ZgPartial*)d_result);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "sampling launch");
  return ZG_OK;
}

extern "C" int zg_run(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample, uint64_t seed,
                      uint32_t stream_id, void* cuda_stream, zg_counters* out) {
  int rc = validate_run(g, p);
  if (rc) return rc;
  if (!out) return zg_set_error(ZG_ERR_INVALID_ARG, "null output"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  uint64_t maxg = (n + kBlock - 1) / kBlock;
  int grid = grid_for_kind(p->kind, rec_layout(g));
  if ((uint64_t)grid > maxg) grid = (int)(maxg ? maxg : 1);
  ZgPartial* parts = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&parts, sizeof(ZgPartial) * (grid + 1), s));
  launch_sample(g, p, n, first_sample, seed, stream_id, s, parts, grid);
  k_finalize<<<1, kBlock, 0, s>>>(parts, grid, parts + grid);
  ZgPartial h;
  cudaError_t ce = cudaMemcpyAsync(&h, parts + grid, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(parts, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_run");
  partial_to_counters(h, den_for(p), out);
  return ZG_OK;
}

static_assert(sizeof(ZgPartial) == ZG_RESULT_BYTES, "result layout");

extern "C" int zg_run_async(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                            uint64_t seed, uint32_t stream_id, void* cuda_stream, void* d_result) {
  int rc = validate_run(g, p);
  if (rc) return rc;
  if (!d_result) return zg_set_error(ZG_ERR_INVALID_ARG, "null device result"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  uint64_t maxg = (n + kBlock - 1) / kBlock;
  int grid = grid_for_kind(p->kind, rec_layout(g));
  if ((uint64_t)grid > maxg) grid = (int)(maxg ? maxg : 1);
  ZgPartial* parts = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&parts, sizeof(ZgPartial) * grid, s));
  launch_sample(g, p, n, first_sample, seed, stream_id, s, parts, grid);
  k_finalize<<<1, kBlock, 0, s>>>(parts, grid, (ZgPartial*)d_result);
  cudaFreeAsync(parts, s);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_run_async");
  return ZG_OK;
}

extern "C" int zg_set_variant(int kind, int variant) {
  if (variant < 0 || variant >= kVariants)
    return zg_set_error(ZG_ERR_INVALID_ARG, "launch variant %d outside [0, %d)", variant, kVariants), ZG_ERR_INVALID_ARG;
  if (kind < ZG_PROG_TRIANGLE || kind > ZG_PROG_FOUR_CLIQUE_UNBIASED)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown program kind %d", kind), ZG_ERR_INVALID_ARG;
  if (int rc = check_device()) return rc;
  variant_for(kind);  // initialise the table
  int d = current_device();
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_variant[d][kind] = variant;
  return ZG_OK;
}

extern "C" int zg_get_variant(int kind, int* variant, int* min_blocks, int* grid) {
  if (kind < ZG_PROG_TRIANGLE || kind > ZG_PROG_FOUR_CLIQUE_UNBIASED)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown program kind %d", kind), ZG_ERR_INVALID_ARG;
  if (int rc = check_device()) return rc;
  int v = variant_for(kind);
  if (variant) *variant = v;
  if (min_blocks) *min_blocks = kMinBlocks[v];
  if (grid) *grid = grid_for_variant(kind, v, false);
  return ZG_OK;
}

// Autotuner: times every launch variant of p's kernel on g (probe_samples estimators each, best
// of `reps`, CUDA events on cuda_stream) and keeps the fastest for this device and program kind.
extern "C" int zg_tune(const zg_graph* g, const zg_program* p, uint64_t probe_samples, void* cuda_stream,
                       int* best_variant, float* ms_per_variant) {
  int rc = validate_run(g, p);
  if (rc) return rc;
  if (probe_samples == 0) probe_samples = 1ull << 22;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  int grid_max = 0;
  for (int v = 0; v < kVariants; ++v) grid_max = std::max(grid_max, grid_for_variant(p->kind, v, rec_layout(g)));
  ZgPartial* parts = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&parts, sizeof(ZgPartial) * (grid_max + 1), s));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bestv = variant_for(p->kind);
  const int reps = 3;
  cudaError_t ce = cudaSuccess;
  for (int v = 0; v < kVariants && ce == cudaSuccess; ++v) {
    int grid = grid_for_variant(p->kind, v, rec_layout(g));
    uint64_t maxg = (probe_samples + kBlock - 1) / kBlock;
    if ((uint64_t)grid > maxg) grid = (int)maxg;
    float vbest = 1e30f;
    launch_variant(g, p, v, probe_samples, 0, 1, 0, s, parts, grid);  // warm
    for (int r = 0; r < reps; ++r) {
      cudaEventRecord(e0, s);
      launch_variant(g, p, v, probe_samples, (uint64_t)(r + 1) * probe_samples, 1, 0, s, parts, grid);
      cudaEventRecord(e1, s);
      ce = cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      vbest = std::min(vbest, ms);
    }
    if (ms_per_variant) ms_per_variant[v] = vbest;
    if (vbest < best) {
      best = vbest;
      bestv = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(parts, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_tune");
  {
    int d = current_device();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_variant[d][kind_slot(p->kind)] = bestv;
  }
  if (best_variant) *best_variant = bestv;
  return ZG_OK;
}

extern "C" int zg_result_to_counters(const void* h_result, const zg_program* p, zg_counters* out) {
  if (!h_result || !p || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  ZgPartial h;
  memcpy(&h, h_result, sizeof(h));
  partial_to_counters(h, den_for(p), out);
  return ZG_OK;
}

extern "C" int zg_run_debug(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                            uint64_t seed, uint32_t stream_id, zg_sample_trace* traces) {
  int rc = validate_run(g, p);
  if (rc) return rc;
  if (!traces && n) return zg_set_error(ZG_ERR_INVALID_ARG, "null traces"), ZG_ERR_INVALID_ARG;
  if (n > (1ull << 22)) return zg_set_error(ZG_ERR_TOO_LARGE, "debug runs take at most 2^22 samples"), ZG_ERR_TOO_LARGE;
  int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((n + kBlock - 1) / kBlock, 4096));
  ZgPartial* parts = nullptr;
  zg_sample_trace* dt = nullptr;
  ZG_CUDA(cudaMalloc((void**)&parts, sizeof(ZgPartial) * (grid + 1)));
  cudaError_t ce = cudaMalloc((void**)&dt, sizeof(zg_sample_trace) * (n ? n : 1));
  if (ce != cudaSuccess) {
    cudaFree(parts);
    return zg_check_cuda(ce, "debug traces");
  }
  ce = cudaMemset(dt, 0, sizeof(zg_sample_trace) * (n ? n : 1));
  ZgProgParams pp = params_for(p);
  k_sample_debug<<<grid, kBlock>>>(g->d, pp, n, first_sample, seed, stream_id, parts, dt);
  if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce == cudaSuccess && n) ce = cudaMemcpy(traces, dt, sizeof(zg_sample_trace) * n, cudaMemcpyDeviceToHost);
  cudaFree(parts);
  cudaFree(dt);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_run_debug");
  return ZG_OK;
}

static int run_motif(const zg_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed, uint32_t sc, uint32_t st,
                     cudaStream_t s, zg_counters* oc, zg_counters* ot, zg_sample_trace* tc, zg_sample_trace* tt) {
  if (!g) return zg_set_error(ZG_ERR_INVALID_ARG, "null graph"), ZG_ERR_INVALID_ARG;
  bool dbg = tc || tt;
  uint64_t n = std::max(n_chain, n_tri);
  if (dbg && n > (1ull << 22)) return zg_set_error(ZG_ERR_TOO_LARGE, "debug runs take at most 2^22 samples"), ZG_ERR_TOO_LARGE;
  if (dbg && (!tc || !tt)) return zg_set_error(ZG_ERR_INVALID_ARG, "both trace arrays are required"), ZG_ERR_INVALID_ARG;
  int grid = dbg ? (int)std::max<uint64_t>(1, std::min<uint64_t>((n + kBlock - 1) / kBlock, 4096))
                 : std::min<int>(grid_of(k_three_motif<false>), (int)std::max<uint64_t>(1, (n + kBlock - 1) / kBlock));
  ZgPartial* parts = nullptr;
  zg_sample_trace *dtc = nullptr, *dtt = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&parts, sizeof(ZgPartial) * (2 * grid + 2), s));
  cudaError_t ce = cudaSuccess;
  if (dbg) {
    ce = zg_malloc_async((void**)&dtc, sizeof(zg_sample_trace) * (n_chain ? n_chain : 1), s);
    if (ce == cudaSuccess) ce = zg_malloc_async((void**)&dtt, sizeof(zg_sample_trace) * (n_tri ? n_tri : 1), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(dtc, 0, sizeof(zg_sample_trace) * (n_chain ? n_chain : 1), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(dtt, 0, sizeof(zg_sample_trace) * (n_tri ? n_tri : 1), s);
  }
  if (ce == cudaSuccess) {
    if (dbg)
      k_three_motif<true><<<grid, kBlock, 0, s>>>(g->d, n_chain, n_tri, seed, sc, st, parts, parts + grid, dtc, dtt);
    else
      k_three_motif<false><<<grid, kBlock, 0, s>>>(g->d, n_chain, n_tri, seed, sc, st, parts, parts + grid, nullptr,
                                                   nullptr);
    k_finalize<<<1, kBlock, 0, s>>>(parts, grid, parts + 2 * grid);
    k_finalize<<<1, kBlock, 0, s>>>(parts + grid, grid, parts + 2 * grid + 1);
  }
  ZgPartial h[2];
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(h, parts + 2 * grid, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess && dbg && n_chain)
    ce = cudaMemcpyAsync(tc, dtc, sizeof(zg_sample_trace) * n_chain, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess && dbg && n_tri)
    ce = cudaMemcpyAsync(tt, dtt, sizeof(zg_sample_trace) * n_tri, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(parts, s);
  if (dtc) cudaFreeAsync(dtc, s);
  if (dtt) cudaFreeAsync(dtt, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "three motif");
  if (oc) partial_to_counters(h[0], 1, oc);
  if (ot) partial_to_counters(h[1], 1, ot);
  return ZG_OK;
}

extern "C" int zg_run_three_motif(const zg_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                                  uint32_t stream_chain, uint32_t stream_tri, void* cuda_stream, zg_counters* out_chain,
                                  zg_counters* out_tri) {
  return run_motif(g, n_chain, n_tri, seed, stream_chain, stream_tri, (cudaStream_t)cuda_stream, out_chain, out_tri,
                   nullptr, nullptr);
}

extern "C" int zg_run_three_motif_debug(const zg_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                                        uint32_t stream_chain, uint32_t stream_tri, zg_sample_trace* chain_traces,
                                        zg_sample_trace* tri_traces) {
  zg_counters a, b;
  return run_motif(g, n_chain, n_tri, seed, stream_chain, stream_tri, nullptr, &a, &b, chain_traces, tri_traces);
}
