// zg_elp.cu — error-latency profiles and bounded queries on the device.
//
//   zg_elp_plain     ErrorProfile<E>::get_num_estimators (src/ErrorLatencyProfile.cpp:72-207): 10 %
//                    edge subsample (zg_graph_subsample), 2^14 groups of 16 estimators plus 2^23
//                    estimators in two launches instead of 2^14 + 1 calculate() calls, then the
//                    moving-average regression and the Chernoff-style bound, host side.
//   zg_elp_solve     the host half alone (testable without a GPU).
//   zg_time_profile  TimeProfile<E>::run (:25-47): doubling runs under a wall-clock budget.
//   zg_query         run a budget, check the answer's empirical CLT half-width at the requested
//                    confidence and keep sampling until the bound holds: the delivered error never
//                    depends on how the budget was chosen.
#include <math.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "zg_internal.cuh"

int zg_graph_filter_sampling(const zg_graph* g, int pred_op, int64_t t0, int64_t t1, uint64_t shuffle_seed,
                             cudaStream_t s, uint64_t* out_m, zg_graph** out);
int zg_graph_subsample_sampling(const zg_graph* g, double rate, uint64_t keep_seed, uint64_t shuffle_seed,
                                cudaStream_t s, uint64_t* out_m, zg_graph** out);
int zg_launch_groups(const zg_graph* g, const zg_program* p, uint64_t n_groups, uint32_t group, uint64_t first,
                     uint64_t seed, uint32_t stream_id, cudaStream_t s, double* out);
double zg_exact_mean_host(const uint64_t s[5], uint32_t den, uint64_t n);

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Estimation::update (src/ZGraphInstance.cpp:24-27)
struct Est {
  unsigned long long n = 0;
  double cur = 0;
  void update(unsigned long long k, double v) {
    cur = (1. * n / (n + k)) * cur + (1. * k / (n + k)) * v;
    n += k;
  }
};

// Acklam's rational approximation of the standard normal quantile (relative error < 1.2e-9),
// refined by one Halley step on erfc.
double normal_quantile(double p) {
  static const double a[6] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                              1.383577518672690e+02,  -3.066479806614716e+01, 2.506628277459239e+00};
  static const double b[5] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                              6.680131188771972e+01,  -1.328068155288572e+01};
  static const double c[6] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                              -2.549732539343734e+00, 4.374664141464968e+00,  2.938163982698783e+00};
  static const double d[4] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                              3.754408661907416e+00};
  double q, r, x;
  if (p < 0.02425) {
    q = sqrt(-2 * log(p));
    x = (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
        ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
  } else if (p > 1 - 0.02425) {
    q = sqrt(-2 * log(1 - p));
    x = -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
        ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
  } else {
    q = p - 0.5;
    r = q * q;
    x = (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
        (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1);
  }
  double e = 0.5 * erfc(-x / sqrt(2.0)) - p;
  double u = e * sqrt(2 * M_PI) * exp(x * x / 2);
  return x - u / (1 + x * u / 2);
}

}  // namespace

// ErrorProfile::calculate_bound (src/ErrorLatencyProfile.cpp:52-59)
extern "C" double zg_calculate_bound(double epsilon, double delta, double nse, double ncse, double estimation,
                                     uint64_t max_degree, uint64_t num_edges) {
  double factor_0 = 1. / pow(epsilon, 2.);
  double factor_1 = pow(double(max_degree), ncse) * pow(double(num_edges), nse) / estimation;
  double factor_2 = log(2. / delta);
  return factor_0 * factor_1 * factor_2;
}

extern "C" double zg_normal_quantile(double p) { return normal_quantile(p); }

// The host half of get_num_estimators (:115-206) on given group estimates, with the reference's
// long double intermediates (UnbiasedLinearRegression::solve, src/Regression.cpp:17-28).
extern "C" int zg_elp_solve(const double* groups, uint64_t n_groups, uint32_t group_size, double big_estimate,
                            uint64_t big_n, double nse, double ncse, uint64_t sampled_m, uint64_t sampled_max_degree,
                            uint64_t orig_m, uint64_t orig_max_degree, double eps, double conf, zg_elp_result* out) {
  if (!groups || !out || n_groups == 0 || group_size == 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_elp_solve: empty input"), ZG_ERR_INVALID_ARG;
  std::vector<long double> estimations(n_groups), X(n_groups), Y(n_groups);
  Est estimation;
  for (uint64_t i = 0; i < n_groups; ++i) {
    long double v = groups[i];
    estimation.update(group_size, (double)v);
    estimations[i] = estimation.cur;
  }
  estimation.update(big_n, big_estimate);
  const double est = estimation.cur;
  long double ema = 100;
  const double error_times = 1, alpha = 0.04;
  for (uint64_t i = 0; i < n_groups; ++i) {
    long double error = (estimations[i] - est) / est * 5;
    if (error < 0) error = -error;
    ema = ema * (1 - alpha) + error * alpha;
    double x_tmp = zg_calculate_bound((double)(ema * error_times), 1 - conf, nse, ncse, est, sampled_max_degree,
                                      sampled_m) *
                   pow(ema * error_times, 2);
    X[i] = sqrt(x_tmp / ((i + 1) * (unsigned long long)group_size));
    Y[i] = ema;
  }
  long double t0 = 0, t1 = 0;
  for (uint64_t i = 0; i < n_groups; ++i) t0 += X[i] * Y[i];
  for (uint64_t i = 0; i < n_groups; ++i) t1 += X[i] * X[i];
  double K = (double)(t0 / t1);
  long double sample_rate = 0.1;
  long double rough = est / pow(sample_rate, nse + ncse);
  double n = zg_calculate_bound(eps, 1. - conf, nse, ncse, (double)rough, orig_max_degree, orig_m);
  n *= (K * K);
  memset(out, 0, sizeof(*out));
  out->n_required = (uint64_t)n;
  out->n_required_f = n;
  out->K = K;
  out->estimate_sampled = est;
  out->rough_estimate = (double)rough;
  out->nse = nse;
  out->ncse = ncse;
  out->sampled_edges = sampled_m;
  out->sampled_max_degree = sampled_max_degree;
  return ZG_OK;
}

extern "C" int zg_run_groups(const zg_graph* g, const zg_program* p, uint64_t n_groups, uint32_t group_size,
                             uint64_t first_sample, uint64_t seed, uint32_t stream_id, void* cuda_stream,
                             double* group_estimates) {
  if (!g || !p || (n_groups && !group_estimates) || group_size == 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_run_groups: invalid argument"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  double* d = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&d, sizeof(double) * (n_groups ? n_groups : 1), s));
  int rc = zg_launch_groups(g, p, n_groups, group_size, first_sample, seed, stream_id, s, d);
  cudaError_t ce = cudaSuccess;
  if (rc == ZG_OK && n_groups)
    ce = cudaMemcpyAsync(group_estimates, d, sizeof(double) * n_groups, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (rc) return rc;
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_run_groups");
  return ZG_OK;
}

extern "C" int zg_elp_plain(const zg_graph* g, const zg_program* p, int pred_op, int64_t t0, int64_t t1, double eps,
                            double conf, uint64_t seed, void* cuda_stream, zg_elp_result* out,
                            double* group_estimates) {
  if (!g || !p || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_elp_plain: null argument"), ZG_ERR_INVALID_ARG;
  if (!(eps > 0) || !(conf > 0 && conf < 1))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_elp_plain: error %g / confidence %g", eps, conf), ZG_ERR_INVALID_ARG;
  double tstart = now_ms();
  uint32_t cc = 0;
  zg_program_info(p, nullptr, &cc, nullptr);
  const double nse = 1.0, ncse = (double)cc;
  const uint64_t n_groups = 1ull << 14, big_n = 1ull << 23;
  const uint32_t group = 16;
  zg_graph *sub = nullptr, *fsub = nullptr;
  uint64_t m_s = 0;
  int rc = zg_graph_subsample_sampling(g, 0.1, seed + ZG_ELP_KEEP_OFFSET, seed + ZG_ELP_SHUFFLE_OFFSET,
                                       (cudaStream_t)cuda_stream, &m_s, &sub);
  if (rc) return rc;
  const zg_graph* run_g = sub;
  if (pred_op) {
    uint64_t mf = 0;
    rc = zg_graph_filter_sampling(sub, pred_op, t0, t1, seed + ZG_ELP_FILTER_OFFSET, (cudaStream_t)cuda_stream, &mf,
                                  &fsub);
    if (rc) {
      zg_graph_free(sub);
      return rc;
    }
    run_g = fsub;
  }
  std::vector<double> groups(n_groups);
  rc = zg_run_groups(run_g, p, n_groups, group, 0, seed, ZG_ELP_STREAM, cuda_stream, groups.data());
  zg_counters big;
  if (rc == ZG_OK) rc = zg_run(run_g, p, big_n, n_groups * group, seed, ZG_ELP_STREAM, cuda_stream, &big);
  if (rc == ZG_OK) {
    rc = zg_elp_solve(groups.data(), n_groups, group, big.estimate, big_n, nse, ncse, sub->num_edges,
                      sub->max_degree, g->num_edges, g->max_degree, eps, conf, out);
    if (group_estimates) memcpy(group_estimates, groups.data(), sizeof(double) * n_groups);
    out->big_estimate = big.estimate;
  }
  if (fsub) zg_graph_free(fsub);
  zg_graph_free(sub);
  out->profile_ms = now_ms() - tstart;
  return rc;
}

extern "C" int zg_time_profile(const zg_graph* g, const zg_program* p, uint32_t time_limit_ms, uint64_t seed,
                               uint32_t stream_id, void* cuda_stream, double* estimate, uint64_t* samples_used) {
  if (!g || !p || !estimate) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_time_profile: null argument"), ZG_ERR_INVALID_ARG;
  Est est;
  unsigned int used_time = 0, curr_used_time = 0;
  unsigned long long next = 64;  // BASIC_NUM_ESTIMATORS_PER_THREAD x one sampling "thread" (the device)
  uint64_t cursor = 0;
  zg_counters c;
  while (used_time + curr_used_time * 2 <= time_limit_ms && next < (1ull << 40)) {
    double t = now_ms();
    int rc = zg_run(g, p, next, cursor, seed, stream_id, cuda_stream, &c);
    if (rc) return rc;
    t = now_ms() - t;
    cursor += next;
    est.update(next, c.estimate);
    next <<= 1;
    curr_used_time = (unsigned int)t;
    used_time += curr_used_time;
  }
  if (curr_used_time > 0 && used_time < time_limit_ms) {
    unsigned long long remained = next * (time_limit_ms - used_time) / (curr_used_time * 2);
    if (remained) {
      int rc = zg_run(g, p, remained, cursor, seed, stream_id, cuda_stream, &c);
      if (rc) return rc;
      cursor += remained;
      est.update(remained, c.estimate);
    }
  }
  *estimate = est.cur;
  if (samples_used) *samples_used = cursor;
  return ZG_OK;
}

// The largest weight one estimator of this program can carry on g (the Bernstein bound's range):
// m (3m for the four-chain) times, per conditional step i, at most min((i + 1) max_degree, 2m).
int zg_weight_range(const zg_graph* g, int kind, uint32_t param, uint32_t pattern_edges, cudaStream_t s,
                    double* range) {
  uint64_t dmax = 0;
  int rc = zg_graph_max_degree(g, s, &dmax);
  if (rc) return rc;
  uint32_t steps;  // conditional_sample_edge calls after the first sample_edge
  switch (kind) {
    case ZG_PROG_TRIANGLE:
    case ZG_PROG_THREE_CHAIN: steps = 1; break;
    case ZG_PROG_FOUR_CLIQUE:
    case ZG_PROG_FOUR_CLIQUE_UNBIASED:
    case ZG_PROG_FOUR_CHAIN: steps = 2; break;
    case ZG_PROG_CHAIN: steps = param >= 2 ? param - 2 : 0; break;
    default: steps = pattern_edges ? pattern_edges - 1 : 0; break;
  }
  const double m = (double)g->d.m;
  double r = (kind == ZG_PROG_FOUR_CHAIN ? 3.0 : 1.0) * m;
  for (uint32_t i = 1; i <= steps; ++i) r *= std::min((double)(i + 1) * (double)dmax, 2.0 * m);
  *range = r;
  return ZG_OK;
}

double zg_variance_bound(double mean, double var, double ew4, uint64_t n, double conf) {
  // unknown (0) or overflowed (weights past 1e77): no inflation, the plain variance
  if (n == 0 || !(ew4 > 0) || !isfinite(ew4)) return var;
  const double z = normal_quantile(1.0 - (1.0 - conf) / 2.0);
  const double m4 = ew4 + 2.0 * mean * mean * var;  // >= the fourth central moment for w >= 0
  const double spread = m4 - var * var;
  return spread > 0 ? var + z * sqrt(spread / (double)n) : var;
}

bool zg_bound_check(double mean, double var, double ew4, uint64_t n, uint64_t hits, double eps, double conf,
                    double range, double* half, uint32_t* method) {
  const double z = normal_quantile(1.0 - (1.0 - conf) / 2.0);
  const double x = log(3.0 / (1.0 - conf));
  const double dn = (double)n;
  const double bern = n ? sqrt(2.0 * var * x / dn) + 3.0 * range * x / dn : INFINITY;
  const double clt = n ? z * sqrt(zg_variance_bound(mean, var, ew4, n, conf) / dn) : INFINITY;
  if (hits >= 30 && clt <= bern) {
    *half = clt;
    *method = ZG_BOUND_CLT;
  } else {
    *half = bern;
    *method = ZG_BOUND_BERNSTEIN;
  }
  return mean > 0 && *half <= eps * mean;
}

extern "C" int zg_bound_half_width(double mean, double var, double fourth_moment, uint64_t n, uint64_t hits,
                                   double error, double confidence, double weight_range, double* half_width,
                                   uint32_t* method, uint32_t* met) {
  if (!half_width || !method || !met || !(confidence > 0 && confidence < 1) || !(error > 0) || var < 0 ||
      fourth_moment < 0 || weight_range < 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_bound_half_width: invalid argument"), ZG_ERR_INVALID_ARG;
  *met = zg_bound_check(mean, var, fourth_moment, n, hits, error, confidence, weight_range, half_width, method) ? 1 : 0;
  return ZG_OK;
}

double zg_samples_needed(double mean, double var, double ew4, uint64_t n, uint64_t hits, double eps, double conf) {
  if (hits < 30 || !(mean > 0)) return 2.0 * (double)n;
  const double z = normal_quantile(1.0 - (1.0 - conf) / 2.0);
  const double v = zg_variance_bound(mean, var, ew4, n, conf);
  return z * z * v / (eps * eps * mean * mean) * (1.0 + 0.5 / sqrt((double)hits));
}

// Bounded query: sample n_initial estimators (the sizing step's budget), then check the answer with
// zg_bound_check at `conf`; while its half-width exceeds eps * estimate, extend with more estimators
// (never reusing sample indices) sized by zg_samples_needed, up to max_samples.
extern "C" int zg_query(const zg_graph* g, const zg_program* p, double eps, double conf, uint64_t n_initial,
                        uint64_t max_samples, uint64_t seed, uint32_t stream_id, void* cuda_stream,
                        zg_query_result* out) {
  if (!g || !p || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_query: null argument"), ZG_ERR_INVALID_ARG;
  if (!(eps > 0) || !(conf > 0 && conf < 1))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_query: error %g / confidence %g", eps, conf), ZG_ERR_INVALID_ARG;
  double tstart = now_ms();
  memset(out, 0, sizeof(*out));
  double range = 0;
  int rc = zg_weight_range(g, p->kind, p->param, p->pe, (cudaStream_t)cuda_stream, &range);
  if (rc) return rc;
  out->weight_range = range;
  uint64_t n_total = 0, hits = 0;
  uint64_t sum[5] = {0, 0, 0, 0, 0};
  uint32_t den = 0;
  double sw2 = 0, sw4 = 0;
  uint64_t next = std::max<uint64_t>(n_initial, 1ull << 16);
  if (max_samples == 0) max_samples = 1ull << 40;
  for (uint32_t round = 0; round < 64; ++round) {
    next = std::min(next, max_samples - n_total);
    if (next == 0) break;
    zg_counters c;
    rc = zg_run(g, p, next, n_total, seed, stream_id, cuda_stream, &c);
    if (rc) return rc;
    // a weight past 192 bits makes the sums inexact: no bound can be claimed on them (programs
    // with at most six weight factors, every factor below 2^32, never get here)
    if (c.overflow)
      return zg_set_error(ZG_ERR_OVERFLOW, "zg_query: an estimator's exact weight exceeded 192 bits"), ZG_ERR_OVERFLOW;
    den = c.den_log2;
    unsigned __int128 carry = 0;
    for (int i = 0; i < 5; ++i) {
      unsigned __int128 s = (unsigned __int128)sum[i] + c.sum_num[i] + carry;
      sum[i] = (uint64_t)s;
      carry = s >> 64;
    }
    n_total += next;
    hits += c.hits;
    sw2 += c.sum_w2;
    sw4 += c.sum_w4;
    out->rounds = round + 1;
    // exact mean of all samples, then the empirical variance
    double mean = zg_exact_mean_host(sum, den, n_total);
    double var = sw2 / (double)n_total - mean * mean;
    if (var < 0) var = 0;
    double half = INFINITY;
    uint32_t method = 0;
    const double ew4 = sw4 / (double)n_total;
    const bool met = zg_bound_check(mean, var, ew4, n_total, hits, eps, conf, range, &half, &method);
    out->estimate = mean;
    out->half_width = half;
    out->rel_half_width = mean > 0 ? half / mean : INFINITY;
    out->bound_method = method;
    out->samples = n_total;
    out->hits = hits;
    if (met) {
      out->bound_met = 1;
      break;
    }
    double need = zg_samples_needed(mean, var, ew4, n_total, hits, eps, conf);
    uint64_t want = need > 1e15 ? (uint64_t)1e15 : (uint64_t)need;
    next = want > n_total ? want - n_total : n_total / 4 + 1;
  }
  out->n_sized = n_initial;
  out->ms_total = now_ms() - tstart;
  return ZG_OK;
}
