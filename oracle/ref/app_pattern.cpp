/* Oracle driver around SamplerGenerator<Empty> (src/SamplerGenerator.cpp) for a Pattern given as
 * (src,dst) pairs with edge_id = index, as applications/FiveStar.cpp:18-26 and FiveHouse.cpp:18-27
 * build theirs.  Also exposes UnbiasedLinearRegression, ErrorProfile::calculate_bound and
 * Estimation::update for the ELP checks.  Test infrastructure. */
#include <assert.h>
#include <math.h>
#include <functional>
#include <iostream>
#include <random>
#include <string>
#include <utility>
#include <vector>
#define ZGREF_E Empty
#include "SamplerGenerator.hpp"
#include "Regression.hpp"
#define private public
#include "ErrorLatencyProfile.hpp"
#undef private
#include "zgref_driver.hpp"
static ZGraphInstance<Empty>* zgref_make(Graph<Empty>* g, uint32_t, const uint32_t* pedges,
                                         uint32_t pv, uint32_t pe) {
  std::vector<Edge<Empty>> es(pe);
  for (uint32_t i = 0; i < pe; ++i) {
    es[i].src = pedges[2 * i];
    es[i].dst = pedges[2 * i + 1];
    es[i].edge_id = i;
  }
  Pattern pat(pv, pe, es.data());
  return new SamplerGenerator<Empty>(g, &pat);
}

ZGREF_API double zgref_regression_k(const double* x, const double* y, uint32_t len) {
  std::vector<long double> lx(x, x + len), ly(y, y + len);
  UnbiasedLinearRegression r;
  r.solve(lx.data(), ly.data(), len);
  return (double)r.get_k();
}

ZGREF_API double zgref_calculate_bound(double eps, double delta, double nse, double ncse,
                                       double est, uint64_t maxdeg, uint64_t m) {
  ErrorProfile<Empty> ep;
  return ep.calculate_bound(eps, delta, nse, ncse, est, maxdeg, m);
}

/* Estimation::update folded over a sequence (src/ZGraphInstance.cpp:24-27). */
ZGREF_API double zgref_estimation_fold(const uint64_t* ns, const double* vals, uint32_t len) {
  Estimation e;
  for (uint32_t i = 0; i < len; ++i) e.update(ns[i], vals[i]);
  return e.get_currnet_estimation();
}
