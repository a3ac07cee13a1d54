/* Oracle driver around applications/AllPredicateWeightedTriangle.cpp
 * (WeightedTriangleCoutingInstance over AllPredicateZGraphInstance<VertexId>).
 * param = (op << 24) | threshold, op = ZG_PRED_GE (the app's w >= 50) or ZG_PRED_LT (the
 * inverted predicate of AtLeastOnePredicateWeightedTriangle.cpp:138-140). Test infrastructure. */
#define main zgref_app_main
#include "applications/AllPredicateWeightedTriangle.cpp"
#undef main
#define ZGREF_E VertexId
#include "zgref_driver.hpp"
static ZGraphInstance<VertexId>* zgref_make(Graph<VertexId>* g, uint32_t param, const uint32_t*,
                                            uint32_t, uint32_t) {
  uint32_t op = param >> 24, t = param & 0xFFFFFFu;
  std::function<bool(VertexId)> pred;
  if (op == ZG_PRED_LT) pred = [t](VertexId w) { return w < t; };
  else pred = [t](VertexId w) { return w >= t; };
  return new WeightedTriangleCoutingInstance<VertexId>(g, pred);
}
