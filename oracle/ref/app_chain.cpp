/* Oracle driver around applications/ChainMining.cpp (ChainMiningInstance, param = order). Test infrastructure. */
#define main zgref_app_main
#include "applications/ChainMining.cpp"
#undef main
#define ZGREF_E Empty
#include "zgref_driver.hpp"
static ZGraphInstance<Empty>* zgref_make(Graph<Empty>* g, uint32_t order, const uint32_t*, uint32_t,
                                         uint32_t) {
  return new ChainMiningInstance<Empty>(g, (int)order);
}
