/* Oracle driver around applications/FourChain.cpp (FourChainCountingInstance). Test infrastructure. */
#define main zgref_app_main
#include "applications/FourChain.cpp"
#undef main
#define ZGREF_E Empty
#include "zgref_driver.hpp"
static ZGraphInstance<Empty>* zgref_make(Graph<Empty>* g, uint32_t, const uint32_t*, uint32_t,
                                         uint32_t) {
  return new FourChainCountingInstance<Empty>(g);
}
