/* Zero-filling operator new[] linked into the naive counters of the oracle build: several of
 * them read arrays they never initialise (naive_implementation/TriangleCounting.cpp:36,
 * FiveHouse.cpp:64-65).  Test infrastructure. */
#include <cstdlib>
#include <new>
int zgref_num_cpus = 1;
void* operator new[](std::size_t n) {
  void* p = std::calloc(n ? n : 1, 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }
