// Host-only check of the sim:: layer's plan cache (include/bartels_sim.hpp,
// detail::PlanCache) with stand-in plans: hits on equal content, misses on a
// changed V or E at the same addresses, the tag separating triangle plans of
// different DOF counts, least-recently-used eviction of the fifth mesh and the
// destruction of every evicted plan. Prints "plan cache ok" and returns 0.
#include <cstdio>
#include <vector>

#include "bartels_sim.hpp"

#define REQUIRE(c)                                                          \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main() {
  sim::detail::PlanCache<int> cache;
  int made = 0;
  std::vector<int> destroyed;
  auto get = [&](int tag, const std::vector<double> &V, const std::vector<int> &E) {
    return cache.get(tag, (int)V.size() / 3, V.data(), V.size(), E.data(), E.size(), [&] { return ++made; },
                     [&](int p) { destroyed.push_back(p); });
  };
  std::vector<double> V = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::vector<int> E = {0, 1, 2, 3};
  const int a = get(0, V, E);
  REQUIRE(a == 1 && get(0, V, E) == 1 && made == 1);  // same content: hit
  V[3] = 2.0;                                          // same buffer, new rest positions
  const int b = get(0, V, E);
  REQUIRE(b == 2 && made == 2);
  E[1] = 3;
  E[3] = 1;                                            // same buffer, new connectivity
  REQUIRE(get(0, V, E) == 3);
  REQUIRE(get(1, V, E) == 4);                          // another tag: another plan
  // 4 plans cached (1..4); a fifth mesh evicts the least recently used one (1)
  std::vector<double> V5 = V;
  V5[0] = -1.0;
  REQUIRE(get(0, V5, E) == 5 && destroyed.size() == 1 && destroyed[0] == 1);
  // 2 is still cached; touching it makes 3 the least recently used
  V[3] = 2.0;
  E = {0, 1, 2, 3};
  REQUIRE(get(0, V, E) == 2);
  std::vector<double> V6 = V;
  V6[0] = -2.0;
  REQUIRE(get(0, V6, E) == 6 && destroyed.size() == 2 && destroyed[1] == 3);
  std::printf("plan cache ok\n");
  return 0;
}
