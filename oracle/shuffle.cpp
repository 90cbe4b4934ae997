/* shuffle.cpp -- the one C++ piece of the oracle (test infrastructure only).
 * Reproduces the particle permutation of the reference's sampling mode,
 * `random_shuffle(Particles.begin(), Particles.end())` at
 * src/subhalo_unbind.cpp:302, by making the same library call after
 * srand(seed); std::random_shuffle draws from the C library's rand(). */
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "hbt_oracle.h"

extern "C" void hbto_reference_shuffle(int64_t n, unsigned seed, int64_t *perm)
{
  std::vector<int64_t> v(n > 0 ? n : 0);
  for (int64_t i = 0; i < n; i++) v[i] = i;
  srand(seed);
  std::random_shuffle(v.begin(), v.end());
  for (int64_t i = 0; i < n; i++) perm[i] = v[i];
}
