// Pass 2 of egb(): GB + Coulomb + Lennard-Jones (src/sff/eff.c:1770-2066).
#include "passes.h"

namespace sffg {

void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t) {
  if (kappa) k_gbpair<true><<<grid, 256, 0, st>>>(t);
  else k_gbpair<false><<<grid, 256, 0, st>>>(t);
}

int pair_blocks_per_sm() {
  int a = 0, b = 0, c = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_gbpair<false>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_gbpair<true>, 256, 0);
  c = a < b ? a : b;
  return c > 0 ? c : 1;
}

}  // namespace sffg
