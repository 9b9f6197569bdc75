// Pass 2 of egb(): GB + Coulomb + Lennard-Jones (src/sff/eff.c:1770-2066).
#include "passes.h"

namespace sffg {

void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t) {
  if (kappa) k_gbpair<true><<<grid, 256, 0, st>>>(t);
  else k_gbpair<false><<<grid, 256, 0, st>>>(t);
}

int gbpair_blocks_per_sm(bool kappa) {
  int occ = 0;
  if (kappa) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gbpair<true>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gbpair<false>, 256, 0);
  return occ > 0 ? occ : 1;
}

}  // namespace sffg
