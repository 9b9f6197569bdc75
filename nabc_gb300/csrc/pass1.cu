// Pass 1 of egb(): Born-radius descreening (src/sff/eff.c:1566-1709).
#include "passes.h"

namespace sffg {

// Persistent grid: as many 256-thread blocks as fit on the GPU at once.
template <class K>
int full_grid(K kernel, int nsm) {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0);
  return nsm * (occ > 0 ? occ : 1);
}

void launch_born(bool neck, int nsm, cudaStream_t st, const DevTables &t) {
  static const int g1 = full_grid(k_born<true>, nsm), g0 = full_grid(k_born<false>, nsm);
  if (neck) k_born<true><<<g1, 256, 0, st>>>(t);
  else k_born<false><<<g0, 256, 0, st>>>(t);
}

}  // namespace sffg
