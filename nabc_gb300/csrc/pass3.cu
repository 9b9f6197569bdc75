// Pass 3 of egb(): chain rule through the Born radii
// (src/sff/eff.c:2131-2405).
#include "passes.h"

namespace sffg {

// Persistent grid: as many 256-thread blocks as fit on the GPU at once.
template <class K>
int full_grid(K kernel, int nsm) {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0);
  return nsm * (occ > 0 ? occ : 1);
}

void launch_chain(bool neck, int nsm, cudaStream_t st, const DevTables &t) {
  static const int g1 = full_grid(k_chain<true>, nsm), g0 = full_grid(k_chain<false>, nsm);
  if (neck) k_chain<true><<<g1, 256, 0, st>>>(t);
  else k_chain<false><<<g0, 256, 0, st>>>(t);
}

}  // namespace sffg
