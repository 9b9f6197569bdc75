// Pass 3 of egb(): chain rule through the Born radii
// (src/sff/eff.c:2131-2405).
#include "passes.h"

namespace sffg {

void launch_chain(bool neck, bool poly, int grid, cudaStream_t st, const DevTables &t) {
  if (neck) {
    if (poly) launch_pdl(k_chain<true, true>, grid, 256, st, t);
    else launch_pdl(k_chain<true, false>, grid, 256, st, t);
  } else {
    if (poly) launch_pdl(k_chain<false, true>, grid, 256, st, t);
    else launch_pdl(k_chain<false, false>, grid, 256, st, t);
  }
}

int chain_blocks_per_sm(bool neck, bool poly) {
  int occ = 0;
  if (neck) {
    if (poly) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_chain<true, true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_chain<true, false>, 256, 0);
  } else {
    if (poly) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_chain<false, true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_chain<false, false>, 256, 0);
  }
  return occ > 0 ? occ : 1;
}

int pass3_check_code() {
#ifdef SFFG_CHECKED
  int c = 0;
  cudaMemcpyFromSymbol(&c, g_check_code, sizeof(int));
  return c;
#else
  return 0;
#endif
}

}  // namespace sffg
