// Pass 1 of egb(): Born-radius descreening (src/sff/eff.c:1566-1709).
#include "passes.h"

namespace sffg {

void launch_born(bool neck, bool poly, int grid, cudaStream_t st, const DevTables &t) {
  if (neck) {
    if (poly) launch_pdl(k_born<true, true>, grid, 256, st, t);
    else launch_pdl(k_born<true, false>, grid, 256, st, t);
  } else {
    if (poly) launch_pdl(k_born<false, true>, grid, 256, st, t);
    else launch_pdl(k_born<false, false>, grid, 256, st, t);
  }
}

int born_blocks_per_sm(bool neck, bool poly) {
  int occ = 0;
  if (neck) {
    if (poly) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_born<true, true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_born<true, false>, 256, 0);
  } else {
    if (poly) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_born<false, true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_born<false, false>, 256, 0);
  }
  return occ > 0 ? occ : 1;
}

int pass1_check_code() {
#ifdef SFFG_CHECKED
  int c = 0;
  cudaMemcpyFromSymbol(&c, g_check_code, sizeof(int));
  return c;
#else
  return 0;
#endif
}

}  // namespace sffg
