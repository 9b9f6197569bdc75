// Pass 2 of egb(): GB + Coulomb + Lennard-Jones (src/sff/eff.c:1770-2066).
#include "passes.h"

namespace sffg {

void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t) {
  const bool ljs = t.lj_shared && t.lj_n <= kLjShared;  // one more entry: the zero one
  if (kappa) {
    if (ljs) launch_pdl(k_gbpair<true, true>, grid, 256, st, t);
    else launch_pdl(k_gbpair<true, false>, grid, 256, st, t);
  } else {
    if (ljs) launch_pdl(k_gbpair<false, true>, grid, 256, st, t);
    else launch_pdl(k_gbpair<false, false>, grid, 256, st, t);
  }
}

// Resident blocks per SM of the shared-table form (the one the tuner and
// the default grid size use; the global-table form fits at least as many).
int gbpair_blocks_per_sm(bool kappa) {
  int occ = 0;
  if (kappa) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gbpair<true, true>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gbpair<false, true>, 256, 0);
  return occ > 0 ? occ : 1;
}

int pass2_check_code() {
#ifdef SFFG_CHECKED
  int c = 0;
  cudaMemcpyFromSymbol(&c, g_check_code, sizeof(int));
  return c;
#else
  return 0;
#endif
}

}  // namespace sffg
