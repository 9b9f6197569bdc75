// Pass 1 of egb(): Born-radius descreening (src/sff/eff.c:1566-1709).
#include "passes.h"

namespace sffg {

void launch_born(bool neck, int grid, cudaStream_t st, const DevTables &t) {
  if (neck) k_born<true><<<grid, 256, 0, st>>>(t);
  else k_born<false><<<grid, 256, 0, st>>>(t);
}

}  // namespace sffg
