// Launchers of the three pair passes, each compiled in its own
// translation unit (pass1.cu, pass2.cu, pass3.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace sffg {

// grid: 256-thread blocks of the persistent kernel.
void launch_born(bool neck, int grid, cudaStream_t st, const DevTables &t);
void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t);
void launch_chain(bool neck, int grid, cudaStream_t st, const DevTables &t);
// Resident 256-thread blocks per SM of each pair kernel.
int born_blocks_per_sm(bool neck);
int gbpair_blocks_per_sm(bool kappa);
int chain_blocks_per_sm(bool neck);

}  // namespace sffg
