// Launchers of the three pair passes, each compiled in its own
// translation unit (pass1.cu, pass2.cu, pass3.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace sffg {

// Passes 1 and 3 size their persistent grids from the occupancy of the
// kernel launched (nsm: multiprocessors of the device).
void launch_born(bool neck, int nsm, cudaStream_t st, const DevTables &t);
void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t);
void launch_chain(bool neck, int nsm, cudaStream_t st, const DevTables &t);
// Resident 256-thread blocks per SM of the pair kernels.
int pair_blocks_per_sm();

}  // namespace sffg
