// Launchers of the three pair passes, each compiled in its own
// translation unit (pass1.cu, pass2.cu, pass3.cu).
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "kernels.cuh"

namespace sffg {

// Launches kernel k with programmatic stream serialization: it may be
// scheduled while the previous kernel on the stream drains, hiding the
// launch gap; k must call pdl_wait() before reading that kernel's output.
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t st, A &&...args) {
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = 0;
  c.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  c.attrs = at;
  c.numAttrs = 1;
  return cudaLaunchKernelEx(&c, k, std::forward<A>(args)...);
}

// grid: 256-thread blocks of the persistent kernel.
void launch_born(bool neck, bool poly, int grid, cudaStream_t st, const DevTables &t);
void launch_gbpair(bool kappa, int grid, cudaStream_t st, const DevTables &t);
void launch_chain(bool neck, bool poly, int grid, cudaStream_t st, const DevTables &t);
// Resident 256-thread blocks per SM of each pair kernel.
int born_blocks_per_sm(bool neck, bool poly);
int gbpair_blocks_per_sm(bool kappa);
int chain_blocks_per_sm(bool neck, bool poly);
// The checked build's error word of each pass's translation unit (0 when
// no check failed, and always 0 in the normal build).
int pass1_check_code();
int pass2_check_code();
int pass3_check_code();

}  // namespace sffg
