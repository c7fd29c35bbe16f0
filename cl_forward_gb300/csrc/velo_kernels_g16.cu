// velo_kernels_g16.cu -- the search kernel builds that seed with 16 lanes per
// h0 (velo_search_kernel.cuh); a translation unit of its own so that the
// widths compile in parallel.
#include "velo_search_kernel.cuh"

namespace velo {

int launch_search_g16(const SearchParams& p, int grid, int block, uint32_t smem, void* stream, int reg_ctas,
                     bool compact) {
  return SearchBuilds<16>::launch(p, grid, block, smem, (cudaStream_t)stream, reg_ctas, compact);
}
int configure_search_g16(uint32_t smem) { return SearchBuilds<16>::configure(smem); }
int search_occupancy_g16(int block, uint32_t smem, int reg_ctas, int mode, bool compact, int* ctas) {
  return SearchBuilds<16>::occupancy(block, smem, reg_ctas, mode, compact, ctas);
}
#ifdef VELO_PHASE_CLOCKS
int phase_cycles_g16(unsigned long long* out) { return SearchBuilds<16>::phase_cycles(out); }
#endif

}  // namespace velo
