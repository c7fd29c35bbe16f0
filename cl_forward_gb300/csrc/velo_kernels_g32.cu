// velo_kernels_g32.cu -- the search kernel builds that seed with 32 lanes per
// h0 (velo_search_kernel.cuh); a translation unit of its own so that the
// widths compile in parallel.
#include "velo_search_kernel.cuh"

namespace velo {

int launch_search_g32(const SearchParams& p, int grid, int block, uint32_t smem, void* stream, int reg_ctas,
                     bool compact) {
  return SearchBuilds<32>::launch(p, grid, block, smem, (cudaStream_t)stream, reg_ctas, compact);
}
int configure_search_g32(uint32_t smem) { return SearchBuilds<32>::configure(smem); }
int search_occupancy_g32(int block, uint32_t smem, int reg_ctas, int mode, bool compact, int* ctas) {
  return SearchBuilds<32>::occupancy(block, smem, reg_ctas, mode, compact, ctas);
}
#ifdef VELO_PHASE_CLOCKS
int phase_cycles_g32(unsigned long long* out) { return SearchBuilds<32>::phase_cycles(out); }
#endif

}  // namespace velo
