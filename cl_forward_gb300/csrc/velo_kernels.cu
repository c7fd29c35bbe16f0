// velo_kernels.cu -- host side of the search kernel: picks the build of a
// launch (seeding width, register budget, threads, shared-state size, mode)
// and keeps the per-device dynamic shared-memory limit.  The device code is
// velo_search_kernel.cuh, compiled once per seeding width
// (velo_kernels_g8.cu, _g16.cu, _g32.cu).
#include <cuda_runtime.h>

#include <mutex>

#include "velo_internal.h"

namespace velo {

int launch_search_g8(const SearchParams&, int, int, uint32_t, void*, int, bool);
int launch_search_g16(const SearchParams&, int, int, uint32_t, void*, int, bool);
int launch_search_g32(const SearchParams&, int, int, uint32_t, void*, int, bool);
int configure_search_g8(uint32_t);
int configure_search_g16(uint32_t);
int configure_search_g32(uint32_t);
int search_occupancy_g8(int, uint32_t, int, int, bool, int*);
int search_occupancy_g16(int, uint32_t, int, int, bool, int*);
int search_occupancy_g32(int, uint32_t, int, int, bool, int*);

// The training-data dump records doublets independently of the seeding
// width, so it always runs the 32-lane build.
int launch_search(const SearchParams& p, int grid, int block, uint32_t smem_bytes, void* stream, int reg_ctas,
                  bool compact) {
  if (p.seed_lanes == 8 && !p.dump_features)
    return launch_search_g8(p, grid, block, smem_bytes, stream, reg_ctas, compact);
  if (p.seed_lanes == 16 && !p.dump_features)
    return launch_search_g16(p, grid, block, smem_bytes, stream, reg_ctas, compact);
  return launch_search_g32(p, grid, block, smem_bytes, stream, reg_ctas, compact);
}

int configure_search_kernel(uint32_t smem_bytes) {
  // Only ever raised, per device, so that no caller lowers it under another.
  static std::mutex mu;
  static uint32_t configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && configured[dev] >= smem_bytes) return 0;
  int r = configure_search_g8(smem_bytes);
  if (r == 0) r = configure_search_g16(smem_bytes);
  if (r == 0) r = configure_search_g32(smem_bytes);
  if (r == 0 && dev >= 0 && dev < 64) configured[dev] = smem_bytes;
  return r;
}

int search_occupancy(int block, uint32_t smem_bytes, int reg_ctas, int mode, bool compact, int seed_lanes,
                     int* ctas_per_sm) {
  if (seed_lanes == 8 && mode != kModeDump)
    return search_occupancy_g8(block, smem_bytes, reg_ctas, mode, compact, ctas_per_sm);
  if (seed_lanes == 16 && mode != kModeDump)
    return search_occupancy_g16(block, smem_bytes, reg_ctas, mode, compact, ctas_per_sm);
  return search_occupancy_g32(block, smem_bytes, reg_ctas, mode, compact, ctas_per_sm);
}

#ifdef VELO_PHASE_CLOCKS
int phase_cycles_g8(unsigned long long*);
int phase_cycles_g16(unsigned long long*);
int phase_cycles_g32(unsigned long long*);
// Reads and clears the per-phase cycle counters (diagnostic builds only).
extern "C" int velo_debug_phase_cycles(unsigned long long* out) {
  for (int k = 0; k < 8; ++k) out[k] = 0;
  int e = phase_cycles_g8(out);
  if (e == 0) e = phase_cycles_g16(out);
  if (e == 0) e = phase_cycles_g32(out);
  return e;
}
#endif

}  // namespace velo
