// velo_sort.cu -- the reference's per-module x-sort (preorder_by_x,
// Tools.cpp:46-66) on the device, in place on staged events.
//
// Output hit indices refer to the sorted order, so the permutation has to be
// the reference's, equal x values included.  The reference sorts each module
// with a first-element-pivot quicksort (Tools.cpp:125-157).  Where a
// module's x values are all distinct its result is the one ascending order
// there is, which any sort reaches; only equal x values make the
// reference's partition steps visible (it swaps equal neighbours).  So:
//
//  * one warp per module stages the module's hits (x, y, z, ID) in shared
//    memory, and each hit's destination is its rank, the number of hits of
//    the module with a smaller x; one pass over the staged module per hit;
//  * a module with two equal x values (+0 and -0 count as equal), or with
//    more hits than a warp's staging buffer holds, replays the reference's
//    partition steps in one thread instead, on the event in global memory
//    (taking the smaller side first bounds the explicit stack at 2 log2(n)
//    entries);
//  * a module whose x values strictly increase is already in the
//    reference's order (its partitions keep every pivot first and move
//    nothing) and is not written;
//  * a module with a non-finite x is left alone: the reference's sort does
//    not return on a NaN, and the search marks such an event invalid.
//
// velo_sort_search sorts inside the search kernel instead, while it stages
// each event (velo_search_kernel.cuh: sort_arena), with the same rules.
#include <cuda_runtime.h>

#include "velo_internal.h"
#include "velo_partition.cuh"

namespace velo {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kSortThreads = 128;              // 4 warps per event
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kRankMax = 256;                  // hits a warp stages (16 B each)

struct SortStage {
  float x[kSortWarps][kRankMax];
  float y[kSortWarps][kRankMax];
  float z[kSortWarps][kRankMax];
  uint32_t id[kSortWarps][kRankMax];
};

// Sorts the modules of one event in place (all threads of the CTA call it);
// returns, in every thread, whether any byte moved.  Events whose module
// table does not tile their hits are left alone.
__device__ bool sort_event(uint8_t* event, SortStage& st) {
  int32_t* hdr = reinterpret_cast<int32_t*>(event);
  const int S = hdr[0], H = hdr[1];
  const int32_t* start = hdr + 2 + S;
  const int32_t* num = start + S;
  uint32_t* id = reinterpret_cast<uint32_t*>(hdr + 2 + 3 * S);
  float* x = reinterpret_cast<float*>(id + H);
  float* y = x + H;
  float* z = y + H;
  // the module table must tile [0, H) in order before anything moves
  bool bad = threadIdx.x == 0 && S == 0 && H != 0;
  for (int m = threadIdx.x; m < S; m += blockDim.x) {
    const int64_t expect = m == 0 ? 0 : (int64_t)start[m - 1] + (int64_t)num[m - 1];
    bad |= num[m] < 0 || num[m] > VELO_MAX_MODULE_HITS || (int64_t)start[m] != expect ||
           (m == S - 1 && (int64_t)start[m] + (int64_t)num[m] != (int64_t)H);
  }
  if (__syncthreads_or(bad)) return false;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* sx = st.x[w];
  float* sy = st.y[w];
  float* sz = st.z[w];
  uint32_t* sid = st.id[w];
  bool wrote = false;
  for (int m = w; m < S; m += kSortWarps) {   // warp-uniform
    const int s0 = start[m], n = num[m];
    if (n < 2) continue;
    if (n > kRankMax) {
      // large module: one thread checks it and, unless it is in order
      // already or holds a non-finite x, replays the reference's partitions
      bool changed = false;
      if (lane == 0) {
        bool finite = true, increasing = true;
        for (int i = s0; i < s0 + n; ++i) {
          finite &= isfinite(x[i]) != 0;
          if (i > s0) increasing &= x[i - 1] < x[i];
        }
        if (finite && !increasing) {
          quicksort4(x, y, z, id, s0, s0 + n - 1);
          changed = true;
        }
      }
      wrote |= changed;
      continue;
    }
    bool finite = true, moved = false;
    for (int i = lane; i < n; i += 32) {
      const float xi = x[s0 + i];
      sx[i] = xi;
      sy[i] = y[s0 + i];
      sz[i] = z[s0 + i];
      sid[i] = id[s0 + i];
      finite &= isfinite(xi) != 0;
    }
    __syncwarp();
    if (!__all_sync(kFullMask, finite)) continue;   // left alone
    // rank of each hit; `tie` when another hit has the same x
    bool tie = false;
    int rank_of[kRankMax / 32];
#pragma unroll
    for (int k = 0; k < kRankMax / 32; ++k) {
      const int i = lane + 32 * k;
      rank_of[k] = i;
      if (i < n) {
        const float xi = sx[i];
        int r = 0, eq = 0;
        for (int j = 0; j < n; ++j) {
          const float xj = sx[j];
          r += xj < xi;
          eq += xj == xi;
        }
        rank_of[k] = r;
        tie |= eq > 1;
        moved |= r != i;
      }
    }
    if (__any_sync(kFullMask, tie)) {
      // equal x values: the reference's partition steps decide their order
      if (lane == 0) {
        quicksort4(x, y, z, id, s0, s0 + n - 1);
        wrote = true;
      }
      __syncwarp();
      continue;
    }
    if (!__any_sync(kFullMask, moved)) continue;   // strictly increasing already
    wrote = true;
#pragma unroll
    for (int k = 0; k < kRankMax / 32; ++k) {
      const int i = lane + 32 * k;
      if (i < n) {
        const int r = s0 + rank_of[k];
        x[r] = sx[i];
        y[r] = sy[i];
        z[r] = sz[i];
        id[r] = sid[i];
      }
    }
    __syncwarp();   // the staging buffer is refilled for the next module
  }
  return __syncthreads_or(wrote) != 0;
}

__global__ void __launch_bounds__(kSortThreads) sort_modules_kernel(uint8_t* input, const uint64_t* offsets,
                                                                    const uint32_t* valid, int n_events) {
  __shared__ SortStage st;
  const int e = blockIdx.x;
  if (e >= n_events || !valid[e]) return;
  sort_event(input + offsets[e], st);
}

}  // namespace

int launch_sort_modules(uint8_t* input, const uint64_t* offsets, const uint32_t* valid, int n_events, void* stream) {
  if (n_events <= 0) return 0;
  sort_modules_kernel<<<n_events, kSortThreads, 0, (cudaStream_t)stream>>>(input, offsets, valid, n_events);
  return (int)cudaGetLastError();
}

}  // namespace velo
