// velo_internal.h -- definitions shared by the host orchestration
// (velo_capi.cpp) and the sm_103a kernels (velo_kernels.cu).
#pragma once

#include <stdint.h>

#include "../../include/velo_search.h"

#ifdef __CUDACC__
#define VELO_HD __host__ __device__ __forceinline__
#else
#define VELO_HD inline
#endif

namespace velo {

// Physics cuts and capacities of the reference, KernelDefinitions.h:15-33.
constexpr float kTolerance = 0.6f;             // PARAM_TOLERANCE
constexpr float kToleranceCandidates = 0.6f;   // PARAM_TOLERANCE_CANDIDATES
constexpr float kMaxXSlopeCandidates = 0.7f;   // PARAM_MAXXSLOPE_CANDIDATES
constexpr float kMaxYSlope = 0.7f;             // PARAM_MAXYSLOPE
constexpr float kMaxScatter = 0.000016f;       // MAX_SCATTER
constexpr uint32_t kMaxSkippedModules = 3;     // MAX_SKIPPED_MODULES
constexpr int kMaxModules = VELO_MAX_MODULES;
constexpr int kMaxModuleHits = VELO_MAX_MODULE_HITS;

// Ring entry encoding, Kernel.cl:222-225,351,566: bit 31 = tracklet (3 hits,
// index into the tracklet list), bits 28-30 = skipped modules, bits 0-27 =
// track or tracklet number.
constexpr uint32_t kTrackletFlag = 0x80000000u;
constexpr uint32_t kSkipMask = 0x70000000u;
constexpr uint32_t kNumberMask = 0x0FFFFFFFu;
constexpr uint64_t kNoArena = ~0ull;

// Per-event working set ("arena"): staged in dynamic shared memory when it
// fits the launch's shared-memory size, else carved from global scratch.
// Offsets are bytes, each array 16-byte aligned.
struct ArenaLayout {
  uint32_t x, y, z;              // float[H]   hit coordinates (x-sorted per module)
  uint32_t h1f, h1l, h2f, h2l;   // int32[H]   candidate windows, absolute hit index or -1
  uint32_t used;                 // uint8[H]   hit_used
  uint32_t ring0, ring1;         // uint32[H+1] tracks-to-follow, double-buffered
  uint32_t slot_h0;              // int32[M]   seeding: unused h0 of the module
  uint32_t slot_pref;            // uint32[M+1] seeding: prefix of h1-window sizes
  uint32_t cutoff;               // uint32[M*Y] seeding: first dead element per lane
  uint32_t best;                 // uint64[M]  seeding: packed best key per h0
  uint32_t total;
};

VELO_HD uint32_t align16(uint32_t v) { return (v + 15u) & ~15u; }

VELO_HD ArenaLayout arena_layout(uint32_t H, uint32_t M, uint32_t Y) {
  ArenaLayout L;
  uint32_t o = 0;
  L.x = o; o = align16(o + 4u * H);
  L.y = o; o = align16(o + 4u * H);
  L.z = o; o = align16(o + 4u * H);
  L.h1f = o; o = align16(o + 4u * H);
  L.h1l = o; o = align16(o + 4u * H);
  L.h2f = o; o = align16(o + 4u * H);
  L.h2l = o; o = align16(o + 4u * H);
  L.used = o; o = align16(o + H);
  L.ring0 = o; o = align16(o + 4u * (H + 1u));
  L.ring1 = o; o = align16(o + 4u * (H + 1u));
  L.slot_h0 = o; o = align16(o + 4u * M);
  L.slot_pref = o; o = align16(o + 4u * (M + 1u));
  L.cutoff = o; o = align16(o + 4u * M * Y);
  L.best = o; o = align16(o + 8u * M);
  L.total = o;
  return L;
}

struct SearchParams {
  // input: packed event blobs, event e at input + ev_offset[e]
  const uint8_t* input;
  const uint64_t* ev_offset;
  const uint32_t* ev_hits;        // H per event (0 for invalid events)
  const uint32_t* ev_maxmod;      // largest module occupancy per event
  const uint32_t* ev_valid;       // 1 = passed host validation
  const uint64_t* hit_base;       // prefix sum of max(H, 1): per-event scratch row
  const uint64_t* arena_off;      // byte offset into global_arena, or kNoArena (shared memory)
  const int32_t* order;           // persistent mode: event processing order
  int32_t n_events;
  int32_t y_lanes;
  int32_t narrow;                 // 1 = binary-search narrowing of sorted modules
  int32_t persistent;
  uint32_t smem_arena_bytes;      // dynamic shared memory per CTA
  // global scratch
  uint8_t* global_arena;
  uint32_t* tracklets;            // 3 hit indices per tracklet, row hit_base[e]
  uint32_t* weak;                 // weak-track list, row hit_base[e]
  velo_track* tracks;             // working tracks, row hit_base[e]
  // outputs
  velo_track* out_tracks;         // compacted: event e at out_first[e]
  uint32_t* out_counts;
  uint64_t* out_first;
  uint32_t* out_status;
  unsigned long long* out_cursor; // running total of compacted tracks
  int32_t* work_counter;          // persistent mode queue head
};

// Launches the search kernel (velo_kernels.cu).  Returns a cudaError_t value.
int launch_search(const SearchParams& p, int grid, int block, uint32_t smem_bytes, void* stream);
// Sets the kernel's maximum dynamic shared memory.  Returns a cudaError_t value.
int configure_search_kernel(uint32_t smem_bytes);
// Maximum resident CTAs per SM for a block size and shared-memory size.
int search_occupancy(int block, uint32_t smem_bytes, int* ctas_per_sm);

}  // namespace velo
