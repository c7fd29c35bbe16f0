// velo_internal.h -- definitions shared by the host orchestration
// (velo_capi.cpp) and the sm_103a kernels (velo_search_kernel.cuh, launched
// from velo_kernels.cu).
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

// Tracks-to-follow entry bits shared with the reference (Kernel.cl:222-225,
// 351,566): bit 31 = tracklet, bits 28-30 = skipped modules.
constexpr uint32_t kTrackletFlag = 0x80000000u;
constexpr uint32_t kSkipMask = 0x70000000u;
constexpr uint64_t kNoArena = ~0ull;
// Module-table capacity of the compact shared-state build of the search
// kernel (events with fewer modules; the full build takes kMaxModules).
constexpr int kCompactModules = 64;

// MLP parameter layout (velo_search.h): W1[32][10] b1[32] W2[32][32] b2[32]
// W3[2][32] b3[2]
constexpr int kMlpIn = VELO_MLP_INPUTS;
constexpr int kMlpHidden = VELO_MLP_HIDDEN;
constexpr int kMlpOut = VELO_MLP_OUTPUTS;
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHidden * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpOut * kMlpHidden;
static_assert(kMlpB3 + kMlpOut == VELO_MLP_PARAMS, "MLP parameter count");

// The same weights in FP16 tensor-core fragment order for inference
// (velo_mlp_warp.cuh): B fragments of W1^T (K 16 x N 32), W2^T (K 32 x N 32)
// and W3^T (K 32 x N 8, 2 used) per n-tile and lane, biases in FP32.  Leads
// the dynamic shared memory of a learned launch.
struct alignas(8) MlpPair {
  uint32_t x, y;
};
struct MlpFrag {
  MlpPair w1[4][32], w2[2][4][32], w3[2][32];
  float b1[kMlpHidden], b2[kMlpHidden], b3[8];
};
constexpr uint32_t kMlpSmemBytes = (sizeof(MlpFrag) + 15) & ~15u;

// Per-event working set ("arena"): staged in dynamic shared memory when it
// fits the launch's shared-memory size, else carved from global scratch.
// Offsets are bytes, each array 16-byte aligned.  21 bytes per hit.  (The
// tracks-to-follow rings live with the per-row scratch in global memory.)
struct ArenaLayout {
  uint32_t x, y, z;              // float[H]    hit coordinates (x-sorted per module)
  uint32_t win;                  // uint2[H]    candidate windows, 16-bit offsets into module f-2
  uint32_t used;                 // uint8[H]    hit_used
  uint32_t total;
};

VELO_HD uint32_t align16(uint32_t v) { return (v + 15u) & ~15u; }

// M (largest module) and Y (lanes) are accepted for callers that size by
// them; the layout depends on H only.
VELO_HD ArenaLayout arena_layout(uint32_t H, uint32_t M, uint32_t Y) {
  (void)M;
  (void)Y;
  ArenaLayout L;
  uint32_t o = 0;
  // one stride P for every array, so a view of the arena is its base and P
  const uint32_t P = align16(4u * H);
  L.x = 0;
  L.y = P;
  L.z = 2u * P;
  L.win = 3u * P;      // 8H bytes <= 2P
  L.used = 5u * P;
  o = 5u * P + align16(H);
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
  uint64_t out_capacity;          // rows of out_tracks; rows past it are not written
  int32_t n_events;
  int32_t y_lanes;
  int32_t seed_lanes;             // lanes per h0 in seeding: 8, 16 or 32 (a multiple of y_lanes below 32)
  int32_t narrow;                 // 1 = binary-search narrowing of sorted modules
  int32_t persistent;
  uint32_t smem_arena_bytes;      // dynamic shared memory per CTA
  // global scratch
  uint8_t* global_arena;
  uint32_t* tracklets;            // 4 words per tracklet {h0, h1, h2, 0}, row hit_base[e]
  uint32_t* rings;                // 8 words per row: the two tracks-to-follow rings of event e
                                  // (max(H, 1) entries each) from row hit_base[e], entries
                                  // {entry word, first hit, previous hit, last hit}
  uint32_t* weak;                 // weak-track list, row hit_base[e]
  velo_track* tracks;             // working tracks, row hit_base[e]
  // outputs
  velo_track* out_tracks;         // compacted: event e at out_first[e]
  uint32_t* out_counts;
  uint64_t* out_first;
  uint32_t* out_status;
  unsigned long long* out_cursor; // running total of compacted tracks
  velo_event_result* results;     // streaming (velo_search_begin): per-event records in host memory, or null
  // velo_sort_search / velo_search_begin with sort: each event's modules are
  // x-sorted (the reference's permutation) while the event is staged, and
  // the sorted hit arrays are written back into the input, which is then
  // the caller's buffer read in place
  int32_t sort_events;
  int32_t* work_counter;          // persistent mode queue head
  // training data: features and {event, h0, h1} of sampled doublets
  float* dump_features;
  uint32_t* dump_ids;
  unsigned long long* dump_count;
  uint64_t dump_capacity;
  uint32_t dump_keep;             // one in dump_keep doublets (hash-sampled)
  // learned seeding: MLP weights (null = plain), prefix of the dynamic shared memory
  const float* mlp;
  float keep_threshold;
  float window_margin;
  float min_keep_rate;
  uint32_t learned_max_hits;      // larger events take the plain method (0 = no limit)
  int32_t learned_min_window;     // score only doublets with at least this many h2 candidates
};

// Launches the search kernel (velo_kernels.cu); reg_ctas (4 or 5) picks the
// register budget of the <= 256-thread build, p.seed_lanes the seeding width.  Returns a cudaError_t value.
// compact: every event of the launch has fewer than 64 modules (the compact
// shared-state build).
int launch_search(const SearchParams& p, int grid, int block, uint32_t smem_bytes, void* stream, int reg_ctas,
                  bool compact);
// Sets the kernels' maximum dynamic shared memory.  Returns a cudaError_t value.
int configure_search_kernel(uint32_t smem_bytes);
// Maximum resident CTAs per SM for a block size, shared-memory size and build.
int search_occupancy(int block, uint32_t smem_bytes, int reg_ctas, int mode, bool compact, int seed_lanes,
                     int* ctas_per_sm);
// Straight-line fits of the compacted output tracks (velo_fit.cu).
int launch_fit_tracks(const uint8_t* input, const uint64_t* ev_offset, const uint32_t* ev_valid,
                      const velo_track* tracks, const uint32_t* counts, const uint64_t* first, int n_events,
                      velo_track_fit* fits, void* stream);
// Sorts each module's hits by x in place on staged events (velo_sort.cu).
int launch_sort_modules(uint8_t* input, const uint64_t* offsets, const uint32_t* valid, int n_events, void* stream);
// kernel modes (velo_search_kernel.cuh): plain, plain + training-data dump, learned
constexpr int kModePlain = 0, kModeDump = 1, kModeLearned = 2;

}  // namespace velo
