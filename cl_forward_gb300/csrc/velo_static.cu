// velo_static.cu -- the search without any device allocation.
//
// For callers that cannot allocate device memory themselves: code running
// under a framework that owns every device allocation (a fixed memory budget
// handed out by its own pool), and code that must not call cudaMalloc /
// cudaFree at run time (a trigger path with a fixed footprint, or one that
// enqueues work on a stream it does not own).  They pass device buffers for
// the events and the results; every other byte the search needs comes from
// one file-scope device array of fixed size, g_velo_static_scratch, which
// every GPU that loads the library holds until the process exits.
//
// Limits of one call (checked on the host, with a clear error):
//   n_events                      <= VELO_STATIC_MAX_EVENTS
//   total_hits + n_events         <= VELO_STATIC_MAX_HIT_ROWS
//   max_event_hits                small enough for the event to be staged in
//                                 shared memory (10,676 hits)
// and on the device (events that break them get VELO_EVENT_INVALID and no
// tracks; nothing is written out of bounds): each event's header and module
// table are checked as the host path checks them, and its hit count must not
// exceed max_event_hits.
//
// The array's symbol is a host-side stand-in in host code; its device
// address is taken once per device (cudaGetSymbolAddress, with that device
// current) on the first call made on that device, so that first call should
// come before any stream capture.  All calls share the array and it keeps the
// previous call's contents: the prep kernel clears the counters that must
// start at zero, and calls whose work overlaps on the GPU (different streams,
// or different host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "velo_internal.h"

namespace velo {
namespace {

constexpr uint64_t kRowBytes = 16u + 32u + 4u + sizeof(velo_track);   // tracklet + rings + weak + track per hit row
constexpr uint64_t kEventBytes = 4u + 4u + 4u + 8u + 8u;         // hits, maxmod, valid, hit_base, arena_off
constexpr uint64_t kCounterBytes = 256;
constexpr uint64_t kOffEvents = kCounterBytes;
constexpr uint64_t kOffRows = (kOffEvents + kEventBytes * VELO_STATIC_MAX_EVENTS + 255u) & ~255ull;
constexpr uint64_t kScratchBytes = kOffRows + kRowBytes * VELO_STATIC_MAX_HIT_ROWS;

__device__ __align__(256) uint8_t g_velo_static_scratch[kScratchBytes];

struct StaticView {
  unsigned long long* cursor;   // counters (cleared every call)
  int32_t* work;
  uint32_t* ev_hits;
  uint32_t* ev_maxmod;
  uint32_t* ev_valid;
  uint64_t* hit_base;
  uint64_t* arena_off;
  uint32_t* tracklets;          // 4 words per row
  uint32_t* rings;              // 8 words per row
  uint32_t* weak;               // 1 per row
  velo_track* tracks;           // 1 per row
};

__host__ __device__ StaticView view_of(uint8_t* base) {
  StaticView v;
  v.cursor = reinterpret_cast<unsigned long long*>(base);
  v.work = reinterpret_cast<int32_t*>(base + 32);
  uint8_t* ev = base + kOffEvents;
  v.hit_base = reinterpret_cast<uint64_t*>(ev);
  v.arena_off = reinterpret_cast<uint64_t*>(ev + 8ull * VELO_STATIC_MAX_EVENTS);
  v.ev_hits = reinterpret_cast<uint32_t*>(ev + 16ull * VELO_STATIC_MAX_EVENTS);
  v.ev_maxmod = reinterpret_cast<uint32_t*>(ev + 20ull * VELO_STATIC_MAX_EVENTS);
  v.ev_valid = reinterpret_cast<uint32_t*>(ev + 24ull * VELO_STATIC_MAX_EVENTS);
  uint8_t* rows = base + kOffRows;
  v.tracks = reinterpret_cast<velo_track*>(rows);
  v.tracklets = reinterpret_cast<uint32_t*>(rows + sizeof(velo_track) * VELO_STATIC_MAX_HIT_ROWS);
  v.weak = reinterpret_cast<uint32_t*>(rows + (sizeof(velo_track) + 16u) * VELO_STATIC_MAX_HIT_ROWS);
  v.rings = reinterpret_cast<uint32_t*>(rows + (sizeof(velo_track) + 20u) * VELO_STATIC_MAX_HIT_ROWS);
  return v;
}

// One CTA: validate headers, per-event row offsets (prefix sum of max(H, 1)),
// and clear the counters.  Events whose rows would pass the scratch end, or
// the caller's track buffer (row_limit), are marked invalid.
constexpr int kPrepThreads = 1024;

__global__ void __launch_bounds__(kPrepThreads) static_prep_kernel(const uint8_t* input, const uint64_t* offsets,
                                                                   const uint64_t* sizes, int32_t n,
                                                                   uint32_t max_event_hits, uint64_t row_limit) {
  __shared__ uint64_t part[kPrepThreads];
  const StaticView v = view_of(g_velo_static_scratch);
  const int tid = threadIdx.x;
  if (tid == 0) {
    *v.cursor = 0ull;
    *v.work = 0;
  }
  const int per = (n + kPrepThreads - 1) / kPrepThreads;
  const int a = min(n, tid * per), b = min(n, a + per);
  uint64_t local = 0;
  for (int e = a; e < b; ++e) {
    const uint8_t* blob = input + offsets[e];
    const uint64_t size = sizes[e];
    bool ok = size >= 8 && (offsets[e] & 3u) == 0;
    int32_t S = 0, H = 0, M = 0;
    if (ok) {
      const int32_t* hdr = reinterpret_cast<const int32_t*>(blob);
      S = hdr[0];
      H = hdr[1];
      ok = S >= 0 && S <= VELO_MAX_MODULES && H >= 0 && (uint32_t)H <= max_event_hits &&
           size >= 8ull + 12ull * (uint64_t)S + 16ull * (uint64_t)H;
      int64_t acc = 0;
      for (int m = 0; ok && m < S; ++m) {
        const int32_t st = hdr[2 + S + m], nm = hdr[2 + 2 * S + m];
        ok = nm >= 0 && nm <= VELO_MAX_MODULE_HITS && st == acc;
        acc += nm;
        M = max(M, nm);
      }
      ok = ok && acc == H;
    }
    v.ev_valid[e] = ok ? 1u : 0u;
    v.ev_hits[e] = ok ? (uint32_t)H : 0u;
    v.ev_maxmod[e] = ok ? (uint32_t)M : 0u;
    v.arena_off[e] = kNoArena;
    local += ok && H > 0 ? (uint64_t)H : 1ull;
  }
  part[tid] = local;
  __syncthreads();
  for (int o = 1; o < kPrepThreads; o <<= 1) {   // inclusive scan of the per-thread row counts
    const uint64_t add = tid >= o ? part[tid - o] : 0ull;
    __syncthreads();
    part[tid] += add;
    __syncthreads();
  }
  uint64_t base = part[tid] - local;
  for (int e = a; e < b; ++e) {
    const uint64_t rows = v.ev_hits[e] > 0 ? v.ev_hits[e] : 1ull;
    v.hit_base[e] = base;
    if (base + rows > row_limit) {
      v.ev_valid[e] = 0u;
      v.ev_hits[e] = 0u;
      v.ev_maxmod[e] = 0u;
      v.hit_base[e] = 0u;
    }
    base += rows;
  }
}

std::mutex g_mutex;
// Device address of the array, per device ordinal, taken on the first call
// with that device current and kept for the life of the process: it belongs
// to the device's primary context (the one the CUDA runtime uses), so it
// goes stale if that context is destroyed (cudaDeviceReset) and a new one
// made; the entry point's header says so.
void* g_scratch_ptr[64] = {};
uint32_t g_configured_smem[64] = {};

}  // namespace
}  // namespace velo

extern "C" velo_status velo_search_device_static(const uint8_t* d_input, const uint64_t* d_offsets,
                                                 const uint64_t* d_sizes, int32_t n_events, uint64_t total_hits,
                                                 uint32_t max_event_hits, int32_t y_lanes, velo_track* d_tracks_out,
                                                 uint64_t track_capacity, uint32_t* d_counts, uint64_t* d_first,
                                                 uint32_t* d_status, void* stream) {
  using namespace velo;
  if (n_events < 0 || n_events > VELO_STATIC_MAX_EVENTS) return VELO_ERR_CAPACITY;
  if (total_hits + (uint64_t)n_events > VELO_STATIC_MAX_HIT_ROWS) return VELO_ERR_CAPACITY;
  if (max_event_hits > VELO_STATIC_MAX_HIT_ROWS) return VELO_ERR_CAPACITY;   // no such event can be staged
  if (y_lanes < 1 || y_lanes > 16) return VELO_ERR_INVALID_ARGUMENT;
  if (track_capacity < total_hits + (uint64_t)n_events) return VELO_ERR_CAPACITY;
  if (n_events > 0 && (!d_input || !d_offsets || !d_sizes || !d_tracks_out || !d_counts || !d_first || !d_status))
    return VELO_ERR_INVALID_ARGUMENT;
  const uint32_t M = max_event_hits < (uint32_t)VELO_MAX_MODULE_HITS ? max_event_hits : (uint32_t)VELO_MAX_MODULE_HITS;
  const uint32_t smem = arena_layout(max_event_hits, M, (uint32_t)y_lanes).total;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VELO_ERR_CUDA;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return VELO_ERR_CUDA;
  if (smem > (uint32_t)(optin > 8192 ? optin - 8192 : 0)) return VELO_ERR_CAPACITY;   // event too large to stage
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {   // once per device, with that device current
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_velo_static_scratch) != cudaSuccess || !p) return VELO_ERR_CUDA;
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
    if (g_configured_smem[dev] < smem) {
      if (configure_search_kernel(smem) != 0) return VELO_ERR_CUDA;
      g_configured_smem[dev] = smem;
    }
  }
  if (n_events == 0) return VELO_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t row_limit = track_capacity < (uint64_t)VELO_STATIC_MAX_HIT_ROWS ? track_capacity
                                                                                 : (uint64_t)VELO_STATIC_MAX_HIT_ROWS;
  static_prep_kernel<<<1, kPrepThreads, 0, s>>>(d_input, d_offsets, d_sizes, n_events, max_event_hits, row_limit);
  if (cudaGetLastError() != cudaSuccess) return VELO_ERR_CUDA;
  const StaticView v = view_of(static_cast<uint8_t*>(base));
  SearchParams p{};
  p.input = d_input;
  p.ev_offset = d_offsets;
  p.ev_hits = v.ev_hits;
  p.ev_maxmod = v.ev_maxmod;
  p.ev_valid = v.ev_valid;
  p.hit_base = v.hit_base;
  p.arena_off = v.arena_off;
  p.order = nullptr;
  p.n_events = n_events;
  p.y_lanes = y_lanes;
  p.seed_lanes = 32;
  p.narrow = 1;
  p.persistent = 0;
  p.smem_arena_bytes = smem;
  p.global_arena = nullptr;
  p.tracklets = v.tracklets;
  p.rings = v.rings;
  p.weak = v.weak;
  p.tracks = v.tracks;
  p.out_tracks = d_tracks_out;
  p.out_capacity = track_capacity;
  p.out_counts = d_counts;
  p.out_first = d_first;
  p.out_status = d_status;
  p.out_cursor = v.cursor;
  p.work_counter = v.work;
  if (launch_search(p, n_events, 256, smem, s, 5, false) != 0) return VELO_ERR_CUDA;
  return VELO_OK;
}
