// velo_capi.cpp -- host orchestration behind include/velo_search.h.
//
// Replaces invokeParallelSearch (KernelInvoker.cpp:14-275): instead of a fresh
// OpenCL context, a JIT build and twelve buffers per call, a velo_ctx keeps
// one CUDA stream and grow-only device buffers; event headers are checked on
// the host (module tables and coordinates by the search kernel), the events
// are copied with one H2D transfer (or read in place from mapped pinned host
// memory), searched by one kernel launch, and the tracks come back compacted
// in one D2H transfer (or are written in place).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "velo_internal.h"

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

// Grow-only array in pinned host memory: the per-event metadata goes to the
// device with asynchronous copies (a copy from pageable memory would first
// wait for the stream, serialising the host behind the input transfer).
template <typename T>
struct PinnedVec {
  T* p = nullptr;
  size_t n = 0, cap = 0;
  PinnedVec() = default;
  PinnedVec(const PinnedVec&) = delete;
  PinnedVec& operator=(const PinnedVec&) = delete;
  ~PinnedVec() {
    if (p) cudaFreeHost(p);
  }
  bool resize(size_t m) {
    if (m > cap) {
      T* q = nullptr;
      const size_t nc = m + m / 4 + 64;
      if (cudaHostAlloc(reinterpret_cast<void**>(&q), nc * sizeof(T), cudaHostAllocDefault) != cudaSuccess)
        return false;
      if (p) {
        std::memcpy(q, p, n * sizeof(T));
        cudaFreeHost(p);
      }
      p = q;
      cap = nc;
    }
    n = m;
    return true;
  }
  bool assign(size_t m, T v) {
    if (!resize(m)) return false;
    std::fill(p, p + m, v);
    return true;
  }
  T* data() { return p; }
  const T* data() const { return p; }
  T* begin() { return p; }
  T* end() { return p + n; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
  size_t size() const { return n; }
};

}  // namespace

struct velo_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  // the device reads and writes pageable host memory coherently through the
  // host's page tables (a Grace-coupled GPU over NVLink-C2C)
  bool coherent_host = false;
  int max_smem_optin = 0;
  int l2_bytes = 0;
  std::string err;

  DevBuf d_input, d_ev_offset, d_ev_hits, d_ev_maxmod, d_ev_valid, d_hit_base, d_arena_off, d_order;
  DevBuf d_tracklets, d_rings, d_weak, d_tracks, d_out_tracks, d_out_counts, d_out_first, d_out_status;
  DevBuf d_counters, d_garena, d_flush, d_fits;

  // staged batch
  bool staged = false;
  int32_t n = 0;
  PinnedVec<uint64_t> h_offset;
  PinnedVec<uint32_t> h_hits, h_maxmod, h_valid;
  PinnedVec<uint64_t> h_hit_base;
  cudaEvent_t meta_copied = nullptr;   // after the last copy out of the pinned metadata
  std::vector<uint32_t> h_status, h_counts;
  uint64_t rows = 0;
  uint32_t max_modules = 0;   // largest S among the staged events
  uint64_t input_bytes = 0;
  uint64_t total_hits = 0;

  // per-launch metadata cache
  bool meta_valid = false;
  uint32_t meta_smem = 0;
  int meta_y = 0;
  int meta_persistent = -1;
  uint32_t configured_smem = 0;
  PinnedVec<uint64_t> h_arena_off;
  PinnedVec<int32_t> h_order;
  int32_t events_in_global = 0;

  void* h_stage = nullptr;
  size_t h_stage_cap = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  velo_stats stats{};
  bool ran = false;

  // learned seeding
  DevBuf d_mlp;
  bool mlp_set = false;
  float keep_threshold = 0.f, window_margin = 0.f, min_keep_rate = 0.f;
  uint32_t learned_max_hits = 0;   // 0: no limit
  std::vector<float> h_mlp;        // host copy, handed on to the pipeline contexts
  uint64_t mlp_version = 0;

  // in-place host I/O of the current batch (velo_options.host_direct):
  // device-visible addresses of the caller's pinned buffers, null = copied
  const uint8_t* io_input = nullptr;
  velo_track* io_tracks = nullptr;
  uint64_t io_capacity = 0;
  unsigned long long* io_cursor = nullptr;   // output cursor shared by pipelined parts

  // the next launch x-sorts each event while staging it and writes the
  // sorted hit arrays back into the input, read in place (velo_sort_search,
  // velo_search_begin with sort)
  bool sort_in_search = false;
  // streamed search in flight (velo_search_begin .. velo_search_end)
  velo_event_result* io_results = nullptr;
  bool streaming = false;

  // pipelined searches (velo_options.pipeline_events): two child contexts,
  // each with its own stream and buffers, that alternate over the parts
  velo_ctx* pipe[2] = {nullptr, nullptr};
  uint64_t pipe_mlp_version[2] = {0, 0};
  // training-data dump of the next launch (velo_dump_doublets)
  DevBuf d_dump_features, d_dump_ids;
  uint64_t dump_capacity = 0;
  uint32_t dump_keep = 0;
  bool dump_armed = false;

  // bumped whenever buffers a captured launch refers to may have moved
  uint64_t generation = 0;
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_key[8] = {};
};

namespace {

using velo::ArenaLayout;
using velo::arena_layout;

velo_status cuda_fail(velo_ctx* c, cudaError_t e, const char* what) {
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? VELO_ERR_OUT_OF_MEMORY : VELO_ERR_CUDA;
}

#define VELO_CUDA(c, call)                                   \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return cuda_fail((c), _e, #call); \
  } while (0)

// A streamed search (velo_search_begin .. velo_search_end) owns the
// context's buffers while it runs: every other call that stages, launches or
// reads results waits for velo_search_end.
bool streaming_refused(velo_ctx* c) {
  if (!c->streaming) return false;
  c->err = "a streamed search is in flight: call velo_search_end first";
  return true;
}

velo_status ensure(velo_ctx* c, DevBuf& b, size_t bytes, const char* what) {
  if (bytes == 0) bytes = 16;
  if (bytes <= b.cap) return VELO_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  const size_t nb = bytes + bytes / 4 + 256;
  cudaError_t e = cudaMalloc(&b.p, nb);
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  b.cap = nb;
  return VELO_OK;
}

template <typename T>
T* P(DevBuf& b) { return reinterpret_cast<T*>(b.p); }

// Host wall time of a scope, written to *out (ms) when the scope ends.
struct HostTimer {
  float* out;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit HostTimer(float* o) : out(o) {}
  ~HostTimer() {
    *out = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

int32_t rd_i32(const uint8_t* p) {
  int32_t v;
  std::memcpy(&v, p, 4);
  return v;
}

// Header checks of the staging path: counts in range and the blob long
// enough for them.  The module table (starts contiguous, counts adding up to
// H) and the coordinates are checked by the search kernel, which marks a bad
// event VELO_EVENT_INVALID, so the host reads 8 bytes per event.
bool check_header(const uint8_t* blob, uint64_t size, uint32_t* H_out, uint32_t* S_out) {
  if (!blob || size < 8) return false;
  const int32_t S = rd_i32(blob), H = rd_i32(blob + 4);
  if (S < 0 || S > VELO_MAX_MODULES || H < 0) return false;
  if (size < 8ull + 12ull * (uint64_t)S + 16ull * (uint64_t)H) return false;
  *H_out = (uint32_t)H;
  *S_out = (uint32_t)S;
  return true;
}

// Header and module-table checks (coordinates are checked on the device).
velo_status check_event(const uint8_t* blob, uint64_t size, uint32_t* H_out, uint32_t* M_out) {
  if (!blob || size < 8) return VELO_ERR_INVALID_EVENT;
  const int32_t S = rd_i32(blob), H = rd_i32(blob + 4);
  if (S < 0 || S > VELO_MAX_MODULES || H < 0) return VELO_ERR_INVALID_EVENT;
  if (size < 8ull + 12ull * (uint64_t)S + 16ull * (uint64_t)H) return VELO_ERR_INVALID_EVENT;
  int64_t acc = 0;
  int32_t maxmod = 0;
  for (int m = 0; m < S; ++m) {
    const int32_t st = rd_i32(blob + 8 + 4 * (S + m));
    const int32_t nm = rd_i32(blob + 8 + 4 * (2 * S + m));
    if (nm < 0 || nm > VELO_MAX_MODULE_HITS || st != acc) return VELO_ERR_INVALID_EVENT;
    acc += nm;
    maxmod = std::max(maxmod, nm);
  }
  if (acc != H) return VELO_ERR_INVALID_EVENT;
  if (H_out) *H_out = (uint32_t)H;
  if (M_out) *M_out = (uint32_t)maxmod;
  return VELO_OK;
}

// Reference per-module x-sort: first-element-pivot partition of
// Tools.cpp:125-157, applied per module over the contiguous hit ranges as
// preorder_by_x does (Tools.cpp:53-64).  Same permutation for equal keys.
void swap4(float* a, float* b, float* c, uint32_t* d, int i, int j) {
  std::swap(a[i], a[j]);
  std::swap(b[i], b[j]);
  std::swap(c[i], c[j]);
  std::swap(d[i], d[j]);
}

int partition4(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
  const float pivot = a[lo];
  int l = lo, r = hi;
  while (l < r) {
    while (a[r] > pivot) r--;
    while (l < r && a[l] <= pivot) l++;
    if (l < r) swap4(a, b, c, d, l, r);
  }
  swap4(a, b, c, d, r, lo);
  return r;
}

void sort_range(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
  std::vector<std::pair<int, int>> stack;
  stack.emplace_back(lo, hi);
  while (!stack.empty()) {
    auto [s, e] = stack.back();
    stack.pop_back();
    if (s >= e) continue;
    const int p = partition4(a, b, c, d, s, e);
    stack.emplace_back(s, p - 1);
    stack.emplace_back(p + 1, e);
  }
}

// Seeding lanes per h0 when the caller leaves the choice to the library.
constexpr int32_t kDefaultSeedLanes = 8;

uint32_t resolve_threads(int32_t t) {
  if (t == 32 || t == 64 || t == 128 || t == 256 || t == 512) return (uint32_t)t;
  return 256;
}

}  // namespace

extern "C" {

void velo_default_options(velo_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  // the fastest configuration measured on GB300 for batches of thousands of
  // events: persistent CTAs of 64 threads, per-event state in L1-cached
  // global scratch (only events of <= 50 hits in shared memory)
  o->y_lanes = 4;
  o->threads_per_event = 64;
  o->launch_mode = VELO_LAUNCH_PERSISTENT;
  o->smem_hits = 50;
  o->narrow_windows = 1;
  o->ctas_per_sm = 0;
  o->use_graph = 0;
  o->register_ctas = 0;
}

const char* velo_status_string(velo_status s) {
  switch (s) {
    case VELO_OK: return "ok";
    case VELO_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VELO_ERR_INVALID_EVENT: return "invalid event blob";
    case VELO_ERR_CAPACITY: return "track buffer too small";
    case VELO_ERR_CUDA: return "CUDA error";
    case VELO_ERR_TIMEOUT: return "device wait timed out (reserved)";
    case VELO_ERR_NO_DEVICE: return "no CUDA device";
    case VELO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case VELO_ERR_NOT_STAGED: return "no staged events";
  }
  return "unknown status";
}

velo_status velo_validate_event(const uint8_t* blob, uint64_t size) {
  velo_status st = check_event(blob, size, nullptr, nullptr);
  if (st != VELO_OK) return st;
  const int32_t S = rd_i32(blob), H = rd_i32(blob + 4);
  const uint8_t* xyz = blob + 8 + 12ull * S + 4ull * H;
  for (int64_t i = 0; i < 3ll * H; ++i) {
    float v;
    std::memcpy(&v, xyz + 4 * i, 4);
    if (!std::isfinite(v)) return VELO_ERR_INVALID_EVENT;
  }
  return VELO_OK;
}

velo_status velo_sort_by_x(uint8_t* blob, uint64_t size) {
  velo_status st = velo_validate_event(blob, size);
  if (st != VELO_OK) return st;
  if (reinterpret_cast<uintptr_t>(blob) & 3u) return VELO_ERR_INVALID_ARGUMENT;
  const int32_t S = rd_i32(blob), H = rd_i32(blob + 4);
  const int32_t* num = reinterpret_cast<const int32_t*>(blob + 8 + 8ull * S);
  uint32_t* id = reinterpret_cast<uint32_t*>(blob + 8 + 12ull * S);
  float* x = reinterpret_cast<float*>(id + H);
  float* y = x + H;
  float* z = y + H;
  int acc = 0;
  for (int m = 0; m < S; ++m) {
    // strictly increasing x: the reference's partition moves nothing there
    bool increasing = true;
    for (int i = acc + 1; i < acc + num[m] && increasing; ++i) increasing = x[i - 1] < x[i];
    if (!increasing) sort_range(x, y, z, id, acc, acc + num[m] - 1);
    acc += num[m];
  }
  return VELO_OK;
}

uint64_t velo_track_capacity(const uint8_t* const* events, const uint64_t* sizes, int32_t n) {
  uint64_t total = 0;
  for (int32_t e = 0; e < n; ++e) {
    int32_t H = 0;
    if (events && events[e] && sizes && sizes[e] >= 8) H = rd_i32(events[e] + 4);
    total += H > 0 ? (uint64_t)H : 1ull;
  }
  return total;
}

velo_status velo_create(velo_ctx** out, int32_t device) {
  if (!out) return VELO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return VELO_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return VELO_ERR_INVALID_ARGUMENT;
  velo_ctx* c = new velo_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->l2_bytes, cudaDevAttrL2CacheSize, device);
  if (e == cudaSuccess) {
    int pageable = 0, host_tables = 0;
    e = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
    c->coherent_host = pageable == 1 && host_tables == 1;
  }
  if (e == cudaSuccess) e = cudaEventCreate(&c->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->e1);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->meta_copied, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    velo_destroy(c);
    return VELO_ERR_CUDA;
  }
  *out = c;
  return VELO_OK;
}

void velo_destroy(velo_ctx* c) {
  if (!c) return;
  velo_destroy(c->pipe[0]);
  velo_destroy(c->pipe[1]);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  DevBuf* bufs[] = {&c->d_input, &c->d_ev_offset, &c->d_ev_hits, &c->d_ev_maxmod, &c->d_ev_valid,
                    &c->d_hit_base, &c->d_arena_off, &c->d_order, &c->d_tracklets, &c->d_rings, &c->d_weak,
                    &c->d_tracks, &c->d_out_tracks, &c->d_out_counts, &c->d_out_first,
                    &c->d_out_status, &c->d_counters, &c->d_garena, &c->d_flush, &c->d_mlp,
                    &c->d_dump_features, &c->d_dump_ids, &c->d_fits};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  if (c->meta_copied) cudaEventDestroy(c->meta_copied);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* velo_last_error(const velo_ctx* c) { return c ? c->err.c_str() : "no context"; }

int32_t velo_device_sm_count(const velo_ctx* c) { return c ? c->sm_count : 0; }

namespace {

// Device-visible address of host memory the GPU can access in place (pinned
// memory mapped into the device's address space); null for anything else.
void* device_view(const void* host) {
  if (!host) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();   // clear the (non-sticky) error of an unknown pointer
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
  return a.devicePointer;
}

velo_status stage_impl(velo_ctx* c, const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes,
                       int32_t n, bool direct, bool pageable = false);

}  // namespace

velo_status velo_stage(velo_ctx* c, const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes,
                       int32_t n) {
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  c->io_tracks = nullptr;
  c->io_capacity = 0;
  c->io_cursor = nullptr;
  return stage_impl(c, buf, offsets, sizes, n, false);
}

namespace {

// Stages a batch: host checks, per-event metadata, and the events themselves
// (copied, or with `direct` read in place when buf is mapped pinned memory;
// with `pageable` as well, on a device with coherent access to pageable host
// memory, read in place wherever they are).
velo_status stage_impl(velo_ctx* c, const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes,
                       int32_t n, bool direct, bool pageable) {
  if (!c || n < 0 || (n > 0 && (!buf || !offsets || !sizes))) return VELO_ERR_INVALID_ARGUMENT;
  if (streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  HostTimer timer(&c->stats.host_stage_ms);
  VELO_CUDA(c, cudaSetDevice(c->device));
  c->io_input = nullptr;
  c->staged = false;
  c->meta_valid = false;
  c->ran = false;
  c->generation++;
  c->n = n;
  // the previous batch's metadata copies have left the pinned arrays
  VELO_CUDA(c, cudaEventSynchronize(c->meta_copied));
  if (!c->h_offset.assign(n, 0) || !c->h_hits.assign(n, 0) || !c->h_maxmod.assign(n, 0) ||
      !c->h_valid.assign(n, 0) || !c->h_hit_base.assign(n, 0)) {
    c->err = "pinned host metadata";
    return VELO_ERR_OUT_OF_MEMORY;
  }
  uint64_t lo = ~0ull, hi = 0;
  for (int32_t e = 0; e < n; ++e) {
    if (offsets[e] & 3u) {
      c->err = "event offsets must be 4-byte aligned";
      return VELO_ERR_INVALID_ARGUMENT;
    }
    if (sizes[e] > ~0ull - offsets[e]) {
      c->err = "event offset + size overflows";
      return VELO_ERR_INVALID_ARGUMENT;
    }
    lo = std::min(lo, offsets[e]);
    hi = std::max(hi, offsets[e] + sizes[e]);
  }
  if (n == 0) lo = hi = 0;
  if (reinterpret_cast<uintptr_t>(buf + lo) & 3u) {
    c->err = "event buffer must be 4-byte aligned";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  uint64_t rows = 0, hits = 0;
  uint32_t max_modules = 0;
  for (int32_t e = 0; e < n; ++e) {
    uint32_t H = 0, S = 0;
    const bool ok = check_header(buf + offsets[e], sizes[e], &H, &S);
    if (ok) max_modules = std::max(max_modules, S);
    c->h_valid[e] = ok ? 1u : 0u;
    c->h_hits[e] = ok ? H : 0u;
    c->h_maxmod[e] = 0u;   // the arena layout depends on H only
    c->h_offset[e] = offsets[e] - lo;
    c->h_hit_base[e] = rows;
    rows += std::max<uint64_t>(c->h_hits[e], 1ull);
    hits += c->h_hits[e];
  }
  c->rows = rows;
  c->total_hits = hits;
  c->max_modules = max_modules;
  c->input_bytes = hi - lo;
  velo_status st;
  if (direct && hi > lo) c->io_input = static_cast<const uint8_t*>(device_view(buf + lo));
  if (direct && pageable && hi > lo && !c->io_input && c->coherent_host) c->io_input = buf + lo;
  if (!c->io_input && (st = ensure(c, c->d_input, c->input_bytes + 16, "input")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_ev_offset, 8ull * n, "offsets")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_ev_hits, 4ull * n, "hits")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_ev_maxmod, 4ull * n, "maxmod")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_ev_valid, 4ull * n, "valid")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_hit_base, 8ull * n, "hit_base")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_tracklets, 16ull * rows, "tracklets")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_rings, 32ull * rows, "rings")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_weak, 4ull * rows, "weak")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_tracks, sizeof(velo_track) * rows, "tracks")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_out_tracks, sizeof(velo_track) * rows, "out_tracks")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_out_counts, 4ull * n, "counts")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_out_first, 8ull * n, "first")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_out_status, 4ull * n, "status")) != VELO_OK) return st;
  if ((st = ensure(c, c->d_counters, 64, "counters")) != VELO_OK) return st;
  if (n > 0) {
    VELO_CUDA(c, cudaMemcpyAsync(c->d_ev_offset.p, c->h_offset.data(), 8ull * n, cudaMemcpyHostToDevice, c->stream));
    VELO_CUDA(c, cudaMemcpyAsync(c->d_ev_hits.p, c->h_hits.data(), 4ull * n, cudaMemcpyHostToDevice, c->stream));
    VELO_CUDA(c, cudaMemcpyAsync(c->d_ev_maxmod.p, c->h_maxmod.data(), 4ull * n, cudaMemcpyHostToDevice, c->stream));
    VELO_CUDA(c, cudaMemcpyAsync(c->d_ev_valid.p, c->h_valid.data(), 4ull * n, cudaMemcpyHostToDevice, c->stream));
    VELO_CUDA(c, cudaMemcpyAsync(c->d_hit_base.p, c->h_hit_base.data(), 8ull * n, cudaMemcpyHostToDevice, c->stream));
    VELO_CUDA(c, cudaEventRecord(c->meta_copied, c->stream));
  }
  // the events last, so that waiting for the metadata copies never waits for them
  if (hi > lo && !c->io_input)
    VELO_CUDA(c, cudaMemcpyAsync(c->d_input.p, buf + lo, hi - lo, cudaMemcpyHostToDevice, c->stream));
  c->staged = true;
  return VELO_OK;
}

}  // namespace

namespace {

velo_status prepare_launch(velo_ctx* c, const velo_options& o, uint32_t* smem_out) {
  const uint32_t Y = (uint32_t)o.y_lanes;
  // shared-memory arena size: largest event arena up to the budget
  uint32_t budget;
  if (o.smem_hits > 0) {
    budget = arena_layout((uint32_t)o.smem_hits, std::min<uint32_t>((uint32_t)o.smem_hits, VELO_MAX_MODULE_HITS), Y).total;
  } else {
    // Resident CTAs per SM beat staging every event in shared memory (events
    // over the budget run from a global-memory arena that L1 caches well), so
    // the automatic budget stages the 40th-percentile event, within 16-100 KB.
    std::vector<uint32_t> hits;
    hits.reserve(c->n);
    for (int32_t e = 0; e < c->n; ++e)
      if (c->h_valid[e]) hits.push_back(c->h_hits[e]);
    uint32_t hq = 0;
    if (!hits.empty()) {
      const size_t k = (hits.size() * 4) / 10;
      std::nth_element(hits.begin(), hits.begin() + (std::ptrdiff_t)std::min(k, hits.size() - 1), hits.end());
      hq = hits[std::min(k, hits.size() - 1)];
    }
    budget = std::max(16u * 1024u, std::min(100u * 1024u, arena_layout(hq, hq, Y).total));
  }
  // room for the static shared state, and for the MLP weights ahead of the arena
  const int reserve = 8 * 1024 + (o.learned ? (int)velo::kMlpSmemBytes : 0);
  const uint32_t limit = (uint32_t)std::max(0, c->max_smem_optin - reserve);
  budget = std::min(budget, limit);
  uint32_t smem = 16;
  for (int32_t e = 0; e < c->n; ++e) {
    if (!c->h_valid[e]) continue;
    const uint32_t need = arena_layout(c->h_hits[e], c->h_maxmod[e], Y).total;
    if (need <= budget) smem = std::max(smem, need);
  }
  const bool persistent = o.launch_mode == VELO_LAUNCH_PERSISTENT;
  if (!c->meta_valid || c->meta_smem != smem || c->meta_y != (int)Y || c->meta_persistent != (int)persistent) {
    VELO_CUDA(c, cudaEventSynchronize(c->meta_copied));   // earlier copies have left the pinned arrays
    if (!c->h_arena_off.assign(c->n, velo::kNoArena) || (persistent && !c->h_order.resize(c->n))) {
      c->err = "pinned host metadata";
      return VELO_ERR_OUT_OF_MEMORY;
    }
    uint64_t goff = 0;
    int32_t nglob = 0;
    for (int32_t e = 0; e < c->n; ++e) {
      if (!c->h_valid[e]) continue;
      const uint32_t need = arena_layout(c->h_hits[e], c->h_maxmod[e], Y).total;
      if (need > smem) {
        c->h_arena_off[e] = goff;
        goff += (need + 255u) & ~255ull;
        nglob++;
      }
    }
    velo_status st;
    if ((st = ensure(c, c->d_arena_off, 8ull * c->n, "arena_off")) != VELO_OK) return st;
    if ((st = ensure(c, c->d_garena, goff, "global arena")) != VELO_OK) return st;
    if (c->n > 0)
      VELO_CUDA(c, cudaMemcpyAsync(c->d_arena_off.p, c->h_arena_off.data(), 8ull * c->n,
                                   cudaMemcpyHostToDevice, c->stream));
    if (persistent) {
      // largest events first (load balance of the work queue): a counting
      // sort on the hit count's top bits, stable within a bucket
      constexpr int kBuckets = 1024;
      uint32_t hmax = 1;
      for (int32_t e = 0; e < c->n; ++e) hmax = std::max(hmax, c->h_hits[e]);
      int shift = 0;
      while ((hmax >> shift) >= (uint32_t)kBuckets) ++shift;
      std::vector<int32_t> start(kBuckets + 1, 0);
      for (int32_t e = 0; e < c->n; ++e) start[kBuckets - 1 - (int)(c->h_hits[e] >> shift) + 1]++;
      for (int b = 0; b < kBuckets; ++b) start[b + 1] += start[b];
      for (int32_t e = 0; e < c->n; ++e) c->h_order[start[kBuckets - 1 - (int)(c->h_hits[e] >> shift)]++] = e;
      if ((st = ensure(c, c->d_order, 4ull * c->n, "order")) != VELO_OK) return st;
      if (c->n > 0)
        VELO_CUDA(c, cudaMemcpyAsync(c->d_order.p, c->h_order.data(), 4ull * c->n,
                                     cudaMemcpyHostToDevice, c->stream));
    }
    if (c->n > 0) VELO_CUDA(c, cudaEventRecord(c->meta_copied, c->stream));
    c->events_in_global = nglob;
    c->generation++;
    c->meta_valid = true;
    c->meta_smem = smem;
    c->meta_y = (int)Y;
    c->meta_persistent = persistent ? 1 : 0;
  }
  if (c->configured_smem < smem) {
    int e = velo::configure_search_kernel(smem);
    if (e != 0) return cuda_fail(c, (cudaError_t)e, "cudaFuncSetAttribute");
    c->configured_smem = smem;
  }
  *smem_out = smem;
  return VELO_OK;
}

velo_status check_options(velo_ctx* c, const velo_options* opts, velo_options* o) {
  if (opts) *o = *opts; else velo_default_options(o);
  if (o->y_lanes < 1 || o->y_lanes > 16) {
    c->err = "y_lanes must be in 1..16";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->launch_mode != VELO_LAUNCH_PER_EVENT && o->launch_mode != VELO_LAUNCH_PERSISTENT) {
    c->err = "unknown launch_mode";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  o->threads_per_event = (int32_t)resolve_threads(o->threads_per_event);
  if (o->pipeline_events < 0) {
    c->err = "pipeline_events must be >= 0";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->seed_lanes == 0) o->seed_lanes = kDefaultSeedLanes % o->y_lanes == 0 ? kDefaultSeedLanes : 32;
  if (o->seed_lanes != 8 && o->seed_lanes != 16 && o->seed_lanes != 32) {
    c->err = "seed_lanes must be 8, 16 or 32";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->seed_lanes < 32 && o->seed_lanes % o->y_lanes != 0) {
    c->err = "seed_lanes below 32 must be a multiple of y_lanes";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->register_ctas == 0) o->register_ctas = o->threads_per_event <= 64 ? 18 : 5;
  if (o->register_ctas != 4 && o->register_ctas != 5 && o->register_ctas != 18) {
    c->err = "register_ctas must be 4, 5 or 18";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->register_ctas == 18 && o->threads_per_event > 64) {
    c->err = "register_ctas 18 is the 64-thread build";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->learned_min_window < 0) {
    c->err = "learned_min_window must be >= 0";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->learned && !c->mlp_set) {
    c->err = "learned seeding needs weights (velo_set_mlp)";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (o->learned || c->dump_armed) {
    if (o->threads_per_event > 256) o->threads_per_event = 256;
    o->use_graph = 0;
  }
  return VELO_OK;
}

// Grid of the launch (the occupancy query stays outside any stream capture).
int launch_mode_of(const velo_ctx* c, const velo_options& o) {
  if (o.learned) return velo::kModeLearned;
  if (c->dump_armed) return velo::kModeDump;
  return velo::kModePlain;
}

// Whether every staged event fits the compact shared-state build.
bool compact_of(const velo_ctx* c) { return c->max_modules < (uint32_t)velo::kCompactModules; }

// Dynamic shared memory of the launch: the arena, after the MLP weights when learned.
uint32_t launch_smem(const velo_options& o, uint32_t arena_smem) {
  return arena_smem + (o.learned ? velo::kMlpSmemBytes : 0u);
}

velo_status launch_shape(velo_ctx* c, const velo_options& o, uint32_t smem, int* grid) {
  *grid = c->n;
  const int ce = velo::configure_search_kernel(launch_smem(o, smem));
  if (ce != 0) return cuda_fail(c, (cudaError_t)ce, "cudaFuncSetAttribute");
  if (o.launch_mode == VELO_LAUNCH_PERSISTENT && c->n > 0) {
    int per_sm = o.ctas_per_sm;
    if (per_sm <= 0) {
      int occ = 0;
      int e = velo::search_occupancy(o.threads_per_event, launch_smem(o, smem), o.register_ctas,
                                     launch_mode_of(c, o), compact_of(c), o.seed_lanes, &occ);
      if (e != 0) return cuda_fail(c, (cudaError_t)e, "occupancy");
      per_sm = std::max(occ, 1);
    }
    *grid = (int)std::min<int64_t>((int64_t)c->sm_count * per_sm, c->n);
  }
  return VELO_OK;
}

// memset of the queue head / output cursor, then the search kernel.
velo_status enqueue_kernel(velo_ctx* c, const velo_options& o, uint32_t smem, int grid) {
  VELO_CUDA(c, cudaMemsetAsync(c->d_counters.p, 0, 64, c->stream));
  if (c->n == 0) return VELO_OK;
  velo::SearchParams p{};
  p.input = c->io_input ? c->io_input : P<uint8_t>(c->d_input);
  p.ev_offset = P<uint64_t>(c->d_ev_offset);
  p.ev_hits = P<uint32_t>(c->d_ev_hits);
  p.ev_maxmod = P<uint32_t>(c->d_ev_maxmod);
  p.ev_valid = P<uint32_t>(c->d_ev_valid);
  p.hit_base = P<uint64_t>(c->d_hit_base);
  p.arena_off = P<uint64_t>(c->d_arena_off);
  p.order = P<int32_t>(c->d_order);
  p.n_events = c->n;
  p.y_lanes = o.y_lanes;
  p.seed_lanes = o.seed_lanes;
  p.narrow = o.narrow_windows ? 1 : 0;
  p.persistent = o.launch_mode == VELO_LAUNCH_PERSISTENT ? 1 : 0;
  p.smem_arena_bytes = smem;
  p.global_arena = P<uint8_t>(c->d_garena);
  p.tracklets = P<uint32_t>(c->d_tracklets);
  p.rings = P<uint32_t>(c->d_rings);
  p.weak = P<uint32_t>(c->d_weak);
  p.tracks = P<velo_track>(c->d_tracks);
  p.out_tracks = c->io_tracks ? c->io_tracks : P<velo_track>(c->d_out_tracks);
  p.out_capacity = c->io_tracks ? c->io_capacity : c->rows;
  p.out_counts = P<uint32_t>(c->d_out_counts);
  p.out_first = P<uint64_t>(c->d_out_first);
  p.out_status = P<uint32_t>(c->d_out_status);
  p.out_cursor = c->io_cursor ? c->io_cursor : P<unsigned long long>(c->d_counters);
  p.results = c->io_results;
  p.sort_events = c->sort_in_search && c->io_input ? 1 : 0;
  p.work_counter = reinterpret_cast<int32_t*>(P<uint8_t>(c->d_counters) + 32);
  if (o.learned) {
    p.mlp = P<float>(c->d_mlp);
    p.keep_threshold = c->keep_threshold;
    p.window_margin = c->window_margin;
    p.min_keep_rate = c->min_keep_rate;
    p.learned_max_hits = c->learned_max_hits;
    p.learned_min_window = o.learned_min_window;
  }
  if (c->dump_armed) {
    p.dump_features = P<float>(c->d_dump_features);
    p.dump_ids = P<uint32_t>(c->d_dump_ids);
    p.dump_count = reinterpret_cast<unsigned long long*>(P<uint8_t>(c->d_counters) + 40);
    p.dump_capacity = c->dump_capacity;
    p.dump_keep = c->dump_keep;
  }
  int e = velo::launch_search(p, grid, o.threads_per_event, launch_smem(o, smem), c->stream, o.register_ctas,
                              compact_of(c));
  if (e != 0) return cuda_fail(c, (cudaError_t)e, "search kernel launch");
  return VELO_OK;
}

// One run: directly, or by replaying a CUDA graph of the same two operations
// (captured once per staged batch and launch configuration).
velo_status enqueue_run(velo_ctx* c, const velo_options& o, uint32_t smem) {
  int grid = 0;
  velo_status st = launch_shape(c, o, smem, &grid);
  if (st != VELO_OK) return st;
  c->stats.launches = c->n > 0 ? 1u : 0u;
  c->stats.grid = grid;
  c->stats.block = o.threads_per_event;
  c->stats.smem_bytes_per_cta = (int32_t)smem;
  if (!o.use_graph) return enqueue_kernel(c, o, smem, grid);
  const uint64_t key[8] = {c->generation, smem, (uint64_t)grid, (uint64_t)o.threads_per_event,
                           (uint64_t)o.register_ctas | ((uint64_t)o.learned << 8) | ((uint64_t)o.seed_lanes << 16),
                           (uint64_t)o.y_lanes,
                           (uint64_t)o.narrow_windows, (uint64_t)o.launch_mode};
  if (!c->graph || std::memcmp(key, c->graph_key, sizeof key) != 0) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    cudaGraph_t g = nullptr;
    VELO_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    st = enqueue_kernel(c, o, smem, grid);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (st != VELO_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) return cuda_fail(c, ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      c->graph = nullptr;
      return cuda_fail(c, ce, "cudaGraphInstantiate");
    }
    std::memcpy(c->graph_key, key, sizeof key);
  }
  VELO_CUDA(c, cudaGraphLaunch(c->graph, c->stream));
  return VELO_OK;
}

}  // namespace

velo_status velo_run(velo_ctx* c, const velo_options* opts) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  HostTimer timer(&c->stats.host_launch_ms);
  velo_options o;
  velo_status st = check_options(c, opts, &o);
  if (st != VELO_OK) return st;
  VELO_CUDA(c, cudaSetDevice(c->device));
  uint32_t smem = 0;
  if ((st = prepare_launch(c, o, &smem)) != VELO_OK) return st;
  VELO_CUDA(c, cudaEventRecord(c->e0, c->stream));
  if ((st = enqueue_run(c, o, smem)) != VELO_OK) return st;
  VELO_CUDA(c, cudaEventRecord(c->e1, c->stream));
  c->ran = true;
  c->stats.n_events = (uint32_t)c->n;
  c->stats.total_hits = c->total_hits;
  c->stats.input_bytes = c->input_bytes;
  c->stats.events_in_global = c->events_in_global;
  return VELO_OK;
}

velo_status velo_synchronize(velo_ctx* c) {
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  return VELO_OK;
}

velo_status velo_fetch(velo_ctx* c, velo_track* tracks_out, uint64_t capacity, uint32_t* counts,
                       uint64_t* first, uint32_t* status) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->ran) return VELO_ERR_NOT_STAGED;
  VELO_CUDA(c, cudaSetDevice(c->device));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  HostTimer timer(&c->stats.host_fetch_ms);
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c->e0, c->e1) == cudaSuccess) c->stats.kernel_ms = ms;
  unsigned long long total = 0;
  if (!c->io_cursor)
    VELO_CUDA(c, cudaMemcpyAsync(&total, c->d_counters.p, 8, cudaMemcpyDeviceToHost, c->stream));
  if (c->n > 0) {
    if (counts)
      VELO_CUDA(c, cudaMemcpyAsync(counts, c->d_out_counts.p, 4ull * c->n, cudaMemcpyDeviceToHost, c->stream));
    if (first)
      VELO_CUDA(c, cudaMemcpyAsync(first, c->d_out_first.p, 8ull * c->n, cudaMemcpyDeviceToHost, c->stream));
    c->h_status.resize(c->n);
    VELO_CUDA(c, cudaMemcpyAsync(c->h_status.data(), c->d_out_status.p, 4ull * c->n,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (c->io_cursor && !counts) {
      c->h_counts.resize(c->n);
      VELO_CUDA(c, cudaMemcpyAsync(c->h_counts.data(), c->d_out_counts.p, 4ull * c->n,
                                   cudaMemcpyDeviceToHost, c->stream));
    }
  }
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  if (status && c->n > 0) std::memcpy(status, c->h_status.data(), 4ull * c->n);
  if (c->io_cursor) {   // a part of a pipelined batch: its own tracks are the sum of its counts
    const uint32_t* cn = counts ? counts : c->h_counts.data();
    for (int32_t e = 0; e < c->n; ++e) total += cn[e];
  }
  c->stats.total_tracks = total;
  c->stats.output_bytes = 4ull * c->n + sizeof(velo_track) * total;
  if (c->io_tracks) {   // written in place by the kernel
    if (!c->io_cursor && total > c->io_capacity) {
      c->err = "track buffer holds " + std::to_string(c->io_capacity) + " tracks, " + std::to_string(total) +
               " needed";
      return VELO_ERR_CAPACITY;
    }
    return VELO_OK;
  }
  if (tracks_out == nullptr && capacity == 0) return VELO_OK;
  if (total > capacity) {
    c->err = "track buffer holds " + std::to_string(capacity) + " tracks, " + std::to_string(total) + " needed";
    return VELO_ERR_CAPACITY;
  }
  if (total > 0)
    VELO_CUDA(c, cudaMemcpyAsync(tracks_out, c->d_out_tracks.p, sizeof(velo_track) * total,
                                 cudaMemcpyDeviceToHost, c->stream));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  return VELO_OK;
}

velo_status velo_get_stats(const velo_ctx* c, velo_stats* s) {
  if (!c || !s) return VELO_ERR_INVALID_ARGUMENT;
  *s = c->stats;
  return VELO_OK;
}

namespace {

// A batch cut into parts of o.pipeline_events events that alternate between
// two child contexts: while part k is searched on one stream, part k+1's
// events go up and part k-1's tracks come down on the other.  Each part's
// tracks land after the previous part's in tracks_out; first[] is rebased.
velo_status search_pipelined(velo_ctx* c, const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes,
                             int32_t n, const velo_options& o, velo_track* tracks_out, uint64_t capacity,
                             uint32_t* counts, uint64_t* first, uint32_t* status) {
  velo_options po = o;
  po.pipeline_events = 0;
  po.use_graph = 0;   // parts differ in size; a graph per part would be captured once and replayed once
  for (int k = 0; k < 2; ++k) {
    if (!c->pipe[k]) {
      velo_status st = velo_create(&c->pipe[k], c->device);
      if (st != VELO_OK) {
        c->err = "pipeline context: " + std::string(velo_status_string(st));
        return st;
      }
    }
    if (o.learned && c->pipe_mlp_version[k] != c->mlp_version) {
      velo_status st = velo_set_mlp(c->pipe[k], c->h_mlp.data(), c->keep_threshold, c->window_margin,
                                    c->min_keep_rate, c->learned_max_hits);
      if (st != VELO_OK) {
        c->err = c->pipe[k]->err;
        return st;
      }
      c->pipe_mlp_version[k] = c->mlp_version;
    }
  }
  // the parent holds no batch from here on
  c->staged = false;
  c->ran = false;
  c->generation++;
  // in-place output: all parts reserve rows from one cursor in the caller's
  // buffer, so first[] needs no rebasing
  velo_track* direct_out =
      (o.host_direct && tracks_out && capacity) ? static_cast<velo_track*>(device_view(tracks_out)) : nullptr;
  if (direct_out) {
    velo_status st = ensure(c, c->d_counters, 64, "counters");
    if (st != VELO_OK) return st;
    VELO_CUDA(c, cudaMemsetAsync(c->d_counters.p, 0, 64, c->stream));
    VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  for (int k = 0; k < 2; ++k) {
    c->pipe[k]->io_tracks = direct_out;
    c->pipe[k]->io_capacity = direct_out ? capacity : 0;
    c->pipe[k]->io_cursor = direct_out ? P<unsigned long long>(c->d_counters) : nullptr;
  }
  const int32_t part = o.pipeline_events;
  const int32_t n_parts = (n + part - 1) / part;
  uint64_t base = 0, hits = 0, in_bytes = 0;
  float kernel_ms = 0.f, stage_ms = 0.f, launch_ms = 0.f, fetch_ms = 0.f;
  int32_t bad_event = -1;
  velo_status first_error = VELO_OK;
  auto finish = [&](int32_t k) -> velo_status {
    velo_ctx* ch = c->pipe[k & 1];
    const int32_t a = k * part, b = std::min(n, a + part);
    const bool want_tracks = tracks_out != nullptr || capacity != 0;
    velo_status st = velo_fetch(ch, want_tracks && !direct_out ? tracks_out + base : nullptr,
                                want_tracks && !direct_out ? (capacity > base ? capacity - base : 0) : 0,
                                counts ? counts + a : nullptr, first ? first + a : nullptr,
                                status ? status + a : nullptr);
    if (st != VELO_OK) {
      c->err = ch->err;
      return st;
    }
    if (first && !direct_out)
      for (int32_t e = a; e < b; ++e) first[e] += base;
    for (int32_t e = a; e < b && bad_event < 0; ++e)
      if (ch->h_status[e - a] & VELO_EVENT_INVALID) bad_event = e;
    base += ch->stats.total_tracks;
    hits += ch->stats.total_hits;
    in_bytes += ch->stats.input_bytes;
    kernel_ms += ch->stats.kernel_ms;
    stage_ms += ch->stats.host_stage_ms;
    launch_ms += ch->stats.host_launch_ms;
    fetch_ms += ch->stats.host_fetch_ms;
    return VELO_OK;
  };
  for (int32_t k = 0; k < n_parts; ++k) {
    if (k >= 2 && first_error == VELO_OK) first_error = finish(k - 2);
    if (first_error != VELO_OK) break;
    velo_ctx* ch = c->pipe[k & 1];
    const int32_t a = k * part, b = std::min(n, a + part);
    velo_status st = stage_impl(ch, buf, offsets + a, sizes + a, b - a, o.host_direct != 0);
    if (st == VELO_OK) st = velo_run(ch, &po);
    if (st != VELO_OK) {
      c->err = ch->err;
      first_error = st;
      break;
    }
  }
  // drain: the last two parts (and, after an error, whatever is in flight)
  for (int k = 0; k < 2; ++k) cudaStreamSynchronize(c->pipe[k]->stream);
  auto release = [&]() {   // the children pointed into the caller's buffers
    for (int k = 0; k < 2; ++k) {
      velo_ctx* ch = c->pipe[k];
      ch->io_input = nullptr;
      ch->io_tracks = nullptr;
      ch->io_capacity = 0;
      ch->io_cursor = nullptr;
      ch->staged = false;
      ch->ran = false;
    }
  };
  if (first_error != VELO_OK) {
    release();
    return first_error;
  }
  for (int32_t k = std::max(0, n_parts - 2); k < n_parts; ++k) {
    velo_status st = finish(k);
    if (st != VELO_OK) {
      release();
      return st;
    }
  }
  release();
  if (direct_out && base > capacity) {
    c->err = "track buffer holds " + std::to_string(capacity) + " tracks, " + std::to_string(base) + " needed";
    return VELO_ERR_CAPACITY;
  }
  c->stats.n_events = (uint32_t)n;
  c->stats.total_hits = hits;
  c->stats.input_bytes = in_bytes;
  c->stats.total_tracks = base;
  c->stats.output_bytes = 4ull * n + sizeof(velo_track) * base;
  c->stats.kernel_ms = kernel_ms;
  c->stats.host_stage_ms = stage_ms;
  c->stats.host_launch_ms = launch_ms;
  c->stats.host_fetch_ms = fetch_ms;
  c->stats.launches = (uint32_t)n_parts;
  if (bad_event >= 0) {
    c->err = "event " + std::to_string(bad_event) + " failed validation";
    return VELO_ERR_INVALID_EVENT;
  }
  return VELO_OK;
}

}  // namespace

namespace {

// Upper bound of the device bytes one event takes in a staged batch, from its
// blob size alone (H <= (size - 8) / 16): per hit row 152 B of scratch
// (tracklet, rings, weak, working track), 100 B of output and 21 B of arena,
// plus the blob itself and its metadata.
uint64_t event_device_bytes(uint64_t size) {
  const uint64_t rows = std::max<uint64_t>(size >= 8 ? (size - 8) / 16 : 0, 1);
  return rows * (152 + 100 + 21) + size + 64;
}

// Events per part when the batch would not fit the device budget, else 0.
int32_t budget_part(velo_ctx* c, const uint64_t* sizes, int32_t n, int32_t budget_mb) {
  if (n < 2) return 0;
  uint64_t need = 0;
  for (int32_t e = 0; e < n; ++e) need += event_device_bytes(sizes[e]);
  uint64_t budget = (uint64_t)budget_mb << 20;
  if (budget_mb <= 0) {
    if (need < (256ull << 20)) return 0;   // small batches never ask the driver
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    budget = free_b / 2;
  }
  if (need <= budget) return 0;
  // two parts are in flight at a time, each in its own child context
  const uint64_t part = (uint64_t)n * (budget / 2) / need;
  return (int32_t)std::max<uint64_t>(part, 1);
}

}  // namespace

velo_status velo_search_packed(velo_ctx* c, const uint8_t* buf, const uint64_t* offsets,
                               const uint64_t* sizes, int32_t n, const velo_options* opts,
                               velo_track* tracks_out, uint64_t capacity, uint32_t* counts,
                               uint64_t* first, uint32_t* status) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || n < 0 || (n > 0 && (!buf || !offsets || !sizes))) return VELO_ERR_INVALID_ARGUMENT;
  if (!opts || opts->pipeline_events <= 0) {
    const int32_t part = budget_part(c, sizes, n, opts ? opts->device_budget_mb : 0);
    if (part > 0) {   // too large for one staging: pipelined parts that fit
      velo_options o;
      velo_status st = check_options(c, opts, &o);
      if (st != VELO_OK) return st;
      VELO_CUDA(c, cudaSetDevice(c->device));
      o.pipeline_events = part;
      if (n <= 2 * part) o.pipeline_events = (n + 2) / 3;   // at least three parts
      return search_pipelined(c, buf, offsets, sizes, n, o, tracks_out, capacity, counts, first, status);
    }
  }
  if (opts && opts->pipeline_events > 0 && n > 2 * opts->pipeline_events) {
    velo_options o;
    velo_status st = check_options(c, opts, &o);
    if (st != VELO_OK) return st;
    VELO_CUDA(c, cudaSetDevice(c->device));
    return search_pipelined(c, buf, offsets, sizes, n, o, tracks_out, capacity, counts, first, status);
  }
  if (opts && opts->host_direct) {
    velo_options o;
    velo_status st = check_options(c, opts, &o);
    if (st != VELO_OK) return st;
    VELO_CUDA(c, cudaSetDevice(c->device));
    o.use_graph = 0;   // the buffers change from call to call
    c->io_tracks = (tracks_out && capacity) ? static_cast<velo_track*>(device_view(tracks_out)) : nullptr;
    c->io_capacity = c->io_tracks ? capacity : 0;
    c->io_cursor = nullptr;
    st = stage_impl(c, buf, offsets, sizes, n, true);
    if (st == VELO_OK) st = velo_run(c, &o);
    if (st == VELO_OK) st = velo_fetch(c, tracks_out, capacity, counts, first, status);
    const bool in_place = c->io_input != nullptr || c->io_tracks != nullptr;
    c->io_input = nullptr;
    c->io_tracks = nullptr;
    c->io_capacity = 0;
    if (in_place) {   // the batch pointed into the caller's buffers
      c->staged = false;
      c->ran = false;
      c->generation++;
    }
    if (st != VELO_OK) return st;
    for (int32_t e = 0; e < n; ++e)
      if (c->h_status[e] & VELO_EVENT_INVALID) {
        c->err = "event " + std::to_string(e) + " failed validation";
        return VELO_ERR_INVALID_EVENT;
      }
    return VELO_OK;
  }
  velo_status st = velo_stage(c, buf, offsets, sizes, n);
  if (st != VELO_OK) return st;
  if ((st = velo_run(c, opts)) != VELO_OK) return st;
  st = velo_fetch(c, tracks_out, capacity, counts, first, status);
  if (st != VELO_OK) return st;
  for (int32_t e = 0; e < n; ++e)
    if (c->h_status[e] & VELO_EVENT_INVALID) {
      c->err = "event " + std::to_string(e) + " failed validation";
      return VELO_ERR_INVALID_EVENT;
    }
  return VELO_OK;
}

}  // extern "C"

namespace {

// Runs f(a, b) over [0, n) on up to 16 host threads when `bytes` is large.
template <class F>
void host_parallel(int32_t n, uint64_t bytes, F f) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (bytes <= (64ull << 20) || hw <= 1 || n <= 64) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int32_t chunk = (n + (int32_t)hw - 1) / (int32_t)hw;
  for (unsigned t = 0; t < hw; ++t) {
    const int32_t a = (int32_t)t * chunk, b = std::min(n, a + chunk);
    if (a < b) th.emplace_back(f, a, b);
  }
  for (auto& t : th) t.join();
}

// Packs the events into the context's pinned staging buffer at 16-byte
// aligned offsets (offs_out); returns the buffer, or null on failure.
uint8_t* gather_pinned(velo_ctx* c, const uint8_t* const* events, const uint64_t* sizes, int32_t n,
                       std::vector<uint64_t>& offs, uint64_t* total_out) {
  offs.resize(n);
  uint64_t total = 0;
  for (int32_t e = 0; e < n; ++e) {
    offs[e] = total;
    total += (sizes[e] + 15) & ~15ull;
  }
  if (total + 16 > c->h_stage_cap) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_cap = 0;
    const size_t nb = total + total / 4 + 4096;
    const cudaError_t e = cudaHostAlloc(&c->h_stage, nb, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      cuda_fail(c, e, "cudaHostAlloc");
      c->h_stage = nullptr;
      return nullptr;
    }
    c->h_stage_cap = nb;
  }
  uint8_t* stage = static_cast<uint8_t*>(c->h_stage);
  host_parallel(n, total, [&](int32_t a, int32_t b) {
    for (int32_t e = a; e < b; ++e)
      if (events[e] && sizes[e]) std::memcpy(stage + offs[e], events[e], sizes[e]);
  });
  *total_out = total;
  return stage;
}

// Offsets of the caller's event buffers from the lowest of them, for a batch
// the device reads where it lies; false if an event is not 4-byte aligned.
bool offsets_in_place(const uint8_t* const* events, const uint64_t* sizes, int32_t n, const uint8_t** base,
                      std::vector<uint64_t>& offs) {
  uintptr_t lo = ~(uintptr_t)0;
  for (int32_t e = 0; e < n; ++e) {
    if (!sizes[e]) continue;
    const uintptr_t a = reinterpret_cast<uintptr_t>(events[e]);
    if (!events[e] || (a & 3u)) return false;
    lo = std::min(lo, a);
  }
  if (lo == ~(uintptr_t)0) lo = 0;
  offs.resize(n);
  for (int32_t e = 0; e < n; ++e)
    offs[e] = sizes[e] ? (uint64_t)(reinterpret_cast<uintptr_t>(events[e]) - lo) : 0ull;
  *base = reinterpret_cast<const uint8_t*>(lo);
  return true;
}

// One batch read (and with `sort` x-sorted) in place: the events at
// base + offs[e] are either in the pinned staging buffer or, on a device
// with coherent access to pageable host memory, in the caller's own
// buffers.  Tracks go to tracks_out in place when the device can write it.
velo_status search_in_place(velo_ctx* c, const uint8_t* base, const uint64_t* offs, const uint64_t* sizes,
                            int32_t n, velo_options o, bool sort, velo_track* tracks_out, uint64_t capacity,
                            uint32_t* counts, uint64_t* first, uint32_t* status, bool* read_in_place) {
  o.use_graph = 0;   // the buffers change from call to call
  c->io_tracks = nullptr;
  if (tracks_out && capacity) {
    c->io_tracks = static_cast<velo_track*>(device_view(tracks_out));
    if (!c->io_tracks && c->coherent_host) c->io_tracks = tracks_out;
  }
  c->io_capacity = c->io_tracks ? capacity : 0;
  c->io_cursor = nullptr;
  velo_status st = stage_impl(c, base, offs, sizes, n, true, true);
  *read_in_place = c->io_input != nullptr;
  if (st == VELO_OK && sort && !*read_in_place && n > 0) {   // never: base is device-readable
    c->err = "events to sort are not readable in place";
    st = VELO_ERR_INVALID_ARGUMENT;
  }
  c->sort_in_search = sort;   // the search kernel sorts while staging, and writes back
  if (st == VELO_OK) st = velo_run(c, &o);
  if (st == VELO_OK) st = velo_fetch(c, tracks_out, capacity, counts, first, status);
  uint64_t bytes = 0;
  for (int32_t e = 0; e < n; ++e) bytes += sizes[e];
  c->input_bytes = bytes;
  c->io_input = nullptr;
  c->io_tracks = nullptr;
  c->io_capacity = 0;
  c->sort_in_search = false;
  c->staged = false;   // the batch pointed into the caller's buffers
  c->ran = false;
  c->generation++;
  if (st != VELO_OK) return st;
  for (int32_t e = 0; e < n; ++e)
    if (c->h_status[e] & VELO_EVENT_INVALID) {
      c->err = "event " + std::to_string(e) + " failed validation";
      return VELO_ERR_INVALID_EVENT;
    }
  return VELO_OK;
}

// Device-visible address of a track buffer the kernel writes in place
// (mapped pinned memory, or any host memory on a coherent host), or null.
velo_track* tracks_in_place(velo_ctx* c, velo_track* tracks_out, uint64_t capacity) {
  if (!tracks_out || !capacity) return nullptr;
  velo_track* t = static_cast<velo_track*>(device_view(tracks_out));
  if (!t && c->coherent_host) t = tracks_out;
  return t;
}

// Ends a batch that pointed into the caller's buffers.
velo_status end_in_place(velo_ctx* c, velo_status r) {
  c->io_tracks = nullptr;
  c->io_capacity = 0;
  c->io_results = nullptr;
  c->sort_in_search = false;
  c->streaming = false;
  c->staged = false;
  c->ran = false;
  c->generation++;
  return r;
}

}  // namespace

extern "C" {

velo_status velo_search(velo_ctx* c, const uint8_t* const* events, const uint64_t* sizes, int32_t n,
                        const velo_options* opts, velo_track* tracks_out, uint64_t capacity,
                        uint32_t* counts, uint64_t* first, uint32_t* status) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || n < 0 || (n > 0 && (!events || !sizes))) return VELO_ERR_INVALID_ARGUMENT;
  VELO_CUDA(c, cudaSetDevice(c->device));
  std::vector<uint64_t> offs;
  if (opts && opts->host_direct && opts->pipeline_events <= 0 && c->coherent_host &&
      budget_part(c, sizes, n, opts->device_budget_mb) == 0) {
    // the device reads the caller's buffers where they are: no packing
    const uint8_t* base = nullptr;
    if (offsets_in_place(events, sizes, n, &base, offs)) {
      velo_options o;
      velo_status st = check_options(c, opts, &o);
      if (st != VELO_OK) return st;
      bool in_place = false;
      return search_in_place(c, base, offs.data(), sizes, n, o, false, tracks_out, capacity, counts, first,
                             status, &in_place);
    }
  }
  uint64_t total = 0;
  uint8_t* stage = gather_pinned(c, events, sizes, n, offs, &total);
  if (!stage) return VELO_ERR_OUT_OF_MEMORY;
  return velo_search_packed(c, stage, offs.data(), sizes, n, opts, tracks_out, capacity, counts, first,
                            status);
}

velo_status velo_sort_search(velo_ctx* c, uint8_t* const* events, const uint64_t* sizes, int32_t n,
                             const velo_options* opts, velo_track* tracks_out, uint64_t capacity,
                             uint32_t* counts, uint64_t* first, uint32_t* status) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || n < 0 || (n > 0 && (!events || !sizes))) return VELO_ERR_INVALID_ARGUMENT;
  velo_options o;
  velo_status st = check_options(c, opts, &o);
  if (st != VELO_OK) return st;
  VELO_CUDA(c, cudaSetDevice(c->device));
  for (int32_t e = 0; e < n; ++e)
    if (sizes[e] && (!events[e] || (reinterpret_cast<uintptr_t>(events[e]) & 3u))) {
      c->err = "event " + std::to_string(e) + ": buffer missing or not 4-byte aligned";
      return VELO_ERR_INVALID_ARGUMENT;
    }
  if (budget_part(c, sizes, n, o.device_budget_mb) > 0) {
    c->err = "batch larger than the device budget: call with fewer events";
    return VELO_ERR_OUT_OF_MEMORY;
  }
  std::vector<uint64_t> offs;
  bool in_place = false;
  if (c->coherent_host && o.host_direct) {
    // sorted (while the search kernel stages each event) and searched where
    // the caller's buffers lie
    const uint8_t* base = nullptr;
    offsets_in_place(events, sizes, n, &base, offs);
    st = search_in_place(c, base, offs.data(), sizes, n, o, true, tracks_out, capacity, counts, first, status,
                         &in_place);
    if (in_place || n == 0 || st != VELO_OK) return st;
  }
  // packed into pinned memory, sorted and searched there, the sorted bytes
  // copied back into the caller's buffers
  uint64_t total = 0;
  const uint8_t* const* cev = events;
  uint8_t* stage = gather_pinned(c, cev, sizes, n, offs, &total);
  if (!stage) return VELO_ERR_OUT_OF_MEMORY;
  st = search_in_place(c, stage, offs.data(), sizes, n, o, true, tracks_out, capacity, counts, first, status,
                       &in_place);
  if (st != VELO_OK && st != VELO_ERR_INVALID_EVENT) return st;
  host_parallel(n, total, [&](int32_t a, int32_t b) {
    for (int32_t e = a; e < b; ++e)
      if (sizes[e]) std::memcpy(events[e], stage + offs[e], sizes[e]);
  });
  return st;
}

velo_status velo_search_begin(velo_ctx* c, uint8_t* const* events, const uint64_t* sizes, int32_t n,
                              const velo_options* opts, int32_t sort, velo_track* tracks_out, uint64_t capacity,
                              velo_event_result* results) {
  if (!c || n < 0 || (n > 0 && (!events || !sizes || !tracks_out || !results))) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->coherent_host) {
    c->err = "streamed results need a device with coherent access to host memory";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  if (c->streaming) {
    c->err = "a streamed search is in flight: call velo_search_end first";
    return VELO_ERR_INVALID_ARGUMENT;
  }
  velo_options o;
  velo_status st = check_options(c, opts, &o);
  if (st != VELO_OK) return st;
  o.use_graph = 0;
  VELO_CUDA(c, cudaSetDevice(c->device));
  for (int32_t e = 0; e < n; ++e)
    if (sizes[e] && (!events[e] || (reinterpret_cast<uintptr_t>(events[e]) & 3u))) {
      c->err = "event " + std::to_string(e) + ": buffer missing or not 4-byte aligned";
      return VELO_ERR_INVALID_ARGUMENT;
    }
  if (budget_part(c, sizes, n, o.device_budget_mb) > 0) {
    c->err = "batch larger than the device budget: call with fewer events";
    return VELO_ERR_OUT_OF_MEMORY;
  }
  std::vector<uint64_t> offs;
  const uint8_t* base = nullptr;
  offsets_in_place(events, sizes, n, &base, offs);
  std::memset(results, 0, sizeof(velo_event_result) * (size_t)n);
  c->io_tracks = tracks_in_place(c, tracks_out, capacity);
  c->io_capacity = capacity;
  c->io_cursor = nullptr;
  st = stage_impl(c, base, offs.data(), sizes, n, true, true);   // read in place
  if (st == VELO_OK && c->rows > capacity) {
    c->err = "track buffer holds " + std::to_string(capacity) + " tracks, velo_track_capacity is " +
             std::to_string(c->rows);
    st = VELO_ERR_INVALID_ARGUMENT;
  }
  if (st == VELO_OK && n > 0 && !c->io_input) {
    c->err = "events not readable in place";
    st = VELO_ERR_INVALID_ARGUMENT;
  }
  if (st != VELO_OK) return end_in_place(c, st);
  c->io_results = results;
  c->sort_in_search = sort != 0;   // the search kernel sorts while staging, and writes back
  st = velo_run(c, &o);
  if (st != VELO_OK) {
    cudaStreamSynchronize(c->stream);
    return end_in_place(c, st);
  }
  c->streaming = true;
  return VELO_OK;
}

velo_status velo_search_end(velo_ctx* c, uint32_t* counts, uint64_t* first, uint32_t* status) {
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->streaming) return VELO_ERR_NOT_STAGED;
  c->streaming = false;   // the fetch below is this search's own
  velo_status st = velo_fetch(c, nullptr, 0, counts, first, status);   // waits for the sort and the search
  if (st == VELO_OK)
    for (int32_t e = 0; e < c->n; ++e)
      if (c->h_status[e] & VELO_EVENT_INVALID) {
        c->err = "event " + std::to_string(e) + " failed validation";
        st = VELO_ERR_INVALID_EVENT;
        break;
      }
  return end_in_place(c, st);
}

velo_status velo_time_runs(velo_ctx* c, const velo_options* opts, int32_t warmup, int32_t iters,
                           int32_t flush_l2, float* ms_out) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || iters <= 0 || warmup < 0 || !ms_out) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  velo_options o;
  velo_status st = check_options(c, opts, &o);
  if (st != VELO_OK) return st;
  VELO_CUDA(c, cudaSetDevice(c->device));
  uint32_t smem = 0;
  if ((st = prepare_launch(c, o, &smem)) != VELO_OK) return st;
  const size_t flush_bytes = (size_t)std::max(c->l2_bytes, 1 << 20) * 2;
  if (flush_l2 && (st = ensure(c, c->d_flush, flush_bytes, "l2 flush")) != VELO_OK) return st;
  for (int32_t i = 0; i < warmup; ++i)
    if ((st = enqueue_run(c, o, smem)) != VELO_OK) return st;
  double total = 0.0;
  for (int32_t i = 0; i < iters; ++i) {
    if (flush_l2) VELO_CUDA(c, cudaMemsetAsync(c->d_flush.p, i & 0xff, flush_bytes, c->stream));
    VELO_CUDA(c, cudaEventRecord(c->e0, c->stream));
    if ((st = enqueue_run(c, o, smem)) != VELO_OK) return st;
    VELO_CUDA(c, cudaEventRecord(c->e1, c->stream));
    VELO_CUDA(c, cudaEventSynchronize(c->e1));
    float ms = 0.f;
    VELO_CUDA(c, cudaEventElapsedTime(&ms, c->e0, c->e1));
    total += ms;
  }
  *ms_out = (float)(total / iters);
  c->ran = true;
  c->stats.kernel_ms = *ms_out;
  c->stats.n_events = (uint32_t)c->n;
  c->stats.total_hits = c->total_hits;
  c->stats.input_bytes = c->input_bytes;
  c->stats.events_in_global = c->events_in_global;
  return VELO_OK;
}

velo_status velo_autotune(velo_ctx* c, const velo_options* base, int32_t iters, velo_options* best_out,
                          float* best_ms_out) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || !best_out || iters <= 0) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  velo_options b0;
  velo_status st = check_options(c, base, &b0);
  if (st != VELO_OK) return st;
  // median device milliseconds of `n` runs of `o`, L2 flushed before each
  auto time_median = [&](const velo_options& o, int32_t n, float* med) -> velo_status {
    std::vector<float> ms(n);
    for (int32_t i = 0; i < n; ++i) {
      velo_status s2 = velo_time_runs(c, &o, i == 0 ? 1 : 0, 1, 1, &ms[i]);
      if (s2 != VELO_OK) return s2;
    }
    std::nth_element(ms.begin(), ms.begin() + n / 2, ms.end());
    *med = ms[n / 2];
    return VELO_OK;
  };
  // Stage 1: threads per event x shared-memory tile (hits staged per CTA;
  // 0 = the automatic budget) x register build x launch style, at the
  // caller's seed_lanes; narrowing stays on (it only removes work) and
  // y_lanes is the caller's (it defines results).  32-thread CTAs are
  // supported but measured far slower (1.5x at best).
  static const int32_t kThreads[] = {64, 128, 256, 512};
  static const int32_t kSmemHits[] = {0, 50, 100, 200, 300, 600, 900, 1200, 1600, 2400};
  static const int32_t kRegs[] = {4, 5, 18};
  static const int32_t kModes[] = {VELO_LAUNCH_PER_EVENT, VELO_LAUNCH_PERSISTENT};
  std::vector<std::pair<float, velo_options>> stage1;
  for (int32_t mode : kModes)
    for (int32_t regs : kRegs)
      for (int32_t threads : kThreads)
        for (int32_t hits : kSmemHits) {
          if (threads > 256 && regs != 5) continue;   // one build above 256 threads
          if (regs == 18 && threads != 64) continue;  // the 64-thread build
          velo_options o = b0;
          o.launch_mode = mode;
          o.register_ctas = regs;
          o.threads_per_event = threads;
          o.smem_hits = hits;
          o.narrow_windows = 1;
          float med = 0.f;
          if ((st = time_median(o, iters, &med)) != VELO_OK) return st;
          stage1.emplace_back(med, o);
        }
  std::stable_sort(stage1.begin(), stage1.end(),
                   [](const std::pair<float, velo_options>& a, const std::pair<float, velo_options>& b) {
                     return a.first < b.first;
                   });
  // Stage 2: the three fastest launches x seeding lanes per h0 {8, 16, 32}
  // (the seeding window's width; below 32 only multiples of y_lanes), each
  // re-timed over more runs, so that near-equal launches are told apart.
  const int32_t iters2 = std::max<int32_t>(4 * iters, 12);
  float best = 0.f;
  bool have = false;
  for (size_t k = 0; k < stage1.size() && k < 3; ++k)
    for (int32_t lanes : {8, 16, 32}) {
      if (lanes < 32 && lanes % b0.y_lanes != 0) continue;
      velo_options o = stage1[k].second;
      o.seed_lanes = lanes;
      float med = 0.f;
      if ((st = time_median(o, iters2, &med)) != VELO_OK) return st;
      if (!have || med < best) {
        best = med;
        *best_out = o;
        have = true;
      }
    }
  if (best_ms_out) *best_ms_out = best;
  return VELO_OK;
}

velo_status velo_sort_staged(velo_ctx* c) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  VELO_CUDA(c, cudaSetDevice(c->device));
  // a batch read in place is sorted in place (velo_sort_search)
  uint8_t* events = c->io_input ? const_cast<uint8_t*>(c->io_input) : P<uint8_t>(c->d_input);
  const int e = velo::launch_sort_modules(events, P<uint64_t>(c->d_ev_offset), P<uint32_t>(c->d_ev_valid), c->n,
                                          c->stream);
  if (e != 0) return cuda_fail(c, (cudaError_t)e, "sort kernel launch");
  return VELO_OK;
}

velo_status velo_fit_tracks(velo_ctx* c, velo_track_fit* fits_out, uint64_t capacity) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || (!fits_out && capacity)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->ran) return VELO_ERR_NOT_STAGED;
  VELO_CUDA(c, cudaSetDevice(c->device));
  velo_status st = ensure(c, c->d_fits, sizeof(velo_track_fit) * (c->rows ? c->rows : 1), "fits");
  if (st != VELO_OK) return st;
  unsigned long long total = 0;
  VELO_CUDA(c, cudaMemcpyAsync(&total, c->d_counters.p, 8, cudaMemcpyDeviceToHost, c->stream));
  const int e = velo::launch_fit_tracks(P<uint8_t>(c->d_input), P<uint64_t>(c->d_ev_offset),
                                        P<uint32_t>(c->d_ev_valid), P<velo_track>(c->d_out_tracks),
                                        P<uint32_t>(c->d_out_counts), P<uint64_t>(c->d_out_first), c->n,
                                        P<velo_track_fit>(c->d_fits), c->stream);
  if (e != 0) return cuda_fail(c, (cudaError_t)e, "fit kernel launch");
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  if (total > capacity) {
    c->err = "fit buffer too small";
    return VELO_ERR_CAPACITY;
  }
  if (total)
    VELO_CUDA(c, cudaMemcpyAsync(fits_out, c->d_fits.p, sizeof(velo_track_fit) * total, cudaMemcpyDeviceToHost,
                                 c->stream));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  return VELO_OK;
}

velo_status velo_fetch_staged(velo_ctx* c, uint8_t* buf, uint64_t size) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || (!buf && size)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  if (size < c->input_bytes) {
    c->err = "buffer smaller than the staged events";
    return VELO_ERR_CAPACITY;
  }
  VELO_CUDA(c, cudaSetDevice(c->device));
  if (c->input_bytes)
    VELO_CUDA(c, cudaMemcpyAsync(buf, c->d_input.p, c->input_bytes, cudaMemcpyDeviceToHost, c->stream));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  return VELO_OK;
}

velo_status velo_set_mlp(velo_ctx* c, const float* weights, float keep_threshold, float window_margin,
                         float min_keep_rate, uint32_t max_event_hits) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || !weights) return VELO_ERR_INVALID_ARGUMENT;
  VELO_CUDA(c, cudaSetDevice(c->device));
  velo_status st = ensure(c, c->d_mlp, sizeof(float) * VELO_MLP_PARAMS, "mlp");
  if (st != VELO_OK) return st;
  VELO_CUDA(c, cudaMemcpyAsync(c->d_mlp.p, weights, sizeof(float) * VELO_MLP_PARAMS, cudaMemcpyHostToDevice,
                               c->stream));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  c->keep_threshold = keep_threshold;
  c->window_margin = window_margin;
  c->min_keep_rate = min_keep_rate;
  c->learned_max_hits = max_event_hits;
  c->h_mlp.assign(weights, weights + VELO_MLP_PARAMS);
  c->mlp_version++;
  c->mlp_set = true;
  return VELO_OK;
}

velo_status velo_dump_doublets(velo_ctx* c, const velo_options* opts, uint32_t keep_one_in, float* features_out,
                               uint32_t* ids_out, uint64_t capacity, uint64_t* count_out) {
  if (c && streaming_refused(c)) return VELO_ERR_INVALID_ARGUMENT;
  if (!c || (capacity && (!features_out || !ids_out))) return VELO_ERR_INVALID_ARGUMENT;
  if (!c->staged) return VELO_ERR_NOT_STAGED;
  velo_options o;
  if (opts) o = *opts; else velo_default_options(&o);
  o.learned = 0;   // the training data comes from the plain method
  VELO_CUDA(c, cudaSetDevice(c->device));
  velo_status st;
  if ((st = ensure(c, c->d_dump_features, sizeof(float) * VELO_MLP_INPUTS * (capacity ? capacity : 1),
                   "dump features")) != VELO_OK)
    return st;
  if ((st = ensure(c, c->d_dump_ids, sizeof(uint32_t) * 3 * (capacity ? capacity : 1), "dump ids")) != VELO_OK)
    return st;
  c->dump_capacity = capacity;
  c->dump_keep = keep_one_in ? keep_one_in : 1u;
  c->dump_armed = true;
  c->generation++;
  st = velo_run(c, &o);
  c->dump_armed = false;
  c->generation++;
  if (st != VELO_OK) return st;
  uint64_t count = 0;
  VELO_CUDA(c, cudaMemcpyAsync(&count, P<uint8_t>(c->d_counters) + 40, 8, cudaMemcpyDeviceToHost, c->stream));
  VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  const uint64_t k = count < capacity ? count : capacity;
  if (k) {
    VELO_CUDA(c, cudaMemcpyAsync(features_out, c->d_dump_features.p, sizeof(float) * VELO_MLP_INPUTS * k,
                                 cudaMemcpyDeviceToHost, c->stream));
    VELO_CUDA(c, cudaMemcpyAsync(ids_out, c->d_dump_ids.p, sizeof(uint32_t) * 3 * k, cudaMemcpyDeviceToHost,
                                 c->stream));
    VELO_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (count_out) *count_out = count;
  return VELO_OK;
}

velo_status velo_host_alloc(velo_ctx* c, uint64_t bytes, void** ptr) {
  if (!c || !ptr) return VELO_ERR_INVALID_ARGUMENT;
  VELO_CUDA(c, cudaSetDevice(c->device));
  VELO_CUDA(c, cudaHostAlloc(ptr, bytes ? bytes : 16, cudaHostAllocDefault));
  return VELO_OK;
}

velo_status velo_host_free(velo_ctx* c, void* ptr) {
  if (!c) return VELO_ERR_INVALID_ARGUMENT;
  if (ptr) VELO_CUDA(c, cudaFreeHost(ptr));
  return VELO_OK;
}

}  // extern "C"
