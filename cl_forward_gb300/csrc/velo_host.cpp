// velo_host.cpp -- the reference's C++ host entry points
// (GpuPixelSearchByTriplet.cpp:4-65, KernelInvoker.cpp:14-275,
// Tools.cpp:46-66) on top of the C ABI.  On a GPU with coherent access to
// host memory (GB300 with Grace) the searches stream their results
// (velo_search_begin): the host's cores fill the per-event output vectors
// while the device is still searching.
//
// One process-wide context on device 0 (or $VELO_DEVICE) serves these calls,
// created on first use; like the reference (host globals h_*, Tools.cpp:5-13)
// they are not re-entrant.  The reference's timing sweep over local sizes
// (KernelInvoker.cpp:138-193: four Y values, four launches each, output kept
// from Y = 4) is not repeated: one launch with Y = 4 produces that output.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/GpuPixelSearchByTriplet.h"
#include "../../include/velo_search.h"

namespace {

int g_verbosity = 0;   // 3 in standalone mode, 0 in framework mode (GpuPixelSearchByTriplet.cpp:16,35)
velo_ctx* g_ctx = nullptr;
std::mutex g_mutex;
std::mutex g_call_mutex;   // one search at a time on the shared context (the reference is not re-entrant)
// pinned track buffer the kernel writes in place, kept between calls
velo_track* g_tracks = nullptr;
uint64_t g_tracks_cap = 0;

// Runs f(a, b) over [0, n) on the host's cores when n is large.
template <class F>
void parallel_for(size_t n, size_t grain, F f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t workers = std::min<size_t>(hw, (n + grain - 1) / grain);
  if (workers <= 1) {
    f((size_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  const size_t chunk = (n + workers - 1) / workers;
  for (size_t t = 0; t < workers; ++t) {
    const size_t a = t * chunk, b = std::min(n, a + chunk);
    if (a < b) pool.emplace_back(f, a, b);
  }
  for (std::thread& t : pool) t.join();
}

[[noreturn]] void fail(const char* where, velo_status st, const char* detail) {
  std::cerr << "Error in function " << where << std::endl
            << "Error string: " << velo_status_string(st) << (detail && *detail ? ": " : "")
            << (detail ? detail : "") << std::endl;
  std::exit(-1);   // Tools.h:27-34
}

velo_ctx* context() {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_ctx) {
    int dev = 0;
    if (const char* d = std::getenv("VELO_DEVICE")) dev = std::atoi(d);
    velo_status st = velo_create(&g_ctx, dev);
    if (st != VELO_OK) fail("velo_create", st, nullptr);
  }
  return g_ctx;
}

// Grow-only pinned buffer of at least `bytes` (not zero-filled).
template <typename T>
T* pinned(velo_ctx* c, T*& buf, uint64_t& cap, uint64_t count, const char* where) {
  if (count > cap) {
    if (buf) velo_host_free(c, buf);
    buf = nullptr;
    cap = 0;
    void* p = nullptr;
    const uint64_t want = count + count / 4;
    velo_status st = velo_host_alloc(c, want * sizeof(T), &p);
    if (st != VELO_OK) fail(where, st, velo_last_error(c));
    buf = static_cast<T*>(p);
    cap = want;
  }
  return buf;
}

// Searches (with `sort`, first x-sorts in place) input[a, a + n) with results
// streamed to the host (velo_search_begin): the host's cores fill each
// event's output vector as soon as the device has published it, while the
// search goes on.  Returns false, having started nothing, where the device
// cannot stream (no coherent access to host memory) or the call was refused;
// the caller then takes the synchronous path, which reports any error.
bool streamed_search(velo_ctx* c, std::vector<uint8_t*>& ptrs, std::vector<uint64_t>& sizes, int a, int n,
                     bool sort, std::vector<std::vector<uint8_t> >& output, const char* where) {
  const uint64_t cap = velo_track_capacity(ptrs.data(), sizes.data(), n);
  velo_track* tracks = pinned(c, g_tracks, g_tracks_cap, cap, where);
  std::vector<velo_event_result> results(n);   // written by the device in place
  velo_options opts;
  velo_default_options(&opts);   // Y = 4, the reference's output configuration
  opts.host_direct = 1;
  if (velo_search_begin(c, ptrs.data(), sizes.data(), n, &opts, sort ? 1 : 0, tracks, g_tracks_cap,
                        results.data()) != VELO_OK)
    return false;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::seconds(600);
  std::vector<uint8_t> filled(n, 0);
  parallel_for((size_t)n, 256, [&](size_t lo, size_t hi) {
    std::vector<uint32_t> pending;
    for (size_t i = lo; i < hi; ++i) pending.push_back((uint32_t)i);
    size_t polls = 0;
    while (!pending.empty()) {
      size_t keep = 0;
      for (uint32_t i : pending) {
        velo_event_result& r = results[i];
        if (__atomic_load_n(&r.ready, __ATOMIC_ACQUIRE)) {
          const uint8_t* src = reinterpret_cast<const uint8_t*>(tracks + (r.count ? r.first : 0));
          output[a + i].assign(src, src + (size_t)r.count * sizeof(velo_track));
          filled[i] = 1;
        } else {
          pending[keep++] = i;
        }
      }
      if (keep == pending.size()) {
        std::this_thread::yield();
        if ((++polls & 1023u) == 0 && std::chrono::steady_clock::now() > deadline) break;
      }
      pending.resize(keep);
    }
  });
  std::vector<uint32_t> counts(n), status(n);
  std::vector<uint64_t> first(n);
  const velo_status st = velo_search_end(c, counts.data(), first.data(), status.data());
  if (st == VELO_ERR_INVALID_EVENT)
    for (int i = 0; i < n; ++i)
      if (status[i] & VELO_EVENT_INVALID) {
        const std::string what = "event " + std::to_string(a + i) + " failed validation";
        fail(where, VELO_ERR_INVALID_EVENT, what.c_str());
      }
  if (st != VELO_OK) fail(where, st, velo_last_error(c));
  for (int i = 0; i < n; ++i)   // events the host stopped waiting for (none, unless the deadline passed)
    if (!filled[i]) {
      const uint8_t* src = reinterpret_cast<const uint8_t*>(tracks + (counts[i] ? first[i] : 0));
      output[a + i].assign(src, src + (size_t)counts[i] * sizeof(velo_track));
    }
  return true;
}

// independent_execute's sort and search of input[a, a + n) on the GPU
// (velo_sort_search): each module's hits are x-sorted in the caller's
// buffers with the reference's permutation (velo_sort_staged, byte for byte
// the result of preorder_by_x, which sorts them in place through const
// pointers, Tools.cpp:51-63), then searched.  On a GPU with coherent access
// to pageable host memory (Grace over NVLink-C2C) the device sorts and reads
// the events where they lie; otherwise they go through pinned memory and the
// sorted bytes are copied back.  The tracks land in the pinned track buffer.
void sort_and_search(const std::vector<const std::vector<uint8_t>*>& input, int a, int n,
                     std::vector<std::vector<uint8_t> >& output) {
  if (n <= 0) return;
  velo_ctx* c = context();
  std::lock_guard<std::mutex> call_lock(g_call_mutex);
  std::vector<uint8_t*> ptrs(n);
  std::vector<uint64_t> sizes(n);
  for (int i = 0; i < n; ++i) {
    const std::vector<uint8_t>* v = input[a + i];
    ptrs[i] = v->empty() ? nullptr : const_cast<uint8_t*>(v->data());
    sizes[i] = v->size();
  }
  if (streamed_search(c, ptrs, sizes, a, n, true, output, "independent_execute")) return;
  const uint64_t cap = velo_track_capacity(ptrs.data(), sizes.data(), n);
  velo_track* tracks = pinned(c, g_tracks, g_tracks_cap, cap, "independent_execute");
  std::vector<uint32_t> counts(n), status(n);
  std::vector<uint64_t> first(n);
  velo_options opts;
  velo_default_options(&opts);   // Y = 4, the reference's output configuration
  opts.host_direct = 1;
  velo_status st = velo_sort_search(c, ptrs.data(), sizes.data(), n, &opts, tracks, g_tracks_cap, counts.data(),
                                    first.data(), status.data());
  if (st == VELO_ERR_INVALID_EVENT) {
    for (int i = 0; i < n; ++i)
      if (status[i] & VELO_EVENT_INVALID) {
        const std::string what = "event " + std::to_string(a + i) + " failed validation";
        fail("invokeParallelSearch", VELO_ERR_INVALID_EVENT, what.c_str());
      }
  }
  if (st != VELO_OK) fail("invokeParallelSearch", st, velo_last_error(c));
  parallel_for((size_t)n, 256, [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; ++i) {
      // assign copies the tracks straight in (resize would zero-fill first)
      const uint8_t* src = reinterpret_cast<const uint8_t*>(tracks + (counts[i] ? first[i] : 0));
      output[a + i].assign(src, src + (size_t)counts[i] * sizeof(velo_track));
    }
  });
}

}  // namespace

int invokeParallelSearch(const int startingEvent, const int eventsToProcess,
                         const std::vector<const std::vector<uint8_t>*>& input,
                         std::vector<std::vector<uint8_t> >& output) {
  if (eventsToProcess <= 0) return 0;
  velo_ctx* c = context();
  std::lock_guard<std::mutex> call_lock(g_call_mutex);
  std::vector<const uint8_t*> ptrs(eventsToProcess);
  std::vector<uint64_t> sizes(eventsToProcess);
  for (int i = 0; i < eventsToProcess; ++i) {
    const std::vector<uint8_t>* v = input[startingEvent + i];
    ptrs[i] = v->empty() ? nullptr : v->data();
    sizes[i] = v->size();
  }
  {   // the events are only read (no sort)
    std::vector<uint8_t*> wptrs(eventsToProcess);
    for (int i = 0; i < eventsToProcess; ++i) wptrs[i] = const_cast<uint8_t*>(ptrs[i]);
    if (streamed_search(c, wptrs, sizes, startingEvent, eventsToProcess, false, output, "invokeParallelSearch"))
      return 0;
  }
  // grow-only, not zero-filled: only [first, first + count) is read
  const uint64_t cap = velo_track_capacity(ptrs.data(), sizes.data(), eventsToProcess);
  velo_track* tracks = pinned(c, g_tracks, g_tracks_cap, cap, "invokeParallelSearch");
  std::vector<uint32_t> counts(eventsToProcess), status(eventsToProcess);
  std::vector<uint64_t> first(eventsToProcess);
  velo_options opts;
  // Y = 4 (the reference's output configuration), persistent 64-thread CTAs;
  // the events are gathered into the context's pinned buffer and the tracks
  // land in the pinned track buffer, both accessed by the kernel in place
  velo_default_options(&opts);
  opts.host_direct = 1;
  velo_status st = velo_search(c, ptrs.data(), sizes.data(), eventsToProcess, &opts, tracks, g_tracks_cap,
                               counts.data(), first.data(), status.data());
  if (st != VELO_OK) fail("invokeParallelSearch", st, velo_last_error(c));
  parallel_for((size_t)eventsToProcess, 512, [&](size_t a, size_t b) {
    for (size_t i = a; i < b; ++i) {
      const uint8_t* src = reinterpret_cast<const uint8_t*>(tracks + (counts[i] ? first[i] : 0));
      output[startingEvent + i].assign(src, src + (size_t)counts[i] * sizeof(velo_track));
    }
  });
  if (g_verbosity >= 3) {
    velo_stats s;
    velo_get_stats(c, &s);
    std::cout << "Searched " << eventsToProcess << " events on the GPU: " << s.total_tracks << " tracks, "
              << s.kernel_ms << " ms" << std::endl;
  }
  return 0;
}

int gpuPixelSearchByTripletInvocation(const std::vector<const std::vector<uint8_t>*>& input,
                                      std::vector<std::vector<uint8_t> >& output) {
  if (g_verbosity >= 3)
    std::cout << "Invoking gpuPixelSearchByTriplet with " << input.size() << " events" << std::endl;
  output.resize(input.size());
  const int max_events_to_process_per_kernel = 16000;   // GpuPixelSearchByTriplet.cpp:53
  for (size_t i = 0; i < input.size(); i += max_events_to_process_per_kernel) {
    int n = (int)(input.size() - i);
    if (n > max_events_to_process_per_kernel) n = max_events_to_process_per_kernel;
    invokeParallelSearch((int)i, n, input, output);
  }
  return 0;
}

void preorder_by_x(std::vector<const std::vector<uint8_t>*>& input) {
  // The reference sorts the caller's buffers in place through const
  // pointers (Tools.cpp:51-63), one event after another; so does this, with
  // the events spread over the host's cores (each event is independent, and
  // each event's permutation is the reference's).
  const size_t n = input.size();
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t workers = std::min<size_t>(hw, (n + 63) / 64);
  std::atomic<size_t> next{0};
  std::atomic<int> bad{0};
  auto work = [&]() {
    for (size_t i; (i = next.fetch_add(1)) < n;) {
      const std::vector<uint8_t>* ev = input[i];
      if (!ev || ev->empty()) continue;
      uint8_t* blob = const_cast<uint8_t*>(ev->data());
      const velo_status st = velo_sort_by_x(blob, ev->size());
      if (st != VELO_OK) bad.store((int)st);
    }
  };
  if (workers <= 1) {
    work();
  } else {
    std::vector<std::thread> pool;
    for (size_t t = 0; t < workers; ++t) pool.emplace_back(work);
    for (std::thread& t : pool) t.join();
  }
  if (bad.load() != 0) fail("preorder_by_x", (velo_status)bad.load(), nullptr);
}

// The reference sorts on the host (preorder_by_x), then searches in chunks of
// 16000 events (GpuPixelSearchByTriplet.cpp:4-22,44-65); here each chunk is
// sorted on the GPU as part of its search, with the same bytes left in the
// caller's buffers and the same tracks.
int independent_execute(const std::vector<std::vector<uint8_t> >& input,
                        std::vector<std::vector<uint8_t> >& output) {
  std::vector<const std::vector<uint8_t>*> converted(input.size());
  for (size_t i = 0; i < input.size(); ++i) converted[i] = &input[i];
  g_verbosity = 3;
  const auto t0 = std::chrono::steady_clock::now();
  output.resize(input.size());
  const int max_events_to_process_per_kernel = 16000;   // GpuPixelSearchByTriplet.cpp:53
  for (size_t i = 0; i < input.size(); i += max_events_to_process_per_kernel) {
    int n = (int)(input.size() - i);
    if (n > max_events_to_process_per_kernel) n = max_events_to_process_per_kernel;
    sort_and_search(converted, (int)i, n, output);
  }
  const auto t1 = std::chrono::steady_clock::now();
  const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  std::cout << "Sorted and searched " << input.size() << " events on the GPU in " << ms << " ms ("
            << (double)input.size() / (ms / 1e3) << " events/s end to end)" << std::endl;
  return 0;
}

void independent_post_execute(const std::vector<std::vector<uint8_t> >& output) {
  if (g_verbosity >= 3) std::cout << std::endl << "Size of output: " << output.size() << " entries" << std::endl;
}

int gpuPixelSearchByTriplet(const std::vector<const std::vector<uint8_t>*>& input,
                            std::vector<std::vector<uint8_t> >& output) {
  g_verbosity = 0;
  return gpuPixelSearchByTripletInvocation(input, output);
}
