// velo_api_bench.cpp -- timing harness of the reference-signature entry
// points (libvelo_api_bench.so, loaded by bench.py through ctypes).
//
// It times what a cl_forward caller runs: independent_execute (the
// standalone path: unsorted events, per-module x-sort, search;
// GpuPixelSearchByTriplet.cpp:4-22) and gpuPixelSearchByTriplet (the
// framework path: x-sorted events, no sort; GpuPixelSearchByTriplet.cpp:
// 29-37), both on std::vector<std::vector<uint8_t> > input and output, with
// everything those calls do (host checks, copies, the sort, the search, the
// per-event output vectors) inside the timed region.  Not part of the
// library: a measurement tool beside it.
#include <stdint.h>

#include <chrono>
#include <cstring>
#include <vector>

#include "../../include/GpuPixelSearchByTriplet.h"

namespace {

// Order-independent digest of one event's output (the GPU emits an event's
// tracks in no fixed order): the sum, modulo 2^64, over its 100-byte Track
// records of a 64-bit hash of the record's 25 words; the same function as
// cl_forward_gb300.validation.event_hashes.
uint64_t event_digest(const std::vector<uint8_t>& v) {
  uint64_t sum = 0;
  for (size_t t = 0; t + 100 <= v.size(); t += 100) {
    uint64_t h = 0;
    for (int k = 0; k < 25; ++k) {
      uint32_t w;
      std::memcpy(&w, v.data() + t + 4 * k, 4);
      uint64_t x = ((uint64_t)w + (uint64_t)(k + 1)) * (0x9E3779B97F4A7C15ull * (uint64_t)(2 * k + 1));
      x ^= x >> 29;
      h = (h ^ x) * 0xBF58476D1CE4E5B9ull;
      h ^= h >> 31;
    }
    sum += h;
  }
  return sum;
}

}  // namespace

extern "C" {

// Times `steps` calls (after `warmup` untimed ones) of one entry point on the
// n events of buf (event e at buf + offsets[e], sizes[e] bytes).
//   entry 0: independent_execute on the events as given (unsorted); each
//            call gets a fresh copy of them, made outside the timed region,
//            because the call sorts its input in place;
//   entry 1: gpuPixelSearchByTriplet on the events as given (x-sorted).
// ms_out[i] receives call i's host wall-clock milliseconds; tracks_out the
// track count of the last call; digests_out (optional, n entries) each
// event's output digest; sorted_out (optional, sum of sizes bytes, events
// packed back to back) the input bytes after the last call.  Returns 0, or
// -1 on bad arguments.
int velo_bench_reference_api(const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes, int32_t n,
                             int32_t entry, int32_t warmup, int32_t steps, double* ms_out, uint64_t* tracks_out,
                             uint64_t* digests_out, uint8_t* sorted_out) {
  if (n < 0 || steps < 0 || warmup < 0 || (entry != 0 && entry != 1) || (n > 0 && (!buf || !offsets || !sizes)))
    return -1;
  std::vector<std::vector<uint8_t> > pristine((size_t)n);
  for (int32_t e = 0; e < n; ++e) pristine[e].assign(buf + offsets[e], buf + offsets[e] + sizes[e]);
  std::vector<std::vector<uint8_t> > work = pristine;
  std::vector<std::vector<uint8_t> > output;
  std::vector<const std::vector<uint8_t>*> ptrs((size_t)n);
  for (int32_t i = 0; i < warmup + steps; ++i) {
    if (entry == 0)
      for (int32_t e = 0; e < n; ++e) std::memcpy(work[e].data(), pristine[e].data(), sizes[e]);
    for (int32_t e = 0; e < n; ++e) ptrs[e] = &work[e];
    output.clear();
    output.shrink_to_fit();   // each call allocates its output vectors, as a new caller's would
    const auto t0 = std::chrono::steady_clock::now();
    if (entry == 0)
      independent_execute(work, output);
    else
      gpuPixelSearchByTriplet(ptrs, output);
    const auto t1 = std::chrono::steady_clock::now();
    if (i >= warmup && ms_out) ms_out[i - warmup] = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  uint64_t tracks = 0;
  for (const std::vector<uint8_t>& v : output) tracks += v.size() / 100;
  if (tracks_out) *tracks_out = tracks;
  if (digests_out)
    for (int32_t e = 0; e < n; ++e) digests_out[e] = event_digest(output[e]);
  if (sorted_out) {
    uint64_t o = 0;
    for (int32_t e = 0; e < n; ++e) {
      std::memcpy(sorted_out + o, work[e].data(), sizes[e]);
      o += sizes[e];
    }
  }
  return 0;
}

}  // extern "C"
