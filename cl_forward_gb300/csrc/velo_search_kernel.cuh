// velo_search_kernel.cuh -- sm_103a search-by-triplet kernel (device code).
//
// Included by one translation unit per seeding width (velo_kernels_g8.cu,
// _g16.cu, _g32.cu), each of which instantiates the kernel builds for its
// width; velo_kernels.cu picks the kernel of a launch.
//
// One CTA reconstructs one event (the reference's one work-group per event,
// Kernel.cl:607, KernelInvoker.cpp:26-27), either one CTA per event or
// persistent CTAs pulling events, largest first, from a work queue.  The
// event's hits and its per-hit working state (the "arena": x, y, z,
// candidate windows, used flags) live in dynamic shared memory when the event
// fits the launch's tile, else in global scratch with the same layout, which
// L1 caches.  On GB300 the fastest launch keeps the tile tiny: shared memory
// and L1 share each SM's storage, and resident CTAs are register-bound, so L1
// serves the arenas better than staging does.  The tracks-to-follow rings,
// tracklets and working tracks are per-hit-row global scratch.
//
// Decisions are the reference's, bit for bit:
//  * every FP32 expression is written with round-to-nearest intrinsics
//    (__fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn), term by term as in
//    Kernel.cl, so no contraction into FMA can change a cut;
//  * ties resolve as in the reference: forwarding keeps the first minimum in
//    h2 order (Kernel.cl:302-305); seeding keeps the minimum of the packed
//    key (fit, Y-lane, h1 element, h2), which is the reference's per-lane
//    first minimum followed by its lowest-lane reduction (Kernel.cl:517-545);
//  * a Y-lane stops at its first h1 without an h2 window (the cumulative
//    `inside_bounds` of Kernel.cl:437,457).
// Narrowing: on a module whose hits are x-sorted, x-window searches use
// binary search and skip only hits that provably fail the reference's own
// float predicate (the predicted x is monotone in hit z, so the module's z
// range bounds it; a 0.01 mm guard covers the rounding of the bound).  On an
// unsorted module the full sequential scan runs.  Narrowing changes work, not
// results.
//
// Per module iteration the CTA meets at two barriers: after forwarding (its
// used-hit marks feed seeding) and after seeding (its tracklets feed the next
// forwarding).  Seeding gives each h0 to a group of G lanes of a warp (G =
// 8, 16 or 32, the kernel build's seeding width), whose lanes take the h0's
// h1 candidates; lane cut-offs come from a ballot and the winner from a
// group min-reduction, so seeding itself needs no block barrier.  Each
// tracks-to-follow buffer is filled from both ends (forwarding from the
// front, seeding from the back), which keeps the two counts separate without
// another barrier.
//
// Optional per launch: the x-sort of each event while it is staged, with the
// sorted hit arrays written back into the input (sort_events), and a
// per-event record published in host memory when the event is done
// (results, for a host that consumes events while the search runs).
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "velo_internal.h"
#include "velo_mlp_warp.cuh"
#include "velo_partition.cuh"

namespace velo {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kNone16 = 0xffffu;

// Per-CTA shared state for events of up to kMods modules.  Launches whose
// events all have at most kCompactModules - 1 modules (every VELO geometry)
// use the compact form: 4 KB less static shared memory per CTA, which goes
// to L1 and to more resident CTAs.
template <int kMods>
struct SharedT {
  int32_t start[kMods];
  int32_t num[kMods];
  int32_t sz[kMods];
  float zmin[kMods];
  float zmax[kMods];
  uint8_t sorted[kMods];
  uint32_t ring_lo[2];   // forwarding entries, from the front of ring[i]
  uint32_t ring_hi[2];   // seeding entries, from the back of ring[i]
  uint32_t ntracks, ntracklets, nweak, status;
  uint32_t considered, kept;   // learned seeding: doublets scored / kept
  unsigned long long out_first;
  int32_t next_event;
  int32_t seed_next[2];  // G < 32: next unclaimed h0 of the module being seeded, by ring parity
};

struct EventView {
  int S, H, Y;
  uint32_t cap;             // tracklet / track / weak rows (max(H, 1))
  uint32_t ring_cap;        // entries of each tracks-to-follow buffer (max(H, 1): one per seeded h0 at most)
  // the arena: x, y, z, windows (per hit {h1 first | h1 last << 16, h2 first
  // | h2 last << 16}) and used flags at multiples of one stride P
  uint8_t* arena;
  uint32_t P;
  __device__ __forceinline__ float* xs() const { return reinterpret_cast<float*>(arena); }
  __device__ __forceinline__ float* ys() const { return reinterpret_cast<float*>(arena + P); }
  __device__ __forceinline__ float* zs() const { return reinterpret_cast<float*>(arena + 2u * P); }
  __device__ __forceinline__ uint2* wins() const { return reinterpret_cast<uint2*>(arena + 3u * P); }
  __device__ __forceinline__ uint8_t* useds() const { return arena + 5u * P; }
  uint4* ring0;             // tracks-to-follow buffers, selected by parity:
  uint4* ring1;             //   {entry word, first hit, previous hit, last hit}
  uint4* tracklets;         // {h0, h1, h2, 0} per tracklet
  uint32_t* weak;
  velo_track* tracks;
  bool narrow;
  int event;
  const MlpFrag* mlp;       // learned seeding: weights in shared memory
  float keep_threshold, window_margin;
  int learned_min_window;   // doublets with narrower h2 windows are searched exactly, unscored
  float* dump_features;     // training-data dump
  uint32_t* dump_ids;
  unsigned long long* dump_count;
  uint64_t dump_capacity;
  uint32_t dump_keep;
};

// First index i in [lo, hi) with x[i] > c, for non-decreasing x.
__device__ __forceinline__ int first_gt(const float* x, int lo, int hi, float c) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] > c) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Sub-range [lo, hi) of [lo0, hi0) on a sorted module outside which no hit
// can satisfy |fl(xp - x)| < tol for any predicted xp in [xl, xh].  The upper
// end is usually a few hits past the lower one: walk, then bisect.
// x_first = x[lo0] and x_last = x[hi0 - 1] are passed in (any value when
// lo0 == hi0), so that a caller can load them early.
__device__ __forceinline__ void narrow_range_ends(const float* x, int lo0, int hi0, float x_first, float x_last,
                                                  float xl, float xh, float tol, int* lo, int* hi) {
  const float margin = fadd(0.01f, fmul(1e-5f, fadd(fabsf(xl), fabsf(xh))));
  const float lt = fsub(fsub(xl, tol), margin);
  const float ht = fadd(fadd(xh, tol), margin);
  if (isfinite(lt) && isfinite(ht)) {
    // both ends first: a prediction beyond either end of the module (a track
    // tried on the other detector half) is settled without the bisection,
    // with the bisection's own result
    if (lo0 < hi0 && (x_last <= lt || x_first > ht)) {
      *lo = *hi = x_first > ht ? lo0 : hi0;
      return;
    }
    const int l = first_gt(x, lo0, hi0, lt);
    int h = l;
    const int walk_end = min(hi0, l + 8);
    while (h < walk_end && !(x[h] > ht)) ++h;
    if (h == walk_end && h < hi0) h = first_gt(x, h, hi0, ht);
    *lo = l;
    *hi = h;
  } else {
    *lo = lo0;
    *hi = hi0;
  }
}

__device__ __forceinline__ void narrow_range(const float* x, int lo0, int hi0, float xl, float xh, float tol,
                                             int* lo, int* hi) {
  float x_first = 0.f, x_last = 0.f;
  if (lo0 < hi0) {   // two independent loads
    x_first = x[lo0];
    x_last = x[hi0 - 1];
  }
  narrow_range_ends(x, lo0, hi0, x_first, x_last, xl, xh, tol, lo, hi);
}

// ---------------------------------------------------------------------------
// Candidate windows of hit h on module f (Kernel.cl:50-178), stored relative
// to the start of module f-2 (0xffff = none).
template <class Shared>
__device__ void compute_windows(const EventView& ev, const Shared& s, int h, int f) {
  const int s2 = f - 2;
  const bool proc_h2 = f <= ev.S - 3;
  const int st2 = s.start[s2], n2 = s.num[s2];
  const float x0 = ev.xs()[h], z0 = ev.zs()[h];
  const float* x2 = ev.xs() + st2;
  const float* z2 = ev.zs() + st2;
  const bool sorted = ev.narrow && s.sorted[s2];
  uint32_t r1f = kNone16, r1l = kNone16, r2f = kNone16, r2l = kNone16;

  // h1 window: first hit with |x1-x0| < 0.7|z1-z0|, then the first later hit
  // that fails it (Kernel.cl:115-135,161-165).
  {
    int lo = 0, hi = n2;
    if (sorted && n2 > 0) {
      const float da = fabsf(fsub(s.zmin[s2], z0));
      const float db = fabsf(fsub(s.zmax[s2], z0));
      const float D = fmul(kMaxXSlopeCandidates, fmaxf(da, db));   // >= every hit's dxmax
      narrow_range(x2, 0, n2, x0, x0, D, &lo, &hi);
    }
    if (sorted && n2 > 0 && s.zmin[s2] == s.zmax[s2]) {
      // one z on the module: dxmax is the same for every hit, and
      // d = fl(x2 - x0) is non-decreasing in x2, so the hits passing
      // |d| < dxmax are exactly [A, B): A = first with d > -dxmax, B = first
      // with d >= dxmax -- the scan's first pass and first later failure
      const float dxmax = fmul(kMaxXSlopeCandidates, fabsf(fsub(z2[0], z0)));
      int a = lo, b = hi;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (fsub(x2[mid], x0) > -dxmax) b = mid; else a = mid + 1;
      }
      const int A = a;
      b = hi;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (!(fsub(x2[mid], x0) < dxmax)) b = mid; else a = mid + 1;
      }
      if (A < a) {
        r1f = (uint32_t)A;
        r1l = (uint32_t)a;   // a == hi: hit `hi` provably fails, or hi is the end
      }
    } else {
      bool found = false;
      for (int e = lo; e < hi; ++e) {
        const float h_dist = fabsf(fsub(z2[e], z0));
        const float dxmax = fmul(kMaxXSlopeCandidates, h_dist);
        const bool tol = fabsf(fsub(x2[e], x0)) < dxmax;
        if (!found) {
          if (tol) { found = true; r1f = (uint32_t)e; }
        } else if (!tol) {
          r1l = (uint32_t)e;
          break;
        }
      }
      if (found && r1l == kNone16) r1l = (uint32_t)hi;   // hit `hi` provably fails, or hi is the end
    }
  }

  // h2 window for h taken as the h1 of a seed on f+2 (Kernel.cl:85-102,137-150).
  if (proc_h2) {
    const float fz0 = __int2float_rn(s.sz[f + 2]);
    const float fz2 = __int2float_rn(s.sz[s2]);
    const float h_dist = fabsf(fsub(z0, fz0));
    const float dxmax = fmul(kMaxXSlopeCandidates, h_dist);
    const float x0_min = fsub(x0, dxmax);
    const float x0_max = fadd(x0, dxmax);
    const float z2_tz = fdiv(fsub(fz2, fz0), fsub(z0, fz0));
    const float xmin_h2 = fsub(fadd(x0_max, fmul(fsub(x0, x0_max), z2_tz)), kToleranceCandidates);
    const float xmax_h2 = fadd(fadd(x0_min, fmul(fsub(x0, x0_min), z2_tz)), kToleranceCandidates);
    if (sorted) {   // `x > c` is monotone on a non-decreasing module: exact
      const int a = first_gt(x2, 0, n2, xmin_h2);
      if (a < n2) {
        r2f = (uint32_t)a;
        r2l = (uint32_t)first_gt(x2, a + 1, n2, xmax_h2);
      }
    } else {
      bool found = false;
      for (int e = 0; e < n2; ++e) {
        if (!found) {
          if (x2[e] > xmin_h2) { found = true; r2f = (uint32_t)e; }
        } else if (x2[e] > xmax_h2) {
          r2l = (uint32_t)e;
          break;
        }
      }
      if (found && r2l == kNone16) r2l = (uint32_t)n2;
    }
  }
  ev.wins()[h] = make_uint2(r1f | (r1l << 16), r2f | (r2l << 16));
}

// ---------------------------------------------------------------------------
// Tracks-to-follow entries.  Bit 31 marks a tracklet (3 hits, number = its
// row in the tracklet list) and bits 28-30 count skipped modules, as in the
// reference (Kernel.cl:222-225,351,566).  This kernel also keeps a track's
// hit count in bits 23-27 (the reference re-reads it from the track), so
// numbers use bits 0-22.
constexpr uint32_t kEntryNumber = 0x007FFFFFu;
constexpr uint32_t kEntryCountShift = 23;

__device__ __forceinline__ unsigned lanemask_lt() { return (1u << (threadIdx.x & 31)) - 1u; }

// One shared-memory atomic per warp: lanes with `take` get consecutive slots
// from *counter; returns this lane's slot.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counter, bool take) {
  const unsigned m = __ballot_sync(kFull, take);
  if (m == 0) return 0;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  return base + (uint32_t)__popc(m & lanemask_lt());
}

// (a select, not an indexed array, so the view stays in registers)
__device__ __forceinline__ uint4* ring_buf(const EventView& ev, int b) { return b ? ev.ring1 : ev.ring0; }

// A ring entry carries the track's last two hits (and a tracklet's first), so
// forwarding extrapolates without reading the track or tracklet row first.
template <class Shared>
__device__ __forceinline__ void push_back(Shared& s, const EventView& ev, int b, uint4 v) {
  const uint32_t i = atomicAdd(&s.ring_hi[b], 1u);
  if (i < ev.ring_cap) ring_buf(ev, b)[ev.ring_cap - 1u - i] = v;
}

// i-th entry of ring[b]: the front segment, then the back segment.
__device__ __forceinline__ uint4 ring_entry(const EventView& ev, int b, uint32_t lo, uint32_t i) {
  const uint4* r = ring_buf(ev, b);
  return i < lo ? r[i] : r[ev.ring_cap - 1u - (i - lo)];
}

// Track forwarding onto module m4 (Kernel.cl:210-367), one warp at a time:
// lane j forwards entry i0 + j of ring[b].  Track numbers, ring slots and
// weak slots are reserved with one atomic per warp; new entries go to the
// front of ring[nb].
template <class Shared>
__device__ void forward_warp(const EventView& ev, Shared& s, int b, uint32_t lo_n, uint32_t i0, uint32_t ncur,
                             int m4, int nb) {
  enum { kNone = 0, kPushTrack, kNewTrack, kPushSkip, kWeak };
  const uint32_t i = i0 + (threadIdx.x & 31);
  int action = kNone;
  uint32_t push_value = 0, trackno = 0, best_h2 = 0;
  uint4 en = make_uint4(0, 0, 0, 0);
  // the ends of module m4 for the narrowing, loaded alongside the entry
  // (same addresses in every lane)
  const int st4 = s.start[m4], n4 = s.num[m4];
  const float* x4 = ev.xs() + st4;
  float x4_first = 0.f, x4_last = 0.f;
  if (n4 > 0) {
    x4_first = x4[0];
    x4_last = x4[n4 - 1];
  }
  if (i < ncur) {
    en = ring_entry(ev, b, lo_n, i);
    const uint32_t full = en.x;
    const bool is_tracklet = (full & kTrackletFlag) != 0;
    const uint32_t skipped = (full & kSkipMask) >> 28;
    trackno = full & kEntryNumber;
    const uint32_t n = is_tracklet ? 3u : (full >> kEntryCountShift) & 31u;
    const uint32_t h0 = en.z, h1 = en.w;   // the last two hits
    const float h0x = ev.xs()[h0], h0y = ev.ys()[h0], h0z = ev.zs()[h0];
    const float h1x = ev.xs()[h1], h1y = ev.ys()[h1], h1z = ev.zs()[h1];
    const float td = fdiv(1.0f, fsub(h1z, h0z));
    const float tx = fmul(fsub(h1x, h0x), td);
    const float ty = fmul(fsub(h1y, h0y), td);

    const float* y4 = ev.ys() + st4;
    const float* z4 = ev.zs() + st4;
    int lo = 0, hi = n4;
    if (ev.narrow && s.sorted[m4] && n4 > 0) {
      const float xa = fadd(h0x, fmul(tx, fsub(s.zmin[m4], h0z)));
      const float xb = fadd(h0x, fmul(tx, fsub(s.zmax[m4], h0z)));
      if (isfinite(xa) && isfinite(xb))
        narrow_range_ends(x4, 0, n4, x4_first, x4_last, fminf(xa, xb), fmaxf(xa, xb), kTolerance, &lo, &hi);
    }
    // fitHitToTrack (Kernel.cl:15-35) over the candidates, first minimum wins.
    // The scatter's 1/(z2 - z1) depends only on z2 here: it is recomputed only
    // when z2's bit pattern changes (same operands, same rounded value).
    float best = FLT_MAX;
    int best_k = -1;
    bool degenerate = false;
    uint32_t zc = 0x7fc00001u;   // bit pattern of the z2 the cached factor belongs to (none yet)
    float den = 0.f;
    for (int k = lo; k < hi; ++k) {
      const float h2z = z4[k];
      if (__float_as_uint(h2z) != zc) {
        zc = __float_as_uint(h2z);
        den = fdiv(1.f, fsub(h2z, h1z));
      }
      const float dz = fsub(h2z, h0z);
      const float dx = fabsf(fsub(fadd(h0x, fmul(tx, dz)), x4[k]));
      const float dy = fabsf(fsub(fadd(h0y, fmul(ty, dz)), y4[k]));
      const float scatter = fmul(fmul(fadd(fmul(dx, dx), fmul(dy, dy)), den), den);
      if (dx < kTolerance && dy < kTolerance && scatter < kMaxScatter) {
        if (scatter < best) { best = scatter; best_k = k; }
      } else if (!isfinite(scatter)) {
        degenerate = true;   // the reference's `condition*scatter + !condition*MAX` is NaN here
      }
    }
    if (degenerate) atomicOr(&s.status, VELO_EVENT_DEGENERATE);

    if (best_k >= 0) {
      best_h2 = (uint32_t)(st4 + best_k);
      if (n >= VELO_MAX_TRACK_SIZE) {   // the reference writes past hits[24] here
        atomicOr(&s.status, VELO_EVENT_TRACK_OVERFLOW);
      } else {
        ev.useds()[best_h2] = 1;
        if (is_tracklet) {   // third -> fourth hit: a track is allocated below; hits 0-2 marked
          ev.useds()[en.y] = 1;
          ev.useds()[en.z] = 1;
          ev.useds()[en.w] = 1;
          action = kNewTrack;
        } else {
          velo_track& t = ev.tracks[trackno];
          t.hits[n] = best_h2;
          t.hitsNum = n + 1;
          action = kPushTrack;
          push_value = trackno | ((n + 1u) << kEntryCountShift);
        }
      }
    } else if (skipped <= kMaxSkippedModules) {
      action = kPushSkip;
      push_value = ((skipped + 1u) << 28) | (full & 0x8FFFFFFFu);
    } else if (is_tracklet) {
      action = kWeak;
    }
  }
  // new tracks (Kernel.cl:324-337)
  const uint32_t tn = warp_reserve(&s.ntracks, action == kNewTrack);
  if (action == kNewTrack) {
    if (tn < ev.cap) {
      uint32_t* w = reinterpret_cast<uint32_t*>(&ev.tracks[tn]);
      w[0] = 4; w[1] = en.y; w[2] = en.z; w[3] = en.w; w[4] = best_h2;
#pragma unroll
      for (int k = 5; k < 25; ++k) w[k] = 0;
      push_value = tn | (4u << kEntryCountShift);
    } else {
      action = kNone;
    }
  }
  // tracks to follow in the next iteration (Kernel.cl:344-355)
  const bool push = action == kPushTrack || action == kNewTrack || action == kPushSkip;
  const uint32_t slot = warp_reserve(&s.ring_lo[nb], push);
  if (push && slot < ev.ring_cap)   // a skip keeps the hits; a new hit shifts them
    ring_buf(ev, nb)[slot] = action == kPushSkip ? make_uint4(push_value, en.y, en.z, en.w)
                                                 : make_uint4(push_value, 0u, en.w, best_h2);
  // three-hit tracklets that ran out of skips (Kernel.cl:359-363)
  const uint32_t wi = warp_reserve(&s.nweak, action == kWeak);
  if (action == kWeak && wi < ev.cap) ev.weak[wi] = trackno;
}

// Features of an (h0, h1) doublet seen by the learned seeding (and recorded
// as training data): slopes, h0 radius and azimuth, module, predicted x / y
// at module f-4, z gap, h2 candidates in the exact window, and the y-slope
// cut margin.  Plain FP32; the features steer pruning, not the cuts.  The
// h0 terms (radius, azimuth, module, 1 / dymax) are computed once per h0 by
// h0_features; dz_inv is the seeding's own 1 / (z1 - z0).
struct H0Features {
  float r, phi, module, inv_dymax;
};

__device__ __forceinline__ H0Features h0_features(float h0x, float h0y, int module, int n_modules, float dymax) {
  H0Features g;
  g.r = sqrtf(h0x * h0x + h0y * h0y) * (1.f / 42.f);
  g.phi = atan2f(h0y, h0x) * 0.31830988f;
  g.module = (float)module / (float)n_modules;
  g.inv_dymax = 1.f / dymax;
  return g;
}

__device__ __forceinline__ void doublet_features(float* f, const H0Features& g, float h0x, float h0y, float h0z,
                                                 float h1x, float h1y, float h1z, float dz_inv, float zmid4,
                                                 int h2_window) {
  const float tx = (h1x - h0x) * dz_inv, ty = (h1y - h0y) * dz_inv;
  f[0] = 5.f * tx;
  f[1] = 5.f * ty;
  f[2] = g.r;
  f[3] = g.phi;
  f[4] = g.module;
  f[5] = (h0x + tx * (zmid4 - h0z)) * (1.f / 42.f);
  f[6] = (h0y + ty * (zmid4 - h0z)) * (1.f / 42.f);
  f[7] = (h1z - h0z) * 0.01f;
  f[8] = (float)h2_window * (1.f / 32.f);
  f[9] = fabsf(h1y - h0y) * g.inv_dymax;
}

constexpr int kPlain = 0;    // the reference's seeding
constexpr int kDump = 1;     // plain, recording sampled doublets as training data
constexpr int kLearned = 2;  // MLP-pruned seeding

// Lane constants of the seeding ballots, per event.  With G lanes per h0 (a
// group; G = 32: the whole warp), lane j of a group takes, in chunk c, h1
// element e = G c + j of its h0, which belongs to the reference's Y-lane
// e mod Y.
struct SeedLanes {
  uint32_t below;      // lanes of my group below me whose element shares my Y-lane in a chunk
  uint32_t same_all;   // G < 32 (Y divides G): every lane of my group that shares my Y-lane
  uint32_t lane_mod;   // (lane mod G) mod Y: my Y-lane in chunk 0
};

__device__ __forceinline__ SeedLanes seed_lanes_of(int G, uint32_t Y) {
  SeedLanes sl;
  const int lane = threadIdx.x & 31;
  const int jl = lane & (G - 1), gbase = lane - jl;
  sl.below = 0;
  for (int j = jl - (int)Y; j >= 0; j -= (int)Y) sl.below |= 1u << (gbase + j);
  sl.same_all = 0;
  for (int j = (int)((uint32_t)jl % Y); j < G; j += (int)Y) sl.same_all |= 1u << (gbase + j);
  sl.lane_mod = (uint32_t)jl % Y;
  return sl;
}

// Features and MLP of the learned seeding for the warp's doublets: lanes
// with score == false pass zeros and ignore the result.  All 32 lanes call it
// together.  Kept out of line, so that the seeding loop keeps the plain
// method's registers wherever nothing is scored.
static __device__ __noinline__ float2 score_doublets(const MlpFrag* mlp, bool score, float h0x, float h0y, float h0z,
                                              float h1x, float h1y, float h1z, float dz_inv, float zmid4,
                                              int h2_window, int f, int n_modules, float dymax) {
  float feat[kMlpIn];
  if (score) {
    const H0Features g0 = h0_features(h0x, h0y, f, n_modules, dymax);
    doublet_features(feat, g0, h0x, h0y, h0z, h1x, h1y, h1z, dz_inv, zmid4, h2_window);
  } else {
#pragma unroll
    for (int q = 0; q < kMlpIn; ++q) feat[q] = 0.f;
  }
  float logit, width;
  mlp_eval_warp(*mlp, feat, &logit, &width);
  return make_float2(logit, width);
}

// Seeding of module f: h0 on f, h1 on f-2, h2 on f-4 (Kernel.cl:392-568
// with the unused-h0 gather of :720-764), G lanes per h0 (SeedLanes).
// G = 32: one warp per unused h0.  G = 8 or 16: a warp seeds 32 / G h0s at
// once and walks the chunks of its groups' h1 windows together, so every
// ballot and the groups' minimum reductions run with all lanes present; the
// host allows G < 32 only where Y divides G, so that a lane's Y-lane is the
// same in every chunk.  New tracklets go to the back of ring[nb].
template <int kMode, int G, class Shared>
__device__ void seed_module(const EventView& ev, Shared& s, int f, int nb, const SeedLanes& sl) {
  constexpr int kShift = G == 8 ? 3 : G == 16 ? 4 : 5;
  constexpr int kGroups = 32 / G;
  static_assert(G == 8 || G == 16 || G == 32, "8, 16 or 32 lanes per h0");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int jl = lane & (G - 1);
  const int st0 = s.start[f], n0 = s.num[f];
  const int s1 = f - 2, m4 = f - 4;
  const int st1 = s.start[s1], st4 = s.start[m4], n4 = s.num[m4];
  const uint32_t Y = (uint32_t)ev.Y;
  const uint32_t chunk_step = G == 32 ? 32u % Y : 0u;   // how far the Y-lanes turn per chunk
  const float s1_z = s.num[s1] > 0 ? ev.zs()[st1] : 0.f;   // Kernel.cl:420
  const bool narrow4 = ev.narrow && s.sorted[m4] && n4 > 0;
  const float zmin4 = s.zmin[m4], zmax4 = s.zmax[m4];
  const float* x4 = ev.xs() + st4;
  const float* y4 = ev.ys() + st4;
  const float* z4 = ev.zs() + st4;
  bool degenerate = false;
  // 1 / (z1 - z0) by bit patterns of (z0, z1): hits of a module share few z
  // values, so the division is rarely redone (same operands, same result)
  uint32_t zk0 = 0x7fc00001u, zk1 = 0x7fc00001u;
  float dz_inv_cached = 0.f;

  // G = 32: h0s dealt to the warps in turn; G < 32: each warp claims its
  // next 32 / G h0s from a shared counter (one atomic per warp and claim),
  // which evens out the warps' work before the barrier that ends seeding
  int ib = G == 32 ? warp : 0;
  if constexpr (G < 32) {
    if (lane == 0) ib = atomicAdd(&s.seed_next[nb ^ 1], kGroups);   // seed_next[b] of the module loop
    ib = __shfl_sync(kFull, ib, 0);
  }
  for (; ib < n0;) {   // warp-uniform
    do {   // one claim of h0s; `break` moves on to the next claim
    int h0, n1, c_end;
    uint32_t f1;
    if constexpr (G == 32) {
      h0 = st0 + ib;
      if (ev.useds()[h0]) break;                        // warp-uniform
      const uint32_t w0 = ev.wins()[h0].x;
      f1 = w0 & 0xffffu;
      if (f1 == kNone16) break;
      n1 = (int)(w0 >> 16) - (int)f1;                   // > 0 when a first hit was found
      c_end = n1;
    } else {
      h0 = st0 + ib + (lane >> kShift);
      n1 = 0;
      f1 = 0;
      if (h0 < st0 + n0 && !ev.useds()[h0]) {
        const uint32_t w0 = ev.wins()[h0].x;
        f1 = w0 & 0xffffu;
        if (f1 != kNone16) n1 = (int)(w0 >> 16) - (int)f1;
      }
      const int chunks = (int)__reduce_max_sync(kFull, (uint32_t)((n1 + G - 1) >> kShift));
      if (chunks == 0) break;                           // warp-uniform
      c_end = chunks << kShift;
    }
    float h0x = 0.f, h0y = 0.f, h0z = 0.f;
    if (G == 32 || n1 > 0) {
      h0x = ev.xs()[h0];
      h0y = ev.ys()[h0];
      h0z = ev.zs()[h0];
    }
    const float dymax = fmul(kMaxYSlope, fabsf(fsub(s1_z, h0z)));
    H0Features g0{};
    if constexpr (kMode == kDump) g0 = h0_features(h0x, h0y, f, ev.S, dymax);
    unsigned long long best = ~0ull;
    uint32_t dead_lanes = 0;                         // G = 32: Y-lanes already stopped (bit per lane)
    bool lane_dead = false;                          // G < 32: my Y-lane has stopped
    uint32_t chunk_mod = 0;
    for (int c = 0; c < c_end; c += G) {
      const int e = c + jl;
      const bool in = e < n1;
      uint32_t ly = sl.lane_mod + chunk_mod;
      if (ly >= Y) ly -= Y;
      const int h1 = st1 + (int)f1 + e;
      // everything the cuts read about h1, loaded at once (one round trip)
      uint32_t w1 = 0;
      uint8_t u1 = 1;
      float h1x = 0.f, h1y = 0.f, h1z = 0.f;
      if (in) {
        w1 = ev.wins()[h1].y;
        u1 = ev.useds()[h1];
        h1x = ev.xs()[h1];
        h1y = ev.ys()[h1];
        h1z = ev.zs()[h1];
      }
      const bool dead = in && (w1 & 0xffffu) == kNone16;
      const unsigned dmask = __ballot_sync(kFull, dead);
      bool stopped;
      if constexpr (G == 32) {
        stopped = ((dmask & sl.below) != 0) || ((dead_lanes >> ly) & 1u);
        dead_lanes |= __reduce_or_sync(kFull, dead ? (1u << ly) : 0u);
        chunk_mod += chunk_step;
        if (chunk_mod >= Y) chunk_mod -= Y;
      } else {   // a lane's Y-lane is the same in every chunk
        stopped = (dmask & sl.below) != 0 || lane_dead;
        lane_dead = lane_dead || (dmask & sl.same_all) != 0;
      }
      bool cand = in && !dead && !stopped && !u1;
      if (cand) cand = fabsf(fsub(h1y, h0y)) < dymax;   // h2-independent term of Kernel.cl:509
      int a = (int)(w1 & 0xffffu), b = (int)(w1 >> 16);
      float tol = kTolerance;
      float dz_inverted = 0.f;
      if (cand) {
        if (__float_as_uint(h1z) != zk1 || __float_as_uint(h0z) != zk0) {
          zk0 = __float_as_uint(h0z);
          zk1 = __float_as_uint(h1z);
          dz_inv_cached = fdiv(1.f, fsub(h1z, h0z));
        }
        dz_inverted = dz_inv_cached;
      }
      if constexpr (kMode == kDump) {
        if (cand) {
          float feat[kMlpIn];
          doublet_features(feat, g0, h0x, h0y, h0z, h1x, h1y, h1z, dz_inverted, 0.5f * (zmin4 + zmax4), b - a);
          uint32_t hs = (uint32_t)ev.event * 0x9E3779B1u ^ (uint32_t)h0 * 0x85EBCA77u ^ (uint32_t)h1 * 0xC2B2AE3Du;
          hs ^= hs >> 15;
          hs *= 0x2C1B3C6Du;
          hs ^= hs >> 12;
          if (hs % ev.dump_keep == 0u) {
            const unsigned long long k = atomicAdd(ev.dump_count, 1ull);
            if (k < ev.dump_capacity) {
#pragma unroll
              for (int q = 0; q < kMlpIn; ++q) ev.dump_features[k * kMlpIn + q] = feat[q];
              ev.dump_ids[3 * k + 0] = (uint32_t)ev.event;
              ev.dump_ids[3 * k + 1] = (uint32_t)h0;
              ev.dump_ids[3 * k + 2] = (uint32_t)h1;
            }
          }
        }
      }
      if constexpr (kMode == kLearned) {
        // only doublets with a wide exact h2 window are worth scoring
        const bool score = cand && b - a >= ev.learned_min_window;
        bool keep = true;
        if (__any_sync(kFull, score)) {             // the warp scores its doublets together
          const float2 r = score_doublets(ev.mlp, score, h0x, h0y, h0z, h1x, h1y, h1z, dz_inverted,
                                          0.5f * (zmin4 + zmax4), b - a, f, ev.S, dymax);
          if (score) {
            keep = r.x >= ev.keep_threshold;
            tol = fminf(kTolerance, fmaxf(r.y, 0.f) + ev.window_margin);
          }
        }
        // keep-rate bookkeeping for the guard: the scored doublets
        const unsigned mc = __ballot_sync(kFull, score), mk = __ballot_sync(kFull, score && keep);
        if (lane == 0 && mc) {
          atomicAdd(&s.considered, (uint32_t)__popc(mc));
          atomicAdd(&s.kept, (uint32_t)__popc(mk));
        }
        cand = cand && keep;
      }
      if (!cand) continue;
      const float ddx = fsub(h1x, h0x), ddy = fsub(h1y, h0y);
      if (narrow4) {
        const float xa = fadd(h0x, fmul(ddx, fmul(fsub(zmin4, h0z), dz_inverted)));
        const float xb = fadd(h0x, fmul(ddx, fmul(fsub(zmax4, h0z), dz_inverted)));
        if (isfinite(xa) && isfinite(xb) && a < b) {
          int lo, hi;
          narrow_range(x4, a, b, fminf(xa, xb), fmaxf(xa, xb), tol, &lo, &hi);
          a = lo;
          b = hi;
        }
      }
      float lbest = FLT_MAX;
      int lk = -1;
      uint32_t zc = 0x7fc00001u;
      float z2_tz = 0.f, den = 0.f;
      for (int k = a; k < b; ++k) {
        const float h2z = z4[k];
        if (__float_as_uint(h2z) != zc) {   // both factors depend on h2z only (per h0, h1)
          zc = __float_as_uint(h2z);
          z2_tz = fmul(fsub(h2z, h0z), dz_inverted);
          den = fdiv(1.f, fsub(h2z, h1z));
        }
        const float dx = fsub(fadd(h0x, fmul(ddx, z2_tz)), x4[k]);
        const float dy = fsub(fadd(h0y, fmul(ddy, z2_tz)), y4[k]);
        if (fabsf(dx) < kTolerance && fabsf(dy) < kTolerance) {
          const float scatter = fmul(fmul(fadd(fmul(dx, dx), fmul(dy, dy)), den), den);
          if (scatter < kMaxScatter) {
            if (scatter < lbest) { lbest = scatter; lk = k; }
          } else if (!isfinite(scatter)) {
            degenerate = true;
          }
        }
      }
      if (lk >= 0) {
        const unsigned long long key = ((unsigned long long)__float_as_uint(lbest) << 32) |
                                       ((unsigned long long)ly << 28) | ((unsigned long long)e << 14) |
                                       (unsigned long long)lk;
        best = key < best ? key : best;
      }
    }
    // the group's 64-bit minimum as two 32-bit minima: the high words, then
    // the low words of the lanes that hold the minimal high word
    const uint32_t hi = (uint32_t)(best >> 32);
    uint32_t hmin, lmin;
    if constexpr (G == 32) {
      hmin = __reduce_min_sync(kFull, hi);
      lmin = __reduce_min_sync(kFull, hi == hmin ? (uint32_t)best : 0xffffffffu);
    } else {   // butterflies inside each group
      hmin = hi;
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) hmin = min(hmin, __shfl_xor_sync(kFull, hmin, o));
      lmin = hi == hmin ? (uint32_t)best : 0xffffffffu;
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) lmin = min(lmin, __shfl_xor_sync(kFull, lmin, o));
    }
    best = ((unsigned long long)hmin << 32) | lmin;
    // Kernel.cl:550-567: each group's first lane appends its tracklet
    if constexpr (G == 32) {
      if (lane == 0 && best != ~0ull) {
        const uint32_t e = (uint32_t)(best >> 14) & 0x3fffu;
        const uint32_t h1 = (uint32_t)(st1 + (int)f1) + e;
        const uint32_t h2 = (uint32_t)st4 + (uint32_t)(best & 0x3fffu);
        const uint32_t tp = atomicAdd(&s.ntracklets, 1u);
        if (tp < ev.cap) {
          ev.tracklets[tp] = make_uint4((uint32_t)h0, h1, h2, 0u);
          push_back(s, ev, nb, make_uint4(kTrackletFlag | tp, (uint32_t)h0, h1, h2));
        }
      }
    } else {   // one shared-memory atomic per warp for the tracklet rows, one for the ring
      const bool win = jl == 0 && best != ~0ull;
      const uint32_t tp = warp_reserve(&s.ntracklets, win);
      const bool push = win && tp < ev.cap;
      const uint32_t ri = warp_reserve(&s.ring_hi[nb], push);
      if (push) {
        const uint32_t e = (uint32_t)(best >> 14) & 0x3fffu;
        const uint32_t h1 = (uint32_t)(st1 + (int)f1) + e;
        const uint32_t h2 = (uint32_t)st4 + (uint32_t)(best & 0x3fffu);
        ev.tracklets[tp] = make_uint4((uint32_t)h0, h1, h2, 0u);
        if (ri < ev.ring_cap)
          ring_buf(ev, nb)[ev.ring_cap - 1u - ri] = make_uint4(kTrackletFlag | tp, (uint32_t)h0, h1, h2);
      }
    }
    } while (0);
    if constexpr (G == 32) {
      ib += nwarps;
    } else {
      if (lane == 0) ib = atomicAdd(&s.seed_next[nb ^ 1], kGroups);
      ib = __shfl_sync(kFull, ib, 0);
    }
  }
  if (degenerate) atomicOr(&s.status, VELO_EVENT_DEGENERATE);
}

// Per-phase cycle counters, compiled in only with -DVELO_PHASE_CLOCKS
// (diagnostic builds): thread 0 of every CTA adds the clock64() time between
// the barriers that close each phase; slot 7 counts events.
#ifdef VELO_PHASE_CLOCKS
static __device__ unsigned long long g_phase_cycles[8];   // one per translation unit
#define VELO_PHASE_BEGIN() long long ph_t = clock64(); unsigned long long ph[7] = {0, 0, 0, 0, 0, 0, 0}
#define VELO_PHASE(k)                 \
  do {                                \
    const long long t_ = clock64();   \
    ph[k] += (unsigned long long)(t_ - ph_t); \
    ph_t = t_;                        \
  } while (0)
#define VELO_PHASE_END()                                              \
  do {                                                                \
    if (threadIdx.x == 0) {                                           \
      for (int k_ = 0; k_ < 7; ++k_) atomicAdd(&g_phase_cycles[k_], ph[k_]); \
      atomicAdd(&g_phase_cycles[7], 1ull);                            \
    }                                                                 \
  } while (0)
#else
#define VELO_PHASE_BEGIN() do {} while (0)
#define VELO_PHASE(k) do {} while (0)
#define VELO_PHASE_END() do {} while (0)
#endif

// Hits of a module that one warp sorts by rank in registers (4 per lane).
constexpr int kArenaRankMax = 128;

// The reference's per-module x-sort (preorder_by_x, Tools.cpp:46-66) of the
// event staged in the arena, hit IDs alongside in `ids`; one warp per
// module.  Where a module's x values are distinct the reference's quicksort
// reaches the one ascending order there is, so each hit goes to its rank;
// a module with equal x values, or more than kArenaRankMax hits not already
// in strictly increasing order, replays the reference's partition steps in
// one thread (quicksort4).  x is finite here (the staging checked it).
// Returns, in every thread, whether any hit moved.
template <class Shared>
__device__ bool sort_arena(const EventView& ev, const Shared& s, int S, uint32_t* ids) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  float* x = ev.xs();
  float* y = ev.ys();
  float* z = ev.zs();
  bool moved = false;
  for (int m = warp; m < S; m += nwarps) {   // warp-uniform
    const int s0 = s.start[m], n = s.num[m];
    if (n < 2) continue;
    if (n > kArenaRankMax) {
      bool changed = false;
      if (lane == 0) {
        bool increasing = true;
        for (int i = s0 + 1; i < s0 + n && increasing; ++i) increasing = x[i - 1] < x[i];
        if (!increasing) {
          quicksort4(x, y, z, ids, s0, s0 + n - 1);
          changed = true;
        }
      }
      moved |= __shfl_sync(kFull, changed, 0);
      __syncwarp();
      continue;
    }
    float xr[4];
    int rk[4], eq[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = lane + 32 * k;
      xr[k] = i < n ? x[s0 + i] : 0.f;
      rk[k] = 0;
      eq[k] = 0;
    }
    for (int j = 0; j < n; ++j) {   // the same address in every lane
      const float xj = x[s0 + j];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        rk[k] += xj < xr[k];
        eq[k] += xj == xr[k];
      }
    }
    bool tie = false, mv = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = lane + 32 * k;
      if (i < n) {
        tie |= eq[k] > 1;
        mv |= rk[k] != i;
      }
    }
    if (__any_sync(kFull, tie)) {   // equal x values: the reference's partition steps decide
      if (lane == 0) quicksort4(x, y, z, ids, s0, s0 + n - 1);
      moved = true;
      __syncwarp();
      continue;
    }
    if (!__any_sync(kFull, mv)) continue;   // strictly increasing already
    moved = true;
    float yr[4], zr[4];
    uint32_t ir[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = lane + 32 * k;
      if (i < n) {
        yr[k] = y[s0 + i];
        zr[k] = z[s0 + i];
        ir[k] = ids[s0 + i];
      }
    }
    __syncwarp();   // every lane has read its hits before any is overwritten
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = lane + 32 * k;
      if (i < n) {
        const int r = s0 + rk[k];
        x[r] = xr[k];
        y[r] = yr[k];
        z[r] = zr[k];
        ids[r] = ir[k];
      }
    }
    __syncwarp();
  }
  return __syncthreads_or(moved) != 0;
}

// Streaming results (velo_search_begin): thread 0 writes the event's record,
// its ready flag last, after a system-scope fence; the caller has fenced the
// CTA's track writes before.
__device__ __forceinline__ void publish_result(const SearchParams& p, int e, unsigned long long first,
                                               uint32_t count, uint32_t status) {
  velo_event_result* r = p.results + e;
  r->first = first;
  r->count = count;
  r->status = status;
  __threadfence_system();
  *reinterpret_cast<volatile uint32_t*>(&r->ready) = 1u;
}

// ---------------------------------------------------------------------------
template <int kMode, int kLanes, class Shared>
__device__ void process_event(const SearchParams& p, int e, Shared& s, uint8_t* dyn, const MlpFrag* mlp_smem) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  VELO_PHASE_BEGIN();
  if (!p.ev_valid[e]) {
    if (tid == 0) {
      p.out_counts[e] = 0;
      p.out_first[e] = 0;
      p.out_status[e] = VELO_EVENT_INVALID;
      if (p.results) publish_result(p, e, 0ull, 0u, VELO_EVENT_INVALID);
    }
    return;
  }
  const int32_t* hdr = reinterpret_cast<const int32_t*>(p.input + p.ev_offset[e]);
  EventView ev;
  ev.S = hdr[0];
  ev.H = hdr[1];
  ev.Y = p.y_lanes;
  ev.narrow = p.narrow != 0;
  const int S = ev.S, H = ev.H;
  ev.cap = H > 0 ? (uint32_t)H : 1u;
  ev.ring_cap = ev.cap;
  const int32_t* gZ = hdr + 2;
  const int32_t* gstart = gZ + S;
  const int32_t* gnum = gstart + S;
  const float* gx = reinterpret_cast<const float*>(gnum + S + H);
  const float* gy = gx + H;
  const float* gz = gy + H;

  const ArenaLayout L = arena_layout((uint32_t)H, p.ev_maxmod[e], (uint32_t)ev.Y);
  uint8_t* arena = p.arena_off[e] == kNoArena ? dyn : p.global_arena + p.arena_off[e];
  ev.arena = arena;
  ev.P = L.y;
  const uint64_t hb = p.hit_base[e];
  ev.ring0 = reinterpret_cast<uint4*>(p.rings + 8 * hb);
  ev.ring1 = ev.ring0 + ev.cap;
  ev.tracklets = reinterpret_cast<uint4*>(p.tracklets + 4 * hb);
  ev.weak = p.weak + hb;
  ev.tracks = p.tracks + hb;
  ev.event = e;
  ev.mlp = mlp_smem;
  ev.keep_threshold = p.keep_threshold;
  ev.learned_min_window = p.learned_min_window;
  ev.window_margin = p.window_margin;
  ev.dump_features = p.dump_features;
  ev.dump_ids = p.dump_ids;
  ev.dump_count = p.dump_count;
  ev.dump_capacity = p.dump_capacity;
  ev.dump_keep = p.dump_keep > 0 ? p.dump_keep : 1u;

  // stage the event; the module table must tile [0, H) in order (the host
  // checked only the header and the blob's length)
  bool bad = tid == 0 && S == 0 && H != 0;
  for (int m = tid; m < S; m += nt) {
    const int32_t st = gstart[m], nm = gnum[m];
    const int64_t expect = m == 0 ? 0 : (int64_t)gstart[m - 1] + (int64_t)gnum[m - 1];
    bad |= nm < 0 || nm > VELO_MAX_MODULE_HITS || (int64_t)st != expect ||
           (m == S - 1 && (int64_t)st + (int64_t)nm != (int64_t)H);
    s.start[m] = st;
    s.num[m] = nm;
    s.sz[m] = gZ[m];
  }
  // with sort_events the IDs are staged too, in the window area (written
  // only after the sort)
  const uint32_t* gid = reinterpret_cast<const uint32_t*>(gnum + S);
  uint32_t* ids = reinterpret_cast<uint32_t*>(ev.wins());
  for (int i = tid; i < H; i += nt) {
    const float xv = gx[i], yv = gy[i], zv = gz[i];
    bad |= !(isfinite(xv) && isfinite(yv) && isfinite(zv));
    ev.xs()[i] = xv;
    ev.ys()[i] = yv;
    ev.zs()[i] = zv;
    ev.useds()[i] = 0;
    if (p.sort_events) ids[i] = gid[i];
  }
  if (tid == 0) {
    s.ring_lo[0] = 0; s.ring_lo[1] = 0; s.ring_hi[0] = 0; s.ring_hi[1] = 0;
    s.ntracks = 0; s.ntracklets = 0; s.nweak = 0; s.status = 0;
    s.considered = 0; s.kept = 0;
    s.seed_next[0] = 0; s.seed_next[1] = 0;
  }
  if (__syncthreads_or(bad)) {   // a bad module table, or a non-finite coordinate
    if (tid == 0) {
      p.out_counts[e] = 0;
      p.out_first[e] = 0;
      p.out_status[e] = VELO_EVENT_INVALID;
      if (p.results) publish_result(p, e, 0ull, 0u, VELO_EVENT_INVALID);
    }
    return;
  }
  if (p.sort_events && sort_arena(ev, s, S, ids)) {
    // the sorted hit arrays (IDs, x, y, z) back into the input, the
    // caller's buffer read in place: posted writes across the host link,
    // overlapped with the search of the other resident events
    uint32_t* wid = const_cast<uint32_t*>(gid);
    float* wx = reinterpret_cast<float*>(wid + H);
    float* wy = wx + H;
    float* wz = wy + H;
    for (int i = tid; i < H; i += nt) {
      wid[i] = ids[i];
      wx[i] = ev.xs()[i];
      wy[i] = ev.ys()[i];
      wz[i] = ev.zs()[i];
    }
    __syncthreads();   // the window area is written next
  }
  VELO_PHASE(0);

  // per-module z range and x-sortedness (one warp per module)
  for (int m = warp; m < S; m += nwarps) {
    const int st = s.start[m], n = s.num[m];
    float zmn = FLT_MAX, zmx = -FLT_MAX;
    bool sorted = true;
    for (int i = lane; i < n; i += 32) {
      const float z = ev.zs()[st + i];
      zmn = fminf(zmn, z);
      zmx = fmaxf(zmx, z);
      if (i + 1 < n && !(ev.xs()[st + i] <= ev.xs()[st + i + 1])) sorted = false;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      zmn = fminf(zmn, __shfl_xor_sync(kFull, zmn, o));
      zmx = fmaxf(zmx, __shfl_xor_sync(kFull, zmx, o));
    }
    sorted = __all_sync(kFull, sorted);
    if (lane == 0) {
      s.zmin[m] = zmn;
      s.zmax[m] = zmx;
      s.sorted[m] = sorted ? 1 : 0;
    }
  }
  // windows of modules 0..3 stay empty (Kernel.cl:104 gates the body on f >= 4)
  const int hbeg = S >= 5 ? s.start[4] : H;
  for (int i = tid; i < hbeg; i += nt) ev.wins()[i] = make_uint2(0xffffffffu, 0xffffffffu);
  __syncthreads();
  VELO_PHASE(1);

  // candidate windows for every hit of modules >= 4
  for (int h = hbeg + tid; h < H; h += nt) {
    int lo = 4, hi = S - 1;   // last module whose start is <= h
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s.start[mid] <= h) lo = mid; else hi = mid - 1;
    }
    compute_windows(ev, s, h, lo);
  }

  // per-lane constants of the seeding ballots (the host checked that
  // seed_lanes is 8, 16 or 32, and a multiple of Y below 32)
  const SeedLanes sl = seed_lanes_of(kLanes, (uint32_t)ev.Y);
  __syncthreads();
  VELO_PHASE(2);

  // The learned seeding runs first when enabled; if it kept too small a
  // fraction of the doublets it scored, the event is searched again by the
  // plain method (used flags and lists reset; windows kept).
  bool learned = kMode == kLearned && (p.learned_max_hits == 0 || (uint32_t)H <= p.learned_max_hits);
  uint32_t fallback = (kMode == kLearned && !learned) ? VELO_EVENT_LEARNED_FALLBACK : 0u;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if (attempt > 0) {
      for (int i = tid; i < H; i += nt) ev.useds()[i] = 0;
      if (tid == 0) {
        s.ring_lo[0] = 0; s.ring_lo[1] = 0; s.ring_hi[0] = 0; s.ring_hi[1] = 0;
        s.ntracks = 0; s.ntracklets = 0; s.nweak = 0; s.status = 0;
        s.seed_next[0] = 0; s.seed_next[1] = 0;
      }
      __syncthreads();
    }
    // module loop, Kernel.cl:671-767
    int b = 0;   // ring[b] holds the entries to follow in this iteration
    for (int f = S - 1; f >= 4; --f) {
      const uint32_t lo_n = min(s.ring_lo[b], ev.ring_cap);
      const uint32_t ncur = min(lo_n + s.ring_hi[b], ev.ring_cap);
      if (tid == 0 && s.ring_lo[b] + s.ring_hi[b] > VELO_TTF_MODULO) s.status |= VELO_EVENT_RING_OVERFLOW;
      for (uint32_t i0 = (uint32_t)warp * 32u; i0 < ncur; i0 += (uint32_t)nt)   // warp-uniform
        forward_warp(ev, s, b, lo_n, i0, ncur, f - 4, b ^ 1);
      __syncthreads();
      VELO_PHASE(3);
      if (tid == 0) {
        if (ncur + s.ring_lo[b ^ 1] > VELO_TTF_MODULO) s.status |= VELO_EVENT_RING_OVERFLOW;
        // this iteration's seeding claims h0s from seed_next[b]; the next
        // one (parity b ^ 1) from seed_next[b ^ 1], last used before the
        // barrier that closed the previous iteration
        s.seed_next[b ^ 1] = 0;
        s.ring_lo[b] = 0;   // ring[b] is refilled two iterations on
        s.ring_hi[b] = 0;
      }
      if (s.num[f] > 0) {
        if (learned)
          seed_module<kLearned, kLanes>(ev, s, f, b ^ 1, sl);
        else
          seed_module<kMode == kDump ? kDump : kPlain, kLanes>(ev, s, f, b ^ 1, sl);
      }
      __syncthreads();
      VELO_PHASE(4);
      b ^= 1;
    }

    // leftover tracklets become weak (Kernel.cl:771-792)
    {
      if (tid == 0 && s.ring_lo[b] + s.ring_hi[b] > VELO_TTF_MODULO) s.status |= VELO_EVENT_RING_OVERFLOW;
      const uint32_t lo_n = min(s.ring_lo[b], ev.ring_cap);
      const uint32_t ncur = min(lo_n + s.ring_hi[b], ev.ring_cap);
      for (uint32_t i = tid; i < ncur; i += nt) {
        const uint32_t v = ring_entry(ev, b, lo_n, i).x;
        if (v & kTrackletFlag) {
          const uint32_t wi = atomicAdd(&s.nweak, 1u);
          if (wi < ev.cap) ev.weak[wi] = v & kEntryNumber;
        }
      }
    }
    __syncthreads();
    // weak tracks made of three unused hits (Kernel.cl:796-815)
    {
      const uint32_t nweak = min(s.nweak, ev.cap);
      for (uint32_t i = tid; i < nweak; i += nt) {
        const uint4 t = ev.tracklets[ev.weak[i]];
        const uint32_t a = t.x, bb = t.y, c = t.z;
        if (!ev.useds()[a] && !ev.useds()[bb] && !ev.useds()[c]) {
          const uint32_t tn = atomicAdd(&s.ntracks, 1u);
          if (tn >= ev.cap) continue;
          uint32_t* wr = reinterpret_cast<uint32_t*>(&ev.tracks[tn]);
          wr[0] = 3; wr[1] = a; wr[2] = bb; wr[3] = c;
  #pragma unroll
          for (int k = 4; k < 25; ++k) wr[k] = 0;
        }
      }
    }
    __syncthreads();
    VELO_PHASE(5);
    if (!learned) break;
    const uint32_t considered = s.considered, kept = s.kept;   // final after the barrier above
    if (considered == 0 || (float)kept >= p.min_keep_rate * (float)considered) break;
    learned = false;
    fallback = VELO_EVENT_LEARNED_FALLBACK;
    __syncthreads();   // everyone has read the counters before the reset
  }

  // compacted output: one atomic per event reserves its range
  if (tid == 0) {
    const uint32_t cnt = min(s.ntracks, ev.cap);
    if (s.ntracks > VELO_MAX_TRACKS) s.status |= VELO_EVENT_MAX_TRACKS;
    const unsigned long long first = atomicAdd(p.out_cursor, (unsigned long long)cnt);
    s.out_first = first;
    p.out_counts[e] = cnt;
    p.out_first[e] = first;
    p.out_status[e] = s.status | fallback;
  }
  __syncthreads();
  {
    // rows past out_capacity stay unwritten (the host reports the shortfall)
    const unsigned long long room = s.out_first < p.out_capacity ? p.out_capacity - s.out_first : 0ull;
    const uint32_t words = (uint32_t)min((unsigned long long)min(s.ntracks, ev.cap), room) * 25u;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(ev.tracks);
    uint32_t* dst = reinterpret_cast<uint32_t*>(p.out_tracks + s.out_first);
    for (uint32_t w = tid; w < words; w += nt) dst[w] = src[w];
  }
  if (p.results) {   // streaming: the tracks first, then the record
    __threadfence_system();
    __syncthreads();
    if (tid == 0) publish_result(p, e, s.out_first, min(s.ntracks, ev.cap), s.status | fallback);
  }
  VELO_PHASE(6);
  VELO_PHASE_END();
}

// Builds: up to 256 threads per CTA with registers budgeted for 4 or for 5
// resident 256-thread CTAs per SM (velo_options.register_ctas 4 / 5: 64 / 48
// registers), 64-thread CTAs with 56 registers (18 CTAs per SM,
// register_ctas 18), and 512-thread CTAs; the learned mode in the 64-register
// build of up to 256 threads (a 56-register 64-thread learned build measured
// slower: more of its registers spill around the scorer's calls); each for
// one seeding width kLanes (lanes per h0), so that a kernel holds one copy of
// the seeding loop.
template <int kMaxThreads, int kMinCtas, int kMode, int kMods, int kLanes>
__global__ void __launch_bounds__(kMaxThreads, kMinCtas) search_kernel(const SearchParams p) {
  extern __shared__ __align__(16) uint8_t dyn_smem_raw[];
  __shared__ SharedT<kMods> s;
  // learned seeding: the MLP weights lead the dynamic shared memory
  const MlpFrag* mlp_smem = nullptr;
  uint8_t* dyn_smem = dyn_smem_raw;
  if constexpr (kMode == kLearned) {
    MlpFrag* w = reinterpret_cast<MlpFrag*>(dyn_smem_raw);
    stage_mlp_fragments(p.mlp, w);
    __syncthreads();
    mlp_smem = w;
    dyn_smem = dyn_smem_raw + kMlpSmemBytes;
  }
  if (!p.persistent) {
    if ((int)blockIdx.x < p.n_events) process_event<kMode, kLanes>(p, blockIdx.x, s, dyn_smem, mlp_smem);
    return;
  }
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s.next_event = atomicAdd(p.work_counter, 1);
    __syncthreads();
    const int k = s.next_event;
    if (k >= p.n_events) break;
    process_event<kMode, kLanes>(p, p.order[k], s, dyn_smem, mlp_smem);
  }
}

constexpr int kFullModules = kMaxModules + 1;

// The builds of one seeding width G: launch, dynamic shared-memory limit and
// occupancy, as launch_search / configure_search_kernel / search_occupancy
// (velo_internal.h) take them.  The dump mode exists for G = 32 only.
template <int G>
struct SearchBuilds {
  static int launch(const SearchParams& p, int grid, int block, uint32_t smem, cudaStream_t st, int reg_ctas,
                    bool compact) {
    if (p.mlp && compact)
      search_kernel<256, 4, kLearned, kCompactModules, G><<<grid, min(block, 256), smem, st>>>(p);
    else if (p.mlp)
      search_kernel<256, 4, kLearned, kFullModules, G><<<grid, min(block, 256), smem, st>>>(p);
    else if (G == 32 && p.dump_features)
      search_kernel<256, 4, kDump, kFullModules, 32><<<grid, min(block, 256), smem, st>>>(p);
    else if (block > 256)
      search_kernel<512, 1, kPlain, kFullModules, G><<<grid, block, smem, st>>>(p);
    else if (reg_ctas == 18 && compact)
      search_kernel<64, 18, kPlain, kCompactModules, G><<<grid, block, smem, st>>>(p);
    else if (reg_ctas == 18)
      search_kernel<64, 18, kPlain, kFullModules, G><<<grid, block, smem, st>>>(p);
    else if (reg_ctas == 4 && compact)
      search_kernel<256, 4, kPlain, kCompactModules, G><<<grid, block, smem, st>>>(p);
    else if (reg_ctas == 4)
      search_kernel<256, 4, kPlain, kFullModules, G><<<grid, block, smem, st>>>(p);
    else if (compact)
      search_kernel<256, 5, kPlain, kCompactModules, G><<<grid, block, smem, st>>>(p);
    else
      search_kernel<256, 5, kPlain, kFullModules, G><<<grid, block, smem, st>>>(p);
    return (int)cudaGetLastError();
  }

  static int configure(uint32_t smem) {
    cudaError_t e = cudaSuccess;
#define VELO_LIMIT(...)   \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(__VA_ARGS__, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
    VELO_LIMIT(search_kernel<256, 4, kPlain, kFullModules, G>);
    VELO_LIMIT(search_kernel<256, 5, kPlain, kFullModules, G>);
    VELO_LIMIT(search_kernel<256, 4, kPlain, kCompactModules, G>);
    VELO_LIMIT(search_kernel<256, 5, kPlain, kCompactModules, G>);
    VELO_LIMIT(search_kernel<64, 18, kPlain, kFullModules, G>);
    VELO_LIMIT(search_kernel<64, 18, kPlain, kCompactModules, G>);
    VELO_LIMIT(search_kernel<512, 1, kPlain, kFullModules, G>);
    VELO_LIMIT(search_kernel<256, 4, kLearned, kFullModules, G>);
    VELO_LIMIT(search_kernel<256, 4, kLearned, kCompactModules, G>);
    if (G == 32) VELO_LIMIT(search_kernel<256, 4, kDump, kFullModules, 32>);
#undef VELO_LIMIT
    return (int)e;
  }

  static int occupancy(int block, uint32_t smem, int reg_ctas, int mode, bool compact, int* ctas) {
    if (mode == kModeLearned)
      return compact ? (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<256, 4, kLearned, kCompactModules, G>, min(block, 256), smem)
                     : (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<256, 4, kLearned, kFullModules, G>, min(block, 256), smem);
    if (mode == kModeDump)
      return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, search_kernel<256, 4, kDump, kFullModules, 32>,
                                                                min(block, 256), smem);
    if (block > 256)
      return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, search_kernel<512, 1, kPlain, kFullModules, G>,
                                                                block, smem);
    if (reg_ctas == 18)
      return compact ? (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<64, 18, kPlain, kCompactModules, G>, block, smem)
                     : (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<64, 18, kPlain, kFullModules, G>, block, smem);
    if (reg_ctas == 4)
      return compact ? (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<256, 4, kPlain, kCompactModules, G>, block, smem)
                     : (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           ctas, search_kernel<256, 4, kPlain, kFullModules, G>, block, smem);
    return compact ? (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                         ctas, search_kernel<256, 5, kPlain, kCompactModules, G>, block, smem)
                   : (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                         ctas, search_kernel<256, 5, kPlain, kFullModules, G>, block, smem);
  }

#ifdef VELO_PHASE_CLOCKS
  // Adds this unit's per-phase cycle counters to out[8] and clears them.
  static int phase_cycles(unsigned long long* out) {
    unsigned long long v[8] = {};
    cudaError_t e = cudaMemcpyFromSymbol(v, g_phase_cycles, sizeof v);
    unsigned long long zero[8] = {};
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_phase_cycles, zero, sizeof zero);
    for (int k = 0; k < 8; ++k) out[k] += v[k];
    return (int)e;
  }
#endif
};

}  // namespace velo
