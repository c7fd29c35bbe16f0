// velo_kernels.cu -- sm_103a search-by-triplet kernel.
//
// One CTA reconstructs one event (the reference's one work-group per event,
// Kernel.cl:607, KernelInvoker.cpp:26-27), either one CTA per event or
// persistent CTAs pulling events, largest first, from a work queue.  The
// event's hits and its per-hit working state live in dynamic shared memory
// (the "arena"); events too large for the launch's arena use a global-memory
// arena with the same layout.
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
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <mutex>

#include "velo_internal.h"

namespace velo {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

struct Shared {
  int32_t start[kMaxModules + 1];
  int32_t num[kMaxModules + 1];
  int32_t sz[kMaxModules + 1];
  float zmin[kMaxModules + 1];
  float zmax[kMaxModules + 1];
  uint8_t sorted[kMaxModules + 1];
  uint32_t ncur, nnext, ntracks, ntracklets, nweak, status, nslots, ntasks;
  unsigned long long out_first;
  int32_t next_event;
};

struct EventView {
  int S, H, Y;
  uint32_t cap;             // capacity of tracklet / track / weak rows (max(H, 1))
  uint32_t ring_cap;        // entries of each tracks-to-follow buffer (H + 1)
  float *x, *y, *z;
  int32_t *h1f, *h1l, *h2f, *h2l;
  uint8_t* used;
  uint32_t *ring0, *ring1;
  int32_t* slot_h0;
  uint32_t* slot_pref;
  uint32_t* cutoff;
  unsigned long long* best;
  uint32_t* tracklets;
  uint32_t* weak;
  velo_track* tracks;
  bool narrow;
};

// First index i in [lo, hi) with x[i] > c, for non-decreasing x.
__device__ __forceinline__ int first_gt(const float* x, int lo, int hi, float c) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] > c) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Index range [lo, hi) of a sorted module outside which no hit can satisfy
// |fl(xp - x)| < tol for any predicted xp in [xl, xh].
__device__ __forceinline__ void narrow_range(const float* x, int n, float xl, float xh, float tol,
                                             int* lo, int* hi) {
  const float margin = fadd(0.01f, fmul(1e-5f, fadd(fabsf(xl), fabsf(xh))));
  const float lt = fsub(fsub(xl, tol), margin);
  const float ht = fadd(fadd(xh, tol), margin);
  if (isfinite(lt) && isfinite(ht)) {
    *lo = first_gt(x, 0, n, lt);
    *hi = first_gt(x, *lo, n, ht);
  } else {
    *lo = 0;
    *hi = n;
  }
}

// ---------------------------------------------------------------------------
// Candidate windows of hit h on module f (Kernel.cl:50-178).
__device__ void compute_windows(const EventView& ev, const Shared& s, int h, int f) {
  const int s2 = f - 2;
  const bool proc_h2 = f <= ev.S - 3;
  const int st2 = s.start[s2], n2 = s.num[s2];
  const float x0 = ev.x[h], z0 = ev.z[h];
  const float* x2 = ev.x + st2;
  const float* z2 = ev.z + st2;
  const bool sorted = ev.narrow && s.sorted[s2];
  int r1f = -1, r1l = -1, r2f = -1, r2l = -1;

  // h1 window: first hit with |x1-x0| < 0.7|z1-z0|, then the first later hit
  // that fails it (Kernel.cl:115-135,161-165).
  {
    int lo = 0, hi = n2;
    if (sorted && n2 > 0) {
      const float da = fabsf(fsub(s.zmin[s2], z0));
      const float db = fabsf(fsub(s.zmax[s2], z0));
      const float D = fmul(kMaxXSlopeCandidates, fmaxf(da, db));   // >= every hit's dxmax
      narrow_range(x2, n2, x0, x0, D, &lo, &hi);
    }
    bool found = false;
    for (int e = lo; e < hi; ++e) {
      const float h_dist = fabsf(fsub(z2[e], z0));
      const float dxmax = fmul(kMaxXSlopeCandidates, h_dist);
      const bool tol = fabsf(fsub(x2[e], x0)) < dxmax;
      if (!found) {
        if (tol) { found = true; r1f = st2 + e; }
      } else if (!tol) {
        r1l = st2 + e;
        break;
      }
    }
    if (found && r1l < 0) r1l = st2 + hi;   // hit `hi` provably fails, or hi is the end
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
        r2f = st2 + a;
        r2l = st2 + first_gt(x2, a + 1, n2, xmax_h2);
      }
    } else {
      bool found = false;
      for (int e = 0; e < n2; ++e) {
        if (!found) {
          if (x2[e] > xmin_h2) { found = true; r2f = st2 + e; }
        } else if (x2[e] > xmax_h2) {
          r2l = st2 + e;
          break;
        }
      }
      if (found && r2l < 0) r2l = st2 + n2;
    }
  }
  ev.h1f[h] = r1f;
  ev.h1l[h] = r1l;
  ev.h2f[h] = r2f;
  ev.h2l[h] = r2l;
}

// ---------------------------------------------------------------------------
// fitHitToTrack (Kernel.cl:15-35): the scatter, FLT_MAX when a cut fails, or
// NaN where the reference's `condition*scatter + !condition*MAX` is NaN.
__device__ __forceinline__ float fit_hit(float tx, float ty, float h0x, float h0y, float h0z,
                                         float h1z, float h2x, float h2y, float h2z) {
  const float dz = fsub(h2z, h0z);
  const float dx = fabsf(fsub(fadd(h0x, fmul(tx, dz)), h2x));
  const float dy = fabsf(fsub(fadd(h0y, fmul(ty, dz)), h2y));
  const float num = fadd(fmul(dx, dx), fmul(dy, dy));
  const float den = fdiv(1.f, fsub(h2z, h1z));
  const float scatter = fmul(fmul(num, den), den);
  if (dx < kTolerance && dy < kTolerance && scatter < kMaxScatter) return scatter;
  return isfinite(scatter) ? FLT_MAX : __int_as_float(0x7fc00000);
}

__device__ __forceinline__ void push_ring(Shared& s, const EventView& ev, uint32_t* nxt, uint32_t v) {
  const uint32_t i = atomicAdd(&s.nnext, 1u);
  if (i < ev.ring_cap) nxt[i] = v;
}

// Track forwarding of one tracks-to-follow entry onto module m4
// (Kernel.cl:210-367).
__device__ void forward_entry(const EventView& ev, Shared& s, uint32_t full, int m4, uint32_t* nxt) {
  const bool is_tracklet = (full & kTrackletFlag) != 0;
  const uint32_t skipped = (full & kSkipMask) >> 28;
  uint32_t trackno = full & kNumberMask;
  uint32_t n, h0, h1, t0 = 0, t1 = 0, t2 = 0;
  if (is_tracklet) {
    t0 = ev.tracklets[3 * trackno + 0];
    t1 = ev.tracklets[3 * trackno + 1];
    t2 = ev.tracklets[3 * trackno + 2];
    n = 3;
    h0 = t1;
    h1 = t2;
  } else {
    const velo_track& t = ev.tracks[trackno];
    n = t.hitsNum;
    h0 = t.hits[n - 2];
    h1 = t.hits[n - 1];
  }
  const float h0x = ev.x[h0], h0y = ev.y[h0], h0z = ev.z[h0];
  const float h1x = ev.x[h1], h1y = ev.y[h1], h1z = ev.z[h1];
  const float td = fdiv(1.0f, fsub(h1z, h0z));
  const float tx = fmul(fsub(h1x, h0x), td);
  const float ty = fmul(fsub(h1y, h0y), td);

  const int st4 = s.start[m4], n4 = s.num[m4];
  const float* x4 = ev.x + st4;
  int lo = 0, hi = n4;
  if (ev.narrow && s.sorted[m4] && n4 > 0) {
    const float xa = fadd(h0x, fmul(tx, fsub(s.zmin[m4], h0z)));
    const float xb = fadd(h0x, fmul(tx, fsub(s.zmax[m4], h0z)));
    if (isfinite(xa) && isfinite(xb)) narrow_range(x4, n4, fminf(xa, xb), fmaxf(xa, xb), kTolerance, &lo, &hi);
  }
  float best = FLT_MAX;
  int best_h2 = -1;
  bool degenerate = false;
  for (int k = lo; k < hi; ++k) {
    const int h2 = st4 + k;
    const float fit = fit_hit(tx, ty, h0x, h0y, h0z, h1z, x4[k], ev.y[h2], ev.z[h2]);
    if (isnan(fit)) { degenerate = true; continue; }
    if (fit < best) { best = fit; best_h2 = h2; }
  }
  if (degenerate) atomicOr(&s.status, VELO_EVENT_DEGENERATE);

  if (best != FLT_MAX) {
    if (n >= VELO_MAX_TRACK_SIZE) {   // the reference writes past hits[24] here
      atomicOr(&s.status, VELO_EVENT_TRACK_OVERFLOW);
      return;
    }
    ev.used[best_h2] = 1;
    if (is_tracklet) {   // third -> fourth hit: allocate a track, mark hits 0-2
      ev.used[t0] = 1;
      ev.used[t1] = 1;
      ev.used[t2] = 1;
      const uint32_t tn = atomicAdd(&s.ntracks, 1u);
      if (tn >= ev.cap) return;
      uint32_t* w = reinterpret_cast<uint32_t*>(&ev.tracks[tn]);
      w[0] = 4; w[1] = t0; w[2] = t1; w[3] = t2; w[4] = (uint32_t)best_h2;
#pragma unroll
      for (int i = 5; i < 25; ++i) w[i] = 0;
      trackno = tn;
    } else {
      velo_track& t = ev.tracks[trackno];
      t.hits[n] = (uint32_t)best_h2;
      t.hitsNum = n + 1;
    }
    push_ring(s, ev, nxt, trackno);
  } else if (skipped <= kMaxSkippedModules) {
    push_ring(s, ev, nxt, ((skipped + 1u) << 28) | (full & 0x8FFFFFFFu));
  } else if (is_tracklet) {
    const uint32_t wi = atomicAdd(&s.nweak, 1u);
    if (wi < ev.cap) ev.weak[wi] = trackno;
  }
}

// Last slot whose prefix is <= t (prefixes strictly increase).
__device__ __forceinline__ int slot_of(const uint32_t* pref, int nslots, uint32_t t) {
  int lo = 0, hi = nslots - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Seeding of module f: h0 on f, h1 on f-2, h2 on f-4 (Kernel.cl:392-568
// with the unused-h0 gather of :720-764).  Work is flattened over (h0, h1
// element) pairs; each pair scans its h2 window and folds its first minimum
// into the h0's packed key with a shared-memory atomicMin.
__device__ void seed_module(const EventView& ev, Shared& s, int f, uint32_t* nxt) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  const int st0 = s.start[f], n0 = s.num[f];
  const int Y = ev.Y;

  // S1: unused h0 with a non-empty h1 window, and the prefix of window sizes
  if (tid < 32) {
    uint32_t nslots = 0, ntasks = 0;
    for (int c = 0; c < n0; c += 32) {
      const int i = c + lane;
      const int h0 = st0 + i;
      uint32_t n1 = 0;
      if (i < n0 && !ev.used[h0]) {
        const int a = ev.h1f[h0];
        n1 = a >= 0 ? (uint32_t)(ev.h1l[h0] - a) : 0u;
      }
      const unsigned take = __ballot_sync(0xffffffffu, n1 > 0);
      uint32_t inc = n1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (n1 > 0) {
        const uint32_t pos = nslots + __popc(take & ((1u << lane) - 1u));
        ev.slot_h0[pos] = h0;
        ev.slot_pref[pos] = ntasks + inc - n1;
      }
      nslots += __popc(take);
      ntasks += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) {
      s.nslots = nslots;
      s.ntasks = ntasks;
      ev.slot_pref[nslots] = ntasks;
    }
  }
  __syncthreads();
  const int nslots = (int)s.nslots;
  const uint32_t ntasks = s.ntasks;
  if (nslots == 0) return;   // uniform

  // S2: reset per-slot state
  for (int i = tid; i < nslots * Y; i += nt) ev.cutoff[i] = 0xffffffffu;
  for (int i = tid; i < nslots; i += nt) ev.best[i] = ~0ull;
  __syncthreads();

  // S3: each lane's first h1 element without an h2 window
  for (uint32_t t = tid; t < ntasks; t += nt) {
    const int sl = slot_of(ev.slot_pref, nslots, t);
    const uint32_t e = t - ev.slot_pref[sl];
    const int h1 = ev.h1f[ev.slot_h0[sl]] + (int)e;
    if (ev.h2f[h1] == -1) atomicMin(&ev.cutoff[sl * Y + (int)(e % (uint32_t)Y)], e);
  }
  __syncthreads();

  // S4: triplet scatter search
  const int s1 = f - 2, m4 = f - 4;
  const int st4 = s.start[m4], n4 = s.num[m4];
  const float s1_z = s.num[s1] > 0 ? ev.z[s.start[s1]] : 0.f;   // Kernel.cl:420
  const bool narrow4 = ev.narrow && s.sorted[m4] && n4 > 0;
  const float zmin4 = s.zmin[m4], zmax4 = s.zmax[m4];
  bool degenerate = false;
  for (uint32_t t = tid; t < ntasks; t += nt) {
    const int sl = slot_of(ev.slot_pref, nslots, t);
    const uint32_t e = t - ev.slot_pref[sl];
    const uint32_t lane_y = e % (uint32_t)Y;
    if (e >= ev.cutoff[sl * Y + (int)lane_y]) continue;
    const int h0 = ev.slot_h0[sl];
    const int h1 = ev.h1f[h0] + (int)e;
    if (ev.used[h1]) continue;
    const float h0x = ev.x[h0], h0y = ev.y[h0], h0z = ev.z[h0];
    const float h1x = ev.x[h1], h1y = ev.y[h1], h1z = ev.z[h1];
    const float dymax = fmul(kMaxYSlope, fabsf(fsub(s1_z, h0z)));
    if (!(fabsf(fsub(h1y, h0y)) < dymax)) continue;   // h2-independent term of Kernel.cl:509
    const float dz_inverted = fdiv(1.f, fsub(h1z, h0z));
    const float ddx = fsub(h1x, h0x), ddy = fsub(h1y, h0y);
    int a = ev.h2f[h1], b = ev.h2l[h1];
    if (narrow4) {
      const float xa = fadd(h0x, fmul(ddx, fmul(fsub(zmin4, h0z), dz_inverted)));
      const float xb = fadd(h0x, fmul(ddx, fmul(fsub(zmax4, h0z), dz_inverted)));
      if (isfinite(xa) && isfinite(xb)) {
        int lo, hi;
        narrow_range(ev.x + st4, n4, fminf(xa, xb), fmaxf(xa, xb), kTolerance, &lo, &hi);
        a = max(a, st4 + lo);
        b = min(b, st4 + hi);
      }
    }
    float lbest = FLT_MAX;
    int lh2 = -1;
    for (int h2 = a; h2 < b; ++h2) {
      const float h2x = ev.x[h2], h2y = ev.y[h2], h2z = ev.z[h2];
      const float z2_tz = fmul(fsub(h2z, h0z), dz_inverted);
      const float dx = fsub(fadd(h0x, fmul(ddx, z2_tz)), h2x);
      const float dy = fsub(fadd(h0y, fmul(ddy, z2_tz)), h2y);
      if (fabsf(dx) < kTolerance && fabsf(dy) < kTolerance) {
        const float num = fadd(fmul(dx, dx), fmul(dy, dy));
        const float den = fdiv(1.f, fsub(h2z, h1z));
        const float scatter = fmul(fmul(num, den), den);
        if (scatter < kMaxScatter) {
          if (scatter < lbest) { lbest = scatter; lh2 = h2; }
        } else if (!isfinite(scatter)) {
          degenerate = true;
        }
      }
    }
    if (lh2 >= 0) {
      const unsigned long long key = ((unsigned long long)__float_as_uint(lbest) << 32) |
                                     ((unsigned long long)lane_y << 28) |
                                     ((unsigned long long)e << 14) | (unsigned long long)(lh2 - st4);
      atomicMin(&ev.best[sl], key);
    }
  }
  if (degenerate) atomicOr(&s.status, VELO_EVENT_DEGENERATE);
  __syncthreads();

  // S5: emit one tracklet per h0 with an accepted triplet (Kernel.cl:550-567)
  for (int sl = tid; sl < nslots; sl += nt) {
    const unsigned long long key = ev.best[sl];
    if (key == ~0ull) continue;
    const int h0 = ev.slot_h0[sl];
    const uint32_t e = (uint32_t)(key >> 14) & 0x3fffu;
    const uint32_t h1 = (uint32_t)(ev.h1f[h0] + (int)e);
    const uint32_t h2 = (uint32_t)st4 + (uint32_t)(key & 0x3fffu);
    const uint32_t tp = atomicAdd(&s.ntracklets, 1u);
    if (tp >= ev.cap) continue;
    ev.tracklets[3 * tp + 0] = (uint32_t)h0;
    ev.tracklets[3 * tp + 1] = h1;
    ev.tracklets[3 * tp + 2] = h2;
    push_ring(s, ev, nxt, kTrackletFlag | tp);
  }
}

// ---------------------------------------------------------------------------
__device__ void process_event(const SearchParams& p, int e, Shared& s, uint8_t* dyn) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  if (!p.ev_valid[e]) {
    if (tid == 0) {
      p.out_counts[e] = 0;
      p.out_first[e] = 0;
      p.out_status[e] = VELO_EVENT_INVALID;
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
  ev.ring_cap = (uint32_t)H + 1u;
  const int32_t* gZ = hdr + 2;
  const int32_t* gstart = gZ + S;
  const int32_t* gnum = gstart + S;
  const float* gx = reinterpret_cast<const float*>(gnum + S + H);
  const float* gy = gx + H;
  const float* gz = gy + H;

  const ArenaLayout L = arena_layout((uint32_t)H, p.ev_maxmod[e], (uint32_t)ev.Y);
  uint8_t* arena = p.arena_off[e] == kNoArena ? dyn : p.global_arena + p.arena_off[e];
  ev.x = reinterpret_cast<float*>(arena + L.x);
  ev.y = reinterpret_cast<float*>(arena + L.y);
  ev.z = reinterpret_cast<float*>(arena + L.z);
  ev.h1f = reinterpret_cast<int32_t*>(arena + L.h1f);
  ev.h1l = reinterpret_cast<int32_t*>(arena + L.h1l);
  ev.h2f = reinterpret_cast<int32_t*>(arena + L.h2f);
  ev.h2l = reinterpret_cast<int32_t*>(arena + L.h2l);
  ev.used = arena + L.used;
  ev.ring0 = reinterpret_cast<uint32_t*>(arena + L.ring0);
  ev.ring1 = reinterpret_cast<uint32_t*>(arena + L.ring1);
  ev.slot_h0 = reinterpret_cast<int32_t*>(arena + L.slot_h0);
  ev.slot_pref = reinterpret_cast<uint32_t*>(arena + L.slot_pref);
  ev.cutoff = reinterpret_cast<uint32_t*>(arena + L.cutoff);
  ev.best = reinterpret_cast<unsigned long long*>(arena + L.best);
  const uint64_t hb = p.hit_base[e];
  ev.tracklets = p.tracklets + 3 * hb;
  ev.weak = p.weak + hb;
  ev.tracks = p.tracks + hb;

  // stage the event
  for (int m = tid; m < S; m += nt) {
    s.start[m] = gstart[m];
    s.num[m] = gnum[m];
    s.sz[m] = gZ[m];
  }
  bool bad = false;
  for (int i = tid; i < H; i += nt) {
    const float xv = gx[i], yv = gy[i], zv = gz[i];
    bad |= !(isfinite(xv) && isfinite(yv) && isfinite(zv));
    ev.x[i] = xv;
    ev.y[i] = yv;
    ev.z[i] = zv;
    ev.used[i] = 0;
  }
  if (tid == 0) {
    s.ncur = 0; s.nnext = 0; s.ntracks = 0; s.ntracklets = 0; s.nweak = 0; s.status = 0;
  }
  if (__syncthreads_or(bad)) {   // coordinates must be finite (the host checks only the tables)
    if (tid == 0) {
      p.out_counts[e] = 0;
      p.out_first[e] = 0;
      p.out_status[e] = VELO_EVENT_INVALID;
    }
    return;
  }

  // per-module z range and x-sortedness (one warp per module)
  for (int m = warp; m < S; m += nwarps) {
    const int st = s.start[m], n = s.num[m];
    float zmn = FLT_MAX, zmx = -FLT_MAX;
    bool sorted = true;
    for (int i = lane; i < n; i += 32) {
      const float z = ev.z[st + i];
      zmn = fminf(zmn, z);
      zmx = fmaxf(zmx, z);
      if (i + 1 < n && !(ev.x[st + i] <= ev.x[st + i + 1])) sorted = false;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      zmn = fminf(zmn, __shfl_xor_sync(0xffffffffu, zmn, o));
      zmx = fmaxf(zmx, __shfl_xor_sync(0xffffffffu, zmx, o));
    }
    sorted = __all_sync(0xffffffffu, sorted);
    if (lane == 0) {
      s.zmin[m] = zmn;
      s.zmax[m] = zmx;
      s.sorted[m] = sorted ? 1 : 0;
    }
  }
  // windows of modules 0..3 stay -1 (Kernel.cl:104 gates the body on f >= 4)
  const int hbeg = S >= 5 ? s.start[4] : H;
  for (int i = tid; i < hbeg; i += nt) {
    ev.h1f[i] = -1; ev.h1l[i] = -1; ev.h2f[i] = -1; ev.h2l[i] = -1;
  }
  __syncthreads();

  // candidate windows for every hit of modules >= 4
  for (int h = hbeg + tid; h < H; h += nt) {
    int lo = 4, hi = S - 1;   // last module whose start is <= h
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s.start[mid] <= h) lo = mid; else hi = mid - 1;
    }
    compute_windows(ev, s, h, lo);
  }
  __syncthreads();

  // module loop, Kernel.cl:671-767
  uint32_t* cur = ev.ring0;
  uint32_t* nxt = ev.ring1;
  for (int f = S - 1; f >= 4; --f) {
    const uint32_t ncur = s.ncur;
    for (uint32_t i = tid; i < ncur; i += nt) forward_entry(ev, s, cur[i], f - 4, nxt);
    __syncthreads();
    if (tid == 0 && ncur + s.nnext > VELO_TTF_MODULO) s.status |= VELO_EVENT_RING_OVERFLOW;
    if (s.num[f] > 0) seed_module(ev, s, f, nxt);
    __syncthreads();
    if (tid == 0) {
      if (s.nnext > VELO_TTF_MODULO) s.status |= VELO_EVENT_RING_OVERFLOW;
      s.ncur = min(s.nnext, ev.ring_cap);
      s.nnext = 0;
    }
    uint32_t* tmp = cur; cur = nxt; nxt = tmp;
    __syncthreads();
  }

  // leftover tracklets become weak (Kernel.cl:771-792)
  {
    const uint32_t ncur = s.ncur;
    for (uint32_t i = tid; i < ncur; i += nt) {
      const uint32_t v = cur[i];
      if (v & kTrackletFlag) {
        const uint32_t wi = atomicAdd(&s.nweak, 1u);
        if (wi < ev.cap) ev.weak[wi] = v & kNumberMask;
      }
    }
  }
  __syncthreads();
  // weak tracks made of three unused hits (Kernel.cl:796-815)
  {
    const uint32_t nweak = min(s.nweak, ev.cap);
    for (uint32_t i = tid; i < nweak; i += nt) {
      const uint32_t w = ev.weak[i];
      const uint32_t a = ev.tracklets[3 * w], b = ev.tracklets[3 * w + 1], c = ev.tracklets[3 * w + 2];
      if (!ev.used[a] && !ev.used[b] && !ev.used[c]) {
        const uint32_t tn = atomicAdd(&s.ntracks, 1u);
        if (tn >= ev.cap) continue;
        uint32_t* wr = reinterpret_cast<uint32_t*>(&ev.tracks[tn]);
        wr[0] = 3; wr[1] = a; wr[2] = b; wr[3] = c;
#pragma unroll
        for (int k = 4; k < 25; ++k) wr[k] = 0;
      }
    }
  }
  __syncthreads();

  // compacted output
  if (tid == 0) {
    const uint32_t cnt = min(s.ntracks, ev.cap);
    if (s.ntracks > VELO_MAX_TRACKS) s.status |= VELO_EVENT_MAX_TRACKS;
    const unsigned long long first = atomicAdd(p.out_cursor, (unsigned long long)cnt);
    s.out_first = first;
    p.out_counts[e] = cnt;
    p.out_first[e] = first;
    p.out_status[e] = s.status;
  }
  __syncthreads();
  {
    const uint32_t words = min(s.ntracks, ev.cap) * 25u;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(ev.tracks);
    uint32_t* dst = reinterpret_cast<uint32_t*>(p.out_tracks + s.out_first);
    for (uint32_t w = tid; w < words; w += nt) dst[w] = src[w];
  }
}

__global__ void __launch_bounds__(512) search_kernel(const SearchParams p) {
  extern __shared__ __align__(16) uint8_t dyn_smem[];
  __shared__ Shared s;
  if (!p.persistent) {
    if ((int)blockIdx.x < p.n_events) process_event(p, blockIdx.x, s, dyn_smem);
    return;
  }
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s.next_event = atomicAdd(p.work_counter, 1);
    __syncthreads();
    const int k = s.next_event;
    if (k >= p.n_events) break;
    process_event(p, p.order[k], s, dyn_smem);
  }
}

int launch_search(const SearchParams& p, int grid, int block, uint32_t smem_bytes, void* stream) {
  search_kernel<<<grid, block, smem_bytes, (cudaStream_t)stream>>>(p);
  return (int)cudaGetLastError();
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
  e = cudaFuncSetAttribute(search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  if (e == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = smem_bytes;
  return (int)e;
}

int search_occupancy(int block, uint32_t smem_bytes, int* ctas_per_sm) {
  return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, search_kernel, block,
                                                            smem_bytes);
}

}  // namespace velo
