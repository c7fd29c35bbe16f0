/*
 * velo_oracle.c -- sequential CPU restatement of the reference
 * search-by-triplet (dcampora/cl_forward Kernel.cl), TEST INFRASTRUCTURE
 * ONLY: the parity checker and the timed CPU baseline.  The product never
 * links it.
 *
 * Build with -ffp-contract=off: every cut is an FP32 comparison and the
 * expression shapes below follow the reference term by term, so fused
 * multiply-adds would change decisions.
 *
 * One event at a time, in the order the reference's barriers impose:
 *   1. candidate windows for every module            (Kernel.cl:50-178)
 *   2. for f = S-1 .. 4: forwarding onto f-4           (Kernel.cl:199-368)
 *                        then seeding h0/h1/h2 on f/f-2/f-4 (Kernel.cl:392-568,720-764)
 *   3. leftover tracklets -> weak; weak filter       (Kernel.cl:769-815)
 * Inside a stage the reference's work-items only communicate through
 * append-only lists and hit_used, which forwarding writes and never reads and
 * seeding reads and never writes, so a sequential sweep gives the same track
 * contents as any legal schedule; only track order differs.
 */
#define _GNU_SOURCE
#include "velo_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define PARAM_TOLERANCE 0.6f              /* KernelDefinitions.h:30 */
#define PARAM_TOLERANCE_CANDIDATES 0.6f   /* KernelDefinitions.h:31 */
#define PARAM_MAXXSLOPE_CANDIDATES 0.7f   /* KernelDefinitions.h:28 */
#define PARAM_MAXYSLOPE 0.7f              /* KernelDefinitions.h:27 */
#define MAX_SCATTER 0.000016f             /* KernelDefinitions.h:33 */
#define MAX_SKIPPED_MODULES 3             /* KernelDefinitions.h:22 */

typedef struct {
  int32_t S, H;
  const int32_t* sz;
  const int32_t* start;
  const int32_t* num;
  const uint32_t* id;
  const float* x;
  const float* y;
  const float* z;
} ev_view;

static int read_i32(const uint8_t* p) { int32_t v; memcpy(&v, p, 4); return v; }

int vo_validate_event(const uint8_t* blob, uint64_t size) {
  if (!blob || size < 8) return -1;
  int32_t S = read_i32(blob), H = read_i32(blob + 4);
  if (S < 0 || H < 0 || S > 255) return -1;
  if (size < 8ull + 12ull * (uint64_t)S + 16ull * (uint64_t)H) return -1;
  if (((uintptr_t)blob & 3u) != 0) return -1;
  const int32_t* start = (const int32_t*)(blob + 8 + 4 * S);
  const int32_t* num = start + S;
  int64_t acc = 0;
  for (int m = 0; m < S; ++m) {
    if (num[m] < 0 || start[m] != acc) return -1;  /* contiguous modules, Tools.cpp:53-64 */
    acc += num[m];
  }
  if (acc != H) return -1;
  const float* x = (const float*)(blob + 8 + 12 * S + 4 * H);
  for (int64_t i = 0; i < 3 * (int64_t)H; ++i)
    if (!isfinite(x[i])) return -1;
  return 0;
}

static void view_of(const uint8_t* blob, ev_view* v) {
  v->S = read_i32(blob);
  v->H = read_i32(blob + 4);
  v->sz = (const int32_t*)(blob + 8);
  v->start = v->sz + v->S;
  v->num = v->start + v->S;
  v->id = (const uint32_t*)(v->num + v->S);
  v->x = (const float*)(v->id + v->H);
  v->y = v->x + v->H;
  v->z = v->y + v->H;
}

/* ---------------------------------------------------------------- sort -- */
/* First-element-pivot partition of Tools.cpp:125-157; the permutation of
 * equal keys must match the reference's, because output hit indices refer to
 * the sorted order. */
static void swap4(float* a, float* b, float* c, uint32_t* d, int i, int j) {
  float t = a[i]; a[i] = a[j]; a[j] = t;
  t = b[i]; b[i] = b[j]; b[j] = t;
  t = c[i]; c[i] = c[j]; c[j] = t;
  uint32_t u = d[i]; d[i] = d[j]; d[j] = u;
}

static int partition4(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
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

static void qsort4(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
  /* explicit stack; subranges are disjoint so processing order is free */
  int stack_lo[128], stack_hi[128], sp = 0;
  int* big_lo = NULL; int* big_hi = NULL; int cap = 128;
  int* sl = stack_lo; int* sh = stack_hi;
  sl[sp] = lo; sh[sp] = hi; sp++;
  while (sp) {
    sp--;
    int s = sl[sp], e = sh[sp];
    if (s >= e) continue;
    int p = partition4(a, b, c, d, s, e);
    if (sp + 2 > cap) {
      int ncap = cap * 2;
      int* nl = (int*)malloc(sizeof(int) * ncap);
      int* nh = (int*)malloc(sizeof(int) * ncap);
      memcpy(nl, sl, sizeof(int) * sp); memcpy(nh, sh, sizeof(int) * sp);
      free(big_lo); free(big_hi);
      big_lo = sl = nl; big_hi = sh = nh; cap = ncap;
    }
    sl[sp] = s; sh[sp] = p - 1; sp++;
    sl[sp] = p + 1; sh[sp] = e; sp++;
  }
  free(big_lo); free(big_hi);
}

int vo_sort_by_x(uint8_t* blob, uint64_t size) {
  if (vo_validate_event(blob, size)) return -1;
  int32_t S = read_i32(blob), H = read_i32(blob + 4);
  int32_t* num = (int32_t*)(blob + 8 + 8 * S);
  uint32_t* id = (uint32_t*)(blob + 8 + 12 * S);
  float* x = (float*)(id + H);
  float* y = x + H;
  float* z = y + H;
  int acc = 0;
  for (int m = 0; m < S; ++m) {
    qsort4(x, y, z, id, acc, acc + num[m] - 1);
    acc += num[m];
  }
  return 0;
}

/* ------------------------------------------------------------- search -- */
typedef struct {
  int32_t cap_hits;
  int32_t *h1f, *h1l, *h2f, *h2l;
  uint8_t* used;
  uint32_t *ring_a, *ring_b;
  uint32_t* tracklets;   /* 3 per tracklet */
  uint32_t* weak;
  vo_track* tracks;
} workspace;

static void ws_free(workspace* w) {
  free(w->h1f); free(w->h1l); free(w->h2f); free(w->h2l); free(w->used);
  free(w->ring_a); free(w->ring_b); free(w->tracklets); free(w->weak); free(w->tracks);
  memset(w, 0, sizeof(*w));
}

static int ws_reserve(workspace* w, int32_t H) {
  if (H <= w->cap_hits && w->h1f) return 0;
  ws_free(w);
  int32_t n = H > 16 ? H : 16;
  w->h1f = (int32_t*)malloc(4ull * n); w->h1l = (int32_t*)malloc(4ull * n);
  w->h2f = (int32_t*)malloc(4ull * n); w->h2l = (int32_t*)malloc(4ull * n);
  w->used = (uint8_t*)malloc(n);
  w->ring_a = (uint32_t*)malloc(4ull * (n + 1)); w->ring_b = (uint32_t*)malloc(4ull * (n + 1));
  w->tracklets = (uint32_t*)malloc(12ull * n);
  w->weak = (uint32_t*)malloc(4ull * n);
  w->tracks = (vo_track*)malloc(sizeof(vo_track) * (size_t)n);
  if (!w->h1f || !w->h1l || !w->h2f || !w->h2l || !w->used || !w->ring_a || !w->ring_b ||
      !w->tracklets || !w->weak || !w->tracks) { ws_free(w); return -1; }
  w->cap_hits = n;
  return 0;
}

/* Candidate windows, Kernel.cl:50-178: for h0 on module f (f >= 4), the
 * [first, last) index range of module f-2 from the first hit with
 * |x1-x0| < 0.7|z1-z0| to the first later hit that fails it; and, for
 * f <= S-3, the h2 window on f-2 for h0 taken as an h1 of a seed on f+2. */
static void fill_candidates(const ev_view* v, workspace* w, vo_counters* c) {
  for (int i = 0; i < v->H; ++i) { w->h1f[i] = w->h1l[i] = w->h2f[i] = w->h2l[i] = -1; }
  for (int f = v->S - 1; f >= 4; --f) {
    const int s2 = f - 2;
    const int proc_h2 = f <= v->S - 3;
    const int z_s0 = proc_h2 ? v->sz[f + 2] : 0;
    const int z_s2 = proc_h2 ? v->sz[s2] : 0;
    const int st2 = v->start[s2], n2 = v->num[s2];
    for (int h0 = v->start[f]; h0 < v->start[f] + v->num[f]; ++h0) {
      const float x0 = v->x[h0], z0 = v->z[h0];
      int ff1 = 0, lf1 = 0, ff2 = 0, lf2 = 0;
      float xmin_h2 = 0.f, xmax_h2 = 0.f;
      if (proc_h2) {
        const float h_dist = fabsf(z0 - (float)z_s0);
        const float dxmax = PARAM_MAXXSLOPE_CANDIDATES * h_dist;
        const float x0_min = x0 - dxmax;
        const float x0_max = x0 + dxmax;
        const float z2_tz = ((float)z_s2 - (float)z_s0) / (z0 - (float)z_s0);
        float xv = x0_max + (x0 - x0_max) * z2_tz;
        xmin_h2 = xv - PARAM_TOLERANCE_CANDIDATES;
        xv = x0_min + (x0 - x0_min) * z2_tz;
        xmax_h2 = xv + PARAM_TOLERANCE_CANDIDATES;
      }
      for (int e = 0; e < n2; ++e) {
        const int h1 = st2 + e;
        const float x1 = v->x[h1], z1 = v->z[h1];
        if (c) c->window_evals++;
        if (!lf1) {
          const float h_dist = fabsf(z1 - z0);
          const float dxmax = PARAM_MAXXSLOPE_CANDIDATES * h_dist;
          const int tol = fabsf(x1 - x0) < dxmax;
          if (!ff1 && tol) { w->h1f[h0] = h1; ff1 = 1; }
          else if (ff1 && !tol) { w->h1l[h0] = h1; lf1 = 1; }
        }
        if (proc_h2 && !lf2) {
          if (!ff2 && x1 > xmin_h2) { w->h2f[h0] = h1; ff2 = 1; }
          else if (ff2 && x1 > xmax_h2) { w->h2l[h0] = h1; lf2 = 1; }
        }
        if (lf1 && (!proc_h2 || lf2)) break;
      }
      if (ff1 && !lf1) w->h1l[h0] = st2 + n2;
      if (proc_h2 && ff2 && !lf2) w->h2l[h0] = st2 + n2;
    }
  }
}

/* fitHitToTrack, Kernel.cl:15-35.  Returns the scatter, FLT_MAX when a cut
 * fails, and NAN where the reference's `condition*scatter + ...` would be
 * NaN (scatter not finite with a failed cut). */
static inline float fit_hit(float tx, float ty, float h0x, float h0y, float h0z, float h1z,
                            float h2x, float h2y, float h2z) {
  const float dz = h2z - h0z;
  const float x_prediction = h0x + tx * dz;
  const float dx = fabsf(x_prediction - h2x);
  const int tolx = dx < PARAM_TOLERANCE;
  const float y_prediction = h0y + ty * dz;
  const float dy = fabsf(y_prediction - h2y);
  const int toly = dy < PARAM_TOLERANCE;
  const float scatterNum = (dx * dx) + (dy * dy);
  const float scatterDenom = 1.f / (h2z - h1z);
  const float scatter = scatterNum * scatterDenom * scatterDenom;
  const int cond = tolx && toly && (scatter < MAX_SCATTER);
  if (cond) return scatter;
  return isfinite(scatter) ? FLT_MAX : NAN;
}

static int search_one(const ev_view* v, int Y, workspace* w, vo_track* out, uint32_t cap,
                      uint32_t* count_out, uint32_t* status_out, vo_counters* c) {
  uint32_t status = 0;
  fill_candidates(v, w, c);
  memset(w->used, 0, (size_t)v->H);
  uint32_t* cur = w->ring_a;
  uint32_t* nxt = w->ring_b;
  uint32_t ncur = 0, nxt_n = 0, ntracklets = 0, nweak = 0, ntracks = 0;

  for (int f = v->S - 1; f >= 4; --f) {
    const int m4 = f - 4;
    const int st4 = v->start[m4], n4 = v->num[m4];
    nxt_n = 0;
    /* ---- forwarding, Kernel.cl:199-368 ---- */
    for (uint32_t i = 0; i < ncur; ++i) {
      const uint32_t full = cur[i];
      const int flag = (full & 0x80000000u) != 0;
      const uint32_t skipped = (full & 0x70000000u) >> 28;
      uint32_t trackno = full & 0x0FFFFFFFu;
      vo_track t;
      if (flag) {
        memset(&t, 0, sizeof t);
        t.hitsNum = 3;
        memcpy(t.hits, &w->tracklets[3 * trackno], 12);
      } else {
        t = w->tracks[trackno];
      }
      const uint32_t n = t.hitsNum;
      const uint32_t h0 = t.hits[n - 2], h1 = t.hits[n - 1];
      const float h0x = v->x[h0], h0y = v->y[h0], h0z = v->z[h0];
      const float h1x = v->x[h1], h1y = v->y[h1], h1z = v->z[h1];
      const float td = 1.0f / (h1z - h0z);
      const float txn = (h1x - h0x);
      const float tyn = (h1y - h0y);
      const float tx = txn * td;
      const float ty = tyn * td;
      float best = FLT_MAX;
      int best_h2 = -1;
      for (int k = 0; k < n4; ++k) {
        const int h2 = st4 + k;
        const float fit = fit_hit(tx, ty, h0x, h0y, h0z, h1z, v->x[h2], v->y[h2], v->z[h2]);
        if (c) c->forward_fits++;
        if (isnan(fit)) { status |= VO_EVENT_DEGENERATE; continue; }
        if (fit < best) { best = fit; best_h2 = h2; }
      }
      if (best != FLT_MAX) {
        if (n >= VO_MAX_TRACK_SIZE) {          /* reference writes past hits[24] */
          status |= VO_EVENT_TRACK_OVERFLOW;
          continue;
        }
        w->used[best_h2] = 1;
        t.hits[t.hitsNum++] = (uint32_t)best_h2;
        if (t.hitsNum <= 4) {
          w->used[t.hits[0]] = 1;
          w->used[t.hits[1]] = 1;
          w->used[t.hits[2]] = 1;
          trackno = ntracks++;
        }
        w->tracks[trackno] = t;
        nxt[nxt_n++] = trackno;
      } else if (skipped <= MAX_SKIPPED_MODULES) {
        nxt[nxt_n++] = ((skipped + 1) << 28) | (full & 0x8FFFFFFFu);
      } else if (t.hitsNum == 3) {
        w->weak[nweak++] = trackno;
      }
    }
    const uint32_t n_fwd = nxt_n;
    if (ncur + n_fwd > VO_TTF_MODULO) status |= VO_EVENT_RING_OVERFLOW;

    /* ---- seeding, Kernel.cl:392-568 and the gather at :720-764 ---- */
    const int s1 = f - 2;
    const int st0 = v->start[f], n0 = v->num[f];
    for (int h0 = st0; h0 < st0 + n0; ++h0) {
      if (w->used[h0]) continue;
      const int first_h1 = w->h1f[h0];
      const int n1 = w->h1l[h0] - first_h1;   /* 0 when both are -1 */
      if (n1 <= 0) continue;
      const float h0x = v->x[h0], h0y = v->y[h0], h0z = v->z[h0];
      const float s1_z = v->z[v->start[s1]];
      const float dymax = PARAM_MAXYSLOPE * fabsf(s1_z - h0z);
      float best = FLT_MAX;
      uint32_t bh1 = 0, bh2 = 0;
      for (int ly = 0; ly < Y; ++ly) {
        /* lane ly walks h1 elements ly, ly+Y, ...; `inside_bounds` is
         * cumulative (Kernel.cl:437,457), so the first h1 without an h2
         * window ends the lane */
        float lbest = FLT_MAX;
        uint32_t lh1 = 0, lh2 = 0;
        for (int e = ly; e < n1; e += Y) {
          const int h1 = first_h1 + e;
          const int fh2 = w->h2f[h1], lh2w = w->h2l[h1];
          if (fh2 == -1) break;
          if (w->used[h1]) continue;
          const float h1x = v->x[h1], h1y = v->y[h1], h1z = v->z[h1];
          const float dz_inverted = 1.f / (h1z - h0z);
          if (!(fabsf(h1y - h0y) < dymax)) continue;   /* h2-independent term of :509 */
          for (int h2 = fh2; h2 < lh2w; ++h2) {
            const float h2x = v->x[h2], h2y = v->y[h2], h2z = v->z[h2];
            const float z2_tz = (h2z - h0z) * dz_inverted;
            const float xp = h0x + (h1x - h0x) * z2_tz;
            const float yp = h0y + (h1y - h0y) * z2_tz;
            const float dx = xp - h2x;
            const float dy = yp - h2y;
            if (c) c->seed_fits++;
            if (fabsf(dx) < PARAM_TOLERANCE && fabsf(dy) < PARAM_TOLERANCE) {
              const float scatterNum = (dx * dx) + (dy * dy);
              const float scatterDenom = 1.f / (h2z - h1z);
              const float scatter = scatterNum * scatterDenom * scatterDenom;
              if (c) c->seed_scatters++;
              if (!(scatter < MAX_SCATTER)) {
                if (!isfinite(scatter)) status |= VO_EVENT_DEGENERATE;
                continue;
              }
              if (scatter < lbest) { lbest = scatter; lh1 = (uint32_t)h1; lh2 = (uint32_t)h2; }
            }
          }
        }
        if (lbest < best) { best = lbest; bh1 = lh1; bh2 = lh2; }   /* Kernel.cl:538-545 */
      }
      if (best != FLT_MAX) {
        const uint32_t tp = ntracklets++;
        w->tracklets[3 * tp + 0] = (uint32_t)h0;
        w->tracklets[3 * tp + 1] = bh1;
        w->tracklets[3 * tp + 2] = bh2;
        nxt[nxt_n++] = 0x80000000u | tp;
      }
    }
    if (nxt_n > VO_TTF_MODULO) status |= VO_EVENT_RING_OVERFLOW;   /* n_fwd + n_seed */
    uint32_t* tmp = cur; cur = nxt; nxt = tmp;
    ncur = nxt_n;
  }

  /* ---- leftover tracklets become weak, Kernel.cl:771-792 ---- */
  for (uint32_t i = 0; i < ncur; ++i)
    if (cur[i] & 0x80000000u) w->weak[nweak++] = cur[i] & 0x0FFFFFFFu;
  /* ---- weak tracks with three unused hits, Kernel.cl:796-815 ---- */
  for (uint32_t i = 0; i < nweak; ++i) {
    const uint32_t* th = &w->tracklets[3 * w->weak[i]];
    if (!w->used[th[0]] && !w->used[th[1]] && !w->used[th[2]]) {
      vo_track t;
      memset(&t, 0, sizeof t);
      t.hitsNum = 3;
      memcpy(t.hits, th, 12);
      w->tracks[ntracks++] = t;
    }
  }
  if (ntracks > VO_MAX_TRACKS) status |= VO_EVENT_MAX_TRACKS;
  uint32_t ncopy = ntracks < cap ? ntracks : cap;
  if (out && ncopy) memcpy(out, w->tracks, sizeof(vo_track) * ncopy);
  *count_out = ntracks;
  *status_out = status;
  return ntracks <= cap ? 0 : -2;
}

int vo_search_event(const uint8_t* blob, uint64_t size, int y_lanes, vo_track* out,
                    uint32_t cap, uint32_t* count, uint32_t* status, vo_counters* counters) {
  *count = 0;
  *status = 0;
  if (y_lanes < 1 || y_lanes > 16) return -1;
  if (vo_validate_event(blob, size)) { *status = VO_EVENT_INVALID; return -1; }
  ev_view v;
  view_of(blob, &v);
  workspace w;
  memset(&w, 0, sizeof w);
  if (ws_reserve(&w, v.H)) return -3;
  int rc = search_one(&v, y_lanes, &w, out, cap, count, status, counters);
  ws_free(&w);
  return rc;
}

typedef struct {
  const uint8_t* buf;
  const uint64_t *offsets, *sizes, *out_first;
  const uint32_t* out_cap;
  int n, Y;
  vo_track* out;
  uint32_t *counts, *status;
  vo_counters* counters;
  atomic_int next;
  atomic_int rc;
  pthread_mutex_t lock;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* j = (batch_job*)arg;
  workspace w;
  memset(&w, 0, sizeof w);
  vo_counters local;
  memset(&local, 0, sizeof local);
  for (;;) {
    int e = atomic_fetch_add(&j->next, 1);
    if (e >= j->n) break;
    const uint8_t* blob = j->buf + j->offsets[e];
    j->counts[e] = 0;
    if (vo_validate_event(blob, j->sizes[e])) {
      j->status[e] = VO_EVENT_INVALID;
      atomic_store(&j->rc, -1);
      continue;
    }
    ev_view v;
    view_of(blob, &v);
    if (ws_reserve(&w, v.H)) { atomic_store(&j->rc, -3); continue; }
    int rc = search_one(&v, j->Y, &w, j->out + j->out_first[e], j->out_cap[e], &j->counts[e],
                        &j->status[e], j->counters ? &local : NULL);
    if (rc) atomic_store(&j->rc, rc);
  }
  ws_free(&w);
  if (j->counters) {
    pthread_mutex_lock(&j->lock);
    j->counters->window_evals += local.window_evals;
    j->counters->forward_fits += local.forward_fits;
    j->counters->seed_fits += local.seed_fits;
    j->counters->seed_scatters += local.seed_scatters;
    pthread_mutex_unlock(&j->lock);
  }
  return NULL;
}

int vo_search_batch(const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes, int n,
                    int y_lanes, int threads, vo_track* out, const uint64_t* out_first,
                    const uint32_t* out_cap, uint32_t* counts, uint32_t* status,
                    vo_counters* counters) {
  if (y_lanes < 1 || y_lanes > 16 || n < 0) return -1;
  batch_job j;
  j.buf = buf; j.offsets = offsets; j.sizes = sizes; j.out_first = out_first; j.out_cap = out_cap;
  j.n = n; j.Y = y_lanes; j.out = out; j.counts = counts; j.status = status; j.counters = counters;
  atomic_init(&j.next, 0);
  atomic_init(&j.rc, 0);
  pthread_mutex_init(&j.lock, NULL);
  if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  int started = 0;
  for (int i = 1; i < threads; ++i)
    if (pthread_create(&tid[started], NULL, batch_worker, &j) == 0) started++;
  batch_worker(&j);
  for (int i = 0; i < started; ++i) pthread_join(tid[i], NULL);
  pthread_mutex_destroy(&j.lock);
  return atomic_load(&j.rc);
}
