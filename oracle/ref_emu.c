/*
 * ref_emu.c -- runs the reference's own clSearchByTriplets (Kernel.cl:597-816,
 * compiled as C next to this file by oracle/build_ref.py) on the host CPU.
 * TEST INFRASTRUCTURE ONLY: it pins the oracle restatement (velo_oracle.c)
 * and can serve as a "reference" CPU baseline where the reference sources are
 * present.  Nothing in the product links it.
 *
 * Buffers mirror KernelInvoker.cpp:77-108 and their initial values
 * KernelInvoker.cpp:160-168 (hit_used 0, atomics 0, candidate windows -1,
 * tracks / tracklets / ring 0).  Each work-group (one event) runs as 64*Y
 * fibers on one OS thread; barrier() returns to a scheduler that resumes the
 * fibers in a (optionally seeded-random) order each phase, so repeated runs
 * with different seeds explore different legal schedules.  Work-groups are
 * spread over OS threads through an atomic counter.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <ucontext.h>
#include <unistd.h>

#define REF_NUMTHREADS_X 64
#define REF_MAX_Y 16
#define REF_MAX_TRACKS 3000
#define REF_TTF_MODULO 2000
#define REF_NUM_ATOMICS 5
#define REF_TRACK_BYTES 100
#define STACK_BYTES (64 * 1024)

/* the reference kernel, compiled from Kernel.cl in the same library */
void clSearchByTriplets(void* dev_tracks, const char* dev_input, int* dev_tracks_to_follow,
                        _Bool* dev_hit_used, int* dev_atomicsStorage, void* dev_tracklets,
                        int* dev_weak_tracks, int* dev_event_offsets, int* dev_hit_offsets,
                        float* dev_best_fits, int* dev_hit_candidates, int* dev_hit_h2_candidates);

typedef struct {
  void* tracks;
  const char* input;
  int* ttf;
  _Bool* hit_used;
  int* atomics;
  void* tracklets;
  int* weak;
  int* event_offsets;
  int* hit_offsets;
  float* best_fits;
  int* cand;
  int* cand_h2;
} kargs;

enum { F_READY = 0, F_BARRIER = 1, F_DONE = 2 };

typedef struct {
  ucontext_t ctx;
  int lid0, lid1, state;
} fiber;

typedef struct {
  fiber* fibers;
  char* stacks;
  size_t stack_span;
  int nfib;
  int cur;
  int Y;
  int group, ngroups;
  ucontext_t sched;
  const kargs* args;
} wg_state;

static _Thread_local wg_state* T;

size_t get_local_id(unsigned int d) {
  return d == 0 ? (size_t)T->fibers[T->cur].lid0 : d == 1 ? (size_t)T->fibers[T->cur].lid1 : 0;
}
size_t get_local_size(unsigned int d) { return d == 0 ? REF_NUMTHREADS_X : d == 1 ? (size_t)T->Y : 1; }
size_t get_group_id(unsigned int d) { return d == 0 ? (size_t)T->group : 0; }
size_t get_num_groups(unsigned int d) { return d == 0 ? (size_t)T->ngroups : 1; }

void barrier(int flags) {
  (void)flags;
  fiber* f = &T->fibers[T->cur];
  f->state = F_BARRIER;
  swapcontext(&f->ctx, &T->sched);
}

int ref_atomic_add(volatile int* p, int v) { int o = *p; *p = o + v; return o; }
int ref_atomic_max(volatile int* p, int v) { int o = *p; if (v > o) *p = v; return o; }

static void fiber_main(void) {
  const kargs* a = T->args;
  clSearchByTriplets(a->tracks, a->input, a->ttf, a->hit_used, a->atomics, a->tracklets, a->weak,
                     a->event_offsets, a->hit_offsets, a->best_fits, a->cand, a->cand_h2);
  T->fibers[T->cur].state = F_DONE;
}

static uint64_t lcg(uint64_t* s) {
  *s = *s * 6364136223846793005ull + 1442695040888963407ull;
  return *s >> 33;
}

static int wg_init(wg_state* w, int Y) {
  memset(w, 0, sizeof *w);
  w->Y = Y;
  w->nfib = REF_NUMTHREADS_X * Y;
  w->fibers = (fiber*)calloc((size_t)w->nfib, sizeof(fiber));
  long page = sysconf(_SC_PAGESIZE);
  w->stack_span = STACK_BYTES + (size_t)page;   /* one guard page below each stack */
  w->stacks = (char*)mmap(NULL, w->stack_span * (size_t)w->nfib, PROT_READ | PROT_WRITE,
                          MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (!w->fibers || w->stacks == MAP_FAILED) return -1;
  for (int i = 0; i < w->nfib; ++i) mprotect(w->stacks + w->stack_span * i, (size_t)page, PROT_NONE);
  return 0;
}

static void wg_free(wg_state* w) {
  free(w->fibers);
  if (w->stacks && w->stacks != MAP_FAILED) munmap(w->stacks, w->stack_span * (size_t)w->nfib);
}

/* Run one work-group; returns 0, or -1 if the fibers disagreed on barriers. */
static int run_group(wg_state* w, const kargs* a, int group, int ngroups, uint64_t sched_seed) {
  long page = sysconf(_SC_PAGESIZE);
  w->args = a;
  w->group = group;
  w->ngroups = ngroups;
  for (int i = 0; i < w->nfib; ++i) {
    fiber* f = &w->fibers[i];
    f->lid0 = i % REF_NUMTHREADS_X;
    f->lid1 = i / REF_NUMTHREADS_X;
    f->state = F_READY;
    getcontext(&f->ctx);
    f->ctx.uc_stack.ss_sp = w->stacks + w->stack_span * i + page;
    f->ctx.uc_stack.ss_size = STACK_BYTES;
    f->ctx.uc_link = &w->sched;
    makecontext(&f->ctx, fiber_main, 0);
  }
  int* order = (int*)malloc(sizeof(int) * (size_t)w->nfib);
  for (int i = 0; i < w->nfib; ++i) order[i] = i;
  uint64_t rs = sched_seed * 0x9E3779B97F4A7C15ull + (uint64_t)group;
  int alive = w->nfib, bad = 0;
  T = w;
  while (alive > 0) {
    if (sched_seed) {
      for (int i = w->nfib - 1; i > 0; --i) {
        int j = (int)(lcg(&rs) % (uint64_t)(i + 1));
        int t = order[i]; order[i] = order[j]; order[j] = t;
      }
    }
    int at_barrier = 0, finished = 0;
    for (int k = 0; k < w->nfib; ++k) {
      int i = order[k];
      fiber* f = &w->fibers[i];
      if (f->state == F_DONE) continue;
      f->state = F_READY;
      w->cur = i;
      swapcontext(&w->sched, &f->ctx);
      if (f->state == F_DONE) { alive--; finished++; }
      else at_barrier++;
    }
    if (at_barrier && finished) bad = 1;   /* divergent barrier */
  }
  T = NULL;
  free(order);
  return bad ? -1 : 0;
}

typedef struct {
  kargs a;
  int n, Y;
  uint64_t seed;
  atomic_int next;
  atomic_int rc;
} job;

static void* worker(void* p) {
  job* j = (job*)p;
  wg_state w;
  if (wg_init(&w, j->Y)) { atomic_store(&j->rc, -3); wg_free(&w); return NULL; }
  for (;;) {
    int g = atomic_fetch_add(&j->next, 1);
    if (g >= j->n) break;
    if (run_group(&w, &j->a, g, j->n, j->seed)) atomic_store(&j->rc, -2);
  }
  wg_free(&w);
  return NULL;
}

/*
 * Run the reference kernel over n events packed contiguously in `input`
 * (event e at byte offset offsets[e], as KernelInvoker.cpp:113-117 packs
 * them).  Outputs: counts[e] = atomicsStorage[e] and the first counts[e]
 * Track records of event e's MAX_TRACKS slots, copied to
 * tracks_out + 100 * out_first[e] (at most out_cap[e] of them).
 * Returns 0, or negative on allocation failure / divergent barriers.
 */
int ref_search_batch(const uint8_t* input, const uint64_t* offsets, const int32_t* n_hits, int n,
                     int Y, int threads, uint64_t sched_seed, uint8_t* tracks_out,
                     const uint64_t* out_first, const uint32_t* out_cap, uint32_t* counts) {
  if (Y < 1 || Y > REF_MAX_Y || n <= 0) return -1;
  int64_t acc_hits = 0;
  int* ev_off = (int*)malloc(sizeof(int) * (size_t)n);
  int* hit_off = (int*)malloc(sizeof(int) * (size_t)n);
  for (int e = 0; e < n; ++e) {
    ev_off[e] = (int)offsets[e];
    hit_off[e] = (int)acc_hits;
    acc_hits += n_hits[e];
  }
  const size_t slack = 64;   /* the kernel reads atomicsStorage[6E], one past KernelInvoker's 6E */
  job j;
  memset(&j, 0, sizeof j);
  j.a.tracks = calloc((size_t)n * REF_MAX_TRACKS * REF_TRACK_BYTES + slack, 1);
  j.a.input = (const char*)input;
  j.a.ttf = (int*)calloc((size_t)n * REF_TTF_MODULO + slack, sizeof(int));
  j.a.hit_used = (_Bool*)calloc((size_t)acc_hits + slack, 1);
  j.a.atomics = (int*)calloc((size_t)n * (REF_NUM_ATOMICS + 1) + slack, sizeof(int));
  j.a.tracklets = calloc((size_t)acc_hits * REF_TRACK_BYTES + slack, 1);
  j.a.weak = (int*)calloc((size_t)acc_hits + slack, sizeof(int));
  j.a.event_offsets = ev_off;
  j.a.hit_offsets = hit_off;
  j.a.best_fits = (float*)calloc((size_t)n * REF_NUMTHREADS_X * REF_MAX_Y + slack, sizeof(float));
  j.a.cand = (int*)malloc(sizeof(int) * (2 * (size_t)acc_hits + slack));
  j.a.cand_h2 = (int*)malloc(sizeof(int) * (2 * (size_t)acc_hits + slack));
  int rc = 0;
  if (!j.a.tracks || !j.a.ttf || !j.a.hit_used || !j.a.atomics || !j.a.tracklets || !j.a.weak ||
      !j.a.best_fits || !j.a.cand || !j.a.cand_h2) {
    rc = -3;
  } else {
    for (size_t i = 0; i < 2 * (size_t)acc_hits + slack; ++i) { j.a.cand[i] = -1; j.a.cand_h2[i] = -1; }
    j.n = n;
    j.Y = Y;
    j.seed = sched_seed;
    atomic_init(&j.next, 0);
    atomic_init(&j.rc, 0);
    if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    int started = 0;
    for (int i = 1; i < threads; ++i)
      if (pthread_create(&tid[started], NULL, worker, &j) == 0) started++;
    worker(&j);
    for (int i = 0; i < started; ++i) pthread_join(tid[i], NULL);
    rc = atomic_load(&j.rc);
    for (int e = 0; e < n; ++e) {
      int cnt = j.a.atomics[e];
      counts[e] = (uint32_t)cnt;
      uint32_t ncopy = (uint32_t)cnt < out_cap[e] ? (uint32_t)cnt : out_cap[e];
      if (ncopy > REF_MAX_TRACKS) ncopy = REF_MAX_TRACKS;
      memcpy(tracks_out + REF_TRACK_BYTES * out_first[e],
             (const uint8_t*)j.a.tracks + (size_t)e * REF_MAX_TRACKS * REF_TRACK_BYTES,
             (size_t)ncopy * REF_TRACK_BYTES);
    }
  }
  free(j.a.tracks); free(j.a.ttf); free(j.a.hit_used); free(j.a.atomics); free(j.a.tracklets);
  free(j.a.weak); free(j.a.best_fits); free(j.a.cand); free(j.a.cand_h2);
  free(ev_off); free(hit_off);
  return rc;
}
