/*
 * velo_oracle.h -- CPU restatement of the reference search-by-triplet
 * algorithm (Kernel.cl:15-816 of dcampora/cl_forward), used ONLY as test
 * infrastructure: the parity checker for the CUDA path, and the timed CPU
 * baseline.  Nothing in the product links or calls it.
 *
 * Parity of this restatement is pinned against the reference kernel itself,
 * compiled unmodified as C under a work-group emulator (oracle/ref_emu.c,
 * built from the reference sources by oracle/build_ref.py), on seeded
 * synthetic events and on the reference's own mcdata events; the golden
 * fixtures under tests/golden/ were produced that way.
 */
#ifndef VELO_ORACLE_H
#define VELO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VO_MAX_TRACK_SIZE 24   /* KernelDefinitions.h:16 */
#define VO_MAX_TRACKS 3000     /* KernelDefinitions.h:15 */
#define VO_TTF_MODULO 2000     /* KernelDefinitions.h:23 */

/* Per-event status bits; identical values to VELO_EVENT_* in velo_search.h. */
#define VO_EVENT_RING_OVERFLOW 0x1u   /* reference ring of TTF_MODULO entries would overwrite */
#define VO_EVENT_TRACK_OVERFLOW 0x2u  /* a track needed more than 24 hits */
#define VO_EVENT_MAX_TRACKS 0x4u      /* more than MAX_TRACKS tracks */
#define VO_EVENT_INVALID 0x8u         /* event blob failed validation */
#define VO_EVENT_DEGENERATE 0x10u     /* a fit produced inf/NaN (hits of two modules at equal z) */

typedef struct vo_track {           /* KernelDefinitions.h:59-62 */
  uint32_t hitsNum;
  uint32_t hits[VO_MAX_TRACK_SIZE];
} vo_track;

typedef struct vo_counters {
  uint64_t window_evals;     /* candidate-window predicate evaluations (fillCandidates) */
  uint64_t forward_fits;     /* fitHitToTrack evaluations (trackForwarding) */
  uint64_t seed_fits;        /* triplet extrapolations inside windows (trackCreation) */
  uint64_t seed_scatters;    /* triplets that passed the tolerance cuts */
} vo_counters;

/* Validate one event blob; returns 0 if valid. */
int vo_validate_event(const uint8_t* blob, uint64_t size);

/* Reference per-module x-sort (Tools.cpp:46-66, 117-157), in place. */
int vo_sort_by_x(uint8_t* blob, uint64_t size);

/* Search one x-sorted event.  `out` holds room for `cap` tracks (cap >= H is
 * always enough).  Track order is this implementation's; compare as sets. */
int vo_search_event(const uint8_t* blob, uint64_t size, int y_lanes, vo_track* out,
                    uint32_t cap, uint32_t* count, uint32_t* status, vo_counters* counters);

/* Search n events over `threads` host threads (0 = all cores).  Event e's
 * tracks go to out + out_first[e] with room for out_cap[e] tracks. */
int vo_search_batch(const uint8_t* buf, const uint64_t* offsets, const uint64_t* sizes, int n,
                    int y_lanes, int threads, vo_track* out, const uint64_t* out_first,
                    const uint32_t* out_cap, uint32_t* counts, uint32_t* status,
                    vo_counters* counters);

#ifdef __cplusplus
}
#endif
#endif
