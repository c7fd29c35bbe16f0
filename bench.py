#!/usr/bin/env python3
"""Throughput of the GB300 search-by-triplet (events/s) on seeded synthetic VELO events.

Default workload: 10,000 events from seeds 1000..10999 of the synthetic VELO
generator (the plain path at scale, Y = 4, no FMA contraction), x-sorted
before timing by the library's host sort (velo_sort_by_x: the reference's
per-module permutation).

The launch configuration is the autotuner's (velo_autotune: threads per
event, shared-memory tile, register build, launch style; cached per workload
shape), unless --no-autotune.  Every configuration gives the same tracks.

Per step the GPU arm searches the whole batch once:
  value  device-resident: one kernel launch over events already in HBM, timed
         with CUDA events on the library's stream; L2 is flushed between steps
         (a 2 x L2 memset) and the input is also larger than L2.
  e2e    the public C ABI (velo_search_packed) from pinned host buffers: the
         kernel reads the events and writes the tracks in place over the host
         link (host_direct; --e2e-copies for H2D / D2H copies instead), plus
         the D2H of counts / offsets / status, all inside the timed region
         (host wall clock).
  cpu_baseline  the oracle restatement of the reference algorithm on all host
         cores over a bounded sample (rank 0 only).
  learned  the learned-pruned search of the same events (committed weights).
  e2e_reference_api  the reference's own C++ entry points on
         std::vector<std::vector<uint8_t>> input: independent_execute (unsorted
         events; the x-sort and the search) and gpuPixelSearchByTriplet
         (x-sorted events), host wall clock per call.
  batched  100,000 uneven events (seeds 2000000..2099999): one persistent
         launch, autotuned (on the first 20,000 events) and replayed from a
         CUDA graph, beside the reference's launch style (one 256-thread CTA
         per event), plus end to end in calls of 16,000 events.
  stress  100,000 events at four times the pile-up (seeds 3000000..3099999):
         plain against learned-pruned seeding, the fallback fraction, and
         both methods' tracking rates on the first 10,000 events.
`--impl reference` times the reference's algorithm on the host CPU instead:
the oracle restatement on all host cores, or with --ref-emulator the
reference kernel itself under the work-group emulator (only where it was
built from the reference sources).

Multi-GPU: weak scaling, every rank searches its own 10,000-event block
(seeds offset by rank) on the GPU of its LOCAL_RANK; no collective touches
the data path, only a barrier and max / sum reductions of the step time and
event counts (gloo).  Under a launcher (torchrun) WORLD_SIZE must equal
--gpus; without one, `--gpus N` (N > 1) starts the N ranks itself through
torch.distributed.run on 127.0.0.1.  `--plan` prints the rank layout (world
size and each rank's seed block) without touching a GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "events/s on 1 GB300: plain vs learned-pruned at <=0.5% eff loss; vs ref on host CPU"

CONFIGS = {
    # name: (first seed, events, generator params attr, launch mode, description)
    "scale": (1000, 10000, "CONFIG_SCALE", 1, "10,000 synthetic VELO events (seeds 1000-10999), plain path"),
    "small": (0, 100, "CONFIG_SMALL", 1, "100 synthetic VELO events (seeds 0-99), plain path"),
    "batched": (2000000, 100000, "CONFIG_BATCHED", 1,
                "100,000 uneven events, PVs ~ Poisson(U(2,30)), persistent CTAs"),
    "stress": (3000000, 100000, "CONFIG_STRESS", 1,
               "100,000 events at PVs ~ Poisson(30), 2% noise, 0.96 hit efficiency, persistent CTAs"),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="scale")
    ap.add_argument("--events", type=int, default=0, help="override the number of events")
    ap.add_argument("--launch", choices=["per-event", "persistent"], default=None)
    ap.add_argument("--threads", type=int, default=64)
    ap.add_argument("--smem-hits", type=int, default=50)
    ap.add_argument("--no-narrow", action="store_true")
    ap.add_argument("--register-ctas", type=int, default=0, choices=[0, 4, 5, 18],
                    help="register build (0: automatic for the thread count)")
    ap.add_argument("--seed-lanes", type=int, default=0, choices=[0, 8, 16, 32],
                    help="seeding lanes per h0 (0: the library's automatic width)")
    ap.add_argument("--graph", action="store_true", help="replay launches from a CUDA graph")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="use the library's default launch configuration instead of the autotuned one")
    ap.add_argument("--e2e-chunk", type=int, default=16000, help="events per end-to-end call")
    ap.add_argument("--e2e-pipeline", type=int, default=0,
                    help="events per overlapped part inside an end-to-end call (0: one part)")
    ap.add_argument("--e2e-copies", action="store_true",
                    help="end-to-end: stage copies instead of reading / writing pinned host buffers in place")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-pruning leg")
    ap.add_argument("--no-stages", action="store_true", help="skip the device sort / fit leg")
    ap.add_argument("--no-reference-api", action="store_true",
                    help="skip the end-to-end leg through the reference-signature C++ entry points")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched leg (100,000 uneven events, autotuned persistent launch + CUDA graph)")
    ap.add_argument("--no-stress", action="store_true",
                    help="skip the high-occupancy leg (100,000 events at 4x pile-up, plain vs learned)")
    ap.add_argument("--batched-events", type=int, default=100000)
    ap.add_argument("--stress-events", type=int, default=100000)
    ap.add_argument("--plan", action="store_true",
                    help="print the rank layout (world size, seed block per rank) and exit; no GPU work")
    ap.add_argument("--ref-emulator", action="store_true",
                    help="reference arm: time the reference kernel under the work-group emulator "
                         "(oracle/_ref, only where it was built) instead of the oracle restatement")
    return ap.parse_args()


# ----------------------------------------------------------------- ranks --
class Ranks:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def shard_seeds(first_seed: int, n_events: int, rank: int) -> range:
    """Weak scaling: rank r owns its own block of n_events seeds."""
    start = first_seed + rank * n_events
    return range(start, start + n_events)


def launch_ranks(args):
    """Ranks for --gpus N: under a launcher WORLD_SIZE must equal N (else exit
    with an error); without one, N > 1 ranks are started here through
    torch.distributed.run and their exit code is returned.  None: this
    process is the (only) rank."""
    world = os.environ.get("WORLD_SIZE")
    if world is not None:
        if int(world) != args.gpus:
            sys.exit(f"bench.py: --gpus {args.gpus} but the launcher started WORLD_SIZE={world} ranks")
        return None
    if args.gpus <= 1:
        return None
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def plan(args, ranks: "Ranks"):
    """The rank layout this invocation would run, gathered on rank 0."""
    first, n, _, _, _ = CONFIGS[args.config]
    n = args.events or n
    seeds = shard_seeds(first, n, ranks.rank)
    mine = [ranks.rank, ranks.local, seeds.start, seeds.stop]
    rows = [mine]
    if ranks.pg:
        rows = [None] * ranks.world
        ranks.pg.all_gather_object(rows, mine)
    return {"plan": True, "n_gpus": args.gpus, "world_size": ranks.world,
            "ranks": [{"rank": r, "device": d, "seeds": [a, b]} for r, d, a, b in rows]}


# -------------------------------------------------------------- workload --
def make_workload(args, rank: int):
    from cl_forward_gb300 import events, generator
    first, n, params_name, _, _ = CONFIGS[args.config]
    n = args.events or n
    raw, truths = generator.generate_parallel(shard_seeds(first, n, rank), getattr(generator, params_name))
    return raw, truths


def sort_events(raw):
    """The library's host x-sort (velo_sort_by_x: the reference's preorder_by_x
    permutation), on the host's cores; pure host code, no CUDA context."""
    from concurrent.futures import ThreadPoolExecutor
    from cl_forward_gb300 import build, native
    build.build()
    native.load()
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(native.sort_by_x, raw))


def sort_events_reference(raw):
    from oracle import oracle   # the reference arm sorts with the reference's sort, restated
    return [oracle.sort_by_x(b) for b in raw]


def workload_stats(blobs):
    import numpy as np
    S = np.array([int(np.frombuffer(b[0:4], "<i4")[0]) for b in blobs])
    H = np.array([int(np.frombuffer(b[4:8], "<i4")[0]) for b in blobs])
    return S, H


# ---------------------------------------------------------------- clocks --
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4], parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        maxp = max(r[2] for r in rows)
        loaded = [r for r in rows if r[2] >= 0.5 * maxp] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in loaded for i, v in enumerate(r[4]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(loaded)}


# ------------------------------------------------------------- baselines --
def cpu_baseline(blobs, seconds: float, raw=None):
    """Oracle restatement over all host cores, repeated passes until `seconds`.

    Also: the other Y-lane counts the reference sweeps (KernelInvoker.cpp:149-153)
    and the host x-sort, each on a 2,000-event sample, and the oracle's count
    of candidate evaluations per event (the reference algorithm's work)."""
    from oracle import oracle
    n = len(blobs)
    passes, elapsed = 0, 0.0
    while elapsed < seconds or passes == 0:
        elapsed += oracle.time_search(blobs, 4, 0)
        passes += 1
    cores = os.cpu_count() or 1
    sample = blobs[:2000]
    per_y = {}
    for y in (1, 2, 3, 4):
        per_y[str(y)] = len(sample) / min(oracle.time_search(sample, y, 0) for _ in range(2))
    sort_s = None
    if raw is not None:
        t0 = time.perf_counter()
        for b in raw[:len(sample)]:
            oracle.sort_by_x(b)
        sort_s = (time.perf_counter() - t0) / len(sample)
    _, _, cnt = oracle.search(blobs[:500], 4, 0, counters=True)
    m = max(min(500, n), 1)
    work = {"window_evals": cnt.window_evals / m, "forward_fits": cnt.forward_fits / m,
            "seed_fits": cnt.seed_fits / m, "seed_scatters": cnt.seed_scatters / m,
            "sample_events": m}
    ev_s = n * passes / elapsed
    return {"value": ev_s, "unit": "events/s", "cores": cores, "kind": "port",
            "sample": f"{passes} pass(es) over the same {n} x-sorted events, Y=4, {cores} threads, "
                      f"{elapsed:.1f} s, search only (sort excluded, as on the GPU)",
            "events_per_s_by_y": per_y, "best_y": max(per_y, key=per_y.get),
            "host_sort_us_per_event_one_thread": None if sort_s is None else 1e6 * sort_s,
            "events_per_s_with_sort": None if sort_s is None else 1.0 / (1.0 / ev_s + sort_s / cores),
            "work_per_event": work}


def reference_arm(args, ranks: Ranks):
    if ranks.rank != 0:
        return None
    raw, _ = make_workload(args, 0)
    blobs = sort_events_reference(raw)
    from oracle import oracle
    n = len(blobs)
    kind = "port"
    run = lambda: oracle.time_search(blobs, 4, 0)
    try:
        if args.ref_emulator and os.path.exists(oracle.REF_LIB):
            oracle.ref_lib()
            kind = "reference"

            def run():
                t0 = time.perf_counter()
                oracle.ref_search(blobs, 4, 0)
                return time.perf_counter() - t0
    except Exception:
        kind = "port"
    for _ in range(args.warmup):
        run()
    total = sum(run() for _ in range(args.steps))
    value = n * args.steps / total
    cores = os.cpu_count() or 1
    what = ("the reference kernel (Kernel.cl) under the work-group emulator" if kind == "reference"
            else "the oracle restatement of the reference algorithm")
    _, _, _, _, desc = CONFIGS[args.config]
    return {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded VELO events (no public dataset)",
        "config": {"workload": desc, "events": n, "y_lanes": 4},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": cores, "kind": kind,
                         "sample": f"each step one pass of {what} over all {n} events on {cores} host "
                                   f"threads ({os.uname().machine})"},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


PROFILES = {"scale": "search_kernel_scale7k_full.md"}


def profiled_traffic(config: str, n_events: int):
    """DRAM bytes of one launch: the ncu capture's bytes per event x events.

    The capture ran on 7,000 events of the same workload (a full 10,000-event
    capture would exceed the size a 45-pass ncu replay can take in minutes);
    DRAM traffic grows in proportion to the events processed, so it scales.
    """
    name = PROFILES.get(config)
    if not name:
        return None, None
    path = os.path.join(ROOT, "profiles", name)
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_event:"):
                per = int(ln.split(":")[1])
                return per * n_events, f"profiles/{name}: {per} B/event x {n_events} events"
    except OSError:
        pass
    return None, None


def stages_leg(ctx, raw, opts, n_tracks_expected):
    """The stages either side of the search, on the GPU: the device x-sort of
    the unsorted events (the reference sorts on the host before every launch),
    then the search of the device-sorted events and the straight-line fit of
    every output track.  Host wall clock with a synchronize on both sides."""
    import numpy as np
    n = len(raw)
    offs = np.zeros(n, np.uint64)
    sizes = np.array([len(b) for b in raw], np.uint64)
    total = 0
    for i, b in enumerate(raw):
        offs[i] = total
        total += (len(b) + 15) // 16 * 16
    hbuf = ctx.host_alloc(max(total, 16))
    for i, b in enumerate(raw):
        hbuf[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(b, np.uint8)
    sort_s = []
    for _ in range(3):   # the sort works in place: staged afresh each time
        ctx.stage(hbuf, offs, sizes)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.sort_staged()
        ctx.synchronize()
        sort_s.append(time.perf_counter() - t0)
    o = type(opts).from_buffer_copy(opts)
    o.use_graph = 0
    ctx.run(o)
    rows = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in raw))
    _, counts, _, _ = ctx.fetch(n, rows)
    total_tracks = int(counts.sum())
    fit_s = []
    for _ in range(3):
        t0 = time.perf_counter()
        fits = ctx.fit_tracks(total_tracks)
        fit_s.append(time.perf_counter() - t0)
    ctx.host_free(hbuf)
    sort_ms, fit_ms = 1e3 * statistics.median(sort_s), 1e3 * statistics.median(fit_s)
    return {"device_sort": {"ms": sort_ms, "events_per_s": n / (sort_ms / 1e3)},
            "fit": {"ms": fit_ms, "tracks_per_s": total_tracks / (fit_ms / 1e3),
                    "note": "includes the device-to-host copy of the fits (20 B per track)"},
            "tracks_after_device_sort": total_tracks,
            "same_track_count_as_host_sort": total_tracks == n_tracks_expected,
            "fits_finite": bool(np.isfinite(fits["x0"][:total_tracks]).all())}


LEARNED_WEIGHTS = os.path.join(ROOT, "cl_forward_gb300", "weights", "doublet_mlp.npz")


def learned_leg(ctx, hbuf, offs, sizes, blobs, truths, opts, tracks, counts, first, plain_ms, args):
    """The learned-pruned search of the same staged events next to the plain one."""
    import numpy as np
    from cl_forward_gb300 import native
    from cl_forward_gb300.validation import rates_fast
    wz = np.load(LEARNED_WEIGHTS)
    max_hits = int(wz["max_event_hits"]) if "max_event_hits" in wz.files else 0
    ctx.set_mlp(wz["weights"], float(wz["keep_threshold"]), float(wz["window_margin"]),
                float(wz["min_keep_rate"]), max_hits)
    o = native.Options.from_buffer_copy(opts)
    o.learned = 1
    o.use_graph = 0
    ctx.stage(hbuf, offs, sizes)
    for _ in range(args.warmup):
        ctx.run(o)
    ctx.synchronize()
    steps_ms = [ctx.time_runs(o, warmup=0, iters=1, flush_l2=True) for _ in range(args.steps)]
    n = len(blobs)
    cap = len(tracks)
    lt, lc, lf, ls = ctx.fetch(n, cap)
    per_l = [lt[int(lf[e]):int(lf[e]) + int(lc[e])] for e in range(n)]
    per_p = [tracks[int(first[e]):int(first[e]) + int(counts[e])] for e in range(n)]
    rp = rates_fast(per_p, blobs, truths)
    rl = rates_fast(per_l, blobs, truths)
    ms = statistics.fmean(steps_ms)
    return {"value": n / (ms / 1e3), "unit": "events/s", "ms_per_step": ms, "speedup_vs_plain": plain_ms / ms,
            "efficiency_plain": rp.efficiency, "efficiency_learned": rl.efficiency,
            "efficiency_loss": rp.efficiency - rl.efficiency, "ghost_rate_plain": rp.ghost_rate,
            "ghost_rate_learned": rl.ghost_rate, "ghost_increase": rl.ghost_rate - rp.ghost_rate,
            "clone_change": rl.clone_rate - rp.clone_rate,
            "fallback_fraction": float(np.mean((ls & native.EVENT_LEARNED_FALLBACK) != 0)),
            "weights": os.path.relpath(LEARNED_WEIGHTS, ROOT), "weights_sha256": str(wz["sha256"]),
            "max_event_hits": max_hits,
            "note": "same events, same launch shape; the network is trained on other seeds (100000-149999)"}


def pinned_pack(ctx, blobs):
    """Events packed at 16-byte-aligned offsets in one pinned host buffer."""
    import numpy as np
    n = len(blobs)
    offs = np.zeros(n, np.uint64)
    sizes = np.array([len(b) for b in blobs], np.uint64)
    total = 0
    for i, b in enumerate(blobs):
        offs[i] = total
        total += (len(b) + 15) // 16 * 16
    hbuf = ctx.host_alloc(max(total, 16))
    for i, b in enumerate(blobs):
        hbuf[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(b, np.uint8)
    return hbuf, offs, sizes


class QuietStdout:
    """Sends file descriptor 1 to /dev/null (the reference-signature entry
    points print what the reference prints; stdout carries the JSON line)."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)
        return self

    def __exit__(self, *a):
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def reference_api_leg(raw, blobs, expected_tracks, args):
    """End to end through the reference's own C++ entry points, on
    std::vector<std::vector<uint8_t> > input and output (the timing harness
    libvelo_api_bench.so): independent_execute on the unsorted events (sort
    and search; GpuPixelSearchByTriplet.cpp:4-22) and gpuPixelSearchByTriplet
    on the x-sorted ones (GpuPixelSearchByTriplet.cpp:29-37).  Host wall clock
    per call; everything the call does is inside it."""
    from cl_forward_gb300 import native
    n = len(raw)
    out = {"unit": "events/s", "events": n,
           "io": "std::vector<std::vector<uint8_t>> per event in, output vectors allocated by each call"}
    for entry, evs in (("independent_execute", raw), ("gpuPixelSearchByTriplet", blobs)):
        with QuietStdout():
            ms, tracks, _, _ = native.reference_api_times(evs, entry, max(args.warmup, 1), args.steps)
        mean = statistics.fmean(ms)
        out[entry] = {"value": n / (mean / 1e3), "ms_per_call": mean,
                      "ms_samples": [round(float(x), 3) for x in ms], "tracks": tracks,
                      "same_tracks_as_device_resident": tracks == expected_tracks}
    return out


def timed_steps(ctx, opts, args):
    """Mean device milliseconds of args.steps runs (L2 flushed before each)."""
    for _ in range(args.warmup):
        ctx.run(opts)
    ctx.synchronize()
    steps_ms = [ctx.time_runs(opts, warmup=0, iters=1, flush_l2=True) for _ in range(args.steps)]
    return statistics.fmean(steps_ms), steps_ms


def tuned_on_sample(ctx, hbuf, offs, sizes, H, base, sample):
    """Autotuned options for a large batch, tuned on its first `sample`
    events (the sweep times 104 + 9 launch configurations)."""
    from cl_forward_gb300 import autotune
    k = min(sample, len(offs))
    ctx.stage(hbuf, offs[:k], sizes[:k])
    ctx.synchronize()
    opts, info = autotune.tuned_options(ctx, k, float(H[:k].mean()), base, iters=3)
    return opts, info


def batched_leg(args, peak, peak_src):
    """The batched configuration: 100,000 events of uneven size (PVs ~
    Poisson(U(2, 30))), one persistent launch over all of them with the
    autotuned configuration replayed from a CUDA graph, next to the launch
    style of the reference's runs (one 256-thread CTA per event), and end to
    end from pinned host buffers in calls of 16,000 events."""
    import numpy as np
    from cl_forward_gb300 import generator, native
    first = CONFIGS["batched"][0]
    raw, _ = generator.generate_parallel(range(first, first + args.batched_events), generator.CONFIG_BATCHED)
    blobs = sort_events(raw)
    del raw
    S, H = workload_stats(blobs)
    n = len(blobs)
    ctx = native.Context(0)
    hbuf, offs, sizes = pinned_pack(ctx, blobs)
    del blobs
    base = native.default_options(use_graph=1)
    opts, tuned = tuned_on_sample(ctx, hbuf, offs, sizes, H, base, 20000)
    opts.use_graph = 1
    ctx.stage(hbuf, offs, sizes)
    ms, samples = timed_steps(ctx, opts, args)
    counts, _, status = ctx.fetch_counts(n)
    T = counts.astype(np.int64)
    alg = int((8 + 12 * S + 16 * H).sum() + (4 + 100 * T).sum())
    style = native.default_options(launch_mode=0, threads_per_event=256, smem_hits=0, register_ctas=5,
                                   seed_lanes=32, use_graph=1)
    ms1, samples1 = timed_steps(ctx, style, args)
    counts1, _, _ = ctx.fetch_counts(n)
    # end to end through the C ABI, pinned host buffers, calls of 16,000 events
    chunk = 16000
    bounds = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
    rows = np.maximum(H, 1).astype(np.int64)
    out_cap = int(max(rows[a:b].sum() for a, b in bounds))
    h_tracks = ctx.host_alloc(out_cap * 100).view(native.TRACK_DTYPE)
    hc = np.zeros(n, np.uint32)
    hf = np.zeros(n, np.uint64)
    hs = np.zeros(n, np.uint32)
    e2e_opts = native.Options.from_buffer_copy(opts)
    e2e_opts.host_direct = 1
    e2e_opts.use_graph = 0

    def e2e_pass():
        for a, b in bounds:
            ctx.search_packed_into(hbuf, offs[a:b], sizes[a:b], e2e_opts, h_tracks, hc[a:b], hf[a:b], hs[a:b])

    e2e_pass()
    t0 = time.perf_counter()
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_pass()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    assert np.array_equal(hc, counts)
    ctx.host_free(h_tracks.view(np.uint8))
    ctx.host_free(hbuf)
    ctx.close()
    achieved = alg / (ms / 1e3) / 1e9
    return {
        "workload": CONFIGS["batched"][4], "events": n, "mean_hits": float(H.mean()), "max_hits": int(H.max()),
        "min_hits": int(H.min()), "value": n / (ms / 1e3), "unit": "events/s", "ms_per_step": ms,
        "ms_per_step_samples": [round(x, 3) for x in samples],
        "launch": {"threads_per_event": opts.threads_per_event, "launch_mode": opts.launch_mode,
                   "smem_hits": opts.smem_hits, "register_ctas": opts.register_ctas,
                   "seed_lanes": opts.seed_lanes, "cuda_graph": True, "autotuned": tuned,
                   "tuned_on": "the first 20,000 events of the batch"},
        "config1_launch_style": {"value": n / (ms1 / 1e3), "ms_per_step": ms1,
                                 "ms_per_step_samples": [round(x, 3) for x in samples1],
                                 "launch": "one 256-thread CTA per event, automatic shared-memory tile, "
                                           "32 seeding lanes per h0, CUDA graph",
                                 "same_track_counts": bool(np.array_equal(counts1, counts))},
        "speedup_vs_config1_launch_style": ms1 / ms,
        "e2e": {"value": n / e2e_s, "unit": "events/s", "calls_of_events": chunk,
                "io": "events read and tracks written in place in pinned host memory (NVLink-C2C)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": alg, "peak_source": peak_src,
                     "achieved_config1_launch_style": alg / (ms1 / 1e3) / 1e9},
        "tracks": int(T.sum()),
        "status_flags": {"ring_overflow": int(np.sum(status & 1 != 0)),
                         "track_overflow": int(np.sum(status & 2 != 0))},
    }


def stress_leg(args):
    """The high-occupancy configuration: 100,000 events at four times the
    pile-up, plain (autotuned, CUDA graph) against learned-pruned seeding on
    the same launch, with the fraction of events that fall back to the plain
    method; tracking rates of both, split at p = 2 GeV, on the first 10,000
    events."""
    import numpy as np
    from cl_forward_gb300 import events as E, generator, native, validation
    first = CONFIGS["stress"][0]
    raw, truths = generator.generate_parallel(range(first, first + args.stress_events), generator.CONFIG_STRESS)
    blobs = sort_events(raw)
    del raw
    S, H = workload_stats(blobs)
    n = len(blobs)
    ctx = native.Context(0)
    hbuf, offs, sizes = pinned_pack(ctx, blobs)
    base = native.default_options(use_graph=1)
    opts, tuned = tuned_on_sample(ctx, hbuf, offs, sizes, H, base, 20000)
    ctx.stage(hbuf, offs, sizes)
    ms, samples = timed_steps(ctx, opts, args)
    wz = np.load(LEARNED_WEIGHTS)
    max_hits = int(wz["max_event_hits"]) if "max_event_hits" in wz.files else 0
    ctx.set_mlp(wz["weights"], float(wz["keep_threshold"]), float(wz["window_margin"]),
                float(wz["min_keep_rate"]), max_hits)
    lo = native.Options.from_buffer_copy(opts)
    lo.learned = 1
    lo.use_graph = 0
    ms_l, samples_l = timed_steps(ctx, lo, args)
    _, _, lstatus = ctx.fetch_counts(n)
    fallback = float(np.mean((lstatus & native.EVENT_LEARNED_FALLBACK) != 0))

    # rates on the first 10,000 events, both methods
    k = min(10000, n)
    ctx.stage(hbuf, offs[:k], sizes[:k])
    ids, base_ids = validation.hit_ids_packed(hbuf, offs[:k])
    rates = {}
    for name, o in (("plain", opts), ("learned", lo)):
        o2 = native.Options.from_buffer_copy(o)
        o2.use_graph = 0
        ctx.run(o2)
        counts, _, _ = ctx.fetch_counts(k)
        cap = int(counts.sum())
        tracks = np.zeros(max(cap, 1), E.TRACK_DTYPE)
        c2 = np.zeros(k, np.uint32)
        f2 = np.zeros(k, np.uint64)
        s2 = np.zeros(k, np.uint32)
        ctx.fetch_into(tracks, c2, f2, s2)
        c64 = c2.astype(np.int64)
        starts = np.concatenate([[0], np.cumsum(c64)[:-1]])
        idx = np.repeat(f2.astype(np.int64) - starts, c64) + np.arange(cap, dtype=np.int64)
        words = tracks.view(np.uint32).reshape(-1, 25)[:cap][idx]
        rates[name] = validation.rates_packed(words, c64, ids, base_ids, truths[:k]).as_dict()
    ctx.host_free(hbuf)
    ctx.close()
    rp, rl = rates["plain"], rates["learned"]
    return {
        "workload": CONFIGS["stress"][4], "events": n, "mean_hits": float(H.mean()), "max_hits": int(H.max()),
        "plain": {"value": n / (ms / 1e3), "unit": "events/s", "ms_per_step": ms,
                  "ms_per_step_samples": [round(x, 3) for x in samples],
                  "launch": {"threads_per_event": opts.threads_per_event, "launch_mode": opts.launch_mode,
                             "smem_hits": opts.smem_hits, "register_ctas": opts.register_ctas,
                             "seed_lanes": opts.seed_lanes, "cuda_graph": True, "autotuned": tuned}},
        "learned": {"value": n / (ms_l / 1e3), "unit": "events/s", "ms_per_step": ms_l,
                    "ms_per_step_samples": [round(x, 3) for x in samples_l],
                    "fallback_fraction": fallback, "max_event_hits": max_hits,
                    "weights": os.path.relpath(LEARNED_WEIGHTS, ROOT)},
        "learned_speedup_vs_plain": ms / ms_l,
        "rates_first_10000_events": {"plain": rp, "learned": rl,
                                     "efficiency_loss": rp["efficiency"] - rl["efficiency"],
                                     "efficiency_loss_p_lt_2": rp["efficiency_p_lt_2"] - rl["efficiency_p_lt_2"],
                                     "efficiency_loss_p_ge_2": rp["efficiency_p_ge_2"] - rl["efficiency_p_ge_2"],
                                     "ghost_increase": rl["ghost_rate"] - rp["ghost_rate"],
                                     "clone_change": rl["clone_rate"] - rp["clone_rate"]},
    }


# ---------------------------------------------------------------- GPU arm --
def gpu_arm(args, ranks: Ranks):
    import numpy as np
    from cl_forward_gb300 import events as E

    if args.config in ("batched", "stress"):   # the batched configurations replay a CUDA graph
        args.graph = True
    raw, truths = make_workload(args, ranks.rank)          # process pool before any GPU call
    blobs = sort_events(raw)
    S, H = workload_stats(blobs)
    n = len(blobs)

    from cl_forward_gb300 import build, native
    build.build()
    ctx = native.Context(ranks.local)
    mode = CONFIGS[args.config][3] if args.launch is None else (1 if args.launch == "persistent" else 0)
    opts = native.default_options(threads_per_event=args.threads, launch_mode=mode,
                                  smem_hits=args.smem_hits, narrow_windows=0 if args.no_narrow else 1,
                                  register_ctas=args.register_ctas, use_graph=1 if args.graph else 0,
                                  seed_lanes=args.seed_lanes)

    # pinned host input, 16-byte aligned events
    offs = np.zeros(n, np.uint64)
    sizes = np.array([len(b) for b in blobs], np.uint64)
    total = 0
    for i, b in enumerate(blobs):
        offs[i] = total
        total += (len(b) + 15) // 16 * 16
    hbuf = ctx.host_alloc(max(total, 16))
    for i, b in enumerate(blobs):
        hbuf[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(b, np.uint8)

    # ---- device-resident value ------------------------------------------
    ctx.stage(hbuf, offs, sizes)
    ctx.synchronize()
    tuned = None
    if args.autotune:
        from cl_forward_gb300 import autotune
        opts, tuned = autotune.tuned_options(ctx, n, float(H.mean()), opts, iters=3)
        mode = opts.launch_mode
    ranks.barrier()
    for _ in range(args.warmup):
        ctx.run(opts)
    ctx.synchronize()
    with Clocks(ranks.local) as clk:
        # one timed run per call: L2 flushed before it, CUDA events around it
        steps_ms = [ctx.time_runs(opts, warmup=0, iters=1, flush_l2=True) for _ in range(args.steps)]
    ms = statistics.fmean(steps_ms)
    ranks.barrier()
    st = ctx.stats()
    launches = st.launches * args.steps
    cap = int(np.maximum(H, 1).sum())
    tracks = np.zeros(cap, E.TRACK_DTYPE)
    counts = np.zeros(n, np.uint32)
    first = np.zeros(n, np.uint64)
    status = np.zeros(n, np.uint32)
    ctx.fetch_into(tracks, counts, first, status)
    T = counts.astype(np.int64)
    alg_bytes = int((8 + 12 * S + 16 * H).sum() + (4 + 100 * T).sum())
    ms_max = ranks.max(ms)
    value = ranks.sum(n) / (ms_max / 1e3)

    # ---- end to end through the C ABI ------------------------------------
    # chunks of at most --e2e-chunk events per call, as the reference's
    # gpuPixelSearchByTripletInvocation chunks at 16000
    chunk = max(1, min(args.e2e_chunk, n))
    bounds = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
    rows = np.maximum(H, 1).astype(np.int64)
    out_cap = int(max(rows[a:b].sum() for a, b in bounds))
    h_tracks = ctx.host_alloc(out_cap * 100).view(E.TRACK_DTYPE)
    h_counts = np.zeros(n, np.uint32)
    h_first = np.zeros(n, np.uint64)
    h_status = np.zeros(n, np.uint32)

    e2e_opts = native.Options.from_buffer_copy(opts)
    e2e_opts.pipeline_events = args.e2e_pipeline
    e2e_opts.host_direct = 0 if args.e2e_copies else 1

    def e2e_pass():
        for a, b in bounds:
            ctx.search_packed_into(hbuf, offs[a:b], sizes[a:b], e2e_opts, h_tracks, h_counts[a:b], h_first[a:b],
                                   h_status[a:b])

    for _ in range(args.warmup):
        e2e_pass()
    ranks.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_pass()
    e2e_s = (time.perf_counter() - t0) / args.steps
    ranks.barrier()
    e2e_max = ranks.max(e2e_s)
    assert np.array_equal(h_counts, counts)
    h2d = int(sum(int(offs[b - 1] + sizes[b - 1] - offs[a]) for a, b in bounds)) + 36 * n
    d2h = 8 * len(bounds) + 16 * n + 100 * int(T.sum())

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg_bytes / (ms / 1e3) / 1e9
    traffic, traffic_src = profiled_traffic(args.config, n)
    _, _, _, _, desc = CONFIGS[args.config]
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic seeded VELO events (no public dataset)",
        "config": {"workload": desc, "events": n, "mean_hits": float(H.mean()), "max_hits": int(H.max()),
                   "y_lanes": 4, "launch": "persistent" if mode else "per-event",
                   "threads_per_event": opts.threads_per_event, "smem_bytes_per_cta": st.smem_bytes_per_cta,
                   "events_in_global_arena": st.events_in_global, "tracks": int(T.sum()),
                   "ms_per_step_samples": [round(x, 4) for x in steps_ms],
                   "register_ctas": opts.register_ctas,
                   "seed_lanes": opts.seed_lanes or "automatic (16 when Y divides 16, else 32)",
                   "cuda_graph": bool(opts.use_graph),
                   "smem_hits_option": opts.smem_hits, "autotuned": tuned,
                   "e2e_chunk_events": chunk, "e2e_pipeline_events": args.e2e_pipeline,
                   "e2e_io": ("H2D / D2H copies" if args.e2e_copies else
                              "events read and tracks written in place in pinned host memory by the kernel "
                              "(NVLink-C2C); per-event counts / offsets / status copied"),
                   "l2": "flushed between timed steps (2 x L2 memset); input also larger than L2",
                   "parallelism": f"weak scaling over {args.gpus} GPU(s), event blocks per rank"},
        "impl": "gb300",
        "e2e": {"value": ranks.sum(n) / e2e_max, "unit": "events/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_bytes": alg_bytes, "peak_source": peak_src,
                     "note": "algorithmic bytes = input blobs + 4 B count + 100 B per track",
                     "limiter": ("not HBM: a latency- and issue-bound search (the ncu capture in "
                                 "traffic_source: ~60% of issue slots busy, DRAM ~3%, L2 ~6%, L1 hit rate "
                                 "~87%)")},
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "status_flags": {"ring_overflow": int(np.sum(status & 1 != 0)),
                         "track_overflow": int(np.sum(status & 2 != 0))},
    }
    if not args.no_stages:
        line["pipeline_stages"] = stages_leg(ctx, raw, opts, int(T.sum()))
    if not args.no_learned and os.path.exists(LEARNED_WEIGHTS):
        line["learned"] = learned_leg(ctx, hbuf, offs, sizes, blobs, truths, opts, tracks, counts, first, ms,
                                      args)
    if ranks.rank == 0 and args.gpus == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(blobs, args.cpu_seconds, raw)
        wk = line["cpu_baseline"]["work_per_event"]
        # candidate evaluations of the reference algorithm per event x events/s of the
        # GPU (the GPU skips most of them: narrowed windows)
        line["work"] = {"reference_evals_per_event": wk["window_evals"] + wk["forward_fits"] + wk["seed_fits"],
                        "reference_evals_per_s": (wk["window_evals"] + wk["forward_fits"] + wk["seed_fits"])
                        * value, "counted_by": "oracle restatement on 500 of the events"}
    if ranks.rank == 0 and args.gpus == 1 and not args.no_reference_api:
        line["e2e_reference_api"] = optional_leg(reference_api_leg, raw, blobs, int(T.sum()), args)
    ctx.host_free(hbuf)
    ctx.host_free(h_tracks.view(np.uint8))
    ctx.close()
    if ranks.rank == 0 and args.gpus == 1 and args.config == "scale":
        del raw, blobs
        if not args.no_batched:
            line["batched"] = optional_leg(batched_leg, args, peak, peak_src)
        if not args.no_stress and os.path.exists(LEARNED_WEIGHTS):
            line["stress"] = optional_leg(stress_leg, args)
    return line if ranks.rank == 0 else None


def optional_leg(fn, *a):
    """A leg beside the headline: its failure is reported in the line
    (with the error) instead of costing the line itself."""
    try:
        return fn(*a)
    except Exception as exc:   # noqa: BLE001 -- reported, not hidden
        import traceback
        traceback.print_exc(file=sys.stderr)
        return {"error": f"{type(exc).__name__}: {exc}"[:500]}


def main():
    args = parse_args()
    rc = launch_ranks(args)
    if rc is not None:
        sys.exit(rc)
    ranks = Ranks()
    try:
        if args.plan:
            line = plan(args, ranks)
        elif args.impl == "reference":
            line = reference_arm(args, ranks)
        else:
            line = gpu_arm(args, ranks)
        if line is not None and ranks.rank == 0:
            print(json.dumps(line), flush=True)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
