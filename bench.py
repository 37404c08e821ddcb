"""BC7 throughput benchmark: batched vs plain per-image encoding at -q 50.

Workload (the batched configuration): 512 RGBA8 textures whose sides are
drawn log-uniformly from {16, ..., 2048} per axis, filled with the seeded
tile_mix content (fastc_gb300.synth), 115.6 MP / 7.22 M blocks in total,
encoded at 50 annealing steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --serve [--serve-rates 20,60,120] [--serve-seconds 4]
    python bench.py --profile-case [--case-kind tile_mix|radial|gradient]
        [--case-size 4096] [--case-steps 50] [--case-repeat 1]

--profile-case encodes one seeded texture through the device-memory C ABI
`--case-repeat` times and prints each encode's wall time: the small,
self-contained command that the ncu captures under profiles/ run.

A step is one pass of the encoder over the whole texture set:
  * value       -- batched: one graph launch of the captured plan over all
                   512 device-resident textures (CUDA events, max over ranks)
  * plain_*     -- the same textures, one encode call per texture
  * e2e         -- fastc_bc7_compress_batch with pinned host buffers: the
                   host->device copy of all texels, the encode and the
                   device->host copy of all blocks inside the timed region
  * cpu_baseline -- the oracle (C port of FasTC's encoder) on the host cores,
                   on a bounded sample of the same textures
Inputs (462 MB) are larger than L2, so no flush runs between steps.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SET_SEED = 3
SET_COUNT = 512
STEPS_Q = 50
ANNEAL_SEED = 1
METRIC = "BC7 MPix/s at -q50, batched vs plain per-image on 1 GB300, PSNR within 0.05dB"
SMALL_PIXELS = 64 * 64  # "small textures": at most 4096 texels


def _gen(args):
    from fastc_gb300 import synth

    i, w, h = args
    return synth.tile_mix(SET_SEED * 1000 + i, w, h)


def make_texture_set(workers: int):
    from fastc_gb300 import synth

    sides = synth.texture_sides(SET_SEED, SET_COUNT)
    jobs = [(i, w, h) for i, (w, h) in enumerate(sides)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, workers)) as pool:
        imgs = pool.map(_gen, jobs, chunksize=4)
    return imgs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unparsed"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_per_block():
    """(DRAM bytes, warp instructions) per block from the committed ncu
    summaries: the instructions from the launch list of this workload's own
    timed step (profiles/bc7_encode_texture_set_512_q50.json, one pass), the
    DRAM bytes from a multi-pass capture of a 4096x4096 tile-mix launch
    (profiles/bc7_encode_traffic.json), scaled per block."""
    traffic = inst = None
    try:
        with open(os.path.join(ROOT, "profiles", "bc7_encode_traffic.json")) as f:
            traffic = float(json.load(f)["dram_bytes_per_block"])
    except Exception:
        pass
    try:
        with open(os.path.join(ROOT, "profiles", "bc7_encode_texture_set_512_q50.json")) as f:
            inst = float(json.load(f)["warp_instructions_per_block"])
    except Exception:
        pass
    return traffic, inst


# The CPU legs encode a uniform sample of the set's blocks: every
# BAND_STRIDE-th block row of the 512 textures, rows counted across the set
# in texture order (89 rows, 9,368 blocks, 149,888 texels). A block's
# cost depends only on its texels, so this is the set's content mix at
# 1/720 of its size.
BAND_STRIDE = 720


def band_sample(stride: int = BAND_STRIDE):
    """[(texture index, first texel row, the 4-row band as RGBA8)] of every
    stride-th block row of the texture set."""
    from fastc_gb300 import synth

    out, g = [], 0
    for i, (w, h) in enumerate(synth.texture_sides(SET_SEED, SET_COUNT)):
        for r in range(h // 4):
            if g % stride == stride // 2:
                out.append((i, 4 * r, synth.tile_mix(SET_SEED * 1000 + i, w, 4, 0, 4 * r)))
            g += 1
    return out


def _single_colour_blocks_before(tex, y0: int, x0: int = 0) -> int:
    """Single-colour blocks of `tex` before the block at texel (x0, y0) in
    raster order."""
    import numpy as np

    def count(region):
        px = region.view("<u4")[..., 0]
        if px.size == 0:
            return 0
        h, w = px.shape
        blk = px.reshape(h // 4, 4, w // 4, 4).transpose(0, 2, 1, 3).reshape(h // 4, w // 4, 16)
        return int((blk == blk[..., :1]).all(-1).sum())

    return count(tex[:y0]) + count(tex[y0:y0 + 4, :x0])


# Work items of the CPU legs: pieces of at most PIECE texels of a row, so
# that the host threads stay balanced whatever the rows' widths.
PIECE = 256


def encode_bands(bands, threads: int, kind: str, textures=None, steps: int = STEPS_Q):
    """One pass over the bands on `threads` host threads, which take pieces
    of at most PIECE texels of a row in turn from a shared cursor: FasTC's
    own encoder (kind "reference", the in-place build; its global RNG is
    shared by the threads, as under tc -t N) or the oracle port (kind
    "port", per-fit streams). With the whole `textures` the port encodes
    each piece inside its texture (the texture's block coordinates seed the
    annealing, the watermark counter continues from the blocks before it),
    giving the GPU's bytes. Returns (seconds, the blocks of each band)."""
    import concurrent.futures as cf
    import itertools

    import numpy as np

    from oracle import oracle as O

    enc = O.Reference() if kind == "reference" else O.Port()
    if kind == "reference":
        enc.lib.ref_set_seed(ANNEAL_SEED)
    items = [(k, x0, min(x0 + PIECE, band.shape[1]))
             for k, (_, _, band) in enumerate(bands) for x0 in range(0, band.shape[1], PIECE)]
    prior = {}
    if textures is not None:
        for k, x0, _ in items:
            i, y0, _ = bands[k]
            prior[(k, x0)] = _single_colour_blocks_before(textures[i], y0, x0)
    outs = [np.zeros(b.shape[0] * b.shape[1], dtype=np.uint8) for _, _, b in bands]
    bufs = [np.ascontiguousarray(b) for _, _, b in bands]
    cursor = itertools.count()
    # per thread, one whole-texture block buffer per texture, reused by the
    # pieces of that texture (only each piece's blocks are written), so that
    # the timing is the encoder's and not the allocation of large buffers
    local = threading.local()

    def texture_out(i, size):
        cache = getattr(local, "cache", None)
        if cache is None:
            cache = local.cache = {}
        if i not in cache:
            cache[i] = np.empty(size, dtype=np.uint8)
        return cache[i]

    def work(_):
        while True:
            n = next(cursor)
            if n >= len(items):
                return
            k, x0, x1 = items[n]
            i, y0, band = bands[k]
            if textures is None:
                # the piece as its own 4-texel-high image
                piece = np.ascontiguousarray(bufs[k][:, x0:x1])
                pw = x1 - x0
                if kind == "reference":
                    o = np.zeros(pw * 4, dtype=np.uint8)
                    enc.lib.ref_compress(O._ptr(piece), O._ptr(o), pw, 4, 0, 0, pw, 4, steps, 0xFF, 0)
                else:
                    o = enc.compress(piece, steps=steps, seed=ANNEAL_SEED)
                outs[k][x0 * 4:x1 * 4] = o
            else:
                # the piece inside its texture: row y0, texels [x0, x1)
                tex = textures[i]
                w = tex.shape[1]
                if y0 > 0:
                    o = enc.compress(tex, steps=steps, seed=ANNEAL_SEED, rect=(x0, y0, x1, y0),
                                     state=np.array([0, prior[(k, x0)]], np.uint32),
                                     out=texture_out(i, tex.shape[0] * w))
                    outs[k][x0 * 4:x1 * 4] = o[y0 * w + x0 * 4:y0 * w + x1 * 4]
                else:
                    # the first block row: the texture cut to that row and to
                    # x1 (a rect cannot end on row 0; the blocks keep their
                    # coordinates, which seed the annealing)
                    head = np.ascontiguousarray(tex[:4, :x1])
                    o = enc.compress(head, steps=steps, seed=ANNEAL_SEED, rect=(x0, 0, 0, 0),
                                     state=np.array([0, prior[(k, x0)]], np.uint32))
                    outs[k][x0 * 4:x1 * 4] = o[x0 * 4:x1 * 4]

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(threads)))
    return time.perf_counter() - t0, outs


def band_texels(bands) -> int:
    return sum(b[2].shape[0] * b[2].shape[1] for b in bands)


def run_cpu_baseline(textures=None):
    """The oracle port on all host cores over the row sample; also FasTC's
    work on that sample in its own unit, texel-bucket evaluations of
    QuantizedError (the port runs FasTC's search, so it counts them)."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    bands = band_sample()
    px = band_texels(bands)
    O.Port().qe_counters(reset=True)
    dt, outs = encode_bands(bands, cores, "port", textures)
    calls, evals = O.Port().qe_counters(reset=True)
    return {"value": px / dt / 1e6, "unit": "MPix/s", "cores": cores, "kind": "port",
            "sample": f"every {BAND_STRIDE}th block row of the set: {len(bands)} rows, {px} texels, "
                      f"q50, one pass",
            "host_cpus": host_cpus(),
            "qe_calls_per_block": calls / (px / 16), "qe_evaluations_per_block": evals / (px / 16)}, bands, outs


def host_cpus() -> dict:
    """What the host grants this process: CPUs in its affinity mask and the
    cgroup CPU quota, if any (the CPU legs' speed depends on both)."""
    info = {"cpu_count": os.cpu_count()}
    try:
        info["affinity"] = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        pass
    try:
        with open("/sys/fs/cgroup/cpu.max") as f:
            quota, period = f.read().split()[:2]
        info["cgroup_cpus"] = None if quota == "max" else int(quota) / int(period)
    except (OSError, ValueError):
        pass
    return info


def reference_impl(args):
    """--impl reference: FasTC's CPU encoder on the host cores (the in-place
    reference build where it exists, else the oracle port)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    bands = band_sample()
    px = band_texels(bands)
    cores = os.cpu_count() or 1
    kind = "port"
    if os.path.exists(O.REF_SO):
        try:
            O.Reference()
            kind = "reference"
        except OSError:
            kind = "port"
    for _ in range(args.warmup):
        encode_bands(bands, cores, kind)
    times = [encode_bands(bands, cores, kind)[0] for _ in range(args.steps)]
    dt = sum(times) / len(times)
    v = px / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "MPix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "texture_set_512_q50", "sample_rows": len(bands), "texels": px,
                   "steps_q": STEPS_Q},
        "cpu_baseline": {"value": v, "unit": "MPix/s", "cores": cores, "kind": kind,
                         "sample": f"every {BAND_STRIDE}th block row of the set: {len(bands)} rows, "
                                   f"{px} texels per step", "host_cpus": host_cpus()},
        "e2e": {"value": v, "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def calibrate_cpu(args):
    """--calibrate-cpu (where FasTC's encoder is built in place, oracle/_ref):
    FasTC's own encoder and the oracle port on the same sampled rows and
    thread count, `--steps` passes each after `--warmup`; prints both rates
    and their ratio, which says how far the port's speed stands for
    FasTC's on the GPU machine, where only the port exists."""
    from oracle import oracle as O

    if not os.path.exists(O.REF_SO):
        print(json.dumps({"calibrate_cpu": "unavailable", "why": "oracle/_ref not built here"}))
        return
    bands = band_sample()
    px = band_texels(bands)
    threads = args.threads or (os.cpu_count() or 1)
    res = {}
    for kind in ("reference", "port"):
        for _ in range(args.warmup):
            encode_bands(bands, threads, kind)
        ts = [encode_bands(bands, threads, kind)[0] for _ in range(args.steps)]
        res[kind] = px / statistics.median(ts) / 1e6
    print(json.dumps({"calibrate_cpu": {"reference_mpix_s": res["reference"], "port_mpix_s": res["port"],
                                        "port_over_reference": res["port"] / res["reference"],
                                        "threads": threads, "passes": args.steps, "texels": px,
                                        "rows": len(bands), "steps_q": STEPS_Q}}))


def cpu_configs(args):
    """--cpu-configs: the CPU encoder (FasTC's own where oracle/_ref is built
    here, else the port) on each configuration, all host threads unless
    --threads: config 1 (256x256 gradient, q0, also on 1 thread), config 2
    (2048x2048 tile mix, q50), config 3 (the texture set's row sample, q50)
    and config 5 (rows 3840..3903 of the 8192x8192 radial-alpha image,
    q100). Threads take block rows in turn, as tc -t N splits an image.
    One JSON line of MPix/s."""
    import numpy as np

    from fastc_gb300 import synth
    from oracle import oracle as O

    kind = "reference" if os.path.exists(O.REF_SO) else "port"
    threads = args.threads or (os.cpu_count() or 1)

    def rows_of(img):
        h = img.shape[0]
        return [(0, y, np.ascontiguousarray(img[y:y + 4])) for y in range(0, h, 4)]

    def rate(bands, steps, nthreads):
        dt, _ = encode_bands(bands, nthreads, kind, steps=steps)
        return band_texels(bands) / dt / 1e6

    c1 = rows_of(synth.gradient_noise_alpha_ramp(1, 256, 256))
    out = {"kind": kind, "threads": threads,
           "c1_256_q0_t1": rate(c1, 0, 1), "c1_256_q0": rate(c1, 0, threads),
           "c2_2048_q50": rate(rows_of(synth.tile_mix(2, 2048, 2048)), 50, threads),
           "c3_row_sample_q50": rate(band_sample(), 50, threads),
           "c5_rows_3840_3903_q100": rate(rows_of(synth.tile_mix_radial_alpha(5, 8192, 64, 0, 3840)), 100,
                                          threads)}
    print(json.dumps({"cpu_configs": out}))


def max_over_ranks(seconds: float, dist, device: str) -> float:
    """The job's time: the slowest replica's (all ranks take part)."""
    if dist is None:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mpix_s(texels_per_replica: int, world: int, steps: int, seconds: float) -> float:
    """Whole-job throughput: every rank encodes its own replica of the set."""
    return texels_per_replica * world * steps / seconds / 1e6


SERVE_SEED = 11


def _gen_serve(args):
    from fastc_gb300 import synth

    i, w, h = args
    return synth.tile_mix(SERVE_SEED * 1000 + i, w, h)


def serve_pool(npool: int = 48):
    """The seeded texture pool the serving requests draw from (sides
    log-uniform in 32..4096, multiples of 4), generated on host processes."""
    import numpy as np

    rng = np.random.default_rng(SERVE_SEED)
    sides = [(int(4 * round(32 * (128 ** rng.random()) / 4)), int(4 * round(32 * (128 ** rng.random()) / 4)))
             for _ in range(npool)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        return pool.map(_gen_serve, [(i, w, h) for i, (w, h) in enumerate(sides)], chunksize=1)


def serve_sweep(imgs, rates, seconds: float):
    """The request server under Poisson arrivals at each rate for `seconds`
    (q from {0, 16, 50} w.p. {0.3, 0.4, 0.3}, 8 GB budget, 3 batches in
    flight): per rate the offered and the served MPix/s (texels over the
    time from the first arrival to the last completion), p50/p99 latency.
    The requests' texels are in page-locked host memory (as a server that
    receives into registered buffers has them), so the uploads are DMA
    copies that do not hold the server's worker thread."""
    import numpy as np
    import torch

    from fastc_gb300 import CompressionSettings
    from fastc_gb300.serve import Server

    pinned = [torch.from_numpy(np.ascontiguousarray(im)).pin_memory() for im in imgs]
    imgs = [t.numpy() for t in pinned]

    rng = np.random.default_rng(SERVE_SEED + 1)
    qs = [0, 16, 50]
    with Server(memory_budget=8 << 30) as srv:  # warm the device (tables, allocator)
        srv.wait(srv.submit(imgs[0], CompressionSettings(num_simulated_annealing_steps=0)))
    mean_px = float(np.mean([im.shape[0] * im.shape[1] for im in imgs]))
    results = []
    for rate in rates:
        n = max(8, int(rate * seconds))
        picks = rng.integers(0, len(imgs), n)
        qsel = rng.choice(qs, size=n, p=[0.3, 0.4, 0.3])
        gaps = rng.exponential(1.0 / rate, n)
        with Server(memory_budget=8 << 30, max_inflight=3) as srv:
            reqs = []
            t0 = time.perf_counter()
            due = t0
            for k in range(n):
                due += gaps[k]
                wait = due - time.perf_counter()
                if wait > 0:
                    time.sleep(wait)
                reqs.append(srv.submit(imgs[picks[k]],
                                       CompressionSettings(num_simulated_annealing_steps=int(qsel[k]),
                                                           seed=k)))
            t_sub = time.perf_counter() - t0
            for r in reqs:
                srv.wait(r)
            dt = time.perf_counter() - t0
            st = srv.stats()
        px = sum(imgs[i].shape[0] * imgs[i].shape[1] for i in picks)
        results.append({"rate_per_s": rate, "requests": n, "offered_mpix_s": rate * mean_px / 1e6,
                        "submitted_in_s": t_sub, "mpix_s": px / dt / 1e6,
                        "p50_ms": st["p50_latency_ms"], "p99_ms": st["p99_latency_ms"],
                        "batches": st["batches"], "peak_bytes": st["peak_bytes"]})
    return results


def serve_bench(args):
    """--serve: the request server under a Poisson stream of requests (sides
    log-uniform in 32..4096 rounded to multiples of 4, q drawn from
    {0, 16, 50} with probabilities {0.3, 0.4, 0.3}, 8 GB device budget) at a
    sweep of arrival rates. Prints one JSON line with p50/p99 latency and
    MP/s per rate. Textures come from a pool of seeded images that requests
    draw from."""
    imgs = serve_pool()
    import torch

    torch.cuda.init()
    results = serve_sweep(imgs, [float(r) for r in args.serve_rates.split(",")], args.serve_seconds)
    print(json.dumps({"metric": "BC7 serving: p50/p99 latency and MPix/s under Poisson arrivals",
                      "config": {"workload": "poisson_mixed_q_8gb", "sides": "log-uniform 32..4096",
                                 "q": "{0,16,50} w.p. {0.3,0.4,0.3}", "budget_bytes": 8 << 30,
                                 "texture_pool": len(imgs), "request_buffers": "page-locked"},
                      "sweep": results}))


def _gen_stripe(args):
    from fastc_gb300 import synth

    y0, rows = args
    return synth.tile_mix_radial_alpha(5, 8192, rows, 0, y0)


def config5_image():
    """The 8192x8192 radial-alpha image of the large q100 configuration,
    generated as 16 stripes on host processes."""
    import numpy as np

    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, min(8, os.cpu_count() or 1))) as pool:
        parts = pool.map(_gen_stripe, [(512 * k, 512) for k in range(16)], chunksize=1)
    return np.concatenate(parts, axis=0)


def single_launch(img, steps: int, warmup: int, reps: int):
    """One texture encoded by one device-memory call per launch (inputs
    resident): MPix/s by CUDA events over `reps` launches, the blocks, and
    their PSNR computed on the GPU."""
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, compress_jobs, psnr

    h, w = img.shape[:2]
    din = torch.from_numpy(img).cuda()
    dout = torch.zeros(w * h, dtype=torch.uint8, device="cuda")
    job = CompressionJob(din, dout, w, h)
    st = CompressionSettings(num_simulated_annealing_steps=steps, seed=ANNEAL_SEED)
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        compress_jobs([job], st)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        compress_jobs([job], st)
    e1.record(stream)
    torch.cuda.synchronize()
    dt = e0.elapsed_time(e1) / 1e3 / reps
    return w * h / dt / 1e6, dt, din, dout, psnr(dout, din, w, h)


def dxt_bench(imgs, din, hin, c2_img, reps: int = 5, clocks=None):
    """DXT1 and DXT5 (FasTC's CompressImageDXT1 / DXT5) over the texture set:
    device-resident jobs through fastc_dxt_compress_device (launches of up
    to 32 jobs), timed by CUDA events over `reps` passes; the same set end
    to end through the batched host-memory entry point (pinned buffers,
    copies included); parity of every texture against the GPU's
    own device path and of a band of the 2048x2048 tile mix against the
    oracle, which is also timed on one host core for the CPU figure."""
    import ctypes as C

    import numpy as np
    import torch

    from fastc_gb300 import CompressionFormat, CompressionJob
    from fastc_gb300._lib import Job, check, load
    from oracle import oracle as O

    lib = load()
    stream = torch.cuda.current_stream()
    total_px = sum(im.shape[0] * im.shape[1] for im in imgs)
    blocks = total_px // 16
    peak, peak_kind = measured_peaks()
    # warp instructions per block of each format's encode kernel, from the
    # committed launch list of this workload (one ncu pass)
    try:
        with open(os.path.join(ROOT, "profiles", "dxt_encode_texture_set_512.json")) as f:
            dxt_ipb = {k: float(v["warp_instructions_per_block"]) for k, v in json.load(f)["formats"].items()}
    except Exception:
        dxt_ipb = {}
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    # the host link's own rates (one 256 MB page-locked buffer copied up and
    # down by cudaMemcpyAsync, 3 times each): the end-to-end figures below
    # move the texels up and the blocks down across this link
    link = {}
    hbuf = torch.empty(256 << 20, dtype=torch.uint8).pin_memory()
    dbuf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for name, fn in (("h2d_gb_s", lambda: dbuf.copy_(hbuf, non_blocking=True)),
                     ("d2h_gb_s", lambda: hbuf.copy_(dbuf, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(3):
            fn()
        t1.record(stream)
        torch.cuda.synchronize()
        link[name] = 3 * hbuf.numel() / (t0.elapsed_time(t1) / 1e3) / 1e9
    del hbuf, dbuf
    port = O.Port()
    band = np.ascontiguousarray(c2_img[:256])
    res = {"workload": "texture_set_512", "texels": total_px, "blocks": blocks,
           "l2": "inputs 462 MB > L2, no flush",
           "host_link": dict(link, note="cudaMemcpyAsync of one 256 MB page-locked buffer")}
    for fmt in (CompressionFormat.DXT1, CompressionFormat.DXT5):
        bsz = 8 if fmt == CompressionFormat.DXT1 else 16
        outs = [torch.zeros(im.shape[0] * im.shape[1] * bsz // 16, dtype=torch.uint8, device="cuda")
                for im in imgs]
        jobs = [CompressionJob(a, o, im.shape[1], im.shape[0], format=fmt) for a, o, im in zip(din, outs, imgs)]
        jarr = (Job * len(jobs))(*[j.to_c() for j in jobs])

        def launch():
            check(lib.fastc_dxt_compress_device(jarr, len(jobs), int(fmt), C.c_void_p(stream.cuda_stream)),
                  "fastc_dxt_compress_device")

        for _ in range(3):
            launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            launch()
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3 / reps
        # end to end: pinned host buffers, the whole set in one batched call
        houts = [torch.zeros(im.shape[0] * im.shape[1] * bsz // 16, dtype=torch.uint8).pin_memory()
                 for im in imgs]
        hj = (Job * len(imgs))(*[CompressionJob(a.numpy(), o.numpy(), im.shape[1], im.shape[0],
                                                format=fmt).to_c() for a, o, im in zip(hin, houts, imgs)])
        check(lib.fastc_dxt_compress_batch(hj, len(imgs), int(fmt)), "fastc_dxt_compress_batch")
        e2e_reps = 3
        t0 = time.perf_counter()
        for _ in range(e2e_reps):
            check(lib.fastc_dxt_compress_batch(hj, len(imgs), int(fmt)), "fastc_dxt_compress_batch")
        e2e_dt = (time.perf_counter() - t0) / e2e_reps
        same = all(np.array_equal(h.numpy(), o.cpu().numpy()) for h, o in zip(houts, outs))
        # the oracle on one core: a 2048x256 band of the 2048x2048 tile mix
        t0 = time.perf_counter()
        want = port.dxt_compress(band, fmt == CompressionFormat.DXT5)
        cpu_dt = time.perf_counter() - t0
        got = np.zeros(band.shape[0] * band.shape[1] * bsz // 16, np.uint8)
        bj = CompressionJob(band, got, band.shape[1], band.shape[0], format=fmt).to_c()
        check(lib.fastc_dxt_compress(C.byref(bj), int(fmt)), "fastc_dxt_compress")
        algo = (64 + bsz) * blocks
        res[fmt.name.lower()] = {
            "mpix_s": total_px / dt / 1e6, "ms_per_pass": dt * 1e3, "launches_per_pass": (len(jobs) + 31) // 32,
            "roofline": {"bound": "hbm", "achieved": algo / dt / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / dt / 1e9 / peak, "peak_source": peak_kind,
                         "algorithmic_bytes_per_block": 64 + bsz},
            "e2e": {"value": total_px / e2e_dt / 1e6, "unit": "MPix/s", "h2d_bytes_per_step": total_px * 4,
                    "d2h_bytes_per_step": blocks * bsz, "entry": "fastc_dxt_compress_batch, pinned buffers",
                    "copy_gb_s": (total_px * 4 + blocks * bsz) / e2e_dt / 1e9,
                    # the time the link alone needs (texels up and blocks
                    # down, the two directions concurrent) over the measured
                    "frac_of_link_bound": max(total_px * 4 / (link["h2d_gb_s"] * 1e9),
                                              blocks * bsz / (link["d2h_gb_s"] * 1e9)) / e2e_dt},
            "host_equals_device": bool(same),
            "cpu_port_1core_mpix_s": band.shape[0] * band.shape[1] / cpu_dt / 1e6,
            "band_equals_oracle": bool(np.array_equal(got, want)),
        }
        ipb = dxt_ipb.get(fmt.name.lower())
        if ipb:
            # the encoder is issue-bound: warp instructions per block x
            # blocks/s against 4 schedulers x SMs x the SM clock
            issued = ipb * blocks / dt
            res[fmt.name.lower()]["issue_roofline"] = {
                "achieved": issued, "peak": 4.0 * sms * mhz * 1e6, "unit": "warp-inst/s",
                "frac": issued / (4.0 * sms * mhz * 1e6), "instructions_per_block": ipb,
                "sms": sms, "sm_mhz": mhz}
        del outs
    return res


def fasTC_full_size_psnr(name: str):
    """FasTC's mean PSNR over its pinned seeds for a full-size fixture."""
    with open(os.path.join(ROOT, "tests", "golden", "manifest.json")) as f:
        case = json.load(f)["full_size"][name]
    return sum(case["psnr"]) / len(case["psnr"])


def profile_set(args):
    """The 512-texture set, device-resident, encoded `case_repeat` times per
    format (DXT1 then DXT5 for --case-format dxt): the bench's own DXT
    launches, for ncu captures of that workload."""
    import torch

    from fastc_gb300 import CompressionFormat, CompressionJob, dxt

    imgs = make_texture_set(min(16, os.cpu_count() or 1))
    fmts = ["dxt1", "dxt5"] if args.case_format == "dxt" else [args.case_format]
    if "bptc" in fmts:
        raise SystemExit("the texture-set case covers DXT1 / DXT5 (the BC7 step is bench.py itself)")
    din = [torch.from_numpy(im).cuda() for im in imgs]
    px = sum(im.shape[0] * im.shape[1] for im in imgs)
    for name in fmts:
        fmt = CompressionFormat[name.upper()]
        bsz = 8 if fmt == CompressionFormat.DXT1 else 16
        outs = [torch.zeros(im.shape[0] * im.shape[1] * bsz // 16, dtype=torch.uint8, device="cuda")
                for im in imgs]
        jobs = [CompressionJob(a, o, im.shape[1], im.shape[0], format=fmt) for a, o, im in zip(din, outs, imgs)]
        for _ in range(args.case_repeat):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dxt.compress_dxt_jobs(jobs)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            print(f"texture_set_512 {fmt.name}: {dt * 1e3:.3f} ms, {px / dt / 1e6:.1f} MPix/s")
        del outs


def profile_case(args):
    """One seeded texture encoded `case_repeat` times (for ncu captures)."""
    if args.case_kind == "texture_set":
        profile_set(args)
        return
    n = args.case_size
    from fastc_gb300 import synth

    if args.case_kind == "tile_mix":
        img = synth.tile_mix(21, n, n)
    elif args.case_kind == "radial":
        img = synth.tile_mix_radial_alpha(5, n, n, 0, 0, n, n)
    else:
        img = synth.gradient_noise_alpha_ramp(1, n, n)
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, compress, set_launch_shape

    from fastc_gb300 import CompressionFormat, dxt, set_engine

    set_engine(args.case_engine)
    set_launch_shape(args.case_warps, 0)
    if args.case_format == "dxt":
        raise SystemExit("--case-format dxt (both formats) is for --case-kind texture_set")
    fmt = CompressionFormat[args.case_format.upper()]
    din = torch.from_numpy(img).cuda()
    dout = torch.zeros(n * n * (8 if fmt == CompressionFormat.DXT1 else 16) // 16, dtype=torch.uint8,
                       device="cuda")
    s = CompressionSettings(num_simulated_annealing_steps=args.case_steps, seed=1)
    job = CompressionJob(din, dout, n, n, format=fmt)
    what = f"q{args.case_steps}" if fmt == CompressionFormat.BPTC else fmt.name
    for _ in range(args.case_repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if fmt == CompressionFormat.BPTC:
            compress(job, s)
        else:
            dxt.compress_dxt_jobs([job])
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print(f"{args.case_kind} {n}x{n} {what}: {dt * 1e3:.2f} ms, {n * n / dt / 1e6:.2f} MPix/s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the config-2, config-5 and serving measurements")
    ap.add_argument("--calibrate-cpu", action="store_true",
                    help="time FasTC's own encoder (oracle/_ref) against the port on the CPU sample")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="time the CPU encoder on each configuration (MPix/s)")
    ap.add_argument("--threads", type=int, default=0,
                    help="host threads of --calibrate-cpu and --cpu-configs")
    ap.add_argument("--serve", action="store_true", help="run the serving sweep instead")
    ap.add_argument("--serve-rates", default="20,60,120")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--profile-case", action="store_true",
                    help="encode one texture --case-repeat times (for ncu captures)")
    ap.add_argument("--case-kind", default="tile_mix",
                    choices=["tile_mix", "radial", "gradient", "texture_set"])
    ap.add_argument("--case-size", type=int, default=4096)
    ap.add_argument("--case-steps", type=int, default=50)
    ap.add_argument("--case-format", default="bptc", choices=["bptc", "dxt1", "dxt5", "dxt"])
    ap.add_argument("--case-repeat", type=int, default=1)
    ap.add_argument("--case-engine", type=int, default=0,
                    help="0: pipeline engine, 1: warp-per-block engine")
    ap.add_argument("--case-warps", type=int, default=0,
                    help="warps per CTA of the warp-per-block engine (0: keep)")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    if args.impl == "reference":
        reference_impl(args)
        return
    if args.calibrate_cpu:
        calibrate_cpu(args)
        return
    if args.cpu_configs:
        cpu_configs(args)
        return
    if args.serve:
        serve_bench(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    # host work (texture generation) before the first GPU call
    imgs = make_texture_set(min(16, os.cpu_count() or 1))
    extras = rank == 0 and not args.no_extras
    if extras:
        from fastc_gb300 import synth

        c2_img = synth.tile_mix(2, 2048, 2048)
        c5_img = config5_image()
        pool = serve_pool()

    import numpy as np
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, Plan, compress_jobs

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    settings = CompressionSettings(num_simulated_annealing_steps=STEPS_Q, seed=ANNEAL_SEED)
    total_px = sum(im.shape[0] * im.shape[1] for im in imgs)
    total_blocks = total_px // 16
    din = [torch.from_numpy(im).cuda() for im in imgs]
    dout = [torch.zeros(im.shape[0] * im.shape[1], dtype=torch.uint8, device="cuda") for im in imgs]
    jobs = [CompressionJob(a, b, im.shape[1], im.shape[0]) for a, b, im in zip(din, dout, imgs)]
    plan = Plan(jobs, settings)
    stream = torch.cuda.current_stream()
    tuning = plan.autotune(stream, launches=2)  # outside the timed region

    # --- batched: one graph launch per step ---
    for _ in range(args.warmup):
        plan.launch()
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local_rank) as clocks:
        torch.cuda.nvtx.range_push("timed_steps")  # lets ncu --nvtx-include pick these launches
        ev[0].record(stream)
        for k in range(args.steps):
            plan.launch()
            ev[k + 1].record(stream)
        barrier()
        torch.cuda.nvtx.range_pop()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    dt = sum(step_ms) / 1e3
    dt = max_over_ranks(dt, dist, "cuda")
    value = aggregate_mpix_s(total_px, world, args.steps, dt)
    flags = plan.flags()

    # --- plain: one encode call per texture ---
    def plain_pass(subset):
        for j in subset:
            compress_jobs([j], settings)

    plain_pass(jobs)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plain_pass(jobs)
    e1.record(stream)
    barrier()
    plain_dt = e0.elapsed_time(e1) / 1e3
    plain_value = total_px / plain_dt / 1e6
    ref_blocks = [d.clone() for d in dout]

    # small textures: batched plan over the small subset vs plain loop
    small = [i for i, im in enumerate(imgs) if im.shape[0] * im.shape[1] <= SMALL_PIXELS]
    small_px = sum(imgs[i].shape[0] * imgs[i].shape[1] for i in small)
    small_plan = Plan([jobs[i] for i in small], settings)
    small_tuning = small_plan.autotune(stream, launches=3)  # outside the timed region
    for _ in range(3):
        small_plan.launch()
    barrier()
    e0.record(stream)
    reps = 20
    for _ in range(reps):
        small_plan.launch()
    e1.record(stream)
    barrier()
    small_batched = small_px * reps / (e0.elapsed_time(e1) / 1e3) / 1e6
    small_identical = all(torch.equal(dout[i], ref_blocks[i]) for i in small)
    plain_pass([jobs[i] for i in small])
    barrier()
    e0.record(stream)
    plain_pass([jobs[i] for i in small])
    e1.record(stream)
    barrier()
    small_plain = small_px / (e0.elapsed_time(e1) / 1e3) / 1e6

    # batched == plain, bit for bit
    plan.launch()
    barrier()
    identical = all(torch.equal(a, b) for a, b in zip(ref_blocks, dout))

    # --- e2e through the host-memory C ABI, pinned buffers ---
    hin = [torch.from_numpy(im).pin_memory() for im in imgs]
    hout = [torch.zeros(im.shape[0] * im.shape[1], dtype=torch.uint8).pin_memory() for im in imgs]
    hjobs = [CompressionJob(a.numpy(), b.numpy(), im.shape[1], im.shape[0]) for a, b, im in zip(hin, hout, imgs)]
    compress_jobs(hjobs, settings)
    e2e_steps = max(1, min(args.steps, 3))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        compress_jobs(hjobs, settings)
    barrier()
    e2e_dt = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e_value = aggregate_mpix_s(total_px, world, e2e_steps, e2e_dt)
    e2e_identical = all(np.array_equal(h.numpy(), d.cpu().numpy()) for h, d in zip(hout, dout))

    # --- PSNR of the batched output (FasTC's metric, on the GPU) ---
    from fastc_gb300 import psnr as gpu_psnr

    sse = 0.0
    for a, blk, im in zip(din, dout, imgs):
        sse += float(gpu_psnr(blk, a, im.shape[1], im.shape[0], block_sse=True)[1].sum())
    psnr = 10 * np.log10(3 * 255.0 ** 2 / (sse / total_px))

    peak, peak_kind = measured_peaks()
    step_s = dt / args.steps
    algo_bytes = 80.0 * total_blocks  # 64 B of texels in + 16 B of block out
    achieved = algo_bytes / step_s / 1e9
    tpb, ipb = profile_per_block()

    line = {
        "metric": METRIC, "value": value, "unit": "MPix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "texture_set_512_q50", "textures": len(imgs), "texels": total_px,
                   "blocks": total_blocks, "steps_q": STEPS_Q, "seed": ANNEAL_SEED,
                   "l2": "inputs 462 MB > L2, no flush", "parallelism": f"replica x{world}",
                   "autotuned": tuning},
        "plain_mpix_s": plain_value, "batched_over_plain": value / world / plain_value,
        "small_textures": {"count": len(small), "texels": small_px, "autotuned": small_tuning,
                           "batched_mpix_s": small_batched,
                           "plain_mpix_s": small_plain, "batched_over_plain": small_batched / small_plain,
                           "batched_equals_plain": bool(small_identical)},
        "batched_equals_plain": bool(identical), "psnr_db": psnr, "device_flags": flags,
        "e2e": {"value": e2e_value, "unit": "MPix/s", "h2d_bytes_per_step": total_px * 4,
                "d2h_bytes_per_step": total_blocks * 16, "identical_to_device_path": bool(e2e_identical)},
        "gpu_launches": plan.kernels() * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (tpb * total_blocks) if tpb else None,
                     "note": "issue-bound integer/FP32 search: the annealing kernels issue on 73 % of "
                             "cycles with the ALU pipe 61 % busy, the setup kernels are latency-bound "
                             "(43 % issue), while HBM traffic stays under 1 % of peak; traffic (ncu, "
                             "per block of a 4096x4096 tile-mix launch, scaled to the set's blocks) "
                             "counts the stages' fit state exchanged through HBM and the setup "
                             "kernels' spills; issue_roofline takes the warp instructions per block "
                             "from the launch list of this workload's timed step"},
        "clocks": clocks.summary(),
    }
    if ipb:
        # compute roofline of the issue-bound encoder: warp instructions per
        # block (ncu, committed summary) x blocks/s (this run) against
        # 4 schedulers x SMs x the SM clock seen during the timed region
        cs = line["clocks"]
        mhz = cs.get("sm_mhz") or cs.get("sm_max_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        issued = ipb * total_blocks / step_s
        peak_issue = 4.0 * sms * mhz * 1e6
        line["issue_roofline"] = {"achieved": issued, "peak": peak_issue, "unit": "warp-inst/s",
                                  "frac": issued / peak_issue,
                                  "instructions_per_block": ipb, "sms": sms, "sm_mhz": mhz}
    if rank == 0 and not args.no_cpu_baseline:
        cb, bands, outs = run_cpu_baseline(imgs)
        # same bytes as the GPU on the sampled rows
        cb["identical_to_gpu"] = all(
            np.array_equal(o, dout[i][y0 * imgs[i].shape[1]:(y0 + 4) * imgs[i].shape[1]].cpu().numpy())
            for o, (i, y0, _) in zip(outs, bands))
        line["cpu_baseline"] = cb
        # FasTC's work unit: QuantizedError texel-bucket evaluations (20
        # ops each) per block, counted by the port on the sample, delivered
        # at the GPU's block rate, against one op per lane per cycle
        cs = line["clocks"]
        mhz = cs.get("sm_mhz") or cs.get("sm_max_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        ops = cb["qe_evaluations_per_block"] * 20.0 * total_blocks / step_s
        peak_ops = sms * 128 * mhz * 1e6
        line["work_roofline"] = {
            "unit": "ops/s", "achieved": ops, "peak": peak_ops, "frac": ops / peak_ops,
            "evaluations_per_block": cb["qe_evaluations_per_block"], "ops_per_evaluation": 20,
            "note": "reference-equivalent work: FasTC's QuantizedError texel-bucket evaluations per "
                    "block (counted by the oracle port, which runs FasTC's search, on the CPU sample) "
                    "x 20 ops x the GPU's blocks/s, against SMs x 128 lanes x the SM clock; the GPU "
                    "does fewer evaluations than this (pruned annealing, each distinct subset "
                    "estimated once, integer candidate pairs), so the fraction reads the useful "
                    "work rate in FasTC's units, not the GPU's own instruction rate "
                    "(issue_roofline)"}
    plan.close()
    small_plan.close()
    if extras:
        line["dxt"] = dxt_bench(imgs, din, hin, c2_img, clocks=line["clocks"])
        del din, dout, hin, hout
        torch.cuda.empty_cache()
        # config 2: one 2048x2048 tile-mix texture at q50 in one launch
        mps, dt2, d_in, d_out, db = single_launch(c2_img, STEPS_Q, 2, 3)
        ref_db = fasTC_full_size_psnr("c2_tile2048_q50")
        line["config2"] = {"workload": "tile_mix_2048x2048_q50", "mpix_s": mps, "ms_per_launch": dt2 * 1e3,
                           "psnr_db": db, "psnr_fasTC_db": ref_db, "psnr_delta_db": db - ref_db}
        del d_in, d_out
        # config 5: one 8192x8192 radial-alpha texture at q100 in one launch
        with ClockSampler(local_rank) as c5_clocks:
            mps, dt5, d_in, d_out, db = single_launch(c5_img, 100, 1, 2)
        stripe = gpu_psnr(d_out[3840 * 8192:4352 * 8192], d_in[3840:4352], 8192, 512)
        ref_db = fasTC_full_size_psnr("c5_stripe8192x512_q100")
        line["config5"] = {"workload": "radial_alpha_8192x8192_q100", "mpix_s": mps, "ms_per_launch": dt5 * 1e3,
                           "psnr_db": db, "stripe_rows_3840_4351_psnr_db": stripe,
                           "stripe_psnr_fasTC_db": ref_db, "stripe_psnr_delta_db": stripe - ref_db,
                           "clocks": c5_clocks.summary()}
        del d_in, d_out
        torch.cuda.empty_cache()
        # serving: Poisson arrivals below and above saturation
        sweep = serve_sweep(pool, [60.0, 2000.0], 2.0)
        line["serve"] = {"workload": "poisson_mixed_q_8gb", "sides": "log-uniform 32..4096",
                         "q": "{0,16,50} w.p. {0.3,0.4,0.3}", "request_buffers": "page-locked",
                         "sweep": sweep,
                         "max_sustained_mpix_s": sweep[-1]["mpix_s"], "p99_ms_at_max": sweep[-1]["p99_ms"],
                         "saturated": sweep[-1]["offered_mpix_s"] > sweep[-1]["mpix_s"]}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
