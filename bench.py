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
    """DRAM bytes and warp instructions per block of one encode launch, from
    the committed ncu summary (profiles/bc7_encode_traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "bc7_encode_traffic.json")) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_block"]), float(d["warp_instructions_per_block"])
    except Exception:
        return None, None


def cpu_sample(imgs, budget_px: int):
    """Deterministic sample: textures in set order until the pixel budget."""
    out, px = [], 0
    for im in imgs:
        if px + im.shape[0] * im.shape[1] > budget_px and out:
            continue
        out.append(im)
        px += im.shape[0] * im.shape[1]
        if px >= budget_px:
            break
    return out, px


def run_cpu_baseline(imgs, budget_px: int):
    from oracle import oracle as O

    port = O.Port()
    cores = os.cpu_count() or 1
    sample, px = cpu_sample(imgs, budget_px)
    t0 = time.perf_counter()
    outs = [port.compress_mt(im, steps=STEPS_Q, seed=ANNEAL_SEED, threads=cores) for im in sample]
    dt = time.perf_counter() - t0
    return {"value": px / dt / 1e6, "unit": "MPix/s", "cores": cores, "kind": "port",
            "sample": f"{len(sample)} textures of the set, {px} texels, q50, one pass"}, sample, outs


def reference_impl(args):
    """--impl reference: FasTC's CPU encoder on the host cores (the in-place
    reference build where it exists, else the oracle port)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from fastc_gb300 import synth
    from oracle import oracle as O

    sides = synth.texture_sides(SET_SEED, SET_COUNT)
    imgs = [synth.tile_mix(SET_SEED * 1000 + i, w, h) for i, (w, h) in enumerate(sides[:64])]
    sample, px = cpu_sample(imgs, 160_000)
    cores = os.cpu_count() or 1
    kind = "port"
    ref = None
    if os.path.exists(O.REF_SO):
        try:
            ref = O.Reference()
            kind = "reference"
        except OSError:
            ref = None
    port = O.Port()

    def one_pass():
        if ref is not None:
            # tc -t N: N threads on disjoint block ranges of each image
            for im in sample:
                ref.compress_threads(im, steps=STEPS_Q, threads=cores, seed=ANNEAL_SEED)
        else:
            for im in sample:
                port.compress_mt(im, steps=STEPS_Q, seed=ANNEAL_SEED, threads=cores)

    for _ in range(args.warmup):
        one_pass()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        one_pass()
        times.append(time.perf_counter() - t0)
    dt = sum(times) / len(times)
    v = px / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "MPix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "texture_set_512_q50", "textures": len(sample), "texels": px, "steps_q": STEPS_Q},
        "cpu_baseline": {"value": v, "unit": "MPix/s", "cores": cores, "kind": kind,
                         "sample": f"{len(sample)} textures of the set, {px} texels per step"},
        "e2e": {"value": v, "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


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


def serve_bench(args):
    """--serve: the request server under a Poisson stream of requests (sides
    log-uniform in 32..4096 rounded to multiples of 4, q drawn from
    {0, 16, 50} with probabilities {0.3, 0.4, 0.3}, 8 GB device budget) at a
    sweep of arrival rates. Prints one JSON line with p50/p99 latency and
    MP/s per rate. Textures come from a pool of seeded images that requests
    draw from."""
    import numpy as np

    rng = np.random.default_rng(SERVE_SEED)
    npool = 48
    sides = [(int(4 * round(32 * (128 ** rng.random()) / 4)), int(4 * round(32 * (128 ** rng.random()) / 4)))
             for _ in range(npool)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        imgs = pool.map(_gen_serve, [(i, w, h) for i, (w, h) in enumerate(sides)], chunksize=1)

    import torch

    torch.cuda.init()
    from fastc_gb300 import CompressionSettings
    from fastc_gb300.serve import Server

    qs = [0, 16, 50]
    rates = [float(r) for r in args.serve_rates.split(",")]
    results = []
    # warm the device (tables, allocator)
    with Server(memory_budget=8 << 30) as srv:
        srv.wait(srv.submit(imgs[0], CompressionSettings(num_simulated_annealing_steps=0)))
    for rate in rates:
        n = max(8, int(rate * args.serve_seconds))
        picks = rng.integers(0, npool, n)
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
            for r in reqs:
                srv.wait(r)
            dt = time.perf_counter() - t0
            st = srv.stats()
        px = sum(imgs[i].shape[0] * imgs[i].shape[1] for i in picks)
        results.append({"rate_per_s": rate, "requests": n, "mpix": px / 1e6, "mpix_s": px / dt / 1e6,
                        "p50_ms": st["p50_latency_ms"], "p99_ms": st["p99_latency_ms"],
                        "batches": st["batches"], "peak_bytes": st["peak_bytes"]})
    print(json.dumps({"metric": "BC7 serving: p50/p99 latency and MPix/s under Poisson arrivals",
                      "config": {"workload": "poisson_mixed_q_8gb", "sides": "log-uniform 32..4096",
                                 "q": "{0,16,50} w.p. {0.3,0.4,0.3}", "budget_bytes": 8 << 30,
                                 "texture_pool": npool},
                      "sweep": results}))


def profile_case(args):
    """One seeded texture encoded `case_repeat` times (for ncu captures)."""
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

    from fastc_gb300 import set_engine

    set_engine(args.case_engine)
    set_launch_shape(args.case_warps, 0)
    din = torch.from_numpy(img).cuda()
    dout = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
    s = CompressionSettings(num_simulated_annealing_steps=args.case_steps, seed=1)
    job = CompressionJob(din, dout, n, n)
    for _ in range(args.case_repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        compress(job, s)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print(f"{args.case_kind} {n}x{n} q{args.case_steps}: {dt * 1e3:.2f} ms, "
              f"{n * n / dt / 1e6:.2f} MPix/s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget-px", type=int, default=400_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve", action="store_true", help="run the serving sweep instead")
    ap.add_argument("--serve-rates", default="20,60,120")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--profile-case", action="store_true",
                    help="encode one texture --case-repeat times (for ncu captures)")
    ap.add_argument("--case-kind", default="tile_mix", choices=["tile_mix", "radial", "gradient"])
    ap.add_argument("--case-size", type=int, default=4096)
    ap.add_argument("--case-steps", type=int, default=50)
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
    if args.serve:
        serve_bench(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    # host work (texture generation) before the first GPU call
    imgs = make_texture_set(min(16, os.cpu_count() or 1))

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

    # --- PSNR of the batched output (GPU decoder, reference semantics) ---
    from fastc_gb300 import decompress

    mse, npx = 0.0, 0
    for im, blk in zip(imgs, dout):
        dec = decompress(blk, im.shape[1], im.shape[0]).to(torch.float64)
        src = torch.from_numpy(im).cuda().to(torch.float64)
        a0, a1 = src[..., 3:4] / 255.0, dec[..., 3:4] / 255.0
        mse += float(((a0 * src[..., :3] - a1 * dec[..., :3]) ** 2).sum())
        npx += im.shape[0] * im.shape[1]
    psnr = 10 * np.log10(3 * 255.0 ** 2 / (mse / npx))

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
        "small_textures": {"count": len(small), "texels": small_px, "batched_mpix_s": small_batched,
                           "plain_mpix_s": small_plain, "batched_over_plain": small_batched / small_plain},
        "batched_equals_plain": bool(identical), "psnr_db": psnr, "device_flags": flags,
        "e2e": {"value": e2e_value, "unit": "MPix/s", "h2d_bytes_per_step": total_px * 4,
                "d2h_bytes_per_step": total_blocks * 16, "identical_to_device_path": bool(e2e_identical)},
        "gpu_launches": plan.kernels() * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (tpb * total_blocks) if tpb else None,
                     "note": "issue-bound integer/FP32 search: the annealing and select kernels keep "
                             "the ALU pipe 60-69 % busy and the setup kernels are latency-bound, "
                             "while HBM traffic stays under 1 % of peak; traffic counts the stages' "
                             "fit state exchanged through HBM and the setup kernels' spills"},
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
        cb, sample, outs = run_cpu_baseline(imgs, args.cpu_budget_px)
        # same bytes as the GPU on the sample
        idx = [next(i for i, im in enumerate(imgs) if im is s) for s in sample]
        cb["identical_to_gpu"] = all(np.array_equal(o, dout[i].cpu().numpy()) for o, i in zip(outs, idx))
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line))
    plan.close()
    small_plan.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
