"""Encode one small seeded texture on the GPU, for profiling one launch.

    python -m fastc_gb300.profile_case [--kind tile_mix|radial|gradient]
        [--size 256] [--steps 50] [--repeat 2]

Each repeat is one encode of the whole texture through the device-memory
C ABI (classify, scan and encode kernels), so
``ncu -k regex:encode_kernel -s 1 -c 1`` captures one steady-state launch.
"""
from __future__ import annotations

import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kind", default="tile_mix", choices=["tile_mix", "radial", "gradient"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--warps", type=int, default=0, help="warps per CTA (1, 2, 4, 8)")
    ap.add_argument("--ctas-per-sm", type=int, default=0)
    args = ap.parse_args()
    import torch

    from . import CompressionJob, CompressionSettings, compress, set_launch_shape, synth

    set_launch_shape(args.warps, args.ctas_per_sm)

    n = args.size
    if args.kind == "tile_mix":
        img = synth.tile_mix(21, n, n)
    elif args.kind == "radial":
        img = synth.tile_mix_radial_alpha(5, n, n, 0, 0, n, n)
    else:
        img = synth.gradient_noise_alpha_ramp(1, n, n)
    din = torch.from_numpy(img).cuda()
    dout = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
    s = CompressionSettings(num_simulated_annealing_steps=args.steps, seed=1)
    job = CompressionJob(din, dout, n, n)
    for _ in range(args.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        compress(job, s)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print(f"{args.kind} {n}x{n} q{args.steps}: {dt * 1e3:.2f} ms, {n * n / dt / 1e6:.2f} MPix/s")


if __name__ == "__main__":
    main()
