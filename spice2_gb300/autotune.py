"""Launch-shape autotuner for the delivery kernel of a network.

The delivery kernel accumulates events per (input slot, target tile) in shared memory; its tile
size, CTA size and work mapping change its speed but never its results (the parity tests run every
shape).  The best shape depends on the network (population sizes, out-degree, firing rate), so it
is measured on the network itself: each candidate runs a stretch of simulation steps with per-kernel
CUDA-event timing, the source populations serialised onto the main stream so the delivery timing
is not shared with the overlapped source kernel.  The simulation state advances during tuning (the
steps are real steps of the network).

usage:  python -m spice2_gb300.autotune --brunel 500000 0.002 [--steps 600]
"""
from __future__ import annotations

import argparse
import itertools
import json
import sys

DEFAULT_CANDIDATES = [
    # (tile bytes, threads per CTA, parts per (slot, tile), work mapping: 0 warp-flattened,
    #  1 thread per spike, 2 warp per spike, 3 thread per spike with 16-byte loads,
    #  4 thread per spike, software-pipelined, 5 / 6 four / eight lanes per spike, 7 as 5 with
    #  at most 32 registers, 8 / 9 four lanes per spike with sub-rows staged in shared memory, two /
    #  four sub-rows in flight per group, 10 / 11 / 12 / 13 as 8 / 9 with sub-rows read as aligned
    #  16-byte blocks: 2 x 64, 4 x 32, 1 x 128 and 2 x 96 targets per group and round trip, 14 as 12
    #  with per-sub-row pointers and target ranges precomputed while staging, 15 / 16 / 17 as 14
    #  reading a 16-bit tile-local copy of the targets, 1 x 256, 4 x 64 and 2 x 128 targets per
    #  group and round trip, 18 / 19 as 15 / 17 storing the finished tile by TMA bulk copies,
    #  20 / 21 as 15 / 17 at two 512-thread CTAs per SM)
    (6 * 1024, 128, 1, 1), (12 * 1024, 128, 1, 1), (24 * 1024, 128, 1, 1), (12 * 1024, 256, 1, 1),
    (24 * 1024, 256, 1, 1), (24 * 1024, 512, 1, 1), (48 * 1024, 512, 1, 1), (24 * 1024, 256, 2, 1),
    (24 * 1024, 256, 1, 0), (12 * 1024, 128, 1, 2), (24 * 1024, 256, 1, 2), (48 * 1024, 512, 1, 3),
    (24 * 1024, 256, 1, 4), (12 * 1024, 128, 1, 4), (12 * 1024, 256, 1, 4), (6 * 1024, 128, 1, 4),
    (24 * 1024, 256, 1, 5), (12 * 1024, 128, 1, 5), (48 * 1024, 256, 1, 5), (24 * 1024, 256, 1, 6),
    (48 * 1024, 256, 1, 6), (48 * 1024, 512, 1, 6), (96 * 1024, 512, 1, 6), (12 * 1024, 128, 1, 3),
    (24 * 1024, 512, 1, 7), (26 * 1024, 512, 1, 7), (28 * 1024, 512, 1, 7), (32 * 1024, 512, 1, 7),
    (16 * 1024, 256, 1, 7), (12 * 1024, 128, 1, 7), (112 * 1024, 1024, 1, 4), (112 * 1024, 1024, 1, 6),
    (128 * 1024, 1024, 1, 6), (24 * 1024, 256, 1, 8), (24 * 1024, 512, 1, 8), (12 * 1024, 256, 1, 8),
    (48 * 1024, 512, 1, 8), (112 * 1024, 1024, 1, 8), (96 * 1024, 1024, 1, 8), (100 * 1024, 1024, 1, 8),
    (104 * 1024, 1024, 1, 8), (108 * 1024, 1024, 1, 8), (104 * 1024, 1024, 1, 6),
    (100 * 1024, 1024, 1, 9), (104 * 1024, 1024, 1, 9), (24 * 1024, 256, 1, 9), (48 * 1024, 512, 1, 9),
    (24 * 1024, 256, 1, 10), (48 * 1024, 512, 1, 10), (80 * 1024, 1024, 1, 10), (96 * 1024, 1024, 1, 10),
    (100 * 1024, 1024, 1, 10), (112 * 1024, 1024, 1, 10), (128 * 1024, 1024, 1, 10), (160 * 1024, 1024, 1, 10),
    (24 * 1024, 256, 1, 11), (48 * 1024, 512, 1, 11), (100 * 1024, 768, 1, 11), (112 * 1024, 768, 1, 11),
    (100 * 1024, 1024, 1, 12), (112 * 1024, 1024, 1, 12), (128 * 1024, 1024, 1, 12), (160 * 1024, 1024, 1, 12),
    (48 * 1024, 512, 1, 12), (100 * 1024, 768, 1, 13), (128 * 1024, 768, 1, 13), (160 * 1024, 768, 1, 13),
    (100 * 1024, 1024, 1, 14), (112 * 1024, 1024, 1, 14), (128 * 1024, 1024, 1, 14), (160 * 1024, 1024, 1, 14),
    (48 * 1024, 512, 1, 14), (24 * 1024, 256, 1, 14),
    (100 * 1024, 1024, 1, 15), (112 * 1024, 1024, 1, 15), (128 * 1024, 1024, 1, 15), (160 * 1024, 1024, 1, 15),
    (180 * 1024, 1024, 1, 15), (48 * 1024, 512, 1, 15), (24 * 1024, 256, 1, 15), (80 * 1024, 1024, 1, 15),
    (100 * 1024, 768, 1, 16), (112 * 1024, 768, 1, 16), (128 * 1024, 768, 1, 16), (100 * 1024, 512, 1, 16),
    (100 * 1024, 768, 1, 17), (112 * 1024, 768, 1, 17), (128 * 1024, 768, 1, 17), (48 * 1024, 512, 1, 16),
    (100 * 1024, 1024, 1, 18), (112 * 1024, 1024, 1, 18), (128 * 1024, 1024, 1, 18), (100 * 1024, 768, 1, 19),
    (112 * 1024, 768, 1, 19), (128 * 1024, 768, 1, 19),
    # two CTAs per SM: 50 KiB tiles make 300 (slot, tile) items at Brunel N=5e5, one wave
    (50 * 1024, 512, 1, 15), (50 * 1024, 512, 1, 17), (50 * 1024, 512, 1, 18), (50 * 1024, 512, 1, 19),
    (50 * 1024, 384, 1, 17), (56 * 1024, 512, 1, 15), (64 * 1024, 512, 1, 15),
    # two 512-thread CTAs per SM (at most 64 registers, 1024 staged sub-rows each)
    (48 * 1024, 512, 1, 20), (64 * 1024, 512, 1, 20), (80 * 1024, 512, 1, 20), (88 * 1024, 512, 1, 20),
    (48 * 1024, 512, 1, 21), (64 * 1024, 512, 1, 21), (80 * 1024, 512, 1, 21), (88 * 1024, 512, 1, 21),
]


def autotune(net, steps: int = 600, warm: int = 60, candidates=None, verbose: bool = False) -> dict:
    """Times the delivery kernel of `net` for each candidate shape; applies and returns the best."""
    cands = candidates or DEFAULT_CANDIDATES
    results = []
    net.set_tuning(overlap_sources=False)
    for tb, th, parts, algo in cands:
        net.set_tuning(tile_bytes=tb, deliver_threads=th, deliver_parts=parts, deliver_algo=algo)
        net.run(warm)
        net.synchronize()
        net.set_profiling(True)
        net.run(steps)
        net.synchronize()
        n, ms = net.kernel_stats(1)
        net.set_profiling(False)
        us = 1e3 * ms / max(n, 1)
        results.append({"tile_bytes": tb, "threads": th, "parts": parts, "algo": algo, "deliver_us": us})
        if verbose:
            print(f"tile {tb // 1024:4d} KiB  threads {th:5d}  parts {parts}  algo {algo}:  deliver {us:8.2f} us",
                  flush=True)
    # among the shapes within 2 % of the fastest, the one with the fewest threads per CTA: a delivery
    # CTA that leaves registers free lets the next window's grid become resident under its tail
    # (raster blocks of recorded runs, the neuron blocks' prologues).  On Brunel N=5e5 a 1024-thread
    # CTA as fast as a 768-thread one in isolation cut recorded runs by 18 %.
    fastest = min(r["deliver_us"] for r in results)
    best = min((r for r in results if r["deliver_us"] <= 1.02 * fastest), key=lambda r: (r["threads"], r["deliver_us"]))
    net.set_tuning(tile_bytes=best["tile_bytes"], deliver_threads=best["threads"], deliver_parts=best["parts"],
                   deliver_algo=best["algo"])
    from . import batch
    if not isinstance(net, batch):  # batches run one neuron-update variant
        nres = tune_neurons(net, steps=steps, warm=warm, verbose=verbose)
        best = dict(best, neuron_variant=nres["best"]["variant"], neuron_us=nres["best"]["neuron_us"])
    net.set_tuning(overlap_sources=True)
    return {"best": best, "results": results}


def apply_shape(net, best: dict) -> None:
    """Applies a shape returned by autotune() (delivery shape and, when present, the neuron-update
    variant) to another network of the same structure."""
    net.set_tuning(tile_bytes=best["tile_bytes"], deliver_threads=best["threads"], deliver_parts=best["parts"],
                   deliver_algo=best["algo"])
    if "neuron_variant" in best:
        net.set_tuning(neuron_variant=best["neuron_variant"])


def tune_neurons(net, steps: int = 300, warm: int = 30, variants=(0, 1, 2, 3, 4, 5, 6, 7, 8, 9), verbose: bool = False) -> dict:
    """Times the neuron-update kernel of `net` for each LIF window variant (identical results);
    applies and returns the fastest."""
    results = []
    for v in variants:
        net.set_tuning(neuron_variant=v)
        net.run(warm)
        net.synchronize()
        net.set_profiling(True)
        net.run(steps)
        net.synchronize()
        n, ms = net.kernel_stats(0)
        net.set_profiling(False)
        us = 1e3 * ms / max(n, 1)
        results.append({"variant": v, "neuron_us": us})
        if verbose:
            print(f"neuron variant {v}:  window {us:8.2f} us", flush=True)
    best = min(results, key=lambda r: r["neuron_us"])
    net.set_tuning(neuron_variant=best["variant"])
    return {"best": best, "results": results}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--brunel", nargs=2, metavar=("N", "P"), default=["500000", "0.002"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--mode", type=int, default=0)
    args = ap.parse_args(argv)
    import spice2_gb300 as sp
    net, _ = sp.brunel(int(args.brunel[0]), float(args.brunel[1]), args.seed, mode=args.mode)
    net.run(300)
    rep = autotune(net, steps=args.steps, verbose=True)
    print(json.dumps(rep["best"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
