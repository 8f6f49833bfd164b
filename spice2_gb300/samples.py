"""The reference's sample programs on the GPU engine.

  python -m spice2_gb300.samples brunel [--N 20000] [--p 0.1] [--seed 1337] [--steps 300] [--json]
  python -m spice2_gb300.samples vogels [--N 4000] [--steps 1500] [--json]
  python -m spice2_gb300.samples external_input [--json]
  python -m spice2_gb300.samples plastic_ei [--N 100000] [--seed 1] [--steps 5000] [--persistent 1]

brunel follows samples/brunel.cpp:75-116 (weights scaled by 0.1/p so other p keep the mean input),
vogels samples/vogels.cpp:62-86, external_input samples/external_input.cpp:39-51, plastic_ei the
plastic E/I network (vogels.cpp's conductance LIF, p 0.02, delay 1 step, iSTDP on I->E, atomic
mode; no counterpart sample in the reference).  --json prints the
raster in the format of samples/matplot.cpp:96-134 (populations in the order the sample streams
them, indices offset by the sizes of the populations before); without it a one-line summary with
the synaptic events and the device time is printed.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def _emit(name, raster, order, sizes, skip_empty=False):
    """samples/matplot.cpp:96-134: '\\t\\t[' separated rows of offset spike indices."""
    out = ["{", f'\t"name": "{name}",', '\t"spikes": [']
    rows = []
    for row in raster:
        vals, off, any_ = [], 0, False
        for k in order:
            s = row[k]
            if skip_empty and len(s) == 0:
                continue
            vals.extend(int(x) + off for x in s)
            off += sizes[k]
            any_ = True
        if any_ or not skip_empty:
            rows.append("\t\t[" + ",".join(map(str, vals)) + "]")
    out.append(",\n".join(rows))
    out.append("\t]\n}")
    print("\n".join(out))


def brunel(args):
    import spice2_gb300 as sp
    N, p = args.N, args.p
    net, (P, E, I) = sp.brunel(N, p, args.seed, mode=args.mode)
    if args.tuning:
        tb, th, parts, algo = (int(x) for x in args.tuning.split(","))
        net.set_tuning(tile_bytes=tb, deliver_threads=th, deliver_parts=parts, deliver_algo=algo)
    if args.neuron_variant is not None:
        net.set_tuning(neuron_variant=args.neuron_variant)
    if args.launch_mode is not None:  # 0: neuron update and sources as separate launches, one stream
        net.set_tuning(launch_mode=args.launch_mode, overlap_sources=bool(args.launch_mode))
    if args.pull:
        net.set_tuning(pull=True)
    t = time.perf_counter()
    if args.json:
        raster = net.run_record(args.steps)
        _emit("Brunel", raster, (2, 1, 0), [P.size(), E.size(), I.size()])
    elif args.window_events:
        # one min-delay window (15 steps) per call: one delivery launch each, in launch order
        per, done = [], 0
        while done < args.steps:
            k = min(15, args.steps - done)
            e0 = net.events
            net.run(k)
            per.append(net.events - e0)
            done += k
        print(json.dumps({"sample": "brunel", "N": N, "p": p, "steps": args.steps, "window_steps": 15,
                          "events_per_window": per}))
    else:
        net.run(args.steps)
        net.synchronize()
        dt = time.perf_counter() - t
        print(json.dumps({"sample": "brunel", "N": N, "p": p, "steps": args.steps, "events": net.events,
                          "wall_s": dt, "events_per_s": net.events / dt}))


def vogels(args):
    import spice2_gb300 as sp
    N = args.N
    net = sp.snn(1e-4, 8e-4, [args.seed])
    E = net.add_population(sp.lif_cond(), N * 8 // 10)
    I = net.add_population(sp.lif_cond(), N * 2 // 10)
    we, wi = float(np.float32(6.4e6 / (N * N))), float(np.float32(8.16e7 / (N * N)))
    net.connect(E, E, sp.fixed_probability(0.02), 8e-4, sp.excitatory(we))
    net.connect(E, I, sp.fixed_probability(0.02), 8e-4, sp.excitatory(we))
    net.connect(I, E, sp.fixed_probability(0.02), 8e-4, sp.inhibitory(wi))
    net.connect(I, I, sp.fixed_probability(0.02), 8e-4, sp.inhibitory(wi))
    raster = net.run_record(args.steps)
    if args.json:
        _emit("Vogels", raster, (1, 0), [E.size(), I.size()], skip_empty=True)
    else:
        n = sum(len(r[0]) + len(r[1]) for r in raster)
        print(json.dumps({"sample": "vogels", "N": N, "steps": args.steps, "spikes": n, "events": net.events}))


def plastic_ei(args):
    import spice2_gb300 as sp
    N = args.N
    net = sp.snn(1e-4, 1e-4, [args.seed])
    net.set_mode(sp.MODE_ATOMIC)
    net.set_tuning(persistent=args.persistent)
    E = net.add_population(sp.lif_cond(), N * 8 // 10)
    I = net.add_population(sp.lif_cond(), N * 2 // 10)
    net.connect(E, E, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
    net.connect(E, I, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
    net.connect(I, E, sp.fixed_probability(0.02), 1e-4, sp.istdp(0.3, eta=1e-3, rho0=5.0, tau=0.02))
    net.connect(I, I, sp.fixed_probability(0.02), 1e-4, sp.inhibitory(0.3))
    t = time.perf_counter()
    net.run(args.steps)
    net.synchronize()
    dt = time.perf_counter() - t
    print(json.dumps({"sample": "plastic_ei", "N": N, "steps": args.steps, "events": net.events, "wall_s": dt}))


def external_input(args):
    import spice2_gb300 as sp
    trains = ((4, 5, 8), (5,), (7, 8), (5, 7))
    net = sp.snn(1, 1, [1337])
    I = net.add_population(sp.external_input(trains), 9)
    raster = [[net.spikes(I, 0)] for _ in range(20) if net.step() is None]
    _emit("external_input", raster, (0,), [9]) if args.json else print(json.dumps({"steps": 20}))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="sample", required=True)
    b = sub.add_parser("brunel")
    b.add_argument("--N", type=int, default=20000)
    b.add_argument("--p", type=float, default=0.1)
    b.add_argument("--seed", type=int, default=1337)
    b.add_argument("--steps", type=int, default=300)
    b.add_argument("--mode", type=int, default=0)
    b.add_argument("--json", action="store_true")
    b.add_argument("--window-events", action="store_true",
                   help="run window by window and print the synaptic events of each (profiling aid)")
    b.add_argument("--tuning", default="", metavar="TILE_BYTES,THREADS,PARTS,ALGO",
                   help="delivery launch shape (results do not depend on it)")
    b.add_argument("--neuron-variant", type=int, default=None,
                   help="LIF window variant (results do not depend on it; default: the one the network's size picks)")
    b.add_argument("--pull", action="store_true", help="deliver every population by the pull path over the CSC")
    b.add_argument("--launch-mode", type=int, default=None,
                   help="1: one grid per window for neurons and sources (default); 0: separate launches")
    v = sub.add_parser("vogels")
    v.add_argument("--N", type=int, default=4000)
    v.add_argument("--seed", type=int, default=1337)
    v.add_argument("--steps", type=int, default=1500)
    v.add_argument("--json", action="store_true")
    x = sub.add_parser("external_input")
    x.add_argument("--json", action="store_true")
    e = sub.add_parser("plastic_ei")
    e.add_argument("--N", type=int, default=100000)
    e.add_argument("--seed", type=int, default=1)
    e.add_argument("--steps", type=int, default=5000)
    e.add_argument("--persistent", type=int, default=1, help="SPICE_TUNE_PERSISTENT (0: one launch per phase)")
    args = ap.parse_args(argv)
    {"brunel": brunel, "vogels": vogels, "external_input": external_input, "plastic_ei": plastic_ei}[args.sample](args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
