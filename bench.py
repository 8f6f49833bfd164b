"""Benchmark: synaptic events/s of snn::step on Large Brunel (N=5e5, p=0.002) on one GB300.

One bench "step" = one run of 2000 simulation steps (dt = 1e-4 s, 0.2 s of biological time) of
the Large Brunel network: P = 2.5e5 Poisson (20 Hz), E = 2e5 and I = 5e4 LIF, six
fixed_probability(0.002) projections (2.5e8 synapses), weights scaled by 0.1/p, delay 15 steps,
deterministic delivery (bit-exact with the reference).  The network is generated on the GPU once
and keeps running across bench steps (warm-up steps first), so every timed step is a steady-state
stretch of the same simulation.  The metric counts every synaptic event exactly (sum over spikes
of their CSR row lengths) and divides by device time.

Printed JSON (one line, rank 0):
  value        events/s with the network resident in HBM (CUDA events on the net's stream)
  e2e          the same through the public C ABI call spice_run_record with host buffers: per
               step the dt/seed inputs go host->device and the spike raster comes back
  roofline     the delivery kernel (dominant): algorithmic bytes per launch (8 B per synaptic
               event: int32 target + fp32 weight) / its mean CUDA-event duration, against
               MEASURED_PEAKS.json hbm_gbs; frac_at_4_bytes is the same against the 4-byte target
               alone (a fixed_weight synapse has one weight per projection); frac_span the same
               bytes over the launches' device spans (first CTA start to last CTA end)
  cpu_baseline the CPU restatement of the reference step loop (oracle/oracle_bench, the same
               algorithm as the reference's single-core path) timed on this host's cores
  atomic_mode  value with the fast atomic delivery mode (order-dependent float rounding)
  pull_mode    the deterministic pull path (every population gathers its inputs over the CSC
               adjacency, as per-synapse weights need) on the same network: events/s, synapses
               covered/s, the gather kernels' roofline (8 B per delivered event), the scan-equivalent
               figure (the 4-byte CSC source index of every synapse covered per window), and
               whether its states equal the push path's bit for bit
  batched      the batched sweep (256 Brunel networks, N log-uniform in [5e3, 8e4], 1000 steps):
               events/s as one batch and as the plain path network after network, their ratio,
               and whether both gave bit-identical final states
  adjoint      the differentiable recurrent LIF layer (batch 64, 700 -> 1024, 200 steps): forward and
               adjoint-backward times, their ratio, and plain PyTorch autograd on dense weights
  plastic      the plastic E/I network (N=1e5 conductance LIF, iSTDP on I->E, delay 1 step, 5000
               steps): persistent and launch-per-phase times, roofline, CPU restatement beside it
  seeds        the headline network at seeds 1..10, each timed over the headline's stretch, with
               the CPU restatement of the ten networks beside it
  readme_sample the reference's published sample (Brunel N=2e4, p=0.1, seed 1337, 300 steps) from
               construction, with the CPU restatement on one thread beside it

--impl reference runs the reference's CPU implementation of the path on the host cores (the
reference binary when it was built on this host, else its CPU restatement) and prints the same
metric.  Under torchrun each rank runs an independent replica (seed + rank): replicas only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_NEURONS, P_CONN, SEED, STEPS_PER_RUN = 500000, 0.002, 1, 2000
DT = 1e-4
WORKLOAD = "brunel_large_N5e5_p0.002_2000steps"
# DRAM bytes (read + write) per synaptic event of the delivery kernels measured on this workload:
# dram__bytes_read.sum + dram__bytes_write.sum of one full-size launch
# (profiles/k_deliver_groups_brunel_N5e5_p0.002.md, profiles/k_deliver_staged_brunel_N5e5_p0.002.md,
# profiles/k_deliver_rows16_brunel_N5e5_p0.002.md) divided by its events, keyed by delivery
# mapping.  The bench's traffic per launch is this figure
# times the launch's mean events (None for a mapping without a capture).
DELIVER_DRAM_BYTES_PER_EVENT = {5: (62.261504e6 + 1.521152e6) / 11158496,
                                8: (56.677376e6 + 0.970496e6) / 11158496,
                                # mappings 15-21 read the same 16-bit target copy; measured on 17
                                # (window 30, 10,431,356 events)
                                15: (32.3904e6 + 0.068352e6) / 10431356,
                                16: (32.3904e6 + 0.068352e6) / 10431356,
                                17: (32.3904e6 + 0.068352e6) / 10431356,
                                18: (32.3904e6 + 0.068352e6) / 10431356,
                                19: (32.3904e6 + 0.068352e6) / 10431356,
                                20: (32.3904e6 + 0.068352e6) / 10431356,
                                21: (32.3904e6 + 0.068352e6) / 10431356}
DELIVER_KERNELS = {0: "k_deliver", 1: "k_deliver_tps", 2: "k_deliver_wps", 3: "k_deliver_tps<16-byte loads>",
                   4: "k_deliver_pipe", 5: "k_deliver_groups<4 lanes>", 6: "k_deliver_groups<8 lanes>",
                   7: "k_deliver_groups_occ", 8: "k_deliver_staged<2 in flight>",
                   9: "k_deliver_staged<4 in flight>", 10: "k_deliver_staged_vec<2 sub-rows, 4 blocks>",
                   11: "k_deliver_staged_vec<4 sub-rows, 2 blocks>", 12: "k_deliver_staged_vec<1 sub-row, 8 blocks>",
                   13: "k_deliver_staged_vec<2 sub-rows, 6 blocks>", 14: "k_deliver_rows",
                   15: "k_deliver_rows16<1 sub-row>", 16: "k_deliver_rows16<4 sub-rows>",
                   17: "k_deliver_rows16<2 sub-rows>", 18: "k_deliver_rows16<1 sub-row, TMA store>",
                   19: "k_deliver_rows16<2 sub-rows, TMA store>", 20: "k_deliver_rows16_occ<1 sub-row>",
                   21: "k_deliver_rows16_occ<2 sub-rows>"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce_over_ranks(x: float, ws: int, op: str) -> float:
    """x reduced over the ranks of the process group (NCCL on the GPUs, or gloo on the CPU)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def _max_over_ranks(x: float, ws: int) -> float:
    return _reduce_over_ranks(x, ws, "max")


def _sum_over_ranks(x: float, ws: int) -> float:
    return _reduce_over_ranks(x, ws, "sum")


class ClockSampler:
    """nvidia-smi sampling (every 20 ms) of SM clocks and throttle reasons.  The sampler is started
    during the warm-up (nvidia-smi needs a moment to start); mark() brackets the timed region and
    summary() keeps the samples taken inside it (or, for a region shorter than the sampling period,
    the sample right after its start)."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.out = os.path.join("/tmp", f"spice_clocks_{os.getpid()}.csv")
        self.t0 = self.t1 = None

    def __enter__(self):
        if self.proc is not None:
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=open(self.out, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def mark(self, which: str):
        import datetime
        now = datetime.datetime.now()
        if which == "start":
            self.t0 = now
        else:
            self.t1 = now

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import datetime
        try:
            rows = [[c.strip() for c in r.split(",")] for r in open(self.out).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        stamped = []
        for r in rows:
            try:
                stamped.append((datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f"), r))
            except Exception:
                continue
        inside = [r for t, r in stamped if self.t0 and self.t1 and self.t0 <= t <= self.t1]
        if not inside and self.t0:
            after = [r for t, r in stamped if t >= self.t0]
            inside = after[:1]
        rows = inside
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(threads: int | None = None, steps: int = 200, warmup: int = 50, n_neurons: int = N_NEURONS,
                 samples: int = 1, seed: int = SEED):
    """Times the CPU restatement of the reference step loop (oracle/oracle_bench) on the host cores.
    Every thread runs a replica of the benchmark's network (the same seed): `warmup` untimed steps,
    then `samples` consecutive timed samples of `steps` steps; returns the aggregate, per-core and
    per-sample events/s."""
    from oracle import oracle as o
    if not os.path.exists(o.BENCH_PATH):
        o.build(with_reference=False)
    threads = threads or max(1, min(8, (os.cpu_count() or 1)))
    out = subprocess.run([o.BENCH_PATH, str(n_neurons), repr(P_CONN), str(steps), str(seed), str(threads),
                          str(warmup), str(samples), "1"], check=True, capture_output=True, text=True).stdout
    d = json.loads(out.strip().splitlines()[-1])
    d["kind"] = "port"
    return d


def batched_sweep(n_nets: int, steps: int, warm: int = 60):
    """The batched Brunel sweep: n_nets networks with N log-uniform in [5e3, 8e4] (seeded), p = 0.1 *
    min(1, 2e4/N), seeds 1000 + i, delay 15 steps, deterministic mode.  Two identical sets are built:
    one steps every network on its own, one after the other (the plain path), the other as one batch
    (shared launches per window, CUDA graph replay, launch shape from the autotuner).  Both run the
    same simulated steps; the timed stretch is `steps` steps after warm-up and tuning, and the final
    states of both sets must be bit-identical."""
    import gc
    import numpy as np
    import torch
    import spice2_gb300 as sp
    from spice2_gb300.autotune import autotune
    sizes = sp.brunel_sweep_sizes(n_nets)
    t0 = time.perf_counter()
    A = sp.brunel_sweep(sizes, seed0=1000)
    B = sp.brunel_sweep(sizes, seed0=1000)
    for n, _ in A + B:
        n.csr(0)  # generate the adjacency (construction, not timed)
    syn = sum(n.synapses(c) for n, _ in A for c in range(6))
    batch = sp.batch([n for n, _ in B])
    build_s = time.perf_counter() - t0
    batch.run(warm)
    tuned = autotune(batch, steps=150, warm=15)["best"]
    advanced = batch.nets[0].time
    for n, _ in A:  # bring the plain set to the same step (untimed)
        n.run(advanced)
        n.synchronize()
    # plain path, network after network
    e0 = sum(n.events for n, _ in A)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for n, _ in A:
        n.run(steps)
        n.synchronize()
    plain_s = time.perf_counter() - t
    plain_events = sum(n.events for n, _ in A) - e0
    # batched
    e0 = batch.events
    l0 = batch.launch_count()
    stream = torch.cuda.ExternalStream(batch.stream_handle())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t = time.perf_counter()
    a.record(stream)
    batch.run(steps)
    b.record(stream)
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t
    batch_dev_ms = a.elapsed_time(b)
    batch_events = batch.events - e0
    launches = batch.launch_count() - l0
    same = all(np.array_equal(na.get_state(pa[k], sp.FIELD_V).view(np.uint32), nb.get_state(pb[k], sp.FIELD_V).view(np.uint32))
               for (na, pa), (nb, pb) in zip(A, B) for k in (1, 2))
    same = same and plain_events == batch_events
    out = {"metric": "synaptic_events_per_s", "unit": "events/s", "nets": n_nets, "N_min": min(sizes),
           "N_max": max(sizes), "synapses": syn, "sim_steps": steps,
           "value": batch_events / batch_s, "device_value": batch_events / (batch_dev_ms / 1e3),
           "plain_sequential_value": plain_events / plain_s, "speedup_vs_plain": (batch_events / batch_s) / (plain_events / plain_s),
           "batch_ms": batch_s * 1e3, "plain_ms": plain_s * 1e3, "events": batch_events, "gpu_launches": launches,
           "graph_windows": 8, "delivery_shape": tuned, "bit_identical_to_plain": bool(same),
           "build_seconds": build_s, "timing": "host wall clock around run() with the device synchronised on both sides"}
    del A, B, batch
    gc.collect()
    return out


def adjoint_bench(reps: int = 10):
    """The differentiable recurrent LIF layer (batch 64, 700 Poisson inputs -> 1024 LIF, p = 0.2 / 0.1,
    dt = 1e-3, 200 steps, surrogate slope 25, checkpoint every 20, MSE on the first 128 counts):
    CUDA-event times of the forward kernel and of the adjoint backward (which recomputes every
    20-step segment from its checkpoint), and the same loss and gradients through plain PyTorch
    autograd on dense masked float32 matrices (the surrogate spike as a custom function) for
    comparison."""
    import torch
    from spice2_gb300.lif_layer import RecurrentLIF, count_loss, count_targets, poisson_input, time_step
    torch.backends.cuda.matmul.allow_tf32 = False
    out = time_step(64, 200, reps=reps)
    layer = RecurrentLIF()
    _, x = poisson_input(64, 200, 700, seed=2, return_dense=True)
    target = count_targets(64)
    dev = "cuda"

    def dense(csr, w, ns, nd):
        off, nb = (torch.as_tensor(a, device=dev) for a in csr)
        rows = torch.repeat_interleave(torch.arange(ns, device=dev), off[1:] - off[:-1])
        W = torch.zeros(ns, nd, device=dev)
        W[rows, nb.long()] = w.detach()
        return W.requires_grad_(True)

    class Spike(torch.autograd.Function):
        @staticmethod
        def forward(ctx, xm):
            ctx.save_for_backward(xm)
            return (xm > 0).float()

        @staticmethod
        def backward(ctx, g):
            (xm,) = ctx.saved_tensors
            return g / (1.0 + 25.0 * xm.abs()) ** 2

    xf = x.float()

    def plain():
        Win, Wrec = dense(layer.in_csr, layer.w_in, 700, 1024), dense(layer.rec_csr, layer.w_rec, 1024, 1024)
        th = layer.theta.detach().clone().requires_grad_(True)
        be = layer.beta.detach().clone().requires_grad_(True)
        v = torch.zeros(64, 1024, device=dev)
        s = torch.zeros(64, 1024, device=dev)
        c = torch.zeros(64, 1024, device=dev)
        for t in range(200):
            u = be * v + xf[:, t] @ Win + s @ Wrec
            s = Spike.apply(u - th)
            v = u - th * s
            c = c + s
        count_loss(c, target).backward()

    for _ in range(3):
        plain()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ts = []
    for _ in range(5):
        torch.cuda.synchronize()
        ev[0].record()
        plain()
        ev[1].record()
        torch.cuda.synchronize()
        ts.append(ev[0].elapsed_time(ev[1]))
    ts.sort()
    out["plain_pytorch_fwd_bwd_ms"] = ts[len(ts) // 2]
    out["speedup_vs_plain"] = out["plain_pytorch_fwd_bwd_ms"] / (out["forward_ms"] + out["backward_ms"])
    out["config"] = "batch 64, 700 -> 1024 LIF, p 0.2 / 0.1, 200 steps, checkpoint every 20, slope 25"
    out["plain"] = "PyTorch autograd, dense masked float32 weights (TF32 off), surrogate spike function"
    return out


def plastic_bench(N: int = 100000, steps: int = 5000, peak: float | None = None, cpu_steps: int = 400,
                  cpu_from: int = 1250):
    """The plastic E/I network: N conductance-LIF neurons (80 % E, 20 % I; tau_E 5 ms, tau_I 10 ms,
    the neuron of samples/vogels.cpp), fixed_probability(0.02), delay 1 step, E weights 0.03 and
    I weights 0.3 (0.3 nS and 3 nS over the 10 nS leak), I->E synapses iSTDP (tau 20 ms, rho0 5 Hz,
    eta 1e-3) with lazy event-driven updates, atomic mode, dt 1e-4, `steps` steps after 300 warm-up
    steps.  Windows are one step long, so the net runs persistent steps (cooperative launches split
    at every 64th step for the periodic catch-up, SPICE_TUNE_PERSISTENT); the launch-per-phase path
    is timed beside it.  Reported: synaptic events/s and simulated seconds per wall second (CUDA
    events on the net's stream), firing rates, the I->E weight drift, the roofline of the persistent
    kernel, and the CPU restatement of the same network on the host cores over steps [cpu_from,
    cpu_from + cpu_steps) -- past the opening bursts, where it fires steadily -- with the GPU timed
    on the same steps of a fresh network (`same_stretch`) for the ratio."""
    import numpy as np
    import torch
    import spice2_gb300 as sp

    def build(seed=1):
        net = sp.snn(1e-4, 1e-4, [seed])
        net.set_mode(sp.MODE_ATOMIC)
        E = net.add_population(sp.lif_cond(), N * 8 // 10)
        I = net.add_population(sp.lif_cond(), N * 2 // 10)
        net.connect(E, E, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
        net.connect(E, I, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
        c = net.connect(I, E, sp.fixed_probability(0.02), 1e-4, sp.istdp(0.3, eta=1e-3, rho0=5.0, tau=0.02))
        net.connect(I, I, sp.fixed_probability(0.02), 1e-4, sp.inhibitory(0.3))
        return net, E, I, c

    def timed(net, n):
        stream = torch.cuda.ExternalStream(net.stream_handle())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0, l0 = net.events, net.launch_count()
        torch.cuda.synchronize()
        a.record(stream)
        net.run(n)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b), net.events - e0, net.launch_count() - l0

    warm = 300
    t0 = time.perf_counter()
    net, E, I, c = build()
    net.csr(0)
    syn = sum(net.synapses(k) for k in range(4))
    build_s = time.perf_counter() - t0
    net.run(warm)
    net.synchronize()
    W0 = net.synapse_state(c, 0).astype(np.float64)
    ms, ev, launches = timed(net, steps)
    W = net.synapse_state(c, 0).astype(np.float64)
    raster = net.run_record(1000)  # rates over the next 0.1 s (not timed)
    rE = sum(len(r[0]) for r in raster) / (N * 0.8) / 0.1
    rI = sum(len(r[1]) for r in raster) / (N * 0.2) / 0.1
    net.close()
    # the same stretch through one launch per phase
    net2, *_ = build()
    net2.set_tuning(persistent=0)
    net2.run(warm)
    ms_phase, ev_phase, launches_phase = timed(net2, steps)
    net2.close()
    us_step = 1000.0 * ms / steps
    # algorithmic bytes of a step: the conductance-LIF state read and written (V, Gex, Gin, Tref),
    # the input ring's two sums read and cleared, 8 B per static event (target, weight), 28 B per
    # plastic event (target, W / x_pre / x_post read and written) and every 64 steps the catch-up of
    # every plastic synapse (target 4 B, state 24 B)
    n_plastic = int(0.02 * (N * 2 // 10) * (N * 8 // 10))  # expected I->E synapses
    bytes_step = 32 * N + 16 * N + 8 * ev / steps + 28 * n_plastic / 64.0
    peak = peak or _peaks()[0]
    achieved = bytes_step / (us_step * 1e-6) / 1e9
    out = {"metric": "synaptic_events_per_s", "unit": "events/s", "value": ev / (ms / 1e3), "N": N,
           "synapses": syn, "sim_steps": steps, "warmup_steps": warm, "ms": ms, "us_per_step": us_step,
           "sim_seconds_per_wall_second": steps * 1e-4 / (ms / 1e3),
           "events": ev, "gpu_launches": launches, "rate_E_hz": rE, "rate_I_hz": rI,
           "istdp_weight_mean_start": float(W0.mean()), "istdp_weight_mean_end": float(W.mean()),
           "istdp_weight_std_end": float(W.std()), "build_seconds": build_s, "mode": "atomic",
           "path": "persistent steps (k_persist; launches split at every 64th step for k_plastic_update_all)",
           "launch_per_phase": {"ms": ms_phase, "us_per_step": 1000.0 * ms_phase / steps, "events": ev_phase,
                                "gpu_launches": launches_phase,
                                "sim_seconds_per_wall_second": steps * 1e-4 / (ms_phase / 1e3)},
           "roofline": {"bound": "hbm", "kernel": "k_persist<1>", "achieved": achieved, "peak": peak,
                        "unit": "GB/s", "frac": achieved / peak, "bytes_per_step": bytes_step,
                        "bytes_model": "32 B/neuron state + 16 B/neuron input sums + 8 B/static event + "
                                       "28 B/plastic synapse every 64 steps (catch-up)"},
           "config": "plastic E/I: conductance LIF, p 0.02, delay 1 step, iSTDP on I->E"}
    # the GPU on the CPU sample's steps (fresh seed-1 network, persistent steps)
    net3, *_ = build()
    net3.run(cpu_from)
    net3.synchronize()
    ms3, ev3, _ = timed(net3, cpu_steps)
    net3.close()
    out["same_stretch"] = {"steps": [cpu_from, cpu_from + cpu_steps], "value": ev3 / (ms3 / 1e3),
                           "us_per_step": 1000.0 * ms3 / cpu_steps, "events": ev3}
    try:  # the CPU restatement of the same network over the same steps (same seed)
        from oracle import oracle as o
        if not os.path.exists(o.BENCH_PATH):
            o.build(with_reference=False)
        threads = max(1, min(8, (os.cpu_count() or 1)))
        r = subprocess.run([o.BENCH_PATH, str(N), "0.02", str(cpu_steps), "1", str(threads), str(cpu_from), "1", "1",
                            "plastic_ei"], check=True, capture_output=True, text=True).stdout
        d = json.loads(r.strip().splitlines()[-1])
        out["cpu_baseline"] = {
            "value": d["events_per_s"], "unit": "events/s", "cores": threads, "kind": "port",
            "per_core": d["events_per_s_per_core"],
            "sim_seconds_per_wall_second_per_core": 1e-4 / (d["ms_per_step"] * 1e-3),
            "ms_per_step": d["ms_per_step"],
            "sample": f"steps {cpu_from}..{cpu_from + cpu_steps} of the seed-1 network per thread ({threads} "
                      f"replicas; `same_stretch` is the GPU on those steps); build and warm-up untimed"}
    except Exception as e:  # the oracle could not be built or run here
        out["cpu_baseline"] = {"error": str(e)}
    return out


def pull_bench(steps: int, warmup: int, peak: float):
    """The deterministic per-synapse-weight path on the benchmark's network (SPICE_TUNE_PULL: every
    population gathers its inputs in the reference's order of additions -- connect order, ascending
    source -- and adds them one IEEE addition at a time).  Per window the active synapses are pushed
    into per-target slots with their order keys and ranked per target (the CSC scan of every synapse
    remains the per-target fallback).  Timed like the headline; the final states are compared with
    the push path's after the same steps.  Roofline: 8 B per delivered event (4-byte target, 4-byte
    weight) against the gather's launches (k_pull_masks, k_ps_scatter, k_ps_sort)."""
    import numpy as np
    import torch
    import spice2_gb300 as sp
    net, pops = sp.brunel(N_NEURONS, P_CONN, SEED, mode=sp.MODE_DETERMINISTIC)
    net.set_tuning(pull=True)
    t0 = time.perf_counter()
    net.run(1)
    net.synchronize()
    build_s = time.perf_counter() - t0
    synapses = sum(net.synapses(c) for c in range(6))
    for _ in range(warmup):
        net.run(STEPS_PER_RUN)
    net.synchronize()
    stream = torch.cuda.ExternalStream(net.stream_handle())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0 = net.events
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(steps):
        net.run(STEPS_PER_RUN)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    events = net.events - e0
    net.set_profiling(True)
    for _ in range(steps):
        net.run(STEPS_PER_RUN)
    net.synchronize()
    n_pull, ms_pull = net.kernel_stats(4)
    n_win, ms_win = net.kernel_stats(0)
    net.set_profiling(False)
    total = 1 + (warmup + 2 * steps) * STEPS_PER_RUN
    push, ppops = sp.brunel(N_NEURONS, P_CONN, SEED, mode=sp.MODE_DETERMINISTIC)
    push.run(total)
    same = all(np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32),
                              push.get_state(ppops[k], sp.FIELD_V).view(np.uint32)) for k in (1, 2))
    same = same and net.events == push.events
    windows = n_pull
    t_pull = ms_pull / max(n_pull, 1) / 1e3
    # the profiled run repeats the timed steps: its windows deliver the timed run's events
    ev_window = events / max(windows, 1)
    achieved = 8 * ev_window / t_pull / 1e9 if t_pull > 0 else None
    out = {"metric": "synaptic_events_per_s", "unit": "events/s", "value": events / (ms / 1e3),
           # the inputs of every synapse are settled once per window (a full scan would read each)
           "synapses_covered_per_s": synapses * windows / (ms / 1e3),
           "ms_per_step": ms / steps, "sim_seconds_per_wall_second": STEPS_PER_RUN * steps * DT / (ms / 1e3),
           "pull_launches": n_pull, "pull_mean_us": t_pull * 1e6, "neuron_mean_us": ms_win / max(n_win, 1) * 1e3,
           "roofline": {"bound": "hbm", "kernel": "k_pull_masks + k_ps_scatter + k_ps_sort", "bytes_per_event": 8,
                        "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": (achieved / peak) if achieved else None},
           # pull mode in synapses scanned per second: synapses whose inputs are settled per second at
           # the 4-byte CSC source index a scan of every synapse would read per window (the gather
           # reads only the active ones), against the same bandwidth
           "scan_equivalent": {"bytes_per_synapse": 4, "achieved": 4 * synapses * windows / (ms / 1e3) / 1e9,
                               "peak": peak, "unit": "GB/s",
                               "frac": 4 * synapses * windows / (ms / 1e3) / 1e9 / peak},
           "bit_identical_to_push": bool(same), "build_seconds": build_s,
           "config": "Large Brunel N=5e5 p=0.002 seed 1, every population pulled (SPICE_TUNE_PULL), deterministic"}
    net.close()
    push.close()
    return out


def seed_sweep(tuned: dict, warmup: int, steps: int = 2, seeds=range(1, 11), cpu_steps: int = 100):
    """Large Brunel at seeds 1..10 (the benchmark's seed list): each network built fresh, warm-up
    to the headline's first timed step (warmup x 2000 steps), then `steps` runs of 2000 steps timed
    with CUDA events on its stream, in the headline's launch shape.  Beside it the CPU restatement
    of the same ten networks (one thread per seed) over `cpu_steps` steps from the same step."""
    import torch
    import spice2_gb300 as sp
    from spice2_gb300.autotune import apply_shape
    per_seed = []
    for seed in seeds:
        net, _ = sp.brunel(N_NEURONS, P_CONN, seed, mode=sp.MODE_DETERMINISTIC)
        apply_shape(net, tuned)
        for _ in range(warmup):
            net.run(STEPS_PER_RUN)
        net.synchronize()
        stream = torch.cuda.ExternalStream(net.stream_handle())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0 = net.events
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(steps):
            net.run(STEPS_PER_RUN)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        per_seed.append({"seed": seed, "value": (net.events - e0) / (ms / 1e3), "ms_per_step": ms / steps,
                         "events": net.events - e0})
        net.close()
        del net
    vals = [d["value"] for d in per_seed]
    out = {"metric": "synaptic_events_per_s", "unit": "events/s", "seeds": [d["seed"] for d in per_seed],
           "values": vals, "mean": statistics.fmean(vals), "min": min(vals), "max": max(vals),
           "first_timed_step": warmup * STEPS_PER_RUN, "sim_steps_per_seed": steps * STEPS_PER_RUN,
           "per_seed": per_seed}
    try:
        start = warmup * STEPS_PER_RUN
        d = _oracle_bench([N_NEURONS, P_CONN, cpu_steps, min(seeds), len(seeds), start, 1, 0])
        out["cpu_baseline"] = {"value": d["events_per_s"], "unit": "events/s", "cores": d["threads"], "kind": "port",
                               "per_core": d["events_per_s_per_core"],
                               "sample": f"{cpu_steps} steps of each seed's network from step {start}, one thread "
                                         f"per seed; build and warm-up untimed"}
    except Exception as e:  # reported, never a reason to lose the section
        out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


def readme_sample(repeats: int = 10):
    """The reference's own sample as published (samples/brunel.cpp with its README parameters):
    Brunel N=2e4, p=0.1, weights 2/N and -10/N, delay 15 steps, seed 1337, 300 steps.  A fresh
    network per repetition: construction timed on the host (synchronised), the 300 steps with CUDA
    events on the net's stream after the first call's setup; the best and median repetitions are
    reported, in the launch shape the library picks for the network's sizes.  Beside it the CPU
    restatement of the same sample on one thread (the reference is single-threaded), construction
    and steps timed apart; the speed-up is the ratio of the two times for the 300 steps."""
    import torch
    import spice2_gb300 as sp
    N, p, seed, steps = 20000, 0.1, 1337, 300
    runs = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        net, _ = sp.brunel(N, p, seed, mode=sp.MODE_DETERMINISTIC)
        net.run(0)  # construction: adjacency generation and the first call's setup
        net.synchronize()
        build = time.perf_counter() - t0
        stream = torch.cuda.ExternalStream(net.stream_handle())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        net.run(steps)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        runs.append({"build_s": build, "ms": ms, "events": net.events})
        net.close()
        del net
    ms = sorted(r["ms"] for r in runs)
    events = runs[0]["events"]
    assert all(r["events"] == events for r in runs)
    out = {"metric": "synaptic_events_per_s", "unit": "events/s",
           "config": "Brunel N=2e4 (P 1e4, E 8e3, I 2e3), p=0.1, w 2/N and -10/N, delay 15 steps, seed 1337, "
                     "300 steps from construction",
           "events": events, "value": events / (ms[0] / 1e3), "median_value": events / (statistics.median(ms) / 1e3),
           "ms": ms[0], "sim_seconds_per_wall_second": steps * DT / (ms[0] / 1e3),
           "build_seconds": statistics.median(r["build_s"] for r in runs), "repeats": repeats}
    try:
        d = _oracle_bench([N, p, steps, seed, 1, 0, 1, 0])
        out["cpu_baseline"] = {"value": d["events_per_s"], "unit": "events/s", "cores": 1, "kind": "port",
                               "ms": d["step_seconds"] * 1e3, "build_seconds": d["build_seconds"],
                               "sample": "the 300 steps of the sample on one thread; construction timed apart"}
        # by time for the same 300 steps: the GPU's count includes the events of the spikes of the
        # last window that the reference delivers in later steps (a window delivers all its spikes)
        out["speedup_vs_cpu"] = d["step_seconds"] * 1e3 / out["ms"]
    except Exception as e:
        out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


def _oracle_bench(argv: list) -> dict:
    from oracle import oracle as o
    if not os.path.exists(o.BENCH_PATH):
        o.build(with_reference=False)
    out = subprocess.run([o.BENCH_PATH] + [repr(a) if isinstance(a, float) else str(a) for a in argv],
                         check=True, capture_output=True, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


def reference_arm(args):
    """The reference's CPU implementation of the path (its C restatement: the reference binary is
    built for x86-64 with -march=haswell and its sources are not on the GPU host) on the host cores,
    timing the stretch the GPU arm times: replicas of the seed-1 network, warm-up to the first
    timed step of the GPU arm (warmup x 2000 steps), then one bounded sample of 100 steps per bench
    step."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    threads = max(1, min(16, os.cpu_count() or 1))
    per_step = 100
    start = args.warmup * STEPS_PER_RUN
    d = cpu_baseline(threads=threads, steps=per_step, warmup=start, samples=args.steps)
    vals = d["sample_events_per_s"]
    value = d["events_per_s"]
    line = {"metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "ms_per_step": d["ms_per_step"] * per_step,
            "config": {"workload": WORKLOAD, "N": N_NEURONS, "p": P_CONN, "seed": SEED, "delay_steps": 15,
                       "mode": "deterministic", "sim_steps_per_bench_step": per_step,
                       "first_timed_step": start,
                       "replicas": f"{threads} host threads, each a replica of the seed-{SEED} network"},
            "per_core_value": d["events_per_s_per_core"],
            "sample_values": vals,
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": d["kind"],
                             "per_core": d["events_per_s_per_core"],
                             "sample": f"{args.steps} samples of {per_step} simulation steps of the seed-{SEED} "
                                       f"N=5e5 Brunel network per thread, starting at step {start} (the GPU "
                                       f"arm's first timed step); network build {d['build_seconds']:.1f} s and "
                                       f"warm-up not timed"},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)  # ~115 ms timed: several clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched-nets", type=int, default=256,
                    help="networks of the batched Brunel sweep (0 skips it)")
    ap.add_argument("--batched-steps", type=int, default=1000)
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the batched, adjoint and plastic sections (faster iterations)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    ws, rank, lrank = _dist()
    import torch
    torch.cuda.set_device(lrank)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import spice2_gb300 as sp

    seed = SEED + rank  # replicas: independent networks
    from spice2_gb300.autotune import autotune, apply_shape
    # launch shape of the delivery kernel and neuron update, measured on a copy of the network (the
    # tuning advances the simulation); results do not depend on it
    tnet, _ = sp.brunel(N_NEURONS, P_CONN, seed, mode=sp.MODE_DETERMINISTIC)
    tuned = autotune(tnet, steps=300, warm=30)["best"]
    tnet.close()
    del tnet
    # the benchmarked network: built fresh, so the timed stretch is steps
    # [warmup * 2000, (warmup + steps) * 2000) of the seed's simulation
    t0 = time.perf_counter()
    net, pops = sp.brunel(N_NEURONS, P_CONN, seed, mode=sp.MODE_DETERMINISTIC)
    net.csr(0)
    net.synchronize()
    build_s = time.perf_counter() - t0
    synapses = sum(net.synapses(c) for c in range(6))
    stream = torch.cuda.ExternalStream(net.stream_handle())
    apply_shape(net, tuned)

    clk = ClockSampler(lrank).__enter__()  # sampling starts during the warm-up (nvidia-smi start-up)
    for _ in range(args.warmup):
        net.run(STEPS_PER_RUN)
    net.synchronize()

    # ---- device-resident timed region ----
    ev0, l0 = net.events, net.launch_count()
    _barrier(ws)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clk:
        clk.mark("start")
        torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches
        start.record(stream)
        for _ in range(args.steps):
            net.run(STEPS_PER_RUN)
        end.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        clk.mark("end")
    _barrier(ws)
    ms = start.elapsed_time(end)
    events = net.events - ev0
    launches = net.launch_count() - l0
    # per-kernel CUDA-event times over the same number of steps, run again with an event pair
    # around every launch (the events between kernels cost ~10 % of throughput, so the timed region
    # above runs without them)
    net.set_profiling(True)
    pe0 = net.events
    for _ in range(args.steps):
        net.run(STEPS_PER_RUN)
    net.synchronize()
    prof_events = net.events - pe0
    n_del, ms_del = net.kernel_stats(1)
    n_win, ms_win = net.kernel_stats(0)
    n_span, ms_span = net.kernel_span(1)  # the same launches' device spans (first CTA start to last end)
    n_wspan, ms_wspan = net.kernel_span(0)
    net.set_profiling(False)
    ms_max = _max_over_ranks(ms, ws)
    events_all = _sum_over_ranks(float(events), ws)
    value = events_all / (ms_max / 1e3)

    # ---- end to end through the public C ABI with host buffers (pinned: the GPU writes the raster
    # into them while it steps) ----
    cap = 4_000_000
    counts = torch.zeros((STEPS_PER_RUN, 3), dtype=torch.int64, pin_memory=True)
    spikes = torch.zeros(cap, dtype=torch.int32, pin_memory=True)
    import ctypes as C
    total = C.c_int64()
    L = sp.lib()
    e2e_times, e2e_events, d2h = [], 0, 0
    _barrier(ws)
    for i in range(args.steps + 1):
        e0 = net.events
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = L.spice_run_record(net._h, STEPS_PER_RUN, counts.data_ptr(), spikes.data_ptr(), cap, C.byref(total))
        t = time.perf_counter() - t
        if rc != 0:
            raise RuntimeError(L.spice_last_error().decode())
        if i > 0:  # the first call sizes the device raster buffer
            e2e_times.append(t)
            e2e_events += net.events - e0
            d2h = 4 * int(total.value) + 16 * STEPS_PER_RUN * 3 + 8
    e2e_s = _max_over_ranks(sum(e2e_times), ws)
    e2e_value = _sum_over_ranks(float(e2e_events), ws) / e2e_s

    # ---- atomic mode (fast, order-dependent rounding), timed the same way ----
    atomic = None
    if rank == 0:
        del net
        net2, _ = sp.brunel(N_NEURONS, P_CONN, seed, mode=sp.MODE_ATOMIC)
        autotune(net2, steps=300, warm=30)  # atomic mode has its own fastest shape
        for _ in range(args.warmup):
            net2.run(STEPS_PER_RUN)
        net2.synchronize()
        s2 = torch.cuda.ExternalStream(net2.stream_handle())
        e0 = net2.events
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(s2)
        for _ in range(args.steps):
            net2.run(STEPS_PER_RUN)
        b.record(s2)
        torch.cuda.synchronize()
        atomic = {"value": (net2.events - e0) / (a.elapsed_time(b) / 1e3), "unit": "events/s",
                  "ms_per_step": a.elapsed_time(b) / args.steps}
        del net2

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    peak, peak_kind = _peaks()
    # algorithmic bytes per synaptic event: 8 (int32 target + fp32 weight, the benchmark's per-event
    # figure); Brunel's fixed_weight synapses need only the 4-byte target, so the fraction against
    # that stricter minimum (frac_at_4_bytes) is half of `frac`
    bytes_per_event = 8
    ev_per_launch = prof_events / max(n_del, 1)
    t_launch = ms_del / max(n_del, 1) / 1e3
    achieved = bytes_per_event * ev_per_launch / t_launch / 1e9 if t_launch > 0 else None
    t_span = ms_span / n_span / 1e3 if n_span > 0 else 0.0
    achieved_span = bytes_per_event * ev_per_launch / t_span / 1e9 if t_span > 0 else None
    traffic = None
    if tuned["algo"] in DELIVER_DRAM_BYTES_PER_EVENT:
        traffic = DELIVER_DRAM_BYTES_PER_EVENT[tuned["algo"]] * ev_per_launch

    pull = None
    if rank == 0:
        try:
            pull = pull_bench(args.steps, args.warmup, peak)
        except Exception as e:  # reported, never a reason to lose the headline line
            pull = {"error": str(e)}

    batched = None
    import gc
    gc.collect()  # the N=5e5 nets (populations and nets reference each other)
    if args.batched_nets > 0 and not args.headline_only:
        try:
            batched = batched_sweep(args.batched_nets, args.batched_steps)
        except Exception as e:  # reported, never a reason to lose the headline line
            batched = {"error": str(e)}

    adjoint = plastic = None
    if not args.headline_only:
        try:
            adjoint = adjoint_bench()
        except Exception as e:
            adjoint = {"error": str(e)}
        try:
            plastic = plastic_bench(peak=peak)
        except Exception as e:
            plastic = {"error": str(e)}
    seeds = readme = None
    if not args.headline_only:
        try:
            seeds = seed_sweep(tuned, args.warmup)
        except Exception as e:
            seeds = {"error": str(e)}
        try:
            readme = readme_sample()
        except Exception as e:
            readme = {"error": str(e)}

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        try:
            start = args.warmup * STEPS_PER_RUN
            d = cpu_baseline(steps=200, warmup=start)
            cpu = {"value": d["events_per_s"], "unit": "events/s", "cores": d["threads"], "kind": d["kind"],
                   "per_core": d["events_per_s_per_core"],
                   "sample": f"{d['steps']} steps of the seed-{SEED} N=5e5 Brunel network per thread "
                             f"({d['threads']} replicas) from step {start}, the first step of the GPU timed "
                             f"stretch; build {d['build_seconds']:.1f} s and warm-up untimed"}
        except Exception as e:  # the baseline is reported, never a reason to fail the bench
            cpu = {"value": None, "unit": "events/s", "cores": 0, "kind": "port", "sample": f"failed: {e}"}

    line = {
        "metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "N": N_NEURONS, "p": P_CONN, "synapses": synapses,
                   "sim_steps_per_bench_step": STEPS_PER_RUN, "dt": DT,
                   "delay_steps": 15, "mode": "deterministic", "seed": SEED,
                   "first_timed_step": args.warmup * STEPS_PER_RUN,
                   "parallelism": f"replicas{ws}" if ws > 1 else "single",
                   "delivery_shape": tuned,
                   "l2": "inputs larger than L2 (1 GB of CSR targets; a window reads ~42 MB of random rows)"},
        "sim_seconds_per_wall_second": STEPS_PER_RUN * args.steps * DT / (ms_max / 1e3),
        "ms_per_sim_step": ms_max / args.steps / STEPS_PER_RUN,
        "build_seconds": build_s,
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "events/s", "h2d_bytes_per_step": 20 * STEPS_PER_RUN,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "frac_at_4_bytes": (achieved / peak / 2) if achieved else None,
                     "kernel": DELIVER_KERNELS.get(tuned["algo"], "k_deliver"), "bytes_per_event": bytes_per_event, "peak_source": f"{peak_kind} hbm_gbs",
                     "launches": n_del, "mean_launch_us": t_launch * 1e6,
                     "kernel_timing": "CUDA events around every delivery launch on the net's stream, over a "
                                      "second run of the timed steps (the headline is timed without them)",
                     "neuron_kernel_mean_us": ms_win / max(n_win, 1) * 1e3,
                     "neuron_kernel_span_us": ms_wspan / n_wspan * 1e3 if n_wspan else None,
                     "kernel_span_us": t_span * 1e6 if n_span else None,
                     "achieved_span": achieved_span,
                     "frac_span": (achieved_span / peak) if achieved_span else None,
                     "span_timing": "the same delivery launches from their first CTA's start to their last CTA's "
                                    "end on the GPU's global timer; mean_launch_us - kernel_span_us is the fixed "
                                    "cost of a launch and of the CUDA-event pair around it"},
        "cpu_baseline": cpu,
        "atomic_mode": atomic,
        "pull_mode": pull,
        "batched": batched,
        "adjoint": adjoint,
        "plastic": plastic,
        "seeds": seeds,
        "readme_sample": readme,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
