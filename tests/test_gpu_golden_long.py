"""GPU parity against the reference's own outputs on the conductance LIF and on long Large Brunel runs.

The fixtures (tests/golden/make_golden.py) come from the reference compiled from its own sources
with its Release flags:
  * vogels_n4000.npz: samples/vogels.cpp as published; vogels_c3_n10000.npz: the conductance LIF of
    the plastic E/I network with its static weights and delay 1 step.  Rasters and the final
    V / Gex / Gin / Tref must be equal bit for bit -- the reference's -ffast-math build contracts the
    conductance update into fused multiply-adds, and the engine computes that compiled form.
  * brunel_n500000_long.npz: Large Brunel N=5e5, p=0.002: seed 1 over 50,000 steps (the benchmark
    builds a fresh seed-1 network and times 2000-step runs after 2000-step warm-up runs, all inside
    this stretch) and seeds 2..10 over 2,000 steps; per-step spike counts of P, E, I and per block
    the raster checksum and the E / I state checksums.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _vogels_net(sp, N, seed, we, wi, delay, mode=0):
    net = sp.snn(1e-4, delay, [seed])
    net.set_mode(mode)
    E = net.add_population(sp.lif_cond(), N * 8 // 10)
    I = net.add_population(sp.lif_cond(), N * 2 // 10)
    net.connect(E, E, sp.fixed_probability(0.02), delay, sp.excitatory(we))
    net.connect(E, I, sp.fixed_probability(0.02), delay, sp.excitatory(we))
    net.connect(I, E, sp.fixed_probability(0.02), delay, sp.inhibitory(wi))
    net.connect(I, I, sp.fixed_probability(0.02), delay, sp.inhibitory(wi))
    return net, (E, I)


@pytest.mark.parametrize("name,delay,weights,stepwise", [
    ("vogels_n4000", 8e-4, None, False),
    ("vogels_n4000", 8e-4, None, True),
    ("vogels_c3_n10000", 1e-4, (0.03, 0.3), False),
])
def test_vogels_conductance_lif_golden(engine, name, delay, weights, stepwise):
    sp = engine
    from oracle.oracle import vogels_weights
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    we, wi = weights if weights else vogels_weights(N)
    net, pops = _vogels_net(sp, N, seed, we, wi, delay)
    if stepwise:
        raster = []
        for _ in range(steps):
            net.step()
            raster.append([net.spikes(p, 0) for p in pops])
    else:
        raster = net.run_record(steps)
    counts = np.array([[len(x) for x in row] for row in raster])
    idx = np.concatenate([np.asarray(x) for row in raster for x in row] + [np.zeros(0, np.int32)])
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(idx, g["idx"])
    assert counts.sum() > 100  # the network is active
    for k, p in enumerate(pops):
        st = p.get_neurons()
        for f in ("V", "Gex", "Gin"):
            assert np.array_equal(st[f].view(np.uint32), g[f"{f}{k}"].view(np.uint32)), (k, f)
        assert np.array_equal(st["Tref"], g[f"T{k}"]), k


def _run_blocks(sp, net, steps, block):
    """Runs `steps` steps in recorded blocks; returns the per-step counts and the per-block
    (raster checksum, E state checksum, I state checksum) as the reference's fixture holds them."""
    from oracle.oracle import raster_checksum, state_checksum
    pops = net._pops
    counts, blocks, t = [], [], 0
    while t < steps:
        n = min(block, steps - t)
        raster = net.run_record(n, capacity=n * 3000 + 4096)
        c = np.array([[len(x) for x in row] for row in raster], dtype=np.int32)
        idx = np.concatenate([np.asarray(x) for row in raster for x in row] + [np.zeros(0, np.int32)])
        e, i = pops[1].get_neurons(), pops[2].get_neurons()
        blocks.append((raster_checksum(c, idx), state_checksum(e["V"], e["Tref"]), state_checksum(i["V"], i["Tref"])))
        counts.append(c)
        t += n
    return np.concatenate(counts), blocks


def _check_seed(sp, g, seed, steps=None):
    meta = g[f"meta_s{seed}"]
    steps = int(meta[0]) if steps is None else steps
    block = int(meta[1])
    net, _ = sp.brunel(500000, 0.002, seed)
    counts, blocks = _run_blocks(sp, net, steps, block)
    ref_counts = g[f"counts_s{seed}"][:steps]
    ref_blocks = g[f"blocks_s{seed}"]
    first = next((t for t in range(steps) if not np.array_equal(counts[t], ref_counts[t])), None)
    assert first is None, f"seed {seed}: spike counts differ first at step {first}"
    for b, got in enumerate(blocks):
        assert tuple(int(x) for x in ref_blocks[b]) == got, f"seed {seed}: block {b} checksums differ"


def test_large_brunel_benchmark_stretch_golden(engine):
    """Seed 1, the benchmark's network: 50,000 steps in 2000-step blocks equal the reference's."""
    g = np.load(os.path.join(GOLDEN, "brunel_n500000_long.npz"))
    _check_seed(engine, g, 1)


@pytest.mark.parametrize("seed", list(range(2, 11)))
def test_large_brunel_seeds_golden(engine, seed):
    """Seeds 2..10: 2000 steps in 500-step blocks equal the reference's."""
    g = np.load(os.path.join(GOLDEN, "brunel_n500000_long.npz"))
    _check_seed(engine, g, seed)
