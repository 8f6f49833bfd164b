"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_driver -- spice2's own sources (spice/src/{snn,topology,util/assert}.cpp and
headers) compiled by oracle/Makefile with the reference's Release flags -- and stores its outputs:

  rng.npz                    seed chains, xoroshiro128+ draws, exponential draws, canonical floats
                             and the Kahan dt sequence for seeds 1, 7, 1337
  csr_small.npz              complete fixed_probability CSRs for small (src, dst, p, seed) cases
  brunel_csr_checksums.json  checksums of the six Brunel CSRs at N=2e4 p=0.1 seed 1337 and at
                             N=5e5 p=0.002 seeds 1..10, seeded exactly as snn seeds them
  brunel_n20000.npz          N=2e4 p=0.1 seed 1337, 300 steps: raster (I, E, P) and final V/Tref
  brunel_n5000.npz           N=5e3 p=0.05 seed 7, 500 steps: raster and final V/Tref
  mixed_net.npz              mixed delays (2..7), adj_list edges, three input groups: raster/state
  brunel_n500000_s1.json     N=5e5 p=0.002 seed 1, 300 steps: per-step spike counts and checksums
  brunel_n500000_long.npz    N=5e5 p=0.002: seed 1 over 50,000 steps (the benchmark's warm-up and
                             timed stretch) and seeds 2..10 over 2,000 steps: per-step spike counts
                             of P, E, I and, per block, the raster checksum and E / I state checksums
  vogels_n4000.npz           samples/vogels.cpp as published (N=4000, delay 8 dt, seed 1337), 1000
                             steps: raster (E, I) and final V / Gex / Gin / Tref
  weighted_net.npz           oracle.WEIGHTED_NET (per-synapse weights drawn by PerSynapseInit into LIF
                             and conductance targets, fixed weights, delays 3..12, a population with
                             six distinct input weights), 600 steps: raster and final states
  brunel_plus.npz            samples/brunel+.cpp (N=2e4, STDP on E->E) for seeds 1..10, 1000 steps each:
                             per-step spike counts of P, E, I (plasticity with exp(): compared
                             statistically)
  vogels_c3_n10000.npz       the plastic E/I network's neurons and static weights without plasticity
                             (N=1e4 conductance LIF, p=0.02, E 0.03 / I 0.3, delay 1 step, seed 7),
                             1000 steps: raster and final state
  plastic_ei_n100000.npz     the plastic E/I network (N=1e5 conductance LIF, p=0.02, iSTDP on I->E,
                             eta 1e-3, delay 1 step) for seeds 1..10, 5000 steps each: per-step spike
                             counts of E and I and the pooled inter-spike interval sums (compared
                             statistically: the GPU's atomic-mode sums make the dynamics diverge)

usage: python tests/golden/make_golden.py [GROUP ...]   (needs the reference sources; run from the
       repo root; groups: base, vogels, weighted, brunel_plus, brunel_long, plastic_ei; default: all)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from oracle.oracle import raster_checksum, state_checksum  # noqa: E402


def raster_arrays(res):
    """Flattens a raster into (counts[steps][npop], indices)."""
    counts = np.array([[len(x) for x in row] for row in res["raster"]], dtype=np.int32)
    idx = np.concatenate([x for row in res["raster"] for x in row] + [np.zeros(0, np.int32)]).astype(np.int32)
    return counts, idx


def mixed_spec(steps: int):
    """A network with mixed delays, an adj_list projection and three input groups into E."""
    rng = np.random.default_rng(5)
    pairs = sorted({(int(a), int(b)) for a, b in zip(rng.integers(0, 2000, 6000), rng.integers(0, 1000, 6000))})
    lines = ["0.0001 0.0008 4242 %d 0" % steps,
             "pop poisson 3000 50", "pop lif 2000", "pop lif 1000"]
    lines += ["conn 0 1 0.05 0.0003 0.002",
              "conn 1 1 0.05 0.0005 0.002",
              "conn 2 1 0.1 0.0002 -0.005",
              "conn 0 2 0.02 0.0004 0.004",
              "adj 1 2 0.0006 0.003 %d %s" % (len(pairs), " ".join(f"{a} {b}" for a, b in pairs)),
              "conn 2 2 0.02 0.0007 -0.004",
              "conn 1 1 0.01 0.0008 0.003"]
    return lines, pairs


BRUNEL_LONG_SEED1_STEPS, BRUNEL_LONG_BLOCK = 50000, 2000
BRUNEL_SEEDS_STEPS, BRUNEL_SEEDS_BLOCK = 2000, 500


def vogels_fixtures():
    for name, N, seed, steps, kw in (("vogels_n4000", 4000, 1337, 1000, {}),
                                     ("vogels_c3_n10000", 10000, 7, 1000, {"we": 0.03, "wi": 0.3, "delay": 1e-4})):
        res = O.run_reference_net(O.vogels_spec(N, seed, steps, **kw))
        st, _, _ = O.reference_states(res, [], [0, 1])
        counts, idx = raster_arrays(res)
        arrs = {"counts": counts, "idx": idx, "meta": np.array([N, seed, steps])}
        for k in (0, 1):
            for j, f in enumerate(("V", "Gex", "Gin", "T")):
                arrs[f"{f}{k}"] = st[k][j]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)


def weighted_fixtures(steps: int = 600):
    res = O.run_reference_net(O.weighted_net_spec(steps))
    kinds = [p[0] for p in O.WEIGHTED_NET["pops"]]
    lif = [k for k, x in enumerate(kinds) if x == "lif"]
    cond = [k for k, x in enumerate(kinds) if x == "lif_cond"]
    st, _, _ = O.reference_states(res, lif, cond)
    counts, idx = raster_arrays(res)
    arrs = {"counts": counts, "idx": idx, "steps": np.array([steps])}
    for k in lif:
        arrs[f"V{k}"], arrs[f"T{k}"] = st[k]
    for k in cond:
        arrs[f"V{k}"], arrs[f"Gex{k}"], arrs[f"Gin{k}"], arrs[f"T{k}"] = st[k]
    np.savez_compressed(os.path.join(HERE, "weighted_net.npz"), **arrs)


def brunel_plus_fixtures(steps: int = 1000):
    arrs = {}
    for sd in range(1, 11):
        res = O.run_reference_net(O.brunel_plus_spec(sd, steps))
        arrs[f"counts_s{sd}"] = np.array([[len(x) for x in row] for row in res["raster"]], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "brunel_plus.npz"), **arrs)


def brunel_long_fixtures():
    arrs = {}
    jobs = [(1, BRUNEL_LONG_SEED1_STEPS, BRUNEL_LONG_BLOCK)] + [(sd, BRUNEL_SEEDS_STEPS, BRUNEL_SEEDS_BLOCK)
                                                              for sd in range(2, 11)]
    for sd, steps, block in jobs:
        counts, blocks = O.run_reference_brunel_ck(500000, 0.002, sd, steps, block)
        arrs[f"counts_s{sd}"] = counts
        arrs[f"blocks_s{sd}"] = blocks
        arrs[f"meta_s{sd}"] = np.array([steps, block])
        print("seed", sd, "steps", steps, "spikes", int(counts.sum()), flush=True)
    np.savez_compressed(os.path.join(HERE, "brunel_n500000_long.npz"), **arrs)


def plastic_ei_fixtures(N: int = 100000, steps: int = 5000, seeds=range(1, 11), eta: float = 1e-3):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max(1, min(len(seeds), (os.cpu_count() or 2) - 2))) as ex:
        res = list(ex.map(lambda sd: O.run_reference_plastic_ei(N, sd, steps, eta), seeds))
    arrs = {"meta": np.array([N, steps]), "eta": np.array([eta])}
    for sd, (counts, isi, secs) in zip(seeds, res):
        arrs[f"counts_s{sd}"] = counts
        arrs[f"isi_s{sd}"] = isi
        arrs[f"seconds_s{sd}"] = np.array(secs)
        print("seed", sd, "spikes", counts.sum(0), "run seconds", round(secs[1], 1), flush=True)
    np.savez_compressed(os.path.join(HERE, "plastic_ei_n100000.npz"), **arrs)


def main(groups=("base", "vogels", "weighted", "brunel_plus", "brunel_long", "plastic_ei")):
    if not O.have_reference():
        O.build(with_reference=True, reference_dir=os.environ.get("SPICE_REFERENCE_DIR", "/root/reference"))
    if "vogels" in groups:
        vogels_fixtures()
    if "weighted" in groups:
        weighted_fixtures()
    if "brunel_plus" in groups:
        brunel_plus_fixtures()
    if "brunel_long" in groups:
        brunel_long_fixtures()
    if "plastic_ei" in groups:
        plastic_ei_fixtures()
    if "base" not in groups:
        print("golden fixtures written to", HERE)
        return
    # rng
    rng = {}
    for seed in (1, 7, 1337):
        r = O.run_reference_rng(seed, 2000)
        for k, v in r.items():
            rng[f"{k}_{seed}"] = v
    np.savez_compressed(os.path.join(HERE, "rng.npz"), **rng)
    # small CSRs
    cases = [(1000, 800, 0.1, 1), (100, 5000, 0.002, 7), (50, 50, 1.0, 3), (10, 10, 0.0, 3), (3, 0, 0.5, 1),
             (300, 600, 0.5, 9), (100, 70000, 0.01, 11), (5, 3, 0.9, 2), (1500, 200, 0.3, 5)]
    csr = {}
    for (s, d, p, sd) in cases:
        md, off, nb = O.run_reference_gen(s, d, p, sd)
        key = f"{s}_{d}_{p}_{sd}"
        csr[f"off_{key}"] = off
        csr[f"nb_{key}"] = nb
        csr[f"md_{key}"] = np.array([md])
    np.savez_compressed(os.path.join(HERE, "csr_small.npz"), **csr)
    # full-size checksums
    cs = {}
    for (N, p, seeds) in ((20000, 0.1, [1337]), (500000, 0.002, list(range(1, 11)))):
        key = f"N={N},p={p}"
        cs[key] = {}
        for sd in seeds:
            txt = subprocess.run([O.REF_DRIVER, "bcsr", str(N), repr(p), str(sd)], check=True,
                                 capture_output=True, text=True).stdout
            cs[key][str(sd)] = [[int(x) for x in line.split()] for line in txt.strip().splitlines()]
    json.dump(cs, open(os.path.join(HERE, "brunel_csr_checksums.json"), "w"), indent=1)
    # Brunel rasters
    for (N, p, sd, steps, name) in ((20000, 0.1, 1337, 300, "brunel_n20000"), (5000, 0.05, 7, 500, "brunel_n5000")):
        res = O.run_reference_net(O.brunel_spec(N, p, sd, steps))
        st, _, _ = O.reference_states(res, [1, 2])
        counts, idx = raster_arrays(res)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), counts=counts, idx=idx, dt=res["dt"],
                            V1=st[1][0], T1=st[1][1], V2=st[2][0], T2=st[2][1],
                            meta=np.array([N, sd, steps]), p=np.array([p]))
    # mixed network
    lines, pairs = mixed_spec(400)
    res = O.run_reference_net(lines)
    st, _, _ = O.reference_states(res, [1, 2])
    counts, idx = raster_arrays(res)
    np.savez_compressed(os.path.join(HERE, "mixed_net.npz"), counts=counts, idx=idx, V1=st[1][0], T1=st[1][1],
                        V2=st[2][0], T2=st[2][1], pairs=np.array(pairs, dtype=np.int32))
    # N = 5e5: per-step counts and checksums only (the raster and state are megabytes)
    res = O.run_reference_net(O.brunel_spec(500000, 0.002, 1, 300))
    st, _, step_s = O.reference_states(res, [1, 2])
    counts, idx = raster_arrays(res)
    json.dump({"N": 500000, "p": 0.002, "seed": 1, "steps": 300, "counts": counts.tolist(),
               "raster_checksum": raster_checksum(counts, idx),
               "state_checksum_E": state_checksum(*st[1]), "state_checksum_I": state_checksum(*st[2]),
               "reference_step_seconds": step_s},
              open(os.path.join(HERE, "brunel_n500000_s1.json"), "w"))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("base", "vogels", "weighted", "brunel_plus", "brunel_long", "plastic_ei"))
