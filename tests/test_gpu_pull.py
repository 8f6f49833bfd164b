"""GPU: the CSC adjacency and the deterministic pull path for per-synapse weights.

A population receiving weighted synapses (a weight per synapse, drawn at construction as the
reference's PerSynapseInit concept does) is delivered by the pull path: each target gathers its
inputs from the CSC columns of its connections in connect order and ascending source order and
adds them one IEEE addition at a time.  The results are compared bit for bit with the oracle and
with the reference binary's fixture (tests/golden/weighted_net.npz).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _weighted_net(sp, o, mode=0, pull_all=False, spec=None):
    spec = spec or o.WEIGHTED_NET
    net = sp.snn(spec["dt"], spec["max_delay"], [spec["seed"]])
    net.set_mode(mode)
    if pull_all:
        net.set_tuning(pull=True)
    models = {"poisson": lambda p: sp.poisson(p[2]), "lif": lambda p: sp.lif(), "lif_cond": lambda p: sp.lif_cond()}
    pops = [net.add_population(models[p[0]](p), p[1]) for p in spec["pops"]]
    conns = []
    for kind, s, d, p, delay, w, fl in spec["conns"]:
        syn = sp.weighted(float(np.float32(w)), fl) if kind == "w" else sp.fixed_weight(float(np.float32(w)), fl)
        conns.append(net.connect(pops[s], pops[d], sp.fixed_probability(p), delay, syn))
    return net, pops, conns


def _transpose(off, nb, ndst):
    """Stable transpose: each target's sources in ascending (CSR) order."""
    src = np.repeat(np.arange(len(off) - 1, dtype=np.int64), np.diff(off))
    order = np.argsort(nb, kind="stable")
    col = np.zeros(ndst + 1, dtype=np.int64)
    np.add.at(col, nb.astype(np.int64) + 1, 1)
    return np.cumsum(col), src[order].astype(np.int32)


def test_csc_is_the_stable_transpose(engine):
    sp = engine
    net, pops = sp.brunel(20000, 0.1, 1337)
    for c, (s, d) in enumerate([(0, 1), (0, 2), (1, 1), (1, 2), (2, 1), (2, 2)]):
        off, nb = net.csr(c)
        coff, csrc = net.csc(c)
        eoff, esrc = _transpose(off, nb, pops[d].size())
        assert np.array_equal(coff, eoff), c
        assert np.array_equal(csrc, esrc), c


def test_csc_of_adj_list_with_duplicates(engine):
    sp = engine
    rng = np.random.default_rng(3)
    net = sp.snn(1e-4, 1e-4, [5])
    S = net.add_population(sp.poisson(), 700)
    D = net.add_population(sp.lif(), 300)
    adj = sp.adj_list()
    pairs = list(zip(rng.integers(0, 700, 20000).tolist(), rng.integers(0, 300, 20000).tolist()))
    pairs += pairs[:500]  # duplicate (source, target) pairs
    for a, b in pairs:
        adj.connect(a, b)
    c = net.connect(S, D, adj, 1e-4, sp.fixed_weight(0.1))
    off, nb = net.csr(c)
    coff, csrc = net.csc(c)
    eoff, esrc = _transpose(off, nb, 300)
    assert np.array_equal(coff, eoff) and np.array_equal(csrc, esrc)


def test_weights_equal_the_oracle(engine, oracle_lib):
    sp, o = engine, oracle_lib
    net, pops, conns = _weighted_net(sp, o)
    ref, rpops, rconns = o.weighted_net()
    for c, rc, (kind, *_r) in zip(conns, rconns, o.WEIGHTED_NET["conns"]):
        if kind == "w":
            assert np.array_equal(net.synapse_weights(c).view(np.uint32), ref.syn_weights(rc).view(np.uint32)), c


def _states(pops, kinds):
    out = {}
    for k, (p, kind) in enumerate(zip(pops, kinds)):
        if kind == "poisson":
            continue
        st = p.get_neurons()
        out[k] = {f: st[f] for f in (("V", "Gex", "Gin", "Tref") if kind == "lif_cond" else ("V", "Tref"))}
    return out


@pytest.mark.parametrize("how", ["run_record", "stepwise"])
def test_weighted_net_golden(engine, oracle_lib, how):
    """Raster and final states equal the reference binary's (deterministic mode: populations 1-3 are
    pulled for their weighted inputs, population 4 for its six distinct fixed weights)."""
    sp, o = engine, oracle_lib
    g = np.load(os.path.join(GOLDEN, "weighted_net.npz"))
    steps = int(g["steps"][0])
    net, pops, _ = _weighted_net(sp, o)
    if how == "run_record":
        raster = net.run_record(steps)
    else:
        raster = []
        for _ in range(steps):
            net.step()
            raster.append([net.spikes(p, 0) for p in pops])
    counts = np.array([[len(x) for x in row] for row in raster])
    idx = np.concatenate([np.asarray(x) for row in raster for x in row] + [np.zeros(0, np.int32)])
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(idx, g["idx"])
    kinds = [p[0] for p in o.WEIGHTED_NET["pops"]]
    for k, st in _states(pops, kinds).items():
        for f, v in st.items():
            key = f"T{k}" if f == "Tref" else f"{f}{k}"
            assert np.array_equal(np.asarray(v).view(np.uint32), g[key].view(np.uint32)), (k, f)


def test_weighted_net_state_reads_between_steps(engine, oracle_lib):
    """Reading the state between steps applies the pulled inputs of the next step once (the
    reference has already delivered them): states equal the oracle's after every step."""
    sp, o = engine, oracle_lib
    net, pops, _ = _weighted_net(sp, o)
    ref, rpops, _ = o.weighted_net()
    for t in range(60):
        net.step()
        ref.step()
        for k in (1, 3):
            assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32),
                                  ref.state(rpops[k], 0).view(np.uint32)), (t, k)
        assert np.array_equal(net.get_state(pops[3], sp.FIELD_GIN).view(np.uint32),
                              ref.state(rpops[3], 2).view(np.uint32)), t
    net.run(100)
    ref.run(100)
    for k in range(5):
        assert np.array_equal(net.spikes(pops[k], 0), ref.spikes(rpops[k], 0)), k


def test_weighted_net_atomic_mode(engine, oracle_lib):
    """In atomic mode the pulled populations stay bit-exact (population 4, with fixed weights only,
    takes the atomic push path; nothing depends on it)."""
    sp, o = engine, oracle_lib
    net, pops, _ = _weighted_net(sp, o, mode=sp.MODE_ATOMIC)
    ref, rpops, _ = o.weighted_net()
    raster = net.run_record(400)
    for t, row in enumerate(raster):
        ref.step()
        for k in range(4):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    for k in (1, 2, 3):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))


def test_pull_forced_on_brunel(engine, oracle_lib):
    """Every population pulled (fixed weights through the pull path): bit-exact with the oracle, and
    the events equal the push path's."""
    sp, o = engine, oracle_lib
    N, p, seed = 6000, 0.05, 21
    net, pops = sp.brunel(N, p, seed)
    net.set_tuning(pull=True)
    push, _ = sp.brunel(N, p, seed)
    ref, rpops = o.brunel(N, p, seed)
    raster = net.run_record(500)
    for t, row in enumerate(raster):
        ref.step()
        for k in range(3):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
    push.run(500)
    assert net.events == push.events


@pytest.mark.parametrize("fed", [True, False])
def test_pulled_population_without_neurons(engine, fed):
    """A pulled population of size 0 (the reference allows empty populations), beside a pulled one
    with neurons (fed) or as the only pulled one: many windows run without error and the other
    population matches the push path bit for bit."""
    sp = engine
    nets = []
    for pull in (False, True):
        net = sp.snn(1e-4, 15e-4, [3])
        P = net.add_population(sp.poisson(20.0), 2000)
        E = net.add_population(sp.lif(), 0)
        I = net.add_population(sp.lif(), 400)
        net.connect(P, E, sp.fixed_probability(0.1), 15e-4, sp.fixed_weight(0.02))
        if fed:
            net.connect(P, I, sp.fixed_probability(0.1), 15e-4, sp.fixed_weight(0.02))
            net.connect(I, I, sp.fixed_probability(0.1), 15e-4, sp.fixed_weight(-0.01))
        if pull:
            net.set_tuning(pull=True)
        net.run(1500)
        nets.append((net, I))
    (a, ia), (b, ib) = nets
    assert np.array_equal(a.get_state(ia, sp.FIELD_V).view(np.uint32), b.get_state(ib, sp.FIELD_V).view(np.uint32))
    assert a.events == b.events


def test_pull_ungrouped_bins(engine, oracle_lib):
    """Sources firing at several steps of one window (Poisson at 3 kHz, windows of 16 steps): the
    bins overflow the targets' regions and the neuron update walks the active list instead; still
    bit-exact with the oracle."""
    sp, o = engine, oracle_lib
    spec = {"dt": 1e-4, "max_delay": 16e-4, "seed": 77,
            "pops": [("poisson", 400, 3000.0), ("lif", 300)],
            "conns": [("w", 0, 1, 0.2, 16e-4, 1e-4, 0), ("f", 1, 1, 0.1, 16e-4, 0.001, 0)]}
    net, pops, _ = _weighted_net(sp, o, spec=spec)
    ref, rpops, _ = o.weighted_net(spec)
    raster = net.run_record(200, capacity=200 * 700)
    for t, row in enumerate(raster):
        ref.step()
        for k in range(2):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    assert np.array_equal(net.get_state(pops[1], sp.FIELD_V).view(np.uint32), ref.state(rpops[1], 0).view(np.uint32))


def test_many_distinct_weights_no_longer_refused(engine, oracle_lib):
    """Six fixed_weight connections with distinct weights into one population (deterministic mode):
    pulled instead of refused, bit-exact with the oracle."""
    sp, o = engine, oracle_lib
    spec = {"dt": 1e-4, "max_delay": 6e-4, "seed": 8,
            "pops": [("poisson", 2000, 30.0), ("lif", 1000)],
            "conns": [("f", 0, 1, 0.05, (2 + j) * 1e-4, 0.002 + 0.0007 * j, 0) for j in range(5)]
            + [("f", 1, 1, 0.05, 2e-4, -0.003, 0)]}
    net, pops, _ = _weighted_net(sp, o, spec=spec)
    ref, rpops, _ = o.weighted_net(spec)
    raster = net.run_record(300)
    for t, row in enumerate(raster):
        ref.step()
        for k in range(2):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    assert np.array_equal(net.get_state(pops[1], sp.FIELD_V).view(np.uint32), ref.state(rpops[1], 0).view(np.uint32))


def test_pull_errors(engine):
    sp = engine
    net = sp.snn(1e-4, 1e-4, [1])
    net.set_mode(sp.MODE_ATOMIC)
    S = net.add_population(sp.lif_cond(), 50)
    net.connect(S, S, sp.fixed_probability(0.1), 1e-4, sp.weighted(0.1, sp.FIELD_GEX))
    net.connect(S, S, sp.fixed_probability(0.1), 1e-4, sp.istdp(0.3))
    with pytest.raises(sp.LogicError, match="plastic synapses into a population whose inputs are pulled"):
        net.run(1)
    a, _ = sp.brunel(2000, 0.1, 1)
    a.run(1)
    with pytest.raises(sp.SpiceError, match="fixed once the network steps"):
        a.set_tuning(pull=True)
