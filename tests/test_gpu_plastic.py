"""Plastic synapses on the GPU (lazy catch-up of synapse_population.h:82-140) against the oracle,
whose schedule is pinned to the reference binary (tests/test_oracle_plastic.py).

* counting model (the reference tests' plastic_synapse) on Brunel nets in deterministic mode:
  every per-synapse count, the raster and V/Tref bit for bit;
* iSTDP with one plastic input per target (one addend per target and step, so atomic-mode sums
  are exact): weights, traces, conductances and spikes bit for bit;
* the plastic E/I network (conductance LIF, iSTDP on I->E): firing rates and weight statistics
  within the oracle's seed-to-seed spread (atomic-mode sums make the dynamics diverge)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pdelay", [1e-4, 15e-4])
def test_counting_schedule_matches_oracle(engine, oracle_lib, pdelay):
    sp, o = engine, oracle_lib
    N, p, seed, steps = 4000, 0.05, 7, 300
    net, pops = sp.brunel(N, p, seed)
    c = net.connect(pops[1], pops[1], sp.fixed_probability(0.05), pdelay, sp.count_synapse(0.0))
    ref, rpops = o.brunel(N, p, seed)
    rc = ref.connect(rpops[1], rpops[1], 0.05, pdelay, 0.0)
    ref.set_plastic(rc, o.SYN_COUNT)
    raster = net.run_record(steps)
    for t in range(steps):
        ref.step()
        for k in range(3):
            assert np.array_equal(raster[t][k], ref.spikes(rpops[k], 0)), (t, k)
    assert np.array_equal(net.synapse_state(c, 0), ref.syn_state(rc, 0))
    for k in (1, 2):
        st = pops[k].get_neurons()
        assert np.array_equal(st["V"].view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
        assert np.array_equal(st["Tref"], ref.state(rpops[k], 3))


def test_istdp_single_input_matches_oracle(engine, oracle_lib):
    sp, o = engine, oracle_lib
    n_, steps = 96, 3000
    rng = np.random.default_rng(5)
    pre = [list(np.flatnonzero(rng.random(n_) < 0.01)) for _ in range(500)]
    drive = [list(np.flatnonzero(rng.random(n_) < 0.03)) for _ in range(700)]
    one2one = [(i, i) for i in range(n_)]
    net = sp.snn(1e-4, 1e-4, [3])
    net.set_mode(sp.MODE_ATOMIC)
    S = net.add_population(sp.external_input(tuple(tuple(int(x) for x in t) for t in pre)), n_)
    D = net.add_population(sp.external_input(tuple(tuple(int(x) for x in t) for t in drive)), n_)
    T = net.add_population(sp.lif_cond(), n_)
    adj = sp.adj_list(list(one2one))
    net.connect(D, T, adj, 1e-4, sp.excitatory(2.0))
    c = net.connect(S, T, adj, 1e-4, sp.istdp(0.5, eta=0.05, rho0=5.0, tau=0.02))
    ref = o.Net(1e-4, 1e-4, [3])
    rS = ref.add_population(o.EXTERNAL, n_)
    rD = ref.add_population(o.EXTERNAL, n_)
    rT = ref.add_population(o.LIF_COND, n_)
    ref.set_external(rS, pre)
    ref.set_external(rD, drive)
    ref.connect_adj(rD, rT, one2one, 1e-4, 2.0, 1)
    rc = ref.connect_adj(rS, rT, one2one, 1e-4, 0.5, 2)
    ref.set_plastic(rc, o.SYN_ISTDP, 0.5, 0.05, 5.0, 0.02)
    raster = net.run_record(steps)
    n_post = 0
    for t in range(steps):
        ref.step()
        assert np.array_equal(raster[t][2], ref.spikes(rT, 0)), t
        n_post += len(raster[t][2])
    assert n_post > 100
    for f in range(3):
        g, r = net.synapse_state(c, f), ref.syn_state(rc, f)
        assert np.array_equal(g.view(np.uint32), r.view(np.uint32)), f
    st = T.get_neurons()
    for name, f in (("V", 0), ("Gex", 1), ("Gin", 2)):
        assert np.array_equal(st[name].view(np.uint32), ref.state(rT, f).view(np.uint32)), name
    W = net.synapse_state(c, 0)
    assert np.unique(W).size > 10 and not np.allclose(W, 0.5)  # the weights did move


def _plastic_ei(sp, N, seed):
    net = sp.snn(1e-4, 1e-4, [seed])
    net.set_mode(sp.MODE_ATOMIC)
    E = net.add_population(sp.lif_cond(), N * 8 // 10)
    I = net.add_population(sp.lif_cond(), N * 2 // 10)
    net.connect(E, E, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.3))
    net.connect(E, I, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.3))
    c = net.connect(I, E, sp.fixed_probability(0.02), 1e-4, sp.istdp(3.0, eta=1e-3, rho0=5.0, tau=0.02))
    net.connect(I, I, sp.fixed_probability(0.02), 1e-4, sp.inhibitory(3.0))
    return net, E, I, c


def _plastic_ei_oracle(o, N, seed):
    n = o.Net(1e-4, 1e-4, [seed])
    E = n.add_population(o.LIF_COND, N * 8 // 10)
    I = n.add_population(o.LIF_COND, N * 2 // 10)
    n.connect(E, E, 0.02, 1e-4, 0.3, 1)
    n.connect(E, I, 0.02, 1e-4, 0.3, 1)
    c = n.connect(I, E, 0.02, 1e-4, 3.0, 2)
    n.set_plastic(c, o.SYN_ISTDP, 3.0, 1e-3, 5.0, 0.02)
    n.connect(I, I, 0.02, 1e-4, 3.0, 2)
    return n, E, I, c


def test_plastic_ei_network_statistics(engine, oracle_lib):
    sp, o = engine, oracle_lib
    N, warm, steps = 10000, 1000, 3000
    for seed in (1, 2):
        net, E, I, c = _plastic_ei(sp, N, seed)
        net.run(warm)
        W0 = net.synapse_state(c, 0).astype(np.float64)
        raster = net.run_record(steps)
        gE = sum(len(r[0]) for r in raster) / (N * 0.8) / (steps * 1e-4)
        gI = sum(len(r[1]) for r in raster) / (N * 0.2) / (steps * 1e-4)
        gdW = net.synapse_state(c, 0).astype(np.float64) - W0
        ref, rE, rI, rc = _plastic_ei_oracle(o, N, seed)
        ref.run(warm)
        R0 = ref.syn_state(rc, 0).astype(np.float64)
        cE = cI = 0
        for _ in range(steps):
            ref.step()
            cE += len(ref.spikes(rE, 0))
            cI += len(ref.spikes(rI, 0))
        oE, oI = cE / (N * 0.8) / (steps * 1e-4), cI / (N * 0.2) / (steps * 1e-4)
        odW = ref.syn_state(rc, 0).astype(np.float64) - R0
        assert abs(gE - oE) < 0.15 * oE and abs(gI - oI) < 0.15 * oI, (seed, gE, oE, gI, oI)
        assert abs(gdW.std() - odW.std()) < 0.25 * odW.std(), (seed, gdW.std(), odW.std())
        assert gE > 1.0 and gI > 1.0


def test_trace_decay_rounding_matches_double_multiply(engine):
    """The traces' skip() decay, (float)((double)x * f), is computed in integer arithmetic: equal in
    every bit to the GPU's double multiply on 2^27 random pairs (subnormal x, overflowing products)."""
    m, a, f = engine.selftest_skip_rounding(1 << 27, 12345)
    assert m == 0, f"{m} mismatches, first x bits {a:#010x}, f {f!r}"
