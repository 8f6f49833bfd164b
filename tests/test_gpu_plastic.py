"""Plastic synapses on the GPU (lazy catch-up of synapse_population.h:82-140) against the oracle,
whose schedule is pinned to the reference binary (tests/test_oracle_plastic.py).

* counting model (the reference tests' plastic_synapse) on Brunel nets in deterministic mode:
  every per-synapse count, the raster and V/Tref bit for bit;
* iSTDP with one plastic input per target (one addend per target and step, so atomic-mode sums
  are exact): weights, traces, conductances and spikes bit for bit;
* the plastic E/I network (conductance LIF, iSTDP on I->E) at N=1e5: mean firing rates and ISI CVs
  over ten seeds within 1 % of the reference binary's (atomic-mode sums make the dynamics diverge,
  so the comparison is statistical), and the rule moving the E rate toward its target rate."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

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


def _plastic_ei_c3(sp, N, seed, eta=1e-3):
    """The plastic E/I network as bench.py times it (E 0.03, I 0.3 over the 10 nS leak)."""
    net = sp.snn(1e-4, 1e-4, [seed])
    net.set_mode(sp.MODE_ATOMIC)
    E = net.add_population(sp.lif_cond(), N * 8 // 10)
    I = net.add_population(sp.lif_cond(), N * 2 // 10)
    net.connect(E, E, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
    net.connect(E, I, sp.fixed_probability(0.02), 1e-4, sp.excitatory(0.03))
    c = net.connect(I, E, sp.fixed_probability(0.02), 1e-4, sp.istdp(0.3, eta=eta, rho0=5.0, tau=0.02))
    net.connect(I, I, sp.fixed_probability(0.02), 1e-4, sp.inhibitory(0.3))
    return net, E, I, c


def _isi(raster, k, n):
    """Pooled inter-spike intervals (in steps) of population k: count, sum, sum of squares."""
    last = np.full(n, -1, dtype=np.int64)
    cnt = tot = sq = 0.0
    for t, row in enumerate(raster):
        idx = np.asarray(row[k], dtype=np.int64)
        prev = last[idx]
        d = (t - prev[prev >= 0]).astype(np.float64)
        cnt, tot, sq = cnt + d.size, tot + d.sum(), sq + (d * d).sum()
        last[idx] = t
    return np.array([cnt, tot, sq])


def _cv(isi):
    m = isi[1] / isi[0]
    return np.sqrt(isi[2] / isi[0] - m * m) / m


def test_plastic_ei_network_matches_the_reference_over_ten_seeds(engine):
    """The plastic E/I network at N=1e5 (5000 steps, iSTDP on I->E, atomic mode) against the
    reference binary's runs of the same network (tests/golden/plastic_ei_n100000.npz): over seeds
    1..10, the mean firing rates and pooled ISI CVs of E and I within 1 % of the reference's."""
    sp = engine
    g = np.load(os.path.join(GOLDEN, "plastic_ei_n100000.npz"))
    N, steps = (int(x) for x in g["meta"])
    sizes = (N * 8 // 10, N * 2 // 10)
    ref_rate, ref_cv, gpu_rate, gpu_cv = [], [], [], []
    for sd in range(1, 11):
        counts = g[f"counts_s{sd}"]
        isi = g[f"isi_s{sd}"]
        ref_rate.append([counts[:, k].sum() / sizes[k] / (steps * 1e-4) for k in range(2)])
        ref_cv.append([_cv(isi[k]) for k in range(2)])
        net, E, I, _ = _plastic_ei_c3(sp, N, sd, float(g["eta"][0]))
        raster = net.run_record(steps, capacity=steps * 400 + 4096)
        net.close()
        gpu_rate.append([sum(len(r[k]) for r in raster) / sizes[k] / (steps * 1e-4) for k in range(2)])
        gpu_cv.append([_cv(_isi(raster, k, sizes[k])) for k in range(2)])
    ref_rate, ref_cv = np.array(ref_rate), np.array(ref_cv)
    gpu_rate, gpu_cv = np.array(gpu_rate), np.array(gpu_cv)
    for name, r, q in (("rate", ref_rate, gpu_rate), ("ISI CV", ref_cv, gpu_cv)):
        for k, pop in enumerate("EI"):
            assert abs(q[:, k].mean() - r[:, k].mean()) <= 0.01 * r[:, k].mean(), (
                name, pop, q[:, k].mean(), r[:, k].mean(), q[:, k].std(), r[:, k].std())
    assert ref_rate.min() > 1.0


def test_istdp_moves_the_excitatory_rate_toward_rho0(engine):
    """The plastic E/I network at N=1e5 with a learning rate that acts within seconds (eta 0.05):
    after the opening burst E fires far below rho0 = 5 Hz, so iSTDP depresses the I->E weights
    and the E rate climbs toward 5 Hz over 4 s of simulated time (the oracle's run of the same
    network: 0.5 Hz after the burst, 1.6 Hz after 3.5 s, 3.5 Hz after 4 s; weights 0.336 -> 0.305)."""
    sp = engine
    N = 100000
    net, E, I, c = _plastic_ei_c3(sp, N, 3, eta=0.05)
    rates, wmean = [], []
    for _ in range(16):
        raster = net.run_record(2500, capacity=2500 * 2000 + 4096)
        rates.append(sum(len(r[0]) for r in raster) / (N * 0.8) / 0.25)
        wmean.append(float(net.synapse_state(c, 0).mean()))
    net.close()
    early, late = np.mean(rates[1:4]), np.mean(rates[-4:])
    assert early < 1.5 and late > 2 * early, rates
    assert wmean[-1] < wmean[1] - 0.015, wmean


def test_trace_decay_rounding_matches_double_multiply(engine):
    """The traces' skip() decay, (float)((double)x * f), is computed in integer arithmetic: equal in
    every bit to the GPU's double multiply on 2^27 random pairs (subnormal x, overflowing products)."""
    m, a, f = engine.selftest_skip_rounding(1 << 27, 12345)
    assert m == 0, f"{m} mismatches, first x bits {a:#010x}, f {f!r}"
