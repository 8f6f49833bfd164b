"""GPU: persistent steps (SPICE_TUNE_PERSISTENT) -- networks whose windows are one step long run a
chunk of steps as one cooperative launch with grid-wide barriers between the phases of a step.
Deterministic mode must stay bit-exact with the oracle (and with the launch-per-phase path), with
and without plastic synapses, recorded or not, and when the path is switched off and on between
steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare_brunel(sp, o, N, p, seed, delay, steps, persistent, record=True):
    net, pops = sp.brunel(N, p, seed, delay=delay)
    net.set_tuning(persistent=persistent)
    ref, rpops = o.brunel(N, p, seed, delay=delay)
    net.csr(0)  # the adjacency and the first launches of the net, before counting
    net.run(0)
    l0 = net.launch_count()
    if record:
        raster = net.run_record(steps)
        for t in range(steps):
            ref.step()
            for k in range(3):
                assert np.array_equal(np.asarray(raster[t][k]), ref.spikes(rpops[k], 0)), (t, k)
    else:
        net.run(steps)
        ref.run(steps)
        for k in range(3):  # the spike history holds max_delay steps (ages 0 .. D - 1)
            for age in range(max(1, int(round(delay / 1e-4)))):
                assert np.array_equal(net.spikes(pops[k], age), ref.spikes(rpops[k], age)), (k, age)
    launches = net.launch_count() - l0
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_TREF), ref.state(rpops[k], 3))
    return net, launches


@pytest.mark.parametrize("persistent", [1, 0, 2, 8])
def test_delay_one_brunel_bit_exact(engine, oracle_lib, persistent):
    """Brunel with delay 1 step (windows of one step): raster and V / Tref equal the oracle's,
    persistent (default, 2 and 8 CTAs per SM) or one launch per phase."""
    net, launches = _compare_brunel(engine, oracle_lib, 6000, 0.05, 17, 1e-4, 400, persistent)
    if persistent:
        assert launches <= 4  # jump tables and one cooperative launch per chunk, not launches per step
    else:
        assert launches >= 400


def test_delay_one_brunel_unrecorded_and_stepwise(engine, oracle_lib):
    sp, o = engine, oracle_lib
    _compare_brunel(sp, o, 4000, 0.05, 3, 1e-4, 1500, 1, record=False)  # two chunks of 1024 steps
    _compare_brunel(sp, o, 4000, 0.05, 4, 3e-4, 700, 1, record=False)   # delay 3: K = 3, not persistent
    net, pops = sp.brunel(3000, 0.1, 9, delay=1e-4)
    ref, rpops = o.brunel(3000, 0.1, 9, delay=1e-4)
    for t in range(120):
        net.step()
        ref.step()
        for k in range(3):
            assert np.array_equal(net.spikes(pops[k], 0), ref.spikes(rpops[k], 0)), (t, k)


def test_switching_between_paths(engine, oracle_lib):
    """Persistent steps, then one launch per phase, then persistent again: one network, bit-exact."""
    sp, o = engine, oracle_lib
    net, pops = sp.brunel(5000, 0.05, 23, delay=1e-4)
    ref, rpops = o.brunel(5000, 0.05, 23, delay=1e-4)
    for persistent, steps in ((1, 150), (0, 170), (1, 90)):
        net.set_tuning(persistent=persistent)
        raster = net.run_record(steps)
        for t in range(steps):
            ref.step()
            for k in range(3):
                assert np.array_equal(np.asarray(raster[t][k]), ref.spikes(rpops[k], 0)), (persistent, t, k)
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))


def test_mixed_delays_bit_exact(engine, oracle_lib):
    """Delays of 1, 2 and 5 steps in one network (windows of one step, ring slots ahead of the
    current step): bit-exact with the oracle."""
    sp, o = engine, oracle_lib
    spec = {"dt": 1e-4, "max_delay": 5e-4, "seed": 31,
            "pops": [("poisson", 3000, 25.0), ("lif", 2000), ("lif", 500)],
            "conns": [("f", 0, 1, 0.05, 1e-4, 0.004, 0), ("f", 0, 2, 0.05, 2e-4, 0.004, 0),
                      ("f", 1, 1, 0.05, 5e-4, 0.002, 0), ("f", 1, 2, 0.05, 1e-4, 0.002, 0),
                      ("f", 2, 1, 0.05, 2e-4, -0.01, 0), ("f", 2, 2, 0.05, 1e-4, -0.01, 0)]}
    net = sp.snn(spec["dt"], spec["max_delay"], [spec["seed"]])
    pops = [net.add_population(sp.poisson(25.0), 3000), net.add_population(sp.lif(), 2000),
            net.add_population(sp.lif(), 500)]
    for _, s, d, p, delay, w, _f in spec["conns"]:
        net.connect(pops[s], pops[d], sp.fixed_probability(p), delay, sp.fixed_weight(float(np.float32(w))))
    ref, rpops, _ = o.weighted_net(spec)
    raster = net.run_record(500)
    for t in range(500):
        ref.step()
        for k in range(3):
            assert np.array_equal(np.asarray(raster[t][k]), ref.spikes(rpops[k], 0)), (t, k)
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))


@pytest.mark.parametrize("pdelay", [1e-4, 15e-4])
def test_counting_plastic_schedule_persistent(engine, oracle_lib, pdelay):
    """The counting plastic synapse (lazy catch-up every 64 steps and at each delivery) through the
    persistent path: every per-synapse count, the raster and V / Tref bit for bit."""
    sp, o = engine, oracle_lib
    N, p, seed, steps = 4000, 0.05, 7, 700
    net, pops = sp.brunel(N, p, seed)
    c = net.connect(pops[1], pops[1], sp.fixed_probability(0.05), pdelay, sp.count_synapse(0.0))
    net.set_tuning(persistent=1)
    ref, rpops = o.brunel(N, p, seed)
    rc = ref.connect(rpops[1], rpops[1], 0.05, pdelay, 0.0)
    ref.set_plastic(rc, o.SYN_COUNT)
    net.run(0)
    l0 = net.launch_count()
    raster = net.run_record(steps)
    for t in range(steps):
        ref.step()
        for k in range(3):
            assert np.array_equal(raster[t][k], ref.spikes(rpops[k], 0)), (t, k)
    assert np.array_equal(net.synapse_state(c, 0), ref.syn_state(rc, 0))
    # per 64 steps: one cooperative launch and the periodic catch-up kernel between two of them
    assert net.launch_count() - l0 <= 2 * (steps // 64 + 2)


def test_persistent_knob_errors(engine):
    sp = engine
    net, _ = sp.brunel(2000, 0.1, 1)  # delay 15: windows of 15 steps, not eligible
    net.run(1)
    with pytest.raises(sp.SpiceError, match="persistent steps are set up"):
        net.set_tuning(persistent=1)
    net.set_tuning(persistent=0)
    with pytest.raises(sp.SpiceError, match="persistent must be"):
        net.set_tuning(persistent=99)
