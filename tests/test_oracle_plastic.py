"""CPU pins of the oracle's lazy plasticity (synapse_population.h:82-140) against the reference:
the counting model of the reference's own tests, and the reference binary itself on Brunel nets
with a plastic E->E projection.  The counting model delivers count * 2^-12 to V, so every step of
the lazy schedule (catch-up at delivery, the 64-step periodic update, post spikes from the 64-bit
history) shows in the raster and the membrane potentials."""
import numpy as np
import pytest

from oracle import oracle as o

SCALE = 2.0 ** -12


def _counting_net(trains, post_trains=None, n_src=3, n_dst=5, edges=((0, 0), (0, 1), (0, 3), (1, 3), (2, 4))):
    n = o.Net(1.0, 1.0, [1337])
    S = n.add_population(o.EXTERNAL, n_src)
    T = n.add_population(o.LIF, n_dst)
    c = n.connect_adj(S, T, list(edges), 1.0, 0.0)
    n.set_plastic(c, o.SYN_COUNT)
    n.set_external(S, trains)
    if post_trains is not None:
        D = n.add_population(o.EXTERNAL, n_dst)
        n.connect_adj(D, T, [(j, j) for j in range(n_dst)], 1.0, 1.0)
        n.set_external(D, post_trains)
    return n, c


def test_counting_model_reference_cases():
    """test/detail/synapse_population.cpp:96-167 in network form: sources 1 and 2 spike at step
    9; their synapses have been updated once per step by then (10 updates), the others once (the
    periodic update at step 0)."""
    n, c = _counting_net([[]] * 9 + [[1, 2]])
    n.run(10)
    assert n.syn_state(c).tolist() == [1, 1, 1, 10, 10]
    # spiking at step 0: the periodic update of step 0 (one update), then the delivery of step 0
    # does not update again (synapse_population.cpp:114-123: one update per step)
    n, c = _counting_net([[1, 2]])
    n.run(1)
    assert n.syn_state(c).tolist() == [1, 1, 1, 1, 1]


def test_counting_model_every_step_once():
    """Over any run, a synapse is updated exactly once per step it has been caught up through:
    after the periodic update of step 128 every count equals 129 (plus the pending pre updates of
    deliveries, which replace a skipped step rather than adding one), with post spikes on the way."""
    rng = np.random.default_rng(1)
    trains = [list(np.flatnonzero(rng.random(3) < 0.1)) for _ in range(200)]
    post = [list(np.flatnonzero(rng.random(5) < 0.2)) for _ in range(200)]
    n, c = _counting_net(trains, post)
    n.run(129)
    assert n.syn_state(c).tolist() == [129.0] * 5


def _plastic_brunel_spec(N, p, seed, steps, pp, pdelay):
    lines = o.brunel_spec(N, p, seed, steps)
    lines.append(f"plastic 1 {pp!r} {pdelay!r} {SCALE!r}")
    return lines


def _plastic_brunel_oracle(N, p, seed, pp, pdelay):
    net, (P, E, I) = o.brunel(N, p, seed)
    c = net.connect(E, E, pp, pdelay, SCALE)
    net.set_plastic(c, o.SYN_COUNT)
    return net, (P, E, I), c


@pytest.mark.parametrize("pdelay,N,p,seed,steps", [(1e-4, 4000, 0.05, 7, 400), (15e-4, 4000, 0.05, 7, 400),
                                                  (5e-4, 2500, 0.08, 99, 500), (3e-4, 6000, 0.03, 2024, 300)])
def test_oracle_plastic_matches_reference_binary(pdelay, N, p, seed, steps):
    """The plastic restatement (counting model on E->E, lazy catch-up every 64 steps and at each
    delivery) against the reference binary: rasters, LIF state and the schedule's counts."""
    if not o.have_reference():
        pytest.skip("reference driver not built on this host")
    res = o.run_reference_net(_plastic_brunel_spec(N, p, seed, steps, 0.05, pdelay))
    net, pops, c = _plastic_brunel_oracle(N, p, seed, 0.05, pdelay)
    for t in range(steps):
        net.step()
        for k in range(3):
            assert np.array_equal(net.spikes(pops[k], 0), res["raster"][t][k]), (t, k)
    st, _, _ = o.reference_states(res, [1, 2])
    for k in (1, 2):
        assert np.array_equal(net.state(pops[k], 0).view(np.uint32), st[k][0].view(np.uint32))
        assert np.array_equal(net.state(pops[k], 3), st[k][1])
    counts = net.syn_state(c)
    assert counts.max() > 64  # the schedule ran through several periodic updates
