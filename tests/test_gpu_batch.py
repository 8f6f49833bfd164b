"""Batched networks (spice_batch_*): many uneven Brunel nets stepped by shared launches and CUDA
graph replays give each member exactly the results of running it alone, on the plain GPU path and
on the CPU oracle (deterministic mode: bit for bit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1000, 2530, 4000, 1770, 3210, 5000, 1200, 2890]
# uneven run lengths: partial windows, single steps and graph replays (3 windows per graph)
RUNS = [7, 15, 64, 1, 150, 33]


def _snapshot(sp, net, pops):
    out = {"time": net.time, "events": net.events}
    for i, P in enumerate(pops):
        if i > 0:
            out[f"V{i}"] = net.get_state(P, sp.FIELD_V).view(np.uint32)
            out[f"T{i}"] = net.get_state(P, sp.FIELD_TREF)
        for age in range(15):
            out[f"s{i}_{age}"] = net.spikes(P, age)
    return out


def _assert_same(a, b, what):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), f"{what}: {k} differs"


def test_batch_matches_plain_deterministic(engine):
    sp = engine
    plain = sp.brunel_sweep(SIZES, seed0=77)
    bat = sp.brunel_sweep(SIZES, seed0=77)
    for r in RUNS:
        for net, _ in plain:
            net.run(r)
    b = sp.batch([n for n, _ in bat])
    b.set_tuning(graph_windows=3)
    for r in RUNS:
        b.run(r)
    assert b.launch_count() > 0
    for i, ((n1, p1), (n2, p2)) in enumerate(zip(plain, bat)):
        _assert_same(_snapshot(sp, n1, p1), _snapshot(sp, n2, p2), f"net {i} (N={SIZES[i]})")


def test_batch_member_matches_oracle(engine, oracle_lib):
    sp, o = engine, oracle_lib
    nets = sp.brunel_sweep([2000, 3500, 1500], seed0=5)
    b = sp.batch([n for n, _ in nets])
    b.set_tuning(graph_windows=2)
    b.run(100)
    b.run(37)
    for i, (N, (net, pops)) in enumerate(zip([2000, 3500, 1500], nets)):
        ref, rpops = o.brunel(N, 0.1, 5 + i)
        ref.run(137)
        for k in range(3):
            for age in range(15):
                assert np.array_equal(net.spikes(pops[k], age), ref.spikes(rpops[k], age)), (i, k, age)
        for k in (1, 2):
            assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32),
                                  ref.state(rpops[k], 0).view(np.uint32))
            assert np.array_equal(net.get_state(pops[k], sp.FIELD_TREF), ref.state(rpops[k], 3))
        # the engine counts a spike's events when its window is delivered (into the input ring),
        # the reference when the spike reaches age d - 1 = 14: the engine is ahead by the events of
        # the spikes of ages 0..13
        offs = [net.csr(c)[0] for c in range(6)]
        src_of = [0, 0, 1, 1, 2, 2]
        ahead = sum(int(np.sum(offs[c][net.spikes(pops[src_of[c]], age) + 1] - offs[c][net.spikes(pops[src_of[c]], age)]))
                    for c in range(6) for age in range(14))
        assert net.events == ref.events + ahead


@pytest.mark.parametrize("shape", [
    dict(deliver_algo=0), dict(deliver_algo=2), dict(deliver_algo=3, deliver_threads=512), dict(deliver_algo=4),
    dict(deliver_algo=5), dict(deliver_algo=6, tile_bytes=48 * 1024), dict(deliver_algo=8, deliver_parts=2),
    dict(deliver_algo=9, tile_bytes=100 * 1024, deliver_threads=1024),
    dict(deliver_algo=12, tile_bytes=48 * 1024, deliver_threads=512), dict(deliver_algo=14, deliver_parts=2),
    dict(deliver_algo=15, tile_bytes=24 * 1024, deliver_threads=256), dict(deliver_algo=15, deliver_parts=3),
    dict(deliver_parts=2), dict(tile_bytes=4096, deliver_threads=128), dict(overlap_sources=False),
    dict(graph_windows=0), dict(deliver_algo=20, tile_bytes=48 * 1024, deliver_threads=512),
    dict(deliver_algo=21, tile_bytes=24 * 1024, deliver_threads=512),
])
def test_batch_launch_shapes(engine, shape):
    """Every launch shape gives the same bits (results never depend on the shape)."""
    sp = engine
    sizes = [1500, 4200, 2600]
    ref = sp.brunel_sweep(sizes, seed0=9)
    for net, _ in ref:
        net.run(95)
    bat = sp.brunel_sweep(sizes, seed0=9)
    b = sp.batch([n for n, _ in bat])
    b.set_tuning(**shape)
    b.run(40)
    b.run(55)
    for (n1, p1), (n2, p2) in zip(ref, bat):
        _assert_same(_snapshot(sp, n1, p1), _snapshot(sp, n2, p2), str(shape))


def test_batch_atomic_mode_rates(engine):
    """Atomic mode adds float sums in arbitrary order: firing rates match the plain path's."""
    sp = engine
    sizes = [3000, 5000]
    plain = sp.brunel_sweep(sizes, seed0=21, mode=sp.MODE_ATOMIC)
    bat = sp.brunel_sweep(sizes, seed0=21, mode=sp.MODE_ATOMIC)
    counts_p = np.zeros((2, 3))
    counts_b = np.zeros((2, 3))
    b = sp.batch([n for n, _ in bat])
    for _ in range(20):
        for i, (net, pops) in enumerate(plain):
            net.run(15)
            counts_p[i] += [sum(len(net.spikes(P, a)) for a in range(15)) for P in pops]
        b.run(15)
        for i, (net, pops) in enumerate(bat):
            counts_b[i] += [sum(len(net.spikes(P, a)) for a in range(15)) for P in pops]
    # Poisson sources do not depend on the mode's rounding: identical
    assert np.array_equal(counts_p[:, 0], counts_b[:, 0])
    rel = np.abs(counts_p[:, 1:] - counts_b[:, 1:]) / np.maximum(counts_p[:, 1:], 1)
    assert np.all(rel < 0.1), (counts_p, counts_b)


def test_batch_preconditions(engine):
    sp = engine
    a, _ = sp.brunel(1000, 0.1, 1)
    c = sp.snn(2e-4, 15e-4, [1])
    c.add_population(sp.lif(), 10)
    with pytest.raises(sp.LogicError):
        sp.batch([a, c])  # different dt
    d = sp.snn(1e-4, 15e-4, [1])
    d.add_population(sp.external_input(((1,), ())), 4)
    with pytest.raises(sp.LogicError):
        sp.batch([a, d])
    with pytest.raises(sp.LogicError):
        sp.batch([a, a])
    e, _ = sp.brunel(1200, 0.1, 2)
    b = sp.batch([a, e])
    a.run(3)  # a member stepped on its own is no longer in lockstep
    with pytest.raises(sp.SpiceError):
        b.run(5)
    e.run(3)
    b.run(5)
    assert a.time == e.time == 8
