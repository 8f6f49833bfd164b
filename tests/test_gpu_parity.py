"""GPU parity: the CUDA engine against the CPU oracle (and the reference's golden vectors).

Integer/index results (CSR neighbour lists, spike rasters, Tref) and the float state V are
compared bit for bit: the reference's deterministic path has a single valid answer.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr_cases():
    return [
        (1000, 800, 0.1, 1), (100, 5000, 0.002, 7), (50, 50, 1.0, 3), (10, 10, 0.0, 3),
        (3, 0, 0.5, 1), (0, 10, 0.5, 1), (2000, 2000, 0.5, 9), (300, 70000, 0.01, 11),
        (5, 3, 0.9, 2), (70000, 300, 0.3, 5),
    ]


@pytest.mark.parametrize("src,dst,p,seed", _csr_cases())
def test_fixed_probability_csr_bit_exact(engine, oracle_lib, src, dst, p, seed):
    sp, o = engine, oracle_lib
    net = sp.snn(1e-4, 1e-4, [seed])
    # two stateful populations would consume seeds; use stateless source + lif target and
    # compare against the oracle generator fed the projection's own seed
    S = net.add_population(sp.poisson(), src)
    D = net.add_population(sp.lif(), dst)
    c = net.connect(S, D, sp.fixed_probability(p), 1e-4, sp.fixed_weight(0.0))
    off, nb = net.csr(c)
    chain = o.seed_chain([seed], 2)  # seed 0 -> lif population, seed 1 -> the projection
    roff, rnb, _ = o.fp_generate(src, dst, p, chain[1])
    assert np.array_equal(off, roff)
    assert np.array_equal(nb, rnb)


def _compare_net(sp, o, N, p, seed, steps, use_run=False, mode=0):
    net, pops = sp.brunel(N, p, seed, mode=mode)
    ref, rpops = o.brunel(N, p, seed)
    if use_run:
        raster = net.run_record(steps)
    for t in range(steps):
        if not use_run:
            net.step()
        ref.step()
        for k in range(3):
            a = raster[t][k] if use_run else net.spikes(pops[k], 0)
            b = ref.spikes(rpops[k], 0)
            assert np.array_equal(a, b), f"step {t} pop {k}: {a[:10]} vs {b[:10]}"
    for k in (1, 2):
        st = pops[k].get_neurons()
        assert np.array_equal(st["V"].view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
        assert np.array_equal(st["Tref"], ref.state(rpops[k], 3))
    return net, ref


def test_brunel_step_bit_exact(engine, oracle_lib):
    _compare_net(engine, oracle_lib, 4000, 0.05, 1337, 300)


def test_brunel_run_windows_bit_exact(engine, oracle_lib):
    _compare_net(engine, oracle_lib, 4000, 0.05, 42, 400, use_run=True)


def test_brunel_readme_config(engine, oracle_lib):
    """samples/brunel.cpp as published: N=2e4, p=0.1, seed 1337 (README.md:106-117)."""
    net, ref = _compare_net(engine, oracle_lib, 20000, 0.1, 1337, 300, use_run=True)


# ---- against the reference's golden vectors (independent of the oracle) ------------------------
import json
import os

from conftest import GOLDEN


def _raster_flat(raster):
    counts = np.array([[len(x) for x in row] for row in raster], dtype=np.int32)
    idx = np.concatenate([x for row in raster for x in row] + [np.zeros(0, np.int32)]).astype(np.int32)
    return counts, idx


@pytest.mark.parametrize("name", ["brunel_n20000.npz", "brunel_n5000.npz"])
def test_brunel_golden_raster_and_state(engine, name):
    g = np.load(os.path.join(GOLDEN, name))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    counts, idx = _raster_flat(net.run_record(steps))
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(idx, g["idx"])
    for k in (1, 2):
        st = pops[k].get_neurons()
        assert np.array_equal(st["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))
        assert np.array_equal(st["Tref"], g[f"T{k}"])


def test_mixed_network_golden(engine, oracle_lib):
    """Delays 2..8 steps (window = 2 steps), an adj_list projection, three input groups into E."""
    sp = engine
    g = np.load(os.path.join(GOLDEN, "mixed_net.npz"))
    net = sp.snn(1e-4, 8e-4, [4242])
    P = net.add_population(sp.poisson(50.0), 3000)
    E = net.add_population(sp.lif(), 2000)
    I = net.add_population(sp.lif(), 1000)
    f = lambda x: float(np.float32(x))
    net.connect(P, E, sp.fixed_probability(0.05), 3e-4, sp.fixed_weight(f(0.002)))
    net.connect(E, E, sp.fixed_probability(0.05), 5e-4, sp.fixed_weight(f(0.002)))
    net.connect(I, E, sp.fixed_probability(0.1), 2e-4, sp.fixed_weight(f(-0.005)))
    net.connect(P, I, sp.fixed_probability(0.02), 4e-4, sp.fixed_weight(f(0.004)))
    adj = sp.adj_list()
    for a, b in g["pairs"]:
        adj.connect(a, b)
    net.connect(E, I, adj, 6e-4, sp.fixed_weight(f(0.003)))
    net.connect(I, I, sp.fixed_probability(0.02), 7e-4, sp.fixed_weight(f(-0.004)))
    net.connect(E, E, sp.fixed_probability(0.01), 8e-4, sp.fixed_weight(f(0.003)))
    half = g["counts"].shape[0] // 2
    r1 = net.run_record(half)        # windowed
    r2 = [None] * (g["counts"].shape[0] - half)
    for t in range(len(r2)):         # then single steps
        net.step()
        r2[t] = [net.spikes(p, 0) for p in (P, E, I)]
    counts, idx = _raster_flat(r1 + r2)
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(idx, g["idx"])
    for k, pop in ((1, E), (2, I)):
        st = pop.get_neurons()
        assert np.array_equal(st["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))
        assert np.array_equal(st["Tref"], g[f"T{k}"])


def _checksums_of(net, n):
    from oracle.oracle import csr_checksum
    out = []
    for c in range(n):
        off, nb = net.csr(c)
        out.append((int(off[-1]), csr_checksum(off, nb)))
    return out


def test_csr_checksums_n20000(engine):
    cs = json.load(open(os.path.join(GOLDEN, "brunel_csr_checksums.json")))["N=20000,p=0.1"]["1337"]
    net, _ = engine.brunel(20000, 0.1, 1337)
    assert _checksums_of(net, 6) == [(row[2], row[3]) for row in cs]


@pytest.mark.parametrize("seed", list(range(1, 11)))
def test_csr_checksums_full_size(engine, seed):
    """Large Brunel, N=5e5, p=0.002 (2.5e8 synapses): all six CSRs equal the reference's."""
    cs = json.load(open(os.path.join(GOLDEN, "brunel_csr_checksums.json")))["N=500000,p=0.002"][str(seed)]
    net, _ = engine.brunel(500000, 0.002, seed)
    assert _checksums_of(net, 6) == [(row[2], row[3]) for row in cs]


@pytest.mark.parametrize("mode", [0])
def test_large_brunel_300_steps_golden(engine, mode):
    """N=5e5, p=0.002, seed 1: per-step spike counts, raster and state checksums equal the reference's."""
    from oracle.oracle import raster_checksum, state_checksum
    g = json.load(open(os.path.join(GOLDEN, "brunel_n500000_s1.json")))
    net, pops = engine.brunel(500000, 0.002, 1, mode=mode)
    counts, idx = _raster_flat(net.run_record(g["steps"]))
    assert counts.tolist() == g["counts"]
    assert raster_checksum(counts, idx) == g["raster_checksum"]
    e, i = pops[1].get_neurons(), pops[2].get_neurons()
    assert state_checksum(e["V"], e["Tref"]) == g["state_checksum_E"]
    assert state_checksum(i["V"], i["Tref"]) == g["state_checksum_I"]


def test_long_run_across_chunks_matches_oracle(engine, oracle_lib):
    """2100 steps (dt, seeds and jump tables are prepared in chunks of 1024 steps; windows straddle
    no chunk) in uneven recorded and plain calls, under the default launches (neuron update and
    sources in one grid, programmatic dependent launches) and under mapping 19: raster, spikes of
    every age and the LIF state equal the oracle's bit for bit."""
    sp, o = engine, oracle_lib
    N, p, seed = 5000, 0.1, 11
    net, pops = sp.brunel(N, p, seed)
    net.set_tuning(tile_bytes=8192, deliver_threads=256, deliver_algo=19, neuron_variant=6)
    ref, rpops = o.brunel(N, p, seed)
    raster = list(net.run_record(1000))
    net.run(700)
    raster += list(net.run_record(400))
    for t, row in enumerate(raster):
        if t == 1000:
            ref.run(700)
        ref.step()
        for k in range(3):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    for k in range(3):
        for age in range(15):
            assert np.array_equal(net.spikes(pops[k], age), ref.spikes(rpops[k], age)), (k, age)
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_TREF), ref.state(rpops[k], 3))


def test_large_recorded_raster_equals_piecewise_recording(engine):
    """A 2000-step recording at N=5e5 (an 11.7 MB raster, copied to the caller's buffer by several
    host threads) equals the same network recorded in 200-step pieces, entry for entry."""
    sp = engine
    a, _ = sp.brunel(500000, 0.002, 3)
    b, _ = sp.brunel(500000, 0.002, 3)
    whole = a.run_record(2000)
    pieces = []
    for _ in range(10):
        pieces += list(b.run_record(200))
    assert len(whole) == len(pieces) == 2000
    n = 0
    for t, (r1, r2) in enumerate(zip(whole, pieces)):
        for k in range(3):
            assert np.array_equal(np.asarray(r1[k]), np.asarray(r2[k])), (t, k)
            n += len(r1[k])
    assert n * 4 > (8 << 20)  # large enough for the threaded copy


def _one_wave_tile(sizes, nslots, sms):
    """The tile search of the default shape, restated: from 100 KiB down in 128-byte steps, the
    largest tile (32-neuron multiples, 4 bytes per neuron) giving the most CTAs within one wave."""
    best, tb = -1, 100 * 1024
    for b in range(100 * 1024, 4 * 1024 - 1, -128):
        tile = max(32, b // 4 // 32 * 32)
        m = nslots * sum(-(-n // tile) for n in sizes)
        if m > sms:
            break
        if m > best:
            best, tb = m, b
    return tb


def test_default_shape_follows_the_network_sizes(engine):
    """Knobs left unset are picked when the network is prepared: mapping 17, LIF window 9, the
    largest tile <= 100 KiB giving the most (slot, tile) CTAs within one wave of the SMs, threads by
    tile size; a caller's setting stands, and a tile too large for mapping 17's staging takes
    mapping 1."""
    import torch
    sp = engine
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    big, _ = sp.brunel(500000, 0.002, 1)
    assert big.get_tuning()["deliver_algo"] == 1  # the values that stand before preparation
    big.run(0)
    t = big.get_tuning()
    assert (t["deliver_algo"], t["neuron_variant"], t["deliver_threads"]) == (17, 9, 768)
    assert t["tile_bytes"] == _one_wave_tile([200000, 50000], 15, sms)
    small, _ = sp.brunel(20000, 0.1, 1337)
    small.run(0)
    t = small.get_tuning()
    assert (t["deliver_algo"], t["deliver_threads"]) == (17, 256)
    assert t["tile_bytes"] == _one_wave_tile([8000, 2000], 15, sms)
    own, _ = sp.brunel(20000, 0.1, 1337)
    own.set_tuning(tile_bytes=200 * 1024, neuron_variant=4)
    own.run(0)
    t = own.get_tuning()
    assert (t["tile_bytes"], t["deliver_algo"], t["neuron_variant"]) == (200 * 1024, 1, 4)
    own.set_tuning(tile_bytes=64 * 1024)  # back within the staging budget: mapping 17 again
    assert own.get_tuning()["deliver_algo"] == 17
    own.run(30)


def test_delivery_spans_lie_inside_their_event_pairs(engine):
    """With profiling on, each neuron-update and delivery launch also reports its device span (first
    CTA start to last CTA end on the global timer), which is shorter than the CUDA-event time around
    the launch; the raster and V stay the reference's bit for bit."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    net.set_profiling(True)
    counts, idx = _raster_flat(net.run_record(steps))
    n_ev, ms_ev = net.kernel_stats(1)
    n_sp, ms_sp = net.kernel_span(1)
    n_wev, ms_wev = net.kernel_stats(0)
    n_wsp, ms_wsp = net.kernel_span(0)
    assert net.kernel_span(2) == (0, 0.0)  # raster extraction: no spans
    net.set_profiling(False)
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))
    assert n_ev > 0 and 0 < n_sp <= n_ev
    assert 0 < ms_sp < ms_ev
    assert n_wev > 0 and 0 < n_wsp <= n_wev
    assert 0 < ms_wsp < ms_wev


@pytest.mark.parametrize("persistent", [0, 1])
def test_pinned_caller_buffers_written_in_place(engine, persistent):
    """spice_run_record into pinned host buffers (written by the GPU while it steps) and into
    pageable ones (filled from the staging buffer): equal counts, spikes and totals; a pinned buffer
    that is too small reports the same overflow and total as a pageable one."""
    import ctypes as C
    import torch
    sp = engine
    L = sp.lib()
    delay = 1e-4 if persistent else 15e-4
    a, _ = sp.brunel(20000, 0.02, 5, delay=delay)
    b, _ = sp.brunel(20000, 0.02, 5, delay=delay)
    a.set_tuning(persistent=persistent)
    b.set_tuning(persistent=persistent)
    steps, cap = 300, 400000
    pc = torch.full((steps, 3), -1, dtype=torch.int64, pin_memory=True)
    ps = torch.full((cap,), -1, dtype=torch.int32, pin_memory=True)
    hc = np.full((steps, 3), -1, dtype=np.int64)
    hs = np.full(cap, -1, dtype=np.int32)
    ta, tb = C.c_int64(), C.c_int64()
    for _ in range(2):  # a second call starts from the first's end
        assert L.spice_run_record(a._h, steps, pc.data_ptr(), ps.data_ptr(), cap, C.byref(ta)) == 0
        assert L.spice_run_record(b._h, steps, hc.ctypes.data, hs.ctypes.data, cap, C.byref(tb)) == 0
        assert ta.value == tb.value > 0
        assert np.array_equal(pc.numpy(), hc)
        assert np.array_equal(ps.numpy()[:ta.value], hs[:tb.value])
        assert int(hc.sum()) == ta.value
    small = ta.value // 2
    ra = L.spice_run_record(a._h, steps, pc.data_ptr(), ps.data_ptr(), small, C.byref(ta))
    rb = L.spice_run_record(b._h, steps, hc.ctypes.data, hs.ctypes.data, small, C.byref(tb))
    assert ra == rb == sp.EOVERFLOW and ta.value == tb.value > small


# ---- the reference's own known-answer tests, restated ----------------------------------------------
def test_external_input_sample(engine):
    """samples/external_input.cpp: a per-population update replays a cyclic spike train."""
    sp = engine
    trains = [[4, 5, 8], [5], [7, 8], [5, 7]]
    net = sp.snn(1, 1, [1337])
    I = net.add_population(sp.external_input(tuple(map(tuple, trains))), 9)
    for t in range(20):
        net.step()
        assert net.spikes(I, 0).tolist() == trains[t % 4]


def test_deliver_counts_known_answer(engine):
    """test/detail/synapse_population.cpp:28-57: edges 0->0, 0->1, 0->3, 1->3, 2->4; spikes {0, 1}
    deliver 1, 1, 0, 2, 0 times."""
    sp = engine
    net = sp.snn(1, 1, [1337])
    S = net.add_population(sp.external_input(((0, 1), ())), 3)
    D = net.add_population(sp.lif(Vthres=1e9), 5)
    adj = sp.adj_list()
    for a, b in [(0, 0), (0, 1), (0, 3), (1, 3), (2, 4)]:
        adj.connect(a, b)
    net.connect(S, D, adj, 1, sp.fixed_weight(1.0))
    net.step()
    assert D.get_neurons()["V"].tolist() == [1.0, 1.0, 0.0, 2.0, 0.0]


def test_csr_custom_adjacency(engine):
    """test/detail/csr.cpp:25-58: a 3x10 adj_list keeps sorted neighbour lists per source."""
    sp = engine
    net = sp.snn(1, 1, [1337])
    S = net.add_population(sp.poisson(), 3)
    D = net.add_population(sp.lif(), 10)
    adj = sp.adj_list()
    for a, b in [(0, 9), (0, 0), (2, 2), (0, 7), (2, 1), (0, 2)]:
        adj.connect(a, b)
    c = net.connect(S, D, adj, 1, sp.fixed_weight(0.0))
    off, nb = net.csr(c)
    assert off.tolist() == [0, 4, 4, 6]
    assert nb.tolist() == [0, 2, 7, 9, 1, 2]


def test_empty_and_zero_sized(engine):
    """Empty populations: one as the source of a connection fails the reference's precondition at
    connect (its CSR has no offsets: topology.cpp:82 for fixed_probability, :48 for adj_list); one as
    the target, and a connection without synapses, step and deliver nothing."""
    sp = engine
    net = sp.snn(1e-4, 15e-4, [3])
    P = net.add_population(sp.poisson(), 0)
    E = net.add_population(sp.lif(), 0)
    F = net.add_population(sp.lif(), 5)
    Q = net.add_population(sp.poisson(), 50)
    with pytest.raises(sp.LogicError, match=r"topology\.cpp:82\): offsets\.size\(\) > src_count"):
        net.connect(P, F, sp.fixed_probability(0.5), 15e-4, sp.fixed_weight(1.0))
    with pytest.raises(sp.LogicError, match=r"topology\.cpp:48\): offsets\.size\(\) > src_count"):
        net.connect(P, F, sp.adj_list(), 15e-4, sp.fixed_weight(1.0))
    net.connect(Q, E, sp.fixed_probability(0.5), 15e-4, sp.fixed_weight(1.0))
    net.connect(Q, F, sp.fixed_probability(0.0), 15e-4, sp.fixed_weight(1.0))
    net.run(40)
    assert net.spikes(P, 0).size == 0 and net.spikes(F, 3).size == 0
    assert net.events == 0


def test_events_equal_row_lengths(engine):
    """Synaptic events = sum over delivered spikes of their CSR row lengths."""
    sp = engine
    net, pops = sp.brunel(6000, 0.05, 5)
    raster = net.run_record(200)
    csr = [net.csr(c)[0] for c in range(6)]
    src = [0, 0, 1, 1, 2, 2]
    expect = 0
    for row in raster:
        for c in range(6):
            s = row[src[c]]
            expect += int(np.sum(csr[c][s + 1] - csr[c][s]))
    assert net.events == expect


def test_errors_follow_the_reference(engine):
    sp = engine
    net = sp.snn(1e-4, 15e-4, [1])
    P = net.add_population(sp.poisson(), 10)
    E = net.add_population(sp.lif(), 10)
    with pytest.raises(sp.LogicError, match=r"Assertion failed \(snn.h:35\).*at least 1dt"):
        net.connect(P, E, sp.fixed_probability(0.1), 0.0, sp.fixed_weight(1.0))
    with pytest.raises(sp.LogicError, match="may not exceed the maximum delay"):
        net.connect(P, E, sp.fixed_probability(0.1), 16e-4, sp.fixed_weight(1.0))
    with pytest.raises(sp.LogicError, match=r"Assertion failed \(topology.cpp:73\): 0 <= p && p <= 1"):
        net.connect(P, E, sp.fixed_probability(1.5), 15e-4, sp.fixed_weight(1.0))
    for first, where in ((10, "29"), (12, "18")):  # P has 10 neurons: its adjacency has 11 offsets
        adj = sp.adj_list()
        adj.connect(first, 0)
        with pytest.raises(sp.LogicError, match=r"Assertion failed \(topology.cpp:" + where + r"\)"):
            net.connect(P, E, adj, 15e-4, sp.fixed_weight(1.0))
    with pytest.raises(sp.LogicError, match="stateful"):
        net.connect(E, P, sp.fixed_probability(0.1), 15e-4, sp.fixed_weight(1.0))
    net.connect(P, E, sp.fixed_probability(0.1), 15e-4, sp.fixed_weight(1.0))
    with pytest.raises(sp.LogicError, match="0 <= age"):
        net.spikes(P, 0)
    net.step()
    with pytest.raises(sp.LogicError, match="0 <= age"):
        net.spikes(P, 1)
    with pytest.raises(sp.SpiceError):
        net.set_mode(sp.MODE_ATOMIC)
    with pytest.raises(sp.LogicError, match="stateful"):
        P.get_neurons()
    X = sp.snn(1, 1, [1])
    ext = X.add_population(sp.external_input(), 4)
    with pytest.raises(sp.LogicError, match="ascending"):
        X.set_external_input(ext, [[2, 1]])


def _rate_cv(raster, pop, size, dt):
    spikes = [np.asarray(row[pop]) for row in raster]
    total = sum(len(s) for s in spikes)
    rate = total / (size * len(raster) * dt)
    last = np.full(size, -1, dtype=np.int64)
    isis = []
    for t, s in enumerate(spikes):
        prev = last[s]
        ok = prev >= 0
        isis.append(t - prev[ok])
        last[s] = t
    isi = np.concatenate(isis).astype(np.float64) if isis else np.zeros(1)
    return rate, isi.std() / isi.mean()


def test_atomic_mode_statistics(engine):
    """Atomic mode (float atomics, order-dependent rounding) keeps the firing statistics: per-
    population rate and ISI CV within 1% of the deterministic path over 10 seeds."""
    sp = engine
    res = {0: [], 1: []}
    for mode in (0, 1):
        for seed in range(1, 11):
            net, pops = sp.brunel(20000, 0.1, seed, mode=mode)
            raster = net.run_record(2000)
            res[mode].append([_rate_cv(raster, k, pops[k].size(), 1e-4) for k in (1, 2)])
    det, atom = np.array(res[0]).mean(axis=0), np.array(res[1]).mean(axis=0)
    rel = np.abs(atom - det) / det
    assert (rel < 0.01).all(), (det, atom, rel)


@pytest.mark.parametrize("tile_bytes,threads", [(1024, 32), (4096, 128), (48 * 1024, 512), (200 * 1024, 1024)])
def test_results_independent_of_launch_shape(engine, tile_bytes, threads):
    """Delivery tiles and CTA sizes change how events are accumulated, never the result."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    for mode in (0, 1):
        net, pops = engine.brunel(N, float(g["p"][0]), seed, mode=mode)
        net.set_tuning(tile_bytes=tile_bytes, deliver_threads=threads)
        counts, idx = _raster_flat(net.run_record(steps if mode == 0 else 50))
        if mode == 0:
            assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
            for k in (1, 2):
                assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


@pytest.mark.parametrize("algo,tile_bytes,threads,parts", [
    (0, 24 * 1024, 256, 1), (1, 12 * 1024, 128, 1), (2, 24 * 1024, 256, 1), (3, 48 * 1024, 512, 1),
    (4, 24 * 1024, 256, 1), (4, 6 * 1024, 128, 2), (4, 96 * 1024, 1024, 1), (2, 4096, 64, 3), (0, 8192, 512, 2),
    (5, 24 * 1024, 256, 1), (5, 4096, 64, 2), (6, 48 * 1024, 512, 1), (6, 200 * 1024, 1024, 3),
    (7, 26 * 1024, 512, 1), (7, 8192, 1024, 2), (8, 24 * 1024, 256, 1), (8, 4096, 64, 3),
    (8, 112 * 1024, 1024, 1), (9, 100 * 1024, 1024, 1), (9, 8192, 128, 2),
    (10, 100 * 1024, 1024, 1), (10, 24 * 1024, 256, 1), (10, 4096, 64, 3), (10, 180 * 1024, 1024, 2),
    (11, 100 * 1024, 1024, 1), (11, 8192, 128, 2), (11, 48 * 1024, 512, 1),
    (12, 100 * 1024, 1024, 1), (12, 4096, 64, 3), (12, 24 * 1024, 256, 2),
    (13, 100 * 1024, 768, 1), (13, 8192, 128, 2),
    (14, 100 * 1024, 1024, 1), (14, 4096, 64, 3), (14, 24 * 1024, 256, 2), (14, 4096, 32, 1), (14, 12 * 1024, 32, 2),
    (15, 100 * 1024, 1024, 1), (15, 4096, 64, 3), (15, 24 * 1024, 256, 2), (15, 4096, 32, 1), (15, 160 * 1024, 1024, 1),
    (16, 100 * 1024, 768, 1), (16, 4096, 64, 3), (16, 8192, 32, 1), (17, 100 * 1024, 768, 1), (17, 12 * 1024, 128, 2),
    (18, 100 * 1024, 1024, 1), (18, 4096, 32, 1), (18, 180 * 1024, 1024, 1), (19, 100 * 1024, 768, 1), (19, 8192, 64, 2),
    (20, 64 * 1024, 512, 1), (20, 4096, 32, 1), (20, 8192, 128, 2), (21, 88 * 1024, 512, 1), (21, 4096, 64, 3),
])
def test_results_independent_of_delivery_mapping(engine, algo, tile_bytes, threads, parts):
    """Every work mapping of the delivery kernel (warp-flattened, thread per spike, warp per spike,
    16-byte loads, software-pipelined, lane groups, staged descriptors, aligned-block sub-rows)
    gives the reference's raster and V bit for bit."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    net.set_tuning(tile_bytes=tile_bytes, deliver_threads=threads, deliver_parts=parts, deliver_algo=algo)
    counts, idx = _raster_flat(net.run_record(steps))
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 8, 9])
def test_neuron_variants_match_reference(engine, variant):
    """Every LIF window variant of the neuron update (unrolled or rolled steps, per-lane or
    warp-uniform count replay) gives the reference's raster and V bit for bit."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    net.set_tuning(neuron_variant=variant)
    counts, idx = _raster_flat(net.run_record(steps))
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


@pytest.mark.parametrize("variant", [4, 5, 6, 7, 8, 9])
def test_neuron_variants_with_large_counts(engine, oracle_lib, variant):
    """Inputs of ~2.4 events per neuron and step from one group (counts of 8 or more, which take
    the general replay, in about one warp-step in ten): every variant bit-exact with the oracle."""
    sp, o = engine, oracle_lib
    spec = {"dt": 1e-4, "max_delay": 2e-4, "seed": 12,
            "pops": [("poisson", 4000, 30.0), ("lif", 1000), ("poisson", 3000, 15.0)],
            "conns": [("f", 0, 1, 0.2, 2e-4, 0.003, 0), ("f", 2, 1, 0.3, 2e-4, -0.0011, 0)]}
    net = sp.snn(spec["dt"], spec["max_delay"], [spec["seed"]])
    pops = [net.add_population(sp.poisson(30.0), 4000), net.add_population(sp.lif(), 1000),
            net.add_population(sp.poisson(15.0), 3000)]
    for _, s_, d, p, delay, w, _f in spec["conns"]:
        net.connect(pops[s_], pops[d], sp.fixed_probability(p), delay, sp.fixed_weight(float(np.float32(w))))
    net.set_tuning(neuron_variant=variant)
    ref, rpops, _ = o.weighted_net(spec)
    raster = net.run_record(300)
    for t in range(300):
        ref.step()
        assert np.array_equal(np.asarray(raster[t][1]), ref.spikes(rpops[1], 0)), t
    assert sum(len(r[1]) for r in raster) > 100
    assert np.array_equal(net.get_state(pops[1], sp.FIELD_V).view(np.uint32), ref.state(rpops[1], 0).view(np.uint32))


@pytest.mark.parametrize("mode", [0, 1])
def test_launch_modes_match_reference(engine, mode):
    """Sources on their own stream (0) or fused with the neuron update into programmatic dependent
    launches (1), switched mid-run: the reference's raster and V bit for bit."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    net.set_tuning(launch_mode=mode)
    r1 = list(net.run_record(steps // 2))
    net.set_tuning(launch_mode=1 - mode)
    r2 = list(net.run_record(steps - steps // 2))
    counts, idx = _raster_flat(r1 + r2)
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


def test_compact_targets_follow_retiling(engine):
    """The 16-bit tile-local target copy (mapping 15) is rebuilt whenever the tile size changes, and
    switching mappings mid-run keeps the raster and state bit-exact."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    shapes = [(24 * 1024, 256, 1, 15), (8 * 1024, 128, 1, 15), (16 * 1024, 256, 2, 12), (96 * 1024, 1024, 1, 15),
              (4096, 64, 1, 8)]
    raster = []
    for i, (tb, th, parts, algo) in enumerate(shapes):
        net.set_tuning(tile_bytes=tb, deliver_threads=th, deliver_parts=parts, deliver_algo=algo)
        n = steps // len(shapes) if i < len(shapes) - 1 else steps - len(raster)
        raster += list(net.run_record(n))
    counts, idx = _raster_flat(raster)
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


def test_retuning_mid_run_keeps_results(engine):
    """Switching tile size, threads and parts between steps (including between overwritten and
    accumulated input slots) leaves the raster and state bit-exact."""
    g = np.load(os.path.join(GOLDEN, "brunel_n5000.npz"))
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = engine.brunel(N, float(g["p"][0]), seed)
    shapes = [(48 * 1024, 512, 1), (8 * 1024, 256, 3), (16 * 1024, 128, 1), (96 * 1024, 1024, 2), (4096, 64, 5)]
    raster = []
    for i, (tb, th, parts) in enumerate(shapes):
        net.set_tuning(tile_bytes=tb, deliver_threads=th, deliver_parts=parts)
        n = steps // len(shapes) if i < len(shapes) - 1 else steps - len(raster)
        if i % 2:
            for _ in range(n):
                net.step()
                raster.append([net.spikes(p, 0) for p in pops])
        else:
            raster += net.run_record(n)
    counts, idx = _raster_flat(raster)
    assert np.array_equal(counts, g["counts"]) and np.array_equal(idx, g["idx"])
    for k in (1, 2):
        assert np.array_equal(pops[k].get_neurons()["V"].view(np.uint32), g[f"V{k}"].view(np.uint32))


@pytest.mark.parametrize("steps_per_cta", [0, 1, 3, 7, 15])
def test_results_independent_of_source_steps(engine, oracle_lib, steps_per_cta):
    """Poisson source CTAs drawing several consecutive steps each (0: chosen so the window's grid is
    one wave) give the reference's raster and state bit for bit, recorded and step by step."""
    sp, o = engine, oracle_lib
    N, p, seed = 30000, 0.02, 4
    net, pops = sp.brunel(N, p, seed)
    net.set_tuning(source_steps=steps_per_cta)
    ref, rpops = o.brunel(N, p, seed)
    raster = net.run_record(200)
    for t, row in enumerate(raster):
        ref.step()
        for k in range(3):
            assert np.array_equal(np.asarray(row[k]), ref.spikes(rpops[k], 0)), (t, k)
    for _ in range(7):
        net.step()
        ref.step()
    for k in range(3):
        assert np.array_equal(net.spikes(pops[k], 0), ref.spikes(rpops[k], 0))
    for k in (1, 2):
        assert np.array_equal(net.get_state(pops[k], sp.FIELD_V).view(np.uint32), ref.state(rpops[k], 0).view(np.uint32))
