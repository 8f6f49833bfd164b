"""CPU tests: the oracle against the reference's golden vectors (no GPU needed).

The golden fixtures in tests/golden/ were produced by the reference itself (make_golden.py runs
spice2's own sources compiled by oracle/Makefile).  These tests pin the CPU restatement to them;
the GPU engine is then checked against the restatement and the same fixtures (test_gpu_*.py).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("seed", [1, 7, 1337])
def test_rng_and_seed_chain(oracle_lib, seed):
    o = oracle_lib
    g = _golden("rng.npz")
    n = len(g[f"draws_{seed}"])
    chain = np.array(o.seed_chain([seed], n), dtype=np.uint64)
    assert np.array_equal(chain, g[f"chain_{seed}"])
    s0 = tuple(int(x) for x in chain[0])
    assert np.array_equal(o.xoroshiro_draws(s0, n), g[f"draws_{seed}"])
    # exponential_distribution<double>(499) and generate_canonical<float> on the same stream
    import ctypes as C
    st = (C.c_uint64 * 2)(*s0)
    ex = np.array([o.lib().spo_exponential(499.0, st) for _ in range(n)])
    assert np.array_equal(ex.view(np.uint64), g[f"exp_{seed}"].view(np.uint64))
    canon = np.array([o.lib().spo_canonical_f32(int(u)) for u in g[f"draws_{seed}"]], dtype=np.float32)
    assert np.array_equal(canon.view(np.uint32), g[f"canon_{seed}"].view(np.uint32))


def test_kahan_dt_sequence(oracle_lib):
    g = _golden("rng.npz")
    k = oracle_lib.kahan_dts(len(g["kahan_1337"]))
    assert np.array_equal(k.view(np.uint32), g["kahan_1337"].view(np.uint32))


def test_kahan_known_answer(oracle_lib):
    """test/util/numeric.cpp:9-28: 1000 x 0.001 sums to exactly 1 with compensation."""
    import ctypes as C
    o = oracle_lib
    k = o._Kahan(0.0, 0.0)
    deltas = np.float32(0)
    for _ in range(1000):
        # no reset: the reference test uses kahan_sum directly
        y = np.float32(0.001) - np.float32(k.c)
        t = np.float32(k.sum) + y
        k.c = float((t - np.float32(k.sum)) - y)
        k.sum = float(t)
        deltas += y
    assert np.float32(k.sum) == np.float32(1.0)
    assert deltas == np.float32(1.0)


def test_csr_small_cases(oracle_lib):
    o = oracle_lib
    g = _golden("csr_small.npz")
    keys = sorted({k[4:] for k in g.files if k.startswith("off_")})
    assert len(keys) >= 8
    for key in keys:
        s, d, p, sd = key.split("_")
        s, d, p, sd = int(s), int(d), float(p), int(sd)
        off, nb, _ = o.fp_generate(s, d, p, o.seed_from_list([sd]))
        assert np.array_equal(off, g["off_" + key]), key
        assert np.array_equal(nb, g["nb_" + key]), key
        if s:
            assert o.fp_max_degree(d, p) == int(g["md_" + key][0]), key


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("src,dst,p,seed", [(1, 1, 1.0, 5), (257, 1000, 0.013, 77), (4000, 300, 0.5, 9),
                                            (3, 70000, 0.0007, 123), (1000, 1000, 0.999, 42), (50, 20, 0.0, 1),
                                            (50, 0, 0.3, 2), (2, 5, 1.0, 3), (6000, 2, 0.5, 4)])
def test_csr_vs_live_reference(oracle_lib, src, dst, p, seed):
    """fixed_probability adjacency of the restatement against the reference binary on shapes the
    fixtures do not hold (single synapse, near-empty and near-full rows, very sparse wide rows)."""
    o = oracle_lib
    md, off_r, nb_r = o.run_reference_gen(src, dst, p, seed)
    off, nb, _ = o.fp_generate(src, dst, p, o.seed_from_list([seed]))
    assert np.array_equal(off, off_r) and np.array_equal(nb, nb_r)
    if src:
        assert o.fp_max_degree(dst, p) == md


def test_csr_checksums_n20000(oracle_lib):
    o = oracle_lib
    cs = json.load(open(os.path.join(GOLDEN, "brunel_csr_checksums.json")))["N=20000,p=0.1"]["1337"]
    net, _ = o.brunel(20000, 0.1, 1337)
    sizes = [10000, 8000, 2000]
    for c, (sp, dp, nsyn, h) in enumerate(cs):
        n = net.csr(c)
        off = np.zeros(sizes[sp] + 1, dtype=np.int64)
        nb = np.zeros(n, dtype=np.int32)
        o.lib().spo_conn_csr(net.h, c, off.ctypes.data, nb.ctypes.data)
        assert n == nsyn
        assert o.csr_checksum(off, nb) == h


def _raster_matches(net, pops, counts, idx):
    pos = 0
    for t in range(counts.shape[0]):
        net.step()
        for k, pk in enumerate(pops):
            c = counts[t, k]
            got = net.spikes(pk, 0)
            assert np.array_equal(got, idx[pos:pos + c]), f"step {t} population {k}"
            pos += c


@pytest.mark.parametrize("name", ["brunel_n20000.npz", "brunel_n5000.npz"])
def test_brunel_raster_and_state(oracle_lib, name):
    o = oracle_lib
    g = _golden(name)
    N, seed, steps = (int(x) for x in g["meta"])
    net, pops = o.brunel(N, float(g["p"][0]), seed)
    _raster_matches(net, pops, g["counts"], g["idx"])
    for k in (1, 2):
        assert np.array_equal(net.state(pops[k], 0).view(np.uint32), g[f"V{k}"].view(np.uint32))
        assert np.array_equal(net.state(pops[k], 3), g[f"T{k}"])


def test_readme_raster_head():
    """README.md:110-116 prints the JSON raster of samples/brunel.cpp (I, E, P with offsets):
    the first two steps begin [10533,11015,11209,...] and [10310,11115,11884,...]."""
    g = _golden("brunel_n20000.npz")
    counts, idx = g["counts"], g["idx"]
    rows, pos = [], 0
    for t in range(2):
        per = []
        for k in range(3):
            per.append(idx[pos:pos + counts[t, k]])
            pos += counts[t, k]
        P, E, I = per
        rows.append(list(I) + [x + 2000 for x in E] + [x + 10000 for x in P])
    assert rows[0][:3] == [10533, 11015, 11209]
    assert rows[1][:3] == [10310, 11115, 11884]


def test_mixed_network(oracle_lib):
    o = oracle_lib
    g = _golden("mixed_net.npz")
    net, pops, pairs = o.mixed_net()
    assert np.array_equal(np.array(pairs, dtype=np.int32), g["pairs"])
    _raster_matches(net, pops, g["counts"], g["idx"])
    for k in (1, 2):
        assert np.array_equal(net.state(pops[k], 0).view(np.uint32), g[f"V{k}"].view(np.uint32))
        assert np.array_equal(net.state(pops[k], 3), g[f"T{k}"])


@pytest.mark.parametrize("name,delay,weights", [("vogels_n4000.npz", 8e-4, None),
                                                ("vogels_c3_n10000.npz", 1e-4, (0.03, 0.3))])
def test_vogels_raster_and_state(oracle_lib, name, delay, weights):
    """The conductance LIF of samples/vogels.cpp as the reference's -ffast-math build computes it:
    raster and final V / Gex / Gin / Tref equal the reference binary's bit for bit."""
    o = oracle_lib
    g = _golden(name)
    N, seed, steps = (int(x) for x in g["meta"])
    we, wi = weights if weights else (None, None)
    net, pops = o.vogels(N, seed, delay=delay, we=we, wi=wi)
    _raster_matches(net, pops, g["counts"], g["idx"])
    for k in (0, 1):
        for f, fld in (("V", 0), ("Gex", 1), ("Gin", 2)):
            assert np.array_equal(net.state(pops[k], fld).view(np.uint32), g[f"{f}{k}"].view(np.uint32)), (k, f)
        assert np.array_equal(net.state(pops[k], 3), g[f"T{k}"])


def test_vogels_compiled_form_is_not_source_order():
    """The pin is not vacuous: evaluated in source order without contraction, the conductance update
    differs from the reference's compiled form in a fraction of the states the fixtures cover."""
    f32, f64 = np.float32, np.float64
    rng = np.random.default_rng(0)
    V = rng.uniform(-0.08, -0.05, 200000).astype(f32)
    Gex = rng.uniform(0, 2, V.size).astype(f32)
    Gin = rng.uniform(0, 5, V.size).astype(f32)
    dt = f32(1.00000005e-4)
    strict = V + ((f32(-0.06) - V) + Gex * (f32(0) - V) + Gin * (f32(-0.08) - V) + f32(0.02)) * (dt * f32(50))
    a = Gin * (f32(-0.08) - V)
    b = (-(Gex.astype(f64)) * V.astype(f64) + a.astype(f64)).astype(f32)  # product exact in double
    c = (f32(-0.04) - V) + b
    compiled = (f64(dt * f32(50)) * c.astype(f64) + V.astype(f64)).astype(f32)
    assert 0.001 < np.mean(compiled != strict) < 0.1


def test_large_brunel_seed_block_vs_reference(oracle_lib):
    """N=5e5, p=0.002, seed 2: the first 500-step block (per-step counts, raster and state checksums)
    equals the reference's."""
    o = oracle_lib
    g = _golden("brunel_n500000_long.npz")
    steps, block = 500, int(g["meta_s2"][1])
    assert block == steps
    net, pops = o.brunel(500000, 0.002, 2)
    counts, idx = [], []
    for _ in range(steps):
        net.step()
        row = [net.spikes(pk, 0) for pk in pops]
        counts.append([len(x) for x in row])
        idx += row
    counts = np.array(counts, dtype=np.int32)
    assert np.array_equal(counts, g["counts_s2"][:steps])
    ref = tuple(int(x) for x in g["blocks_s2"][0])
    got = (o.raster_checksum(counts, np.concatenate(idx)), o.state_checksum(net.state(pops[1], 0), net.state(pops[1], 3)),
           o.state_checksum(net.state(pops[2], 0), net.state(pops[2], 3)))
    assert got == ref


def test_weighted_net_raster_and_state(oracle_lib):
    """Per-synapse weights drawn by the PerSynapseInit stream (oracle.WEIGHTED_NET: weighted synapses
    into LIF and conductance targets, fixed weights, delays 3..12 steps, six distinct weights into
    one population): raster and final states equal the reference binary's bit for bit."""
    o = oracle_lib
    g = _golden("weighted_net.npz")
    net, pops, _ = o.weighted_net()
    _raster_matches(net, pops, g["counts"], g["idx"])
    for k, (kind, *_rest) in enumerate(o.WEIGHTED_NET["pops"]):
        if kind == "lif":
            assert np.array_equal(net.state(pops[k], 0).view(np.uint32), g[f"V{k}"].view(np.uint32)), k
            assert np.array_equal(net.state(pops[k], 3), g[f"T{k}"]), k
        elif kind == "lif_cond":
            for f, fld in (("V", 0), ("Gex", 1), ("Gin", 2)):
                assert np.array_equal(net.state(pops[k], fld).view(np.uint32), g[f"{f}{k}"].view(np.uint32)), (k, f)
            assert np.array_equal(net.state(pops[k], 3), g[f"T{k}"]), k


def test_weighted_weights_are_the_init_stream(oracle_lib):
    """The weights are wmax * canonical<float> of consecutive draws of the stream seeded one seed
    after the adjacency's, in CSR order (synapse_population.h:30-41)."""
    o = oracle_lib
    net = o.Net(1e-4, 1e-4, [99])
    S = net.add_population(o.POISSON, 300, (20.0,))
    D = net.add_population(o.LIF, 200)
    c = net.connect_weighted(S, D, 0.1, 1e-4, 0.25)
    chain = o.seed_chain([99], 3)  # 0: the LIF population, 1: the adjacency, 2: the weights
    draws = o.xoroshiro_draws(tuple(int(x) for x in chain[2]), len(net.syn_weights(c)))
    canon = np.array([o.lib().spo_canonical_f32(int(u)) for u in draws], dtype=np.float32)
    assert np.array_equal(net.syn_weights(c).view(np.uint32), (np.float32(0.25) * canon).view(np.uint32))


def test_oracle_errors(oracle_lib):
    o = oracle_lib
    net = o.Net(1e-4, 15e-4, [1])
    P = net.add_population(o.POISSON, 10, (20.0,))
    E = net.add_population(o.LIF, 10)
    with pytest.raises(RuntimeError, match="The delay must be at least 1dt"):
        net.connect(P, E, 0.1, 0.0, 1.0)
    with pytest.raises(RuntimeError, match="may not exceed the maximum delay"):
        net.connect(P, E, 0.1, 16e-4, 1.0)
    with pytest.raises(RuntimeError, match="0 <= age"):
        net.spikes(P, 0)


# ---- jump-ahead math (the method the GPU uses to reproduce serial streams in parallel) --------
def _charpoly():
    """Characteristic polynomial of the xoroshiro128+ transition via Berlekamp-Massey."""
    M = (1 << 64) - 1
    s0, s1 = 0x0123456789ABCDEF, 0xFEDCBA9876543210
    bits = []
    for _ in range(256):
        bits.append(s0 & 1)
        t = s0 ^ s1
        s0 = (((s0 << 24) | (s0 >> 40)) & M) ^ t ^ ((t << 16) & M)
        s1 = ((t << 37) | (t >> 27)) & M
    C, B, L, m = [1] + [0] * 256, [1] + [0] * 256, 0, 1
    for n in range(256):
        d = bits[n]
        for i in range(1, L + 1):
            d ^= C[i] & bits[n - i]
        if not d:
            m += 1
            continue
        T = C[:]
        for i in range(0, 257 - m):
            C[i + m] ^= B[i]
        if 2 * L <= n:
            L, B, m = n + 1 - L, T, 1
        else:
            m += 1
    assert L == 128
    return sum(C[128 - k] << k for k in range(128))


def _xpow_mod(n, P):
    def mulmod(a, b):
        r = 0
        for i in range(127, -1, -1):
            carry = r >> 127
            r = (r << 1) & ((1 << 128) - 1)
            if carry:
                r ^= P
            if (b >> i) & 1:
                r ^= a
        return r
    res, base = 1, 2
    while n:
        if n & 1:
            res = mulmod(res, base)
        base = mulmod(base, base)
        n >>= 1
    return res


@pytest.mark.parametrize("n", [1, 31, 32, 1000, 65536, 123457])
def test_jump_ahead_equals_stepping(oracle_lib, n):
    o = oracle_lib
    P = _charpoly()
    poly = _xpow_mod(n, P)
    start = o.seed_from_list([1337])
    jumped = o.xoroshiro_jump(start, (poly & ((1 << 64) - 1), poly >> 64))
    # stepping n times: the (n+1)-th draw equals s0 + s1 of the jumped state
    draws = o.xoroshiro_draws(start, n + 1)
    assert (jumped[0] + jumped[1]) & ((1 << 64) - 1) == int(draws[n])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("N,p,seed,steps", [(3000, 0.07, 99, 400), (12000, 0.02, 7, 250), (800, 0.3, 2024, 600),
                                           (20000, 0.005, 31337, 150)])
def test_oracle_vs_live_reference(oracle_lib, N, p, seed, steps):
    """The restatement against the reference binary on fresh configurations (sizes, densities and
    seeds the fixtures do not hold): every step's raster and dt, and the final LIF state."""
    o = oracle_lib
    res = o.run_reference_net(o.brunel_spec(N, p, seed, steps))
    st, _, _ = o.reference_states(res, [1, 2])
    net, pops = o.brunel(N, p, seed)
    for t in range(steps):
        net.step()
        for k in range(3):
            assert np.array_equal(net.spikes(pops[k], 0), res["raster"][t][k])
        assert net.last_dt == res["dt"][t]
    for k in (1, 2):
        assert np.array_equal(net.state(pops[k], 0).view(np.uint32), st[k][0].view(np.uint32))


def test_connection_from_an_empty_population_is_refused(oracle_lib):
    """An empty source population has a CSR without offsets (csr.h:70), which generate refuses
    (topology.cpp:82 for fixed_probability, topology.cpp:48 for adj_list); an empty target is kept."""
    o = oracle_lib
    net = o.Net(1e-4, 15e-4, [5])
    P = net.add_population(o.POISSON, 0, (20.0,))
    E = net.add_population(o.LIF, 0)
    F = net.add_population(o.LIF, 40)
    with pytest.raises(RuntimeError, match=r"Assertion failed \(topology\.cpp:82\): offsets\.size\(\) > src_count"):
        net.connect(P, F, 0.5, 15e-4, 0.1)
    with pytest.raises(RuntimeError, match=r"Assertion failed \(topology\.cpp:48\): offsets\.size\(\) > src_count"):
        net.connect_adj(P, F, [], 15e-4, 0.1)
    net.connect(F, E, 0.5, 15e-4, 0.1)
    net.run(20)
    assert net.events == 0


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
def test_empty_source_refused_like_the_reference(oracle_lib):
    """The reference binary fails the same precondition, with the same message, for a connection from
    an empty population."""
    import subprocess
    import tempfile
    o = oracle_lib
    spec = ["0.0001 0.0015 77 10 0", "pop poisson 0 20", "pop lif 30", "conn 0 1 0.1 0.0015 0.02"]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "spec.txt")
        open(path, "w").write("\n".join(spec) + "\n")
        r = subprocess.run([o.REF_DRIVER, "net", path, os.path.join(d, "out.bin")], capture_output=True, text=True)
    assert r.returncode != 0
    assert "Assertion failed (topology.cpp:82): offsets.size() > src_count" in r.stdout + r.stderr
    net = o.Net(1e-4, 15e-4, [77])
    P = net.add_population(o.POISSON, 0, (20.0,))
    L = net.add_population(o.LIF, 30)
    with pytest.raises(RuntimeError, match=r"topology\.cpp:82\): offsets\.size\(\) > src_count"):
        net.connect(P, L, 0.1, 15e-4, 0.02)



def _reference_error(spec_lines):
    """The reference binary's error line for a network spec (None when it runs)."""
    import subprocess
    import tempfile
    from oracle import oracle as o
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "spec.txt")
        open(path, "w").write("\n".join(spec_lines) + "\n")
        r = subprocess.run([o.REF_DRIVER, "net", path, os.path.join(d, "out.bin")], capture_output=True, text=True)
    if r.returncode == 0:
        return None
    lines = [ln for ln in (r.stdout + r.stderr).splitlines() if ln.strip()]
    return next((ln for ln in lines if ln.startswith("Assertion failed")), lines[0])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("pairs", [[(30, 0)], [(31, 0)], [(30, 0), (30, 1)], [(-1, 0)], [(0, -2)], [(3, 1), (29, 0)],
                                   [(29, 2), (0, 0), (29, 2)]])
def test_adj_list_checks_like_the_reference(oracle_lib, pairs):
    """adj_list edges from rows at or beyond the source's size, and negative indices, fail the
    reference's checks (topology.cpp:16, 18, 29, 57, 58) with its messages, in its order."""
    o = oracle_lib
    spec = ["0.0001 0.0015 77 10 0", "pop poisson 30 20", "pop lif 30",
            "adj 0 1 0.0015 0.02 " + " ".join([str(len(pairs))] + [f"{a} {b}" for a, b in pairs])]
    want = _reference_error(spec)
    net = o.Net(1e-4, 15e-4, [77])
    P = net.add_population(o.POISSON, 30, (20.0,))
    L = net.add_population(o.LIF, 30)
    if want is None:
        net.connect_adj(P, L, pairs, 15e-4, 0.02)
    else:
        with pytest.raises(RuntimeError) as err:
            net.connect_adj(P, L, pairs, 15e-4, 0.02)
        assert str(err.value) == want


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
def test_probability_check_like_the_reference(oracle_lib):
    """fixed_probability(p) outside [0, 1] fails the reference's constructor check (topology.cpp:73)."""
    o = oracle_lib
    want = _reference_error(["0.0001 0.0015 77 10 0", "pop poisson 30 20", "pop lif 30", "conn 0 1 1.5 0.0015 0.02"])
    assert want == "Assertion failed (topology.cpp:73): 0 <= p && p <= 1"
    net = o.Net(1e-4, 15e-4, [77])
    P = net.add_population(o.POISSON, 30, (20.0,))
    L = net.add_population(o.LIF, 30)
    with pytest.raises(RuntimeError) as err:
        net.connect(P, L, 1.5, 15e-4, 0.02)
    assert str(err.value) == want


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
def test_adj_list_rows_after_the_last_edge_differ_from_the_reference(oracle_lib):
    """A known difference: the reference's edge stream fills the offsets only up to the row after the
    last edge's source (topology.cpp:15-32) and leaves the later ones 0, so an adj_list whose last
    source is not the source's last row fails its CSR check (csr.h:76); the restatement (like the
    engine) builds the CSR the edges describe."""
    o = oracle_lib
    want = _reference_error(["0.0001 0.0015 77 10 0", "pop poisson 30 20", "pop lif 30", "adj 0 1 0.0015 0.02 1 5 3"])
    assert want == "Assertion failed (csr.h:76): std::is_sorted(_offsets.begin(), _offsets.end())"
    net = o.Net(1e-4, 15e-4, [77])
    P = net.add_population(o.POISSON, 30, (20.0,))
    L = net.add_population(o.LIF, 30)
    c = net.connect_adj(P, L, [(5, 3)], 15e-4, 0.02)
    off, nb = net.csr_arrays(c, 30)
    assert off.tolist() == [0] * 6 + [1] * 25 and nb.tolist() == [3]



@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("header,kind,size", [("0.0001 0.0015 77 10 0", "poisson", -5), ("0.0001 0.0015 77 10 0", "lif", -5),
                                              ("0.0001 0.00001 77 10 0", "lif", 30)])
def test_population_checks_like_the_reference(oracle_lib, header, kind, size):
    """A negative size fails as the reference's neuron adapters fail it (a stateless adapter's check at
    neuron_population.h:35; a stateful adapter's vector throws first); a maximum delay below one
    step fails neuron_population.h:108."""
    o = oracle_lib
    want = _reference_error([header, f"pop {kind} {size}" + (" 20" if kind == "poisson" else "")])
    assert want is not None
    dt, max_delay = (float(x) for x in header.split()[:2])
    net = o.Net(dt, max_delay, [77])
    with pytest.raises(RuntimeError) as err:
        net.add_population(o.POISSON if kind == "poisson" else o.LIF, size, (20.0,) if kind == "poisson" else ())
    assert str(err.value) == want


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_distributions_pass_the_reference_ks_tests(oracle_lib, seed):
    """The reference's own distribution tests (test/util/random.cpp:47-64, 102-105), restated with
    fixed seeds: on a grid of 100 points x over [a, b], the fraction of 1000 fresh draws <= x stays
    within 0.06 of the CDF -- canonical<float> and canonical<double, left-open> on [0, 1) / (0, 1],
    and exponential_distribution<double>(0.2) against 1 - exp(-5 x) on [0, 1], each on
    xoroshiro128+ seeded from a seed_seq."""
    import math
    o = oracle_lib
    state = o.seed_chain([seed], 1)[0]
    u = o.xoroshiro_draws(state, 100 * 1000 * 3)
    f32 = np.array([o.lib().spo_canonical_f32(int(x)) for x in u[:100000]], dtype=np.float64)
    f64 = np.array([o.lib().spo_canonical_f64_leftopen(int(x)) for x in u[100000:200000]])
    ex = np.array([-0.2 * math.log(o.lib().spo_canonical_f64_leftopen(int(x))) for x in u[200000:]])
    for draws, cdf, a, b in ((f32, lambda x: x, 0.0, 1.0), (f64, lambda x: x, 0.0, 1.0),
                             (ex, lambda x: 1 - math.exp(-5 * x), 0.0, 1.0)):
        ks = 0.0
        for i in range(100):
            x = a + (b - a) * i * 0.01
            ks = max(ks, abs(1e-3 * np.count_nonzero(draws[1000 * i:1000 * (i + 1)] <= x) - cdf(x)))
        assert ks <= 0.06, ks


def _random_net_spec(case):
    """A small random network (seeded by `case`): 1-2 Poisson sources and 1-3 LIF populations, 3-7
    fixed_probability projections into LIF populations with delays of 1..8 steps and weights of
    either sign, 250 steps."""
    rng = np.random.default_rng(1000 + case)
    dt, max_delay = 1e-4, 8e-4
    pops = [("poisson", int(rng.integers(50, 400)), float(rng.choice([10.0, 20.0, 40.0])))
            for _ in range(int(rng.integers(1, 3)))]
    pops += [("lif", int(rng.integers(20, 300)), None) for _ in range(int(rng.integers(1, 4)))]
    lifs = [i for i, p in enumerate(pops) if p[0] == "lif"]
    conns = []
    for _ in range(int(rng.integers(3, 8))):
        s, d = int(rng.integers(0, len(pops))), int(rng.choice(lifs))
        p = float(np.float32(rng.choice([0.02, 0.05, 0.1, 0.3])))
        delay = float(np.float32(int(rng.integers(1, 9)) * 1e-4))
        w = float(np.float32(rng.choice([1, 1, -1]) * rng.uniform(0.002, 0.02)))
        conns.append((s, d, p, delay, w))
    seed = int(rng.integers(1, 1 << 31))
    lines = [f"{dt!r} {max_delay!r} {seed} 250 0"]
    lines += [f"pop poisson {n} {r!r}" if k == "poisson" else f"pop lif {n}" for k, n, r in pops]
    lines += [f"conn {s} {d} {p!r} {delay!r} {w!r}" for s, d, p, delay, w in conns]
    return dt, max_delay, seed, pops, conns, lines


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("case", range(12))
def test_random_networks_vs_live_reference(oracle_lib, case):
    """Random small networks (population counts and sizes, rates, densities, delays of 1..8 steps,
    signed weights, connection order) on the restatement and on the reference binary: every step's
    raster and dt, the event count, and the final V / Tref of every LIF population, bit for bit."""
    o = oracle_lib
    dt, max_delay, seed, pops, conns, spec = _random_net_spec(case)
    res = o.run_reference_net(spec)
    lifs = [i for i, p in enumerate(pops) if p[0] == "lif"]
    st, _, _ = o.reference_states(res, lifs)
    net = o.Net(dt, max_delay, [seed])
    for k, n, r in pops:
        net.add_population(o.POISSON if k == "poisson" else o.LIF, n, (r,) if k == "poisson" else ())
    for s, d, p, delay, w in conns:
        net.connect(s, d, p, delay, w)
    spikes = 0
    for t in range(250):
        net.step()
        assert net.last_dt == res["dt"][t]
        for k in range(len(pops)):
            got = net.spikes(k, 0)
            assert np.array_equal(got, res["raster"][t][k]), (t, k)
            spikes += got.size
    assert spikes > 0
    for k in lifs:
        assert np.array_equal(net.state(k, 0).view(np.uint32), st[k][0].view(np.uint32))
        assert np.array_equal(net.state(k, 3), st[k][1])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                                                    "ref_driver")), reason="reference driver not built here")
@pytest.mark.parametrize("case", range(8))
def test_random_conductance_networks_vs_live_reference(oracle_lib, case):
    """Random small networks of the conductance LIF (samples/vogels.cpp, as the reference's fast-math
    build computes it): Poisson drive and recurrent excitatory (Gex) and inhibitory (Gin) projections
    with random densities, delays of 1..8 steps and weights; rasters and final V / Gex / Gin / Tref
    bit for bit against the reference binary."""
    o = oracle_lib
    rng = np.random.default_rng(2000 + case)
    dt, max_delay, steps = 1e-4, 8e-4, 300
    pops = [("poisson", int(rng.integers(100, 400)), float(rng.choice([20.0, 40.0])))]
    pops += [("lif_cond", int(rng.integers(30, 300)), None) for _ in range(int(rng.integers(1, 3)))]
    conds = list(range(1, len(pops)))
    conns = []
    for _ in range(int(rng.integers(2, 6))):
        s, d = int(rng.integers(0, len(pops))), int(rng.choice(conds))
        field = 1 if s == 0 or rng.random() < 0.5 else 2
        w = float(np.float32(rng.uniform(0.05, 0.5) if field == 1 else rng.uniform(0.1, 1.0)))
        conns.append((s, d, float(np.float32(rng.choice([0.05, 0.1, 0.3]))),
                      float(np.float32(int(rng.integers(1, 9)) * 1e-4)), w, field))
    seed = int(rng.integers(1, 1 << 31))
    spec = [f"{dt!r} {max_delay!r} {seed} {steps} 0"]
    spec += [f"pop poisson {n} {r!r}" if k == "poisson" else f"pop lif_cond {n}" for k, n, r in pops]
    spec += [f"conn {s} {d} {p!r} {delay!r} {w!r} {f}" for s, d, p, delay, w, f in conns]
    res = o.run_reference_net(spec)
    st, _, _ = o.reference_states(res, [], conds)
    net = o.Net(dt, max_delay, [seed])
    for k, n, r in pops:
        net.add_population(o.POISSON if k == "poisson" else o.LIF_COND, n, (r,) if k == "poisson" else ())
    for s, d, p, delay, w, f in conns:
        net.connect(s, d, p, delay, w, f)
    for t in range(steps):
        net.step()
        for k in range(len(pops)):
            assert np.array_equal(net.spikes(k, 0), res["raster"][t][k]), (t, k)
    for k in conds:
        for field in range(3):
            assert np.array_equal(net.state(k, field).view(np.uint32), st[k][field].view(np.uint32)), (k, field)
        assert np.array_equal(net.state(k, 3), st[k][3])
