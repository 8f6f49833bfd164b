"""GPU: the user-model contract of include/spice/snn.h (spice2_gb300/examples/user_contract.cu, compiled
with nvcc here): declared draws take the reference's stream positions, init() runs with each
population's own stream, stateful synapses with PerSynapseInit get the reference's per-synapse
values, deliver() is probed for the member it adds to, and undeclared draws come from independent,
uniform streams."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def contract(engine, tmp_path_factory):
    exe = tmp_path_factory.mktemp("uc") / "user_contract"
    libdir = os.path.join(ROOT, "spice2_gb300")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++20", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "spice2_gb300", "examples", "user_contract.cu"),
                    "-L", libdir, "-lspice_gb300", f"-Xlinker=-rpath={libdir}", "-o", str(exe)], check=True)

    def run(*args):
        out = subprocess.run([str(exe)] + [str(a) for a in args], check=True, capture_output=True, text=True).stdout
        return json.loads(out)
    return run


def test_declared_draws_take_the_reference_stream(contract, oracle_lib):
    """A stateful model declaring one draw per update reproduces the Poisson population that follows
    a stateful population of size 0 (the same seeds consumed, the same stream positions)."""
    o = oracle_lib
    N, steps, seed = 3000, 300, 41
    got = contract("stream", N, steps, seed)["raster"]
    ref = o.Net(1e-4, 1e-4, [seed])
    ref.add_population(o.LIF, 0)  # consumes the seed the stateful user population consumes
    P = ref.add_population(o.POISSON, N, (20.0,))
    n = 0
    for t in range(steps):
        ref.step()
        assert got[t][0] == ref.spikes(P, 0).tolist(), t
        n += len(got[t][0])
    assert n > 100


def test_init_runs_with_the_population_stream(contract, oracle_lib):
    o = oracle_lib
    N, seed = 500, 9
    got = contract("init", N, seed)
    chain = o.seed_chain([seed], 2)  # one seed per stateful population, in add order
    draws_a = o.xoroshiro_draws(tuple(int(x) for x in chain[0]), N)
    draws_b = o.xoroshiro_draws(tuple(int(x) for x in chain[1]), N)
    ca = np.array([o.lib().spo_canonical_f32(int(u)) for u in draws_a], dtype=np.float32)
    cb = np.array([o.lib().spo_canonical_f32(int(u)) for u in draws_b], dtype=np.float32)
    assert np.array_equal(np.array(got["V"], dtype=np.float32), np.float32(0.02) * ca)
    assert got["T"] == [i % 7 for i in range(N)]
    assert np.array_equal(np.array(got["U"], dtype=np.float32), cb)


def test_stateful_synapse_init_and_probed_deliver(contract, oracle_lib):
    """A stateful synapse with PerSynapseInit (w = wmax canonical, the weighted synapse) and a stateless
    one adding a constant (probed, no field declared): bit-exact with the oracle's weighted and
    fixed_weight connections."""
    o = oracle_lib
    N, p, steps, seed = 2000, 0.05, 300, 17
    got = contract("weights", N, p, steps, seed)
    ref = o.Net(1e-4, 3e-4, [seed])
    P = ref.add_population(o.POISSON, N, (300.0,))
    E = ref.add_population(o.LIF, N)
    ref.connect_weighted(P, E, p, 3e-4, float(np.float32(0.004)))
    ref.connect(E, E, p, 2e-4, float(np.float32(-0.001)))
    spikes_e = 0
    for t in range(steps):
        ref.step()
        assert got["raster"][t][0] == ref.spikes(P, 0).tolist(), t
        assert got["raster"][t][1] == ref.spikes(E, 0).tolist(), t
        spikes_e += len(got["raster"][t][1])
    assert spikes_e > 0
    assert np.array_equal(np.array(got["V"], dtype=np.float32).view(np.uint32), ref.state(E, 0).view(np.uint32))


def test_undeclared_draws_are_uniform_and_independent(contract):
    """Kolmogorov-Smirnov against U(0, 1) (the reference's test/util/random.cpp uses 0.06 at 1000
    samples; here 20,000 samples), and no correlation between neighbouring neurons or populations."""
    N = 20000
    got = contract("counter", N, 37, 5)
    u, v = np.sort(np.array(got["u"])), np.array(got["v"])
    ks = np.max(np.abs(np.arange(1, N + 1) / N - u))
    assert ks < 0.015, ks
    a = np.array(got["u"])
    assert abs(np.corrcoef(a[:-1], a[1:])[0, 1]) < 0.03
    assert abs(np.corrcoef(a, v)[0, 1]) < 0.03
    assert not np.array_equal(a, v)
