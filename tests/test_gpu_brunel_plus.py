"""GPU: samples/brunel+.cpp (Brunel with the STDP synapse on E->E, N=2e4, p=0.1) with user models --
spice2_gb300/examples/brunel_plus.cu, the sample's network and models against include/spice/snn.h,
its plastic synapse run by the header's lazy catch-up kernels -- against the reference binary
running the same network (tests/golden/brunel_plus.npz, seeds 1..10, 1000 steps).  The plastic rule
calls exp() and pow() and the weighted sums are order-dependent (atomic mode), so the comparison is
statistical: per-population spike counts, averaged over the 10 seeds, per 100-step bin and in total."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

SEEDS, STEPS = list(range(1, 11)), 1000


@pytest.fixture(scope="module")
def gpu_runs(engine, tmp_path_factory):
    exe = tmp_path_factory.mktemp("bp") / "brunel_plus"
    libdir = os.path.join(ROOT, "spice2_gb300")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-fmad=false", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "spice2_gb300", "examples", "brunel_plus.cu"), "-L", libdir, "-lspice_gb300",
                    f"-Xlinker=-rpath={libdir}", "-o", str(exe)], check=True)
    out = {}
    for sd in SEEDS:
        r = subprocess.run([str(exe), "20000", str(STEPS), str(sd)], check=True, capture_output=True, text=True).stdout
        out[sd] = json.loads(r)
    return out


def _stats(counts):  # counts[seed][step][pop] -> per-seed totals and per-bin sums
    c = np.asarray(counts, dtype=np.float64)
    return c.sum(axis=1), c.reshape(c.shape[0], STEPS // 100, 100, 3).sum(axis=2)


def test_brunel_plus_rates_match_the_reference(gpu_runs):
    g = np.load(os.path.join(GOLDEN, "brunel_plus.npz"))
    ref_tot, ref_bins = _stats([g[f"counts_s{sd}"] for sd in SEEDS])
    gpu_tot, gpu_bins = _stats([gpu_runs[sd]["counts"] for sd in SEEDS])
    # the Poisson population draws from the reference's streams: identical spike counts
    assert np.array_equal(gpu_tot[:, 0], ref_tot[:, 0])
    for k, name in ((1, "E"), (2, "I")):
        m_ref, m_gpu = ref_tot[:, k].mean(), gpu_tot[:, k].mean()
        se = np.sqrt(ref_tot[:, k].var(ddof=1) / len(SEEDS) + gpu_tot[:, k].var(ddof=1) / len(SEEDS))
        rel = abs(m_gpu - m_ref) / m_ref
        print(f"{name}: reference {m_ref:.0f} spikes, GPU {m_gpu:.0f}, relative difference {100 * rel:.2f} % "
              f"(standard error of the difference {100 * se / m_ref:.2f} %)")
        assert rel < max(0.01, 3 * se / m_ref)
        # the time course: every 100-step bin's mean within 3 standard errors (or 2 %)
        rb, gb = ref_bins[:, :, k], gpu_bins[:, :, k]
        seb = np.sqrt(rb.var(axis=0, ddof=1) / len(SEEDS) + gb.var(axis=0, ddof=1) / len(SEEDS))
        assert np.all(np.abs(gb.mean(0) - rb.mean(0)) <= np.maximum(0.02 * rb.mean(0), 3 * seb)), name


def test_brunel_plus_weights_stay_in_bounds_and_move(gpu_runs):
    """The rule clamps W to [0, 0.0003f] (the float nearest 3e-4, a little above it); E->E synapses
    start at 1e-4 and plasticity moves them."""
    for sd in SEEDS:
        r = gpu_runs[sd]
        assert r["synapses"] > 3_000_000
        assert 0.0 <= r["W_min"] and np.float32(r["W_max"]) <= np.float32(3e-4)
        assert abs(r["W_mean"] - 1e-4) > 1e-7 and r["W_std"] > 0
