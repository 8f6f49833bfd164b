"""The C++ front end (include/spice/snn.h): the reference's Brunel sample, unchanged in its calls,
compiled with g++ -std=c++20 against the header and run on the GPU; its JSON raster equals the
reference's (tests/golden/brunel_n20000.npz, README.md:110-116)."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADER_USE = r"""
#include "spice/snn.h"
using namespace spice;
using namespace spice::models;
int main() {
	snn net(1e-4f, 8e-4f, {1337});
	auto P = net.add_population<poisson>(10);
	auto E = net.add_population<lif_cond>(10);
	auto L = net.add_population<lif>(5);
	auto X = net.add_population<external_input>(3, {{{1, 2}, {0}}});
	adj_list a;
	a.connect(0, 1);
	net.connect<excitatory>(E, E, a, 8e-4f, {0.1f});
	net.connect<inhibitory>(E, L, fixed_probability(0.5), 8e-4f, {0.1f});
	net.connect<fixed_weight>(P, L, fixed_probability(0.5), 8e-4f, {1.f});
	net.step();
	auto s = X->spikes(0);
	auto v = E->get_neurons();
	auto w = L->get_neurons();
	return int(s.size() + v.size() + w.size() + P->size()) & 0;
}
"""


def test_cxx_header_compiles(tmp_path):
    """Every model, synapse and topology of the header instantiates under g++ -std=c++20 -Wall."""
    src = tmp_path / "use.cpp"
    src.write_text(HEADER_USE)
    subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                    os.path.join(ROOT, "include"), str(src)], check=True)


@pytest.mark.gpu
def test_cxx_brunel_sample_matches_reference(engine, tmp_path):
    exe = tmp_path / "brunel"
    libdir = os.path.join(ROOT, "spice2_gb300")
    subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "spice2_gb300", "examples", "brunel.cpp"), "-L", libdir, "-lspice_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rows = json.loads(out)["spikes"]
    g = np.load(os.path.join(GOLDEN, "brunel_n20000.npz"))
    counts, idx = g["counts"], g["idx"]
    assert len(rows) == counts.shape[0]
    pos = 0
    for t, row in enumerate(rows):
        per = []
        for k in range(3):
            per.append(idx[pos:pos + counts[t, k]])
            pos += counts[t, k]
        P, E, I = per
        expect = [int(x) for x in I] + [int(x) + 2000 for x in E] + [int(x) + 10000 for x in P]
        assert row == expect, f"step {t}"
    assert rows[0][:3] == [10533, 11015, 11209]  # README.md:112


@pytest.mark.gpu
def test_samples_cli_brunel_json(engine, capsys):
    """python -m spice2_gb300.samples brunel --json prints the reference's README raster."""
    from spice2_gb300 import samples
    samples.main(["brunel", "--steps", "5", "--json"])
    rows = json.loads(capsys.readouterr().out)["spikes"]
    assert len(rows) == 5 and rows[0][:3] == [10533, 11015, 11209] and rows[1][:3] == [10310, 11115, 11884]


USER_MODEL_NO_NVCC = r"""
#include "spice/snn.h"
using namespace spice;
struct my_lif {
	struct neuron { float V = 0; int32_t T = 0; };
	SPICE_HD bool update(neuron& n, float, auto&) const { return false; }
};
int main() { snn net(1e-4f, 1e-4f, {1}); net.add_population<my_lif>(4); }
"""


def test_user_models_need_nvcc(tmp_path):
    """A user model compiled by a host-only compiler is rejected at compile time with a clear message."""
    src = tmp_path / "u.cpp"
    src.write_text(USER_MODEL_NO_NVCC)
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "compile this translation unit with nvcc" in r.stderr


@pytest.mark.gpu
def test_user_models_compiled_with_nvcc_match_the_reference(engine, oracle_lib, tmp_path):
    """samples/brunel.cpp with user-defined Poisson, LIF and synapse structs compiled into GPU kernels
    by the header: the raster equals the oracle's (the reference's algorithm)."""
    o = oracle_lib
    exe = tmp_path / "user_models"
    libdir = os.path.join(ROOT, "spice2_gb300")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++20", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "spice2_gb300", "examples", "user_models.cu"),
                    "-L", libdir, "-lspice_gb300", f"-Xlinker=-rpath={libdir}", "-o", str(exe)], check=True)
    N, p, steps, seed = 4000, 0.05, 200, 1337
    out = subprocess.run([str(exe), str(N), str(p), str(steps), str(seed)], check=True, capture_output=True, text=True)
    rows = json.loads(out.stdout)["spikes"]
    ref, pops = o.brunel(N, p, seed)
    n_spikes = 0
    for t, row in enumerate(rows):
        ref.step()
        P, E, I = (ref.spikes(k, 0) for k in pops)
        expect = [int(x) for x in I] + [int(x) + N // 10 for x in E] + [int(x) + N // 2 for x in P]
        assert sorted(row) == expect, f"step {t}"
        n_spikes += len(I) + len(E)
    assert n_spikes > 0


def _reference_samples_dir():
    import __graft_entry__ as g
    d = os.path.join(g.REFERENCE_DIR, "samples")
    return d if os.path.isdir(d) else None


@pytest.mark.skipif(_reference_samples_dir() is None, reason="the reference's sources are not on this machine")
@pytest.mark.parametrize("sample", ["brunel", "brunel+", "vogels", "ping_pong", "sssp"])
def test_reference_samples_compile_against_the_header(engine, tmp_path, sample):
    """The reference's own sample programs, with SPICE_HD added in front of their models' update(),
    deliver() and skip() and nothing else changed, compile with nvcc against
    include/spice/snn.h and spice2_gb300/examples/matplot.h (their output stream) and link against
    the engine: the reference's user API, model concepts and integer names are all there.  init()
    runs on the host in this engine (sssp's reads a host array), so it stays unannotated; ping_pong
    and sssp deliver through deliver() functors that set flags and take minima."""
    import re
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = open(os.path.join(_reference_samples_dir(), sample + ".cpp")).read()
    annotated = re.sub(r"^(\s*)(bool|void) (update|deliver|skip)\(", r"\1SPICE_HD \2 \3(", src, flags=re.M)
    assert annotated.count("SPICE_HD") >= 2
    f = tmp_path / (sample.replace("+", "_plus") + ".cu")
    f.write_text(annotated)
    libdir = os.path.join(ROOT, "spice2_gb300")
    subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-fmad=false", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "spice2_gb300", "examples"),
                    str(f), "-L", libdir, "-lspice_gb300", f"-Xlinker=-rpath={libdir}", "-o", str(tmp_path / "sample")],
                   check=True)
