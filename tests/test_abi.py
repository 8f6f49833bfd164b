"""CPU tests of the drop-in boundary: the C-ABI library loads and exports every declared symbol."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "spice_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(spice_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = _declared()
    for must in ("spice_net_create", "spice_add_population", "spice_connect_fixed_probability",
                 "spice_connect_adj_list", "spice_step", "spice_run", "spice_spikes", "spice_get_state",
                 "spice_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    lib = ctypes.CDLL(engine.LIB_PATH)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_binds_every_entry_point(engine):
    L = engine.lib()
    for n in _declared():
        fn = getattr(L, n)
        assert fn.restype is not None


def test_no_cuda_device_is_reported_not_faked(engine):
    """Without a GPU the engine refuses to create a net (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        return
    import pytest
    with pytest.raises(engine.SpiceError, match="CUDA|device"):
        engine.snn(1e-4, 15e-4, [1])


def test_precondition_messages_without_a_device(engine):
    import pytest
    with pytest.raises(engine.LogicError, match="at least 1 seed"):
        engine.snn(1e-4, 15e-4, [])


def _enum(name_prefix):
    src = open(os.path.join(ROOT, "include", "spice_gb300.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(" + name_prefix + r"[A-Z0-9_]*)\s*=\s*(\d+)", src)}


def _kernels_header_int(name):
    src = open(os.path.join(ROOT, "spice2_gb300", "csrc", "kernels.h")).read()
    return int(re.search(r"constexpr int " + name + r"\s*=\s*(\d+);", src).group(1))


def test_tuning_knobs_reach_the_python_mirror(engine, monkeypatch):
    """Every SPICE_TUNE_* knob of the header is set by snn.set_tuning or batch.set_tuning."""
    knobs = _enum("SPICE_TUNE_")
    seen = []

    class _L:
        def spice_set_tuning(self, h, knob, value):
            seen.append(knob)
            return 0

        def spice_batch_set_tuning(self, h, knob, value):
            seen.append(knob)
            return 0

    monkeypatch.setattr(engine, "lib", lambda: _L())
    net = engine.snn.__new__(engine.snn)
    net._h = None
    net.set_tuning(tile_bytes=4096, deliver_threads=64, deliver_parts=1, deliver_algo=1, overlap_sources=True,
                   neuron_variant=0, launch_mode=1, pull=False, source_steps=0, persistent=1)
    b = engine.batch.__new__(engine.batch)
    b._h = None
    b.set_tuning(graph_windows=2)
    assert sorted(set(seen)) == sorted(knobs.values()), (knobs, seen)


def test_autotune_candidates_are_valid_launch_shapes():
    """Every candidate of the autotuner is a shape spice_set_tuning accepts, and bench.py names the
    kernel of every delivery mapping."""
    import sys
    sys.path.insert(0, ROOT)
    from spice2_gb300.autotune import DEFAULT_CANDIDATES
    import bench
    n_algos = _kernels_header_int("kDeliverAlgos")
    for tb, th, parts, algo in DEFAULT_CANDIDATES:
        assert 1024 <= tb <= 220 * 1024 and 32 <= th <= 1024 and th % 32 == 0 and 1 <= parts <= 64
        assert 0 <= algo < n_algos
    assert sorted(bench.DELIVER_KERNELS) == list(range(n_algos))
    assert set(bench.DELIVER_DRAM_BYTES_PER_EVENT) <= set(range(n_algos))


def test_kernel_timing_entry_points_refuse_a_null_net(engine):
    """The event-pair and device-span readers check their handle before touching a device."""
    import ctypes as C
    n, ms = C.c_int64(7), C.c_double(7.0)
    for fn in ("spice_kernel_stats", "spice_kernel_span"):
        rc = getattr(engine.lib(), fn)(None, 1, C.byref(n), C.byref(ms))
        assert rc == engine.EINVAL and b"NULL" in engine.lib().spice_last_error()
