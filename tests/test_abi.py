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
