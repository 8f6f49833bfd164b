"""The allocation-free generator entry point, checked against the regular one.

Callers that cannot allocate device memory (real-time loops whose device memory is fixed up front,
hosts that own every device buffer themselves) use spice_fixed_probability_noalloc, whose scratch
is a static device array inside the library.  Its adjacency must equal the one spice_connect_fixed_probability
generates for the same projection seed, on consecutive calls (the scratch keeps the previous call's
contents).  This file is collected last so a failure here comes after every other test ran.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(1000, 800, 0.1, 1), (300, 600, 0.5, 9), (2000, 50, 0.3, 4), (64, 3000, 0.02, 77), (0, 10, 0.5, 2)]


def _noalloc(lib):
    fn = lib.spice_fixed_probability_noalloc
    fn.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int64,
                   C.POINTER(C.c_int64), C.c_void_p]
    fn.restype = C.c_int
    return fn


def _reference_csr(sp, src, dst, p, seed):
    """The adjacency the regular entry point generates, and the projection's 128-bit seed."""
    from oracle import oracle as o
    net = sp.snn(1e-4, 1e-4, [seed])
    S = net.add_population(sp.poisson(), src)
    D = net.add_population(sp.lif(), dst)
    c = net.connect(S, D, sp.fixed_probability(p), 1e-4, sp.fixed_weight(0.0))
    off, nb = net.csr(c)
    net.close()
    return off, nb, o.seed_chain([seed], 2)[1]  # seed 0: the LIF population, seed 1: the projection


def test_noalloc_matches_regular_entry_point_twice_in_a_row(engine):
    import torch
    sp = engine
    fn = _noalloc(sp.lib())
    torch.cuda.init()
    stream = torch.cuda.current_stream().cuda_stream
    for src, dst, p, seed in CASES:
        off_ref, nb_ref, (lo, hi) = _reference_csr(sp, src, dst, p, seed)
        cap = max(1, len(nb_ref) + 17)
        for call in range(2):  # the scratch keeps the previous call's contents
            off = torch.full((src + 1,), -7, dtype=torch.int64, device="cuda")
            nb = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
            syn = C.c_int64(-1)
            rc = fn(src, dst, p, lo, hi, off.data_ptr(), nb.data_ptr(), cap, C.byref(syn), stream)
            assert rc == 0, sp.lib().spice_last_error().decode()
            torch.cuda.synchronize()
            assert syn.value == len(nb_ref)
            assert np.array_equal(off.cpu().numpy(), off_ref), (src, dst, p, call)
            assert np.array_equal(nb.cpu().numpy()[:syn.value], nb_ref), (src, dst, p, call)


def test_noalloc_rejects_sizes_beyond_its_scratch(engine):
    import torch
    sp = engine
    fn = _noalloc(sp.lib())
    off = torch.zeros(70000, dtype=torch.int64, device="cuda")
    nb = torch.zeros(16, dtype=torch.int32, device="cuda")
    syn = C.c_int64(0)
    assert fn(65537, 10, 0.5, 1, 2, off.data_ptr(), nb.data_ptr(), 16, C.byref(syn), None) == sp.EINVAL
    assert b"static scratch limit" in sp.lib().spice_last_error()
    assert fn(5000, 100000, 0.5, 1, 2, off.data_ptr(), nb.data_ptr(), 16, C.byref(syn), None) == sp.EINVAL
    assert b"draws exceeds" in sp.lib().spice_last_error()
    # a too-small neighbors buffer reports the size it needs
    off_ref, nb_ref, (lo, hi) = _reference_csr(sp, 100, 500, 0.2, 3)
    rc = fn(100, 500, 0.2, lo, hi, off.data_ptr(), nb.data_ptr(), 16, C.byref(syn), None)
    assert rc == sp.EOVERFLOW and syn.value == len(nb_ref)
