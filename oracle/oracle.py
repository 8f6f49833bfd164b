"""Python access to the parity oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/libspice_oracle.so`` -- the CPU restatement of spice2's
``snn::step`` path in spice_oracle.c -- and reads the output of
``oracle/_ref/ref_driver``, the reference itself compiled from its own sources.
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
module, and only as the checker; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libspice_oracle.so")
BENCH_PATH = os.path.join(HERE, "_build", "oracle_bench")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")
# directory of the reference's sources (only needed to build the reference driver)
REF_SOURCES = os.environ.get("SPICE_REFERENCE_DIR")

POISSON, LIF, LIF_COND, EXTERNAL = 0, 1, 2, 3
SYN_ISTDP, SYN_COUNT = 1, 2  # plastic models of spo_set_plastic


def build(with_reference: bool | None = None, reference_dir: str | None = None) -> None:
    """Compiles the restatement, and the reference driver when the reference's sources are given
    (reference_dir, else the SPICE_REFERENCE_DIR environment variable) and present."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref = reference_dir or REF_SOURCES
    if with_reference is None:
        with_reference = bool(ref) and os.path.isdir(os.path.join(ref, "spice", "src"))
    if with_reference:
        if not ref:
            raise RuntimeError("the reference driver needs the reference's source directory "
                               "(reference_dir or SPICE_REFERENCE_DIR)")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)


class _U128(C.Structure):
    _fields_ = [("lo", C.c_uint64), ("hi", C.c_uint64)]


class _Kahan(C.Structure):
    _fields_ = [("c", C.c_float), ("sum", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_reference=False)
        L = C.CDLL(LIB_PATH)
        L.spo_murmur3_bytes.restype = _U128
        L.spo_murmur3_bytes.argtypes = [C.c_void_p, C.c_uint64]
        L.spo_murmur3_u128.restype = _U128
        L.spo_murmur3_u128.argtypes = [_U128]
        L.spo_seed_from_list.restype = _U128
        L.spo_seed_from_list.argtypes = [C.POINTER(C.c_uint32), C.c_int]
        L.spo_seed_next.restype = _U128
        L.spo_seed_next.argtypes = [C.POINTER(_U128)]
        L.spo_xoroshiro128p_next.restype = C.c_uint64
        L.spo_xoroshiro128p_next.argtypes = [C.POINTER(C.c_uint64)]
        L.spo_xoroshiro128p_jump.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.spo_canonical_f32.restype = C.c_float
        L.spo_canonical_f32.argtypes = [C.c_uint64]
        L.spo_canonical_f64_leftopen.restype = C.c_double
        L.spo_canonical_f64_leftopen.argtypes = [C.c_uint64]
        L.spo_exponential.restype = C.c_double
        L.spo_exponential.argtypes = [C.c_double, C.POINTER(C.c_uint64)]
        L.spo_kahan_step.restype = C.c_float
        L.spo_kahan_step.argtypes = [C.POINTER(_Kahan), C.c_float]
        L.spo_fp_max_degree.restype = C.c_int64
        L.spo_fp_max_degree.argtypes = [C.c_int64, C.c_double]
        L.spo_fp_generate.restype = C.c_int64
        L.spo_fp_generate.argtypes = [C.c_int64, C.c_int64, C.c_double, _U128, C.c_void_p,
                                      C.c_void_p, C.POINTER(C.c_int64)]
        L.spo_net_create.restype = C.c_void_p
        L.spo_net_create.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_uint32), C.c_int]
        L.spo_net_destroy.argtypes = [C.c_void_p]
        L.spo_add_population.restype = C.c_int
        L.spo_add_population.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.POINTER(C.c_float), C.c_int]
        L.spo_set_external.restype = C.c_int
        L.spo_set_external.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.spo_connect.restype = C.c_int
        L.spo_connect.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_float, C.c_int, C.c_float]
        L.spo_connect_weighted.restype = C.c_int
        L.spo_connect_weighted.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_float, C.c_int, C.c_float]
        L.spo_syn_weights.restype = C.c_int
        L.spo_syn_weights.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.spo_connect_adj.restype = C.c_int
        L.spo_connect_adj.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_float,
                                      C.c_int, C.c_float]
        L.spo_step.argtypes = [C.c_void_p]
        L.spo_run.argtypes = [C.c_void_p, C.c_int64]
        for f in ("spo_time", "spo_events"):
            getattr(L, f).restype = C.c_int64
            getattr(L, f).argtypes = [C.c_void_p]
        L.spo_spike_count.restype = C.c_int64
        L.spo_spike_count.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.spo_spikes.restype = C.c_int64
        L.spo_spikes.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.spo_pop_size.restype = C.c_int64
        L.spo_pop_size.argtypes = [C.c_void_p, C.c_int]
        L.spo_get_state.restype = C.c_int
        L.spo_get_state.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.spo_set_state.restype = C.c_int
        L.spo_set_state.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.spo_conn_synapses.restype = C.c_int64
        L.spo_conn_synapses.argtypes = [C.c_void_p, C.c_int]
        L.spo_conn_csr.restype = C.c_int
        L.spo_conn_csr.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.spo_last_dt.restype = C.c_float
        L.spo_last_dt.argtypes = [C.c_void_p]
        L.spo_last_error.restype = C.c_char_p
        L.spo_set_plastic.restype = C.c_int
        L.spo_set_plastic.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]
        L.spo_syn_state.restype = C.c_int
        L.spo_syn_state.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        _lib = L
    return _lib


# ---- RNG helpers ---------------------------------------------------------------------------
def seed_from_list(seeds) -> tuple[int, int]:
    arr = (C.c_uint32 * len(seeds))(*seeds)
    r = lib().spo_seed_from_list(arr, len(seeds))
    return r.lo, r.hi


def seed_chain(seeds, n: int) -> list[tuple[int, int]]:
    """The values returned by n successive seed_seq post-increments."""
    lo, hi = seed_from_list(seeds)
    s = _U128(lo, hi)
    out = []
    for _ in range(n):
        r = lib().spo_seed_next(C.byref(s))
        out.append((r.lo, r.hi))
    return out


def xoroshiro_draws(state: tuple[int, int], n: int) -> np.ndarray:
    s = (C.c_uint64 * 2)(*state)
    return np.array([lib().spo_xoroshiro128p_next(s) for _ in range(n)], dtype=np.uint64)


def xoroshiro_jump(state: tuple[int, int], poly: tuple[int, int]) -> tuple[int, int]:
    s = (C.c_uint64 * 2)(*state)
    p = (C.c_uint64 * 2)(*poly)
    lib().spo_xoroshiro128p_jump(s, p)
    return s[0], s[1]


def kahan_dts(n: int, dt: float = 1e-4) -> np.ndarray:
    k = _Kahan(0.0, 0.0)
    return np.array([lib().spo_kahan_step(C.byref(k), dt) for _ in range(n)], dtype=np.float32)


def fp_max_degree(dst: int, p: float) -> int:
    return lib().spo_fp_max_degree(dst, p)


def fp_generate(src: int, dst: int, p: float, seed: tuple[int, int]):
    """One fixed_probability CSR for an explicit 128-bit seed: (offsets int64, neighbors int32, draws)."""
    md = fp_max_degree(dst, p) if src > 0 else 0
    off = np.zeros(src + 1, dtype=np.int64)
    nb = np.zeros(max(1, src * max(md, 0)), dtype=np.int32)
    draws = C.c_int64(0)
    n = lib().spo_fp_generate(src, dst, p, _U128(*seed), off.ctypes.data, nb.ctypes.data, C.byref(draws))
    return off, nb[:n].copy(), draws.value


# ---- network ---------------------------------------------------------------------------------
class Net:
    """The CPU restatement of an snn with fixed_weight synapses."""

    def __init__(self, dt: float, max_delay: float, seeds):
        seeds = list(seeds) if hasattr(seeds, "__iter__") else [seeds]
        arr = (C.c_uint32 * len(seeds))(*seeds)
        self.h = lib().spo_net_create(dt, max_delay, arr, len(seeds))
        if not self.h:
            raise RuntimeError(lib().spo_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().spo_net_destroy(self.h)
            self.h = None

    def _chk(self, r):
        if r < 0:
            raise RuntimeError(lib().spo_last_error().decode())
        return r

    def add_population(self, kind: int, size: int, params=()):
        arr = (C.c_float * max(1, len(params)))(*params)
        return self._chk(lib().spo_add_population(self.h, kind, size, arr, len(params)))

    def set_external(self, pop: int, trains):
        counts = np.array([len(t) for t in trains], dtype=np.int32)
        idx = np.concatenate([np.asarray(t, dtype=np.int32) for t in trains] + [np.zeros(0, np.int32)])
        self._chk(lib().spo_set_external(self.h, pop, len(trains), counts.ctypes.data, idx.ctypes.data))

    def connect(self, src, dst, p, delay, weight, field=0):
        return self._chk(lib().spo_connect(self.h, src, dst, p, delay, field, weight))

    def connect_weighted(self, src, dst, p, delay, wmax, field=0):
        """fixed_probability with per-synapse weights wmax * canonical<float> (PerSynapseInit)."""
        return self._chk(lib().spo_connect_weighted(self.h, src, dst, p, delay, field, wmax))

    def syn_weights(self, conn) -> np.ndarray:
        m = lib().spo_conn_synapses(self.h, conn)
        out = np.zeros(max(1, m), dtype=np.float32)
        self._chk(lib().spo_syn_weights(self.h, conn, out.ctypes.data))
        return out[:m]

    def csr_arrays(self, conn, src_size):
        m = lib().spo_conn_synapses(self.h, conn)
        off = np.zeros(src_size + 1, dtype=np.int64)
        nb = np.zeros(max(1, m), dtype=np.int32)
        self._chk(lib().spo_conn_csr(self.h, conn, off.ctypes.data, nb.ctypes.data))
        return off, nb[:m]

    def connect_adj(self, src, dst, pairs, delay, weight, field=0):
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        return self._chk(lib().spo_connect_adj(self.h, src, dst, len(pr), pr.ctypes.data, delay, field, weight))

    def step(self):
        lib().spo_step(self.h)

    def run(self, n):
        lib().spo_run(self.h, n)

    @property
    def time(self):
        return lib().spo_time(self.h)

    @property
    def events(self):
        return lib().spo_events(self.h)

    @property
    def last_dt(self):
        return lib().spo_last_dt(self.h)

    def spikes(self, pop, age=0) -> np.ndarray:
        n = self._chk(lib().spo_spike_count(self.h, pop, age))
        out = np.zeros(max(1, n), dtype=np.int32)
        lib().spo_spikes(self.h, pop, age, out.ctypes.data)
        return out[:n]

    def state(self, pop, field):
        n = lib().spo_pop_size(self.h, pop)
        out = np.zeros(n, dtype=np.int32 if field == 3 else np.float32)
        self._chk(lib().spo_get_state(self.h, pop, field, out.ctypes.data))
        return out

    def set_state(self, pop, field, values):
        v = np.ascontiguousarray(values, dtype=np.int32 if field == 3 else np.float32)
        self._chk(lib().spo_set_state(self.h, pop, field, v.ctypes.data))

    def set_plastic(self, conn, model, w0=0.0, eta=0.0, rho0=0.0, tau=0.02):
        """model: SYN_ISTDP or SYN_COUNT (spo_set_plastic)."""
        self._chk(lib().spo_set_plastic(self.h, conn, model, w0, eta, rho0, tau))

    def syn_state(self, conn, field=0) -> np.ndarray:
        out = np.zeros(max(1, lib().spo_conn_synapses(self.h, conn)), dtype=np.float32)
        self._chk(lib().spo_syn_state(self.h, conn, field, out.ctypes.data))
        return out[:lib().spo_conn_synapses(self.h, conn)]

    def csr(self, conn):
        n = lib().spo_conn_synapses(self.h, conn)
        # source size is not stored separately here; read it from the offsets length
        return n


def brunel(N: int, p: float, seed: int, dt=1e-4, delay=15e-4):
    """Brunel (samples/brunel.cpp:75-103) with weights scaled by 0.1/p. Returns (net, (P, E, I))."""
    net = Net(dt, delay, [seed])
    P = net.add_population(POISSON, N // 2, (20.0,))
    E = net.add_population(LIF, N * 4 // 10)
    I = net.add_population(LIF, N // 10)
    we, wi = brunel_weights(N, p)
    for s, d, w in ((P, E, we), (P, I, we), (E, E, we), (E, I, we), (I, E, wi), (I, I, wi)):
        net.connect(s, d, p, delay, w)
    return net, (P, E, I)


def vogels_weights(N: int) -> tuple[float, float]:
    """samples/vogels.cpp:72-75: float(6.4e6 / (N * N)) and float(8.16e7 / (N * N)) (double, then float)."""
    return float(np.float32(6.4e6 / (N * N))), float(np.float32(8.16e7 / (N * N)))


def vogels(N: int, seed: int = 1337, p: float = 0.02, dt=1e-4, delay=8e-4, we=None, wi=None):
    """samples/vogels.cpp:62-86 (E = 0.8 N, I = 0.2 N conductance LIF; E->E, E->I excitatory,
    I->E, I->I inhibitory, fixed_probability(p)).  Returns (net, (E, I))."""
    dwe, dwi = vogels_weights(N)
    we = dwe if we is None else we
    wi = dwi if wi is None else wi
    net = Net(dt, delay, [seed])
    E = net.add_population(LIF_COND, N * 8 // 10)
    I = net.add_population(LIF_COND, N * 2 // 10)
    for s, d, w, fl in ((E, E, we, 1), (E, I, we, 1), (I, E, wi, 2), (I, I, wi, 2)):
        net.connect(s, d, p, delay, w, fl)
    return net, (E, I)


def vogels_spec(N: int, seed: int, steps: int, p: float = 0.02, dt=1e-4, delay=8e-4, we=None,
                wi=None) -> list[str]:
    """The same network as a ref_driver spec."""
    dwe, dwi = vogels_weights(N)
    we = dwe if we is None else we
    wi = dwi if wi is None else wi
    lines = [f"{dt!r} {delay!r} {seed} {steps} 0", f"pop lif_cond {N * 8 // 10}", f"pop lif_cond {N * 2 // 10}"]
    for s, d, w, fl in ((0, 0, we, 1), (0, 1, we, 1), (1, 0, wi, 2), (1, 1, wi, 2)):
        lines.append(f"conn {s} {d} {p!r} {delay!r} {w!r} {fl}")
    return lines


# A network with per-synapse weights (the weighted synapse: PerSynapseInit, w = wmax * canonical
# <float>) into LIF and conductance-LIF targets, mixed with fixed weights and mixed delays; and a
# population with six distinct fixed input weights.  (kind, src, dst, p, delay, weight / wmax,
# field); kind "w" weighted, "f" fixed_weight.
WEIGHTED_NET = {
    "dt": 1e-4, "max_delay": 12e-4, "seed": 2718,
    "pops": [("poisson", 3000, 40.0), ("lif", 2000), ("lif", 500), ("lif_cond", 1000), ("lif", 800)],
    "conns": [("w", 0, 1, 0.05, 5e-4, 0.01, 0), ("f", 1, 1, 0.05, 7e-4, 0.002, 0),
              ("w", 2, 1, 0.1, 4e-4, -0.02, 0), ("f", 0, 2, 0.02, 3e-4, 0.004, 0),
              ("w", 1, 2, 0.05, 6e-4, 0.006, 0), ("f", 2, 2, 0.02, 9e-4, -0.004, 0),
              ("w", 1, 3, 0.02, 4e-4, 0.8, 1), ("w", 2, 3, 0.05, 5e-4, 0.2, 2), ("f", 0, 3, 0.02, 8e-4, 0.03, 1),
              ("f", 0, 4, 0.01, 3e-4, 0.011, 0), ("f", 1, 4, 0.01, 4e-4, 0.0035, 0),
              ("f", 2, 4, 0.02, 5e-4, -0.007, 0), ("f", 0, 4, 0.01, 6e-4, 0.009, 0),
              ("f", 1, 4, 0.02, 3e-4, 0.0021, 0), ("f", 2, 4, 0.01, 12e-4, -0.0105, 0)],
}


def _f32(x):
    return float(np.float32(x))


def weighted_net(spec=WEIGHTED_NET):
    """WEIGHTED_NET on the oracle: returns (net, pops, conns)."""
    net = Net(spec["dt"], spec["max_delay"], [spec["seed"]])
    kinds = {"poisson": POISSON, "lif": LIF, "lif_cond": LIF_COND}
    pops = [net.add_population(kinds[p[0]], p[1], p[2:]) for p in spec["pops"]]
    conns = []
    for kind, s, d, p, delay, w, fl in spec["conns"]:
        if kind == "w":
            conns.append(net.connect_weighted(pops[s], pops[d], p, delay, _f32(w), fl))
        else:
            conns.append(net.connect(pops[s], pops[d], p, delay, _f32(w), fl))
    return net, pops, conns


def weighted_net_spec(steps: int, spec=WEIGHTED_NET) -> list[str]:
    lines = [f"{spec['dt']!r} {spec['max_delay']!r} {spec['seed']} {steps} 0"]
    for p in spec["pops"]:
        lines.append(f"pop poisson {p[1]} {p[2]!r}" if p[0] == "poisson" else f"pop {p[0]} {p[1]}")
    for kind, s, d, p, delay, w, fl in spec["conns"]:
        cond = spec["pops"][d][0] == "lif_cond"
        lines.append(f"{'wconn' if kind == 'w' else 'conn'} {s} {d} {p!r} {delay!r} {_f32(w)!r}" + (f" {fl}" if cond else ""))
    return lines


def brunel_plus_spec(seed: int, steps: int, N: int = 20000) -> list[str]:
    """samples/brunel+.cpp (Brunel at p = 0.1 with the STDP synapse on E->E) as a ref_driver spec."""
    d = 15e-4
    we, wi = float(np.float32(2.0 / N)), float(np.float32(-10.0 / N))
    return [f"{1e-4!r} {d!r} {seed} {steps} 0", f"pop poisson {N // 2} 20", f"pop lif {N * 4 // 10}",
            f"pop lif {N // 10}", f"conn 0 1 0.1 {d!r} {we!r}", f"conn 0 2 0.1 {d!r} {we!r}", f"stdp 1 0.1 {d!r}",
            f"conn 1 2 0.1 {d!r} {we!r}", f"conn 2 1 0.1 {d!r} {wi!r}", f"conn 2 2 0.1 {d!r} {wi!r}"]


def brunel_weights(N: int, p: float) -> tuple[float, float]:
    """float((2/N)(0.1/p)) and float((-10/N)(0.1/p)), computed in double then rounded."""
    return float(np.float32((2.0 / N) * (0.1 / p))), float(np.float32((-10.0 / N) * (0.1 / p)))


# ---- the reference driver ---------------------------------------------------------------------
def have_reference() -> bool:
    return os.path.exists(REF_DRIVER)


def run_reference_net(spec_lines: list[str]):
    """Runs oracle/_ref/ref_driver on a network spec; returns a dict of results."""
    with tempfile.TemporaryDirectory() as d:
        spec = os.path.join(d, "spec.txt")
        out = os.path.join(d, "out.bin")
        open(spec, "w").write("\n".join(spec_lines) + "\n")
        subprocess.run([REF_DRIVER, "net", spec, out], check=True)
        return read_reference_net(open(out, "rb").read())


def read_reference_net(buf: bytes):
    pos = 0

    def take(fmt):
        nonlocal pos
        v = struct.unpack_from(fmt, buf, pos)
        pos += struct.calcsize(fmt)
        return v

    (npop,) = take("<q")
    sizes = list(take(f"<{npop}q"))
    (steps,) = take("<q")
    dts = np.frombuffer(buf, dtype=np.float32, count=steps, offset=pos).copy()
    pos += 4 * steps
    raster = []
    for _ in range(steps):
        row = []
        for _k in range(npop):
            (n,) = take("<q")
            row.append(np.frombuffer(buf, dtype=np.int32, count=n, offset=pos).copy())
            pos += 4 * n
        raster.append(row)
    states = []
    return {"sizes": sizes, "steps": steps, "dt": dts, "raster": raster, "_rest": buf[pos:]}


def reference_states(res, lif_pops, cond_pops=()):
    """Splits the trailing neuron states out of a reference result, populations in add order:
    (V, T) for each LIF population in lif_pops, (V, Gex, Gin, T) for each conductance LIF in
    cond_pops (the ref_driver writes them in population order)."""
    rest = res["_rest"]
    pos = 0
    out = {}
    for k in sorted(set(lif_pops) | set(cond_pops)):
        n = res["sizes"][k]
        if k in cond_pops:
            dt = np.dtype([("V", "<f4"), ("Gex", "<f4"), ("Gin", "<f4"), ("T", "<i4")])
            rec = np.frombuffer(rest, dtype=dt, count=n, offset=pos)
            out[k] = (rec["V"].copy(), rec["Gex"].copy(), rec["Gin"].copy(), rec["T"].copy())
            pos += 16 * n
        else:
            rec = np.frombuffer(rest, dtype=np.dtype([("V", "<f4"), ("T", "<i4")]), count=n, offset=pos)
            out[k] = (rec["V"].copy(), rec["T"].copy())
            pos += 8 * n
    build_s, step_s = struct.unpack_from("<dd", rest, pos)
    return out, build_s, step_s


def run_reference_brunel_ck(N: int, p: float, seed: int, steps: int, block: int):
    """Runs Brunel on oracle/_ref/ref_driver (brunel_ck): returns (counts[steps][3] int32,
    blocks[nblocks][3] uint64 = raster checksum of each block of `block` steps and the E / I state
    checksums at its end)."""
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "ck.bin")
        subprocess.run([REF_DRIVER, "brunel_ck", str(N), repr(p), str(seed), str(steps), str(block), out], check=True)
        buf = open(out, "rb").read()
    counts, blocks, pos, t = [], [], 0, 0
    while t < steps:
        n = min(block, steps - t)
        counts.append(np.frombuffer(buf, dtype=np.int32, count=3 * n, offset=pos).reshape(n, 3))
        pos += 12 * n
        blocks.append(np.frombuffer(buf, dtype=np.uint64, count=3, offset=pos))
        pos += 24
        t += n
    return np.concatenate(counts).copy(), np.array(blocks, dtype=np.uint64)


def run_reference_plastic_ei(N: int, seed: int, steps: int, eta: float = 1e-3):
    """Runs the plastic E/I network on oracle/_ref/ref_driver (plastic_ei): returns (counts[steps][2]
    int32 spike counts of E and I, isi[2][3] pooled inter-spike interval count / sum / sum of
    squares in steps, (build seconds, run seconds))."""
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "pe.bin")
        subprocess.run([REF_DRIVER, "plastic_ei", str(N), str(seed), str(steps), repr(eta), out], check=True)
        buf = open(out, "rb").read()
    counts = np.frombuffer(buf, dtype=np.int32, count=2 * steps).reshape(steps, 2).copy()
    rest = np.frombuffer(buf, dtype=np.float64, offset=8 * steps).copy()
    return counts, rest[:6].reshape(2, 3), (float(rest[6]), float(rest[7]))


def run_reference_gen(src: int, dst: int, p: float, seed: int):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "g.bin")
        subprocess.run([REF_DRIVER, "gen", str(src), str(dst), repr(p), str(seed), out], check=True)
        buf = open(out, "rb").read()
    md, n = struct.unpack_from("<qq", buf, 0)
    off = np.frombuffer(buf, dtype=np.int64, count=src + 1, offset=16).copy()
    nb = np.frombuffer(buf, dtype=np.int32, count=n, offset=16 + 8 * (src + 1)).copy()
    return md, off, nb


def run_reference_rng(seed: int, n: int):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "r.bin")
        subprocess.run([REF_DRIVER, "rng", str(seed), str(n), out], check=True)
        buf = open(out, "rb").read()
    chain = np.frombuffer(buf, dtype=np.uint64, count=2 * n, offset=0).reshape(n, 2).copy()
    o = 16 * n
    draws = np.frombuffer(buf, dtype=np.uint64, count=n, offset=o).copy()
    o += 8 * n
    expo = np.frombuffer(buf, dtype=np.float64, count=n, offset=o).copy()
    o += 8 * n
    canon = np.frombuffer(buf, dtype=np.float32, count=n, offset=o).copy()
    o += 4 * n
    kahan = np.frombuffer(buf, dtype=np.float32, count=n, offset=o).copy()
    return {"chain": chain, "draws": draws, "exp": expo, "canon": canon, "kahan": kahan}


def brunel_spec(N: int, p: float, seed: int, steps: int, dt=1e-4, delay=15e-4) -> list[str]:
    we, wi = brunel_weights(N, p)
    lines = [f"{dt!r} {delay!r} {seed} {steps} 0",
             f"pop poisson {N // 2} 20", f"pop lif {N * 4 // 10}", f"pop lif {N // 10}"]
    for s, d, w in ((0, 1, we), (0, 2, we), (1, 1, we), (1, 2, we), (2, 1, wi), (2, 2, wi)):
        lines.append(f"conn {s} {d} {p!r} {delay!r} {w!r}")
    return lines


def csr_checksum(off: np.ndarray, nb: np.ndarray) -> int:
    """Order-sensitive 64-bit checksum of a CSR (offsets, neighbors), wrapping arithmetic."""
    with np.errstate(over="ignore"):
        o = off.astype(np.uint64)
        i = np.arange(len(o), dtype=np.uint64)
        mo = (i * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x632BE59BD9B4E019)) | np.uint64(1)
        h1 = int(np.sum((o + np.uint64(1)) * mo, dtype=np.uint64))
        n = nb.astype(np.int64).astype(np.uint64)
        j = np.arange(len(n), dtype=np.uint64)
        mn = (j * np.uint64(0xD1B54A32D192ED03) + np.uint64(0x8CB92BA72F3D8DD7)) | np.uint64(1)
        h2 = int(np.sum((n + np.uint64(1)) * mn, dtype=np.uint64))
    return (h1 ^ ((h2 << 1) | (h2 >> 63))) & 0xFFFFFFFFFFFFFFFF


def raster_checksum(counts: np.ndarray, idx: np.ndarray) -> int:
    """Checksum of a raster given as per-step, per-population counts and the flat spike indices."""
    with np.errstate(over="ignore"):
        a = (idx.astype(np.int64).astype(np.uint64) + np.uint64(1)) * (
            (np.arange(len(idx), dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)) | np.uint64(1))
        b = (np.asarray(counts).ravel().astype(np.uint64) + np.uint64(7)) * (
            (np.arange(np.asarray(counts).size, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)) | np.uint64(1))
        return int(np.sum(a, dtype=np.uint64) ^ np.sum(b, dtype=np.uint64))


def state_checksum(V: np.ndarray, T: np.ndarray) -> int:
    """Checksum of a LIF population's (V bits, Tref) state."""
    with np.errstate(over="ignore"):
        v = np.ascontiguousarray(V, dtype=np.float32).view(np.uint32).astype(np.uint64)
        t = np.ascontiguousarray(T, dtype=np.int32).view(np.uint32).astype(np.uint64)
        i = np.arange(len(v), dtype=np.uint64)
        return int(np.sum((v + np.uint64(3)) * ((i * np.uint64(0x9E3779B97F4A7C15)) | np.uint64(1)), dtype=np.uint64)
                   ^ np.sum((t + np.uint64(5)) * ((i * np.uint64(0xD1B54A32D192ED03)) | np.uint64(1)), dtype=np.uint64))


def mixed_net(steps_unused=None):
    """The mixed-delay network of tests/golden/make_golden.py built on the oracle: returns (net, pops, pairs)."""
    rng = np.random.default_rng(5)
    pairs = sorted({(int(a), int(b)) for a, b in zip(rng.integers(0, 2000, 6000), rng.integers(0, 1000, 6000))})
    net = Net(1e-4, 8e-4, [4242])
    P = net.add_population(POISSON, 3000, (50.0,))
    E = net.add_population(LIF, 2000)
    I = net.add_population(LIF, 1000)
    f = lambda x: float(np.float32(x))
    net.connect(P, E, 0.05, 3e-4, f(0.002))
    net.connect(E, E, 0.05, 5e-4, f(0.002))
    net.connect(I, E, 0.1, 2e-4, f(-0.005))
    net.connect(P, I, 0.02, 4e-4, f(0.004))
    net.connect_adj(E, I, pairs, 6e-4, f(0.003))
    net.connect(I, I, 0.02, 7e-4, f(-0.004))
    net.connect(E, E, 0.01, 8e-4, f(0.003))
    return net, (P, E, I), pairs
