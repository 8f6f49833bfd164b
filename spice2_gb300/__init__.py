"""spice2_gb300 -- the GB300-native snn::step engine, driven from Python.

This mirrors the reference's user API (spice/include/spice/snn.h and the sample models of
samples/brunel.cpp, samples/vogels.cpp, samples/external_input.cpp) over the C ABI declared in
include/spice_gb300.h:

    from spice2_gb300 import snn, poisson, lif, fixed_weight, fixed_probability
    brunel = snn(1e-4, 15e-4, [1337])                       # snn(dt, max_delay, seed)
    P = brunel.add_population(poisson(20), N // 2)           # add_population<poisson>(N/2)
    E = brunel.add_population(lif(), N * 4 // 10)
    brunel.connect(P, E, fixed_probability(0.1), 15e-4, fixed_weight(2 / N))
    brunel.step()                                            # snn::step()
    P.spikes(0)                                              # NeuronPopulation::spikes(age)

Every call runs on the GPU through libspice_gb300.so.  There is no CPU fallback: importing the
package fails loudly when the library has not been built (``python -m spice2_gb300.build``).
Failed preconditions raise LogicError with the reference's message
("Assertion failed (file:line): cond", spice/src/util/assert.cpp:8-15).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field as dc_field
from typing import Iterable, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspice_gb300.so")

OK, EINVAL, ECUDA, ENOMEM, ESTATE, EOVERFLOW = 0, 1, 2, 3, 4, 5
NEURON_POISSON, NEURON_LIF, NEURON_LIF_COND, NEURON_EXTERNAL = 0, 1, 2, 3
SYNAPSE_FIXED_WEIGHT, SYNAPSE_ISTDP, SYNAPSE_COUNT, SYNAPSE_WEIGHTED = 0, 1, 2, 3
MODE_DETERMINISTIC, MODE_ATOMIC = 0, 1
FIELD_V, FIELD_GEX, FIELD_GIN, FIELD_TREF = 0, 1, 2, 3


class SpiceError(RuntimeError):
    """A failed call into libspice_gb300; .code is the SPICE_E* status."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class LogicError(SpiceError, ValueError):
    """A violated precondition -- the reference throws std::logic_error for these."""


class CudaError(SpiceError):
    pass


_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA engine first (python -m spice2_gb300.build); "
            "spice2_gb300 has no CPU fallback")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, u32, f32, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint32, C.c_float, C.c_double
    P = C.POINTER
    sig = {
        "spice_net_create": [f32, f32, P(u32), i32, P(vp)],
        "spice_net_destroy": [vp],
        "spice_add_population": [vp, i32, i64, P(f32), i32, P(i32)],
        "spice_connect_fixed_probability": [vp, i32, i32, f64, f32, i32, P(f32), i32, P(i32)],
        "spice_connect_adj_list": [vp, i32, i32, vp, i64, f32, i32, P(f32), i32, P(i32)],
        "spice_set_external_input": [vp, i32, i32, vp, vp],
        "spice_set_mode": [vp, i32],
        "spice_set_window": [vp, i32],
        "spice_step": [vp],
        "spice_run": [vp, i64],
        "spice_run_record": [vp, i64, vp, vp, i64, P(i64)],
        "spice_spike_count": [vp, i32, i64, P(i64)],
        "spice_spikes": [vp, i32, i64, vp, i64, P(i64)],
        "spice_get_state": [vp, i32, i32, vp],
        "spice_set_state": [vp, i32, i32, vp],
        "spice_pop_size": [vp, i32, P(i64)],
        "spice_time": [vp, P(i64)],
        "spice_events": [vp, P(C.c_uint64)],
        "spice_conn_size": [vp, i32, P(i64), P(i64)],
        "spice_get_synapse_state": [vp, i32, i32, vp],
        "spice_get_csr": [vp, i32, vp, vp],
        "spice_get_csc": [vp, i32, vp, vp],
        "spice_set_profiling": [vp, i32],
        "spice_kernel_stats": [vp, i32, P(i64), P(f64)],
        "spice_kernel_span": [vp, i32, P(i64), P(f64)],
        "spice_launch_count": [vp, P(i64)],
        "spice_get_stream": [vp, P(vp)],
        "spice_set_tuning": [vp, i32, i64],
        "spice_get_tuning": [vp, i32, vp],
        "spice_synchronize": [vp],
        "spice_batch_create": [P(vp), i32, P(vp)],
        "spice_batch_destroy": [vp],
        "spice_batch_run": [vp, i64],
        "spice_batch_set_tuning": [vp, i32, i64],
        "spice_batch_set_profiling": [vp, i32],
        "spice_batch_kernel_stats": [vp, i32, P(i64), P(f64)],
        "spice_batch_launch_count": [vp, P(i64)],
        "spice_batch_get_stream": [vp, P(vp)],
        "spice_add_user_population": [vp, i64, i32, i32, vp, vp, vp, P(i32)],
        "spice_user_field": [vp, i32, i32, P(i32)],
        "spice_get_user_state": [vp, i32, vp],
        "spice_set_user_state": [vp, i32, vp],
        "spice_lif_layer_create": [i32, i32, vp, vp, vp, vp, P(vp)],
        "spice_lif_layer_destroy": [vp],
        "spice_lif_layer_synapses": [vp, P(i64), P(i64)],
        "spice_lif_forward": [vp, i32, i32, i32, i32, f32, vp, vp, vp, vp, vp, vp, vp, vp, vp],
        "spice_lif_backward": [vp, i32, i32, i32, i32, f32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp],
        "spice_selftest_skip_rounding": [i64, C.c_uint64, P(i64), P(u32), P(f64)],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.spice_last_error.argtypes = []
    L.spice_last_error.restype = C.c_char_p
    _lib = L
    return L


def lib():
    return _load()


def _check(rc: int):
    if rc == OK:
        return
    msg = (_load().spice_last_error() or b"").decode()
    if rc == EINVAL:
        raise LogicError(rc, msg)
    if rc == ECUDA:
        raise CudaError(rc, msg)
    raise SpiceError(rc, msg)


# ---- models ---------------------------------------------------------------------------------
@dataclass(frozen=True)
class poisson:
    """Stateless Poisson source: fires when canonical<float>(rng) < rate*dt (samples/brunel.cpp:23-31)."""
    rate: float = 20.0
    model = NEURON_POISSON

    def params(self):
        return [self.rate]


@dataclass(frozen=True)
class lif:
    """Brunel LIF {V, Tref} (samples/brunel.cpp:39-62)."""
    Vthres: float = 0.02
    Tref: int = 20
    TmemInv: float = 50.0
    model = NEURON_LIF

    def params(self):
        return [self.Vthres, float(self.Tref), self.TmemInv]


@dataclass(frozen=True)
class lif_cond:
    """Conductance LIF {V, Gex, Gin, Tref} with the constants of samples/vogels.cpp:10-46."""
    model = NEURON_LIF_COND

    def params(self):
        return []


@dataclass(frozen=True)
class external_input:
    """Per-population update replaying a cyclic spike train (samples/external_input.cpp:17-30)."""
    trains: tuple = ()
    model = NEURON_EXTERNAL

    def params(self):
        return []


@dataclass(frozen=True)
class fixed_weight:
    """Adds `weight` to a target state field on every spike (samples/brunel.cpp:67-70)."""
    weight: float
    field: int = FIELD_V

    def params(self):
        return [self.weight, float(self.field)]


@dataclass(frozen=True)
class istdp:
    """Inhibitory symmetric STDP (Vogels et al. 2011) as a plastic synapse with lazy, event-driven
    updates (the reference's PlasticSynapse concept, synapse_population.h:82-140): W starts at w0;
    a pre spike does W = max(0, W + eta (x_post - 2 rho0 tau)), a post spike W += eta x_pre; the
    traces decay with tau.  Delivery adds W to the target field (default Gin).  Needs atomic mode."""
    w0: float
    field: int = FIELD_GIN
    eta: float = 1e-3
    rho0: float = 5.0
    tau: float = 0.02
    model = SYNAPSE_ISTDP

    def params(self):
        return [self.w0, float(self.field), self.eta, self.rho0, self.tau]


@dataclass(frozen=True)
class count_synapse:
    """The counting plastic synapse of the reference's tests (test/detail/synapse_population.cpp:
    84-94): update() adds 1, skip(n) adds n; delivery adds scale * count (scale 0: nothing)."""
    scale: float = 0.0
    field: int = FIELD_V
    model = SYNAPSE_COUNT

    def params(self):
        return [self.scale, float(self.field)]


@dataclass(frozen=True)
class weighted:
    """A synapse with its own weight, drawn when the connection is built: the reference's
    StatefulSynapse + PerSynapseInit concepts (concepts.h:60-104; the synapse_population ctor walks
    the CSR in order with the stream seeded after the adjacency's, synapse_population.h:30-41), here
    w = wmax * canonical<float>(rng).  Delivery adds w to the target field.  Populations receiving
    weighted synapses are delivered by the deterministic pull path."""
    wmax: float
    field: int = FIELD_V
    model = SYNAPSE_WEIGHTED

    def params(self):
        return [self.wmax, float(self.field)]


def excitatory(weight: float) -> fixed_weight:
    """samples/vogels.cpp:48-53: to.Gex += weight."""
    return fixed_weight(weight, FIELD_GEX)


def inhibitory(weight: float) -> fixed_weight:
    """samples/vogels.cpp:55-60: to.Gin += weight."""
    return fixed_weight(weight, FIELD_GIN)


# ---- topologies -----------------------------------------------------------------------------
@dataclass(frozen=True)
class fixed_probability:
    """fixed_probability(p) (spice/include/spice/topology.h:48-58)."""
    p: float


@dataclass
class adj_list:
    """adj_list (spice/include/spice/topology.h:37-46): connect(src, dst) edge by edge."""
    edges: list = dc_field(default_factory=list)

    def connect(self, src: int, dst: int):
        self.edges.append((int(src), int(dst)))

    def size(self) -> int:
        return len(self.edges)


# ---- network --------------------------------------------------------------------------------
class Population:
    """Handle returned by snn.add_population (the neuron_population<Neur>* of snn.h:21-27)."""

    def __init__(self, net: "snn", idx: int, model):
        self._net = net
        self.id = idx
        self.model = model

    def size(self) -> int:
        v = C.c_int64()
        _check(lib().spice_pop_size(self._net._h, self.id, C.byref(v)))
        return v.value

    def spikes(self, age: int = 0) -> np.ndarray:
        return self._net.spikes(self, age)

    def get_neurons(self) -> dict:
        """State of a stateful population as SoA numpy arrays (neuron_population.h:139-145)."""
        fields = {"V": FIELD_V, "Tref": FIELD_TREF}
        if self.model.model == NEURON_LIF_COND:
            fields.update({"Gex": FIELD_GEX, "Gin": FIELD_GIN})
        return {k: self._net.get_state(self, f) for k, f in fields.items()}

    def __repr__(self):
        return f"Population({self.id}, {self.model})"


class snn:
    """snn(dt, max_delay, seed) -- spice/include/spice/snn.h:16-75, running on the GPU."""

    def __init__(self, dt: float, max_delay: float, seed: Sequence[int] | int):
        seeds = [int(seed)] if isinstance(seed, (int, np.integer)) else [int(s) for s in seed]
        arr = (C.c_uint32 * max(1, len(seeds)))(*seeds)
        h = C.c_void_p()
        _check(lib().spice_net_create(dt, max_delay, arr, len(seeds), C.byref(h)))
        self._h = h
        self._pops: list[Population] = []
        self._conns: list[tuple] = []

    def close(self):
        if getattr(self, "_h", None):
            lib().spice_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # construction
    def add_population(self, model, size: int) -> Population:
        prm = model.params()
        arr = (C.c_float * max(1, len(prm)))(*prm)
        out = C.c_int()
        _check(lib().spice_add_population(self._h, model.model, int(size), arr, len(prm), C.byref(out)))
        pop = Population(self, out.value, model)
        self._pops.append(pop)
        if model.model == NEURON_EXTERNAL and model.trains:
            self.set_external_input(pop, model.trains)
        return pop

    def set_external_input(self, pop: Population, trains: Iterable[Iterable[int]]):
        trains = [np.asarray(list(t), dtype=np.int32) for t in trains]
        counts = np.array([len(t) for t in trains], dtype=np.int32)
        idx = np.concatenate(trains + [np.zeros(0, np.int32)]).astype(np.int32)
        _check(lib().spice_set_external_input(self._h, pop.id, len(trains), counts.ctypes.data, idx.ctypes.data))

    def connect(self, source: Population, target: Population, topology, delay: float, syn) -> int:
        prm = syn.params()
        arr = (C.c_float * len(prm))(*prm)
        out = C.c_int()
        if isinstance(topology, fixed_probability):
            _check(lib().spice_connect_fixed_probability(self._h, source.id, target.id, float(topology.p),
                                                         delay, getattr(syn, "model", SYNAPSE_FIXED_WEIGHT), arr,
                                                         len(prm), C.byref(out)))
        elif isinstance(topology, adj_list):
            pairs = np.ascontiguousarray(np.asarray(topology.edges, dtype=np.int32).reshape(-1, 2))
            _check(lib().spice_connect_adj_list(self._h, source.id, target.id, pairs.ctypes.data, len(pairs),
                                                delay, getattr(syn, "model", SYNAPSE_FIXED_WEIGHT), arr, len(prm),
                                                C.byref(out)))
        else:
            raise TypeError("topology must be fixed_probability or adj_list")
        self._conns.append((source, target, topology, delay, syn))
        return out.value

    def set_mode(self, mode: int):
        _check(lib().spice_set_mode(self._h, mode))

    def set_window(self, w: int):
        _check(lib().spice_set_window(self._h, w))

    def set_tuning(self, tile_bytes: int | None = None, deliver_threads: int | None = None,
                   deliver_parts: int | None = None, deliver_algo: int | None = None,
                   overlap_sources: bool | None = None, neuron_variant: int | None = None,
                   launch_mode: int | None = None, pull: bool | None = None, source_steps: int | None = None,
                   persistent: bool | None = None):
        """Delivery launch shape and neuron-update variant (any time between steps); results are
        independent of them.  pull (before the network first steps): deliver every stateful
        population by the pull path over the CSC adjacency (SPICE_TUNE_PULL)."""
        if pull is not None:
            _check(lib().spice_set_tuning(self._h, 8, int(bool(pull))))
        if persistent is not None:  # one cooperative launch per chunk of one-step windows (SPICE_TUNE_PERSISTENT;
            # an int >= 2: CTAs per SM)
            _check(lib().spice_set_tuning(self._h, 10, int(persistent)))
        if source_steps is not None:  # steps per Poisson source CTA (default 1; 0: one-wave grid)
            _check(lib().spice_set_tuning(self._h, 9, int(source_steps)))
        if tile_bytes is not None:
            _check(lib().spice_set_tuning(self._h, 0, int(tile_bytes)))
        if deliver_threads is not None:
            _check(lib().spice_set_tuning(self._h, 1, int(deliver_threads)))
        if deliver_parts is not None:
            _check(lib().spice_set_tuning(self._h, 2, int(deliver_parts)))
        if deliver_algo is not None:
            _check(lib().spice_set_tuning(self._h, 3, int(deliver_algo)))
        if overlap_sources is not None:
            _check(lib().spice_set_tuning(self._h, 4, int(bool(overlap_sources))))
        if neuron_variant is not None:
            _check(lib().spice_set_tuning(self._h, 6, int(neuron_variant)))
        if launch_mode is not None:
            _check(lib().spice_set_tuning(self._h, 7, int(launch_mode)))

    _TUNING_KNOBS = {"tile_bytes": 0, "deliver_threads": 1, "deliver_parts": 2, "deliver_algo": 3,
                     "overlap_sources": 4, "neuron_variant": 6, "launch_mode": 7, "pull": 8, "source_steps": 9,
                     "persistent": 10}

    def get_tuning(self) -> dict:
        """Every knob's current value (spice_get_tuning): the caller's settings, and once the network
        is prepared (its first step) the launch shape picked from its sizes for the others."""
        out = {}
        for name, knob in self._TUNING_KNOBS.items():
            v = C.c_int64()
            _check(lib().spice_get_tuning(self._h, knob, C.byref(v)))
            out[name] = v.value
        return out

    # stepping
    def step(self):
        _check(lib().spice_step(self._h))

    def run(self, steps: int):
        _check(lib().spice_run(self._h, int(steps)))

    def run_record(self, steps: int, capacity: int | None = None):
        """Runs `steps` steps and returns the raster: list over steps of lists over populations."""
        npop = len(self._pops)
        counts = np.zeros((max(1, steps), max(1, npop)), dtype=np.int64)
        if capacity is None:
            capacity = max(1024, steps * sum(p.size() for p in self._pops) // 50)
        while True:
            buf = np.zeros(max(1, capacity), dtype=np.int32)
            total = C.c_int64()
            rc = lib().spice_run_record(self._h, int(steps), counts.ctypes.data, buf.ctypes.data, capacity,
                                        C.byref(total))
            if rc == EOVERFLOW:
                # the steps ran; the raster did not fit -- the caller asked for too little room
                raise SpiceError(rc, f"raster needs {total.value} entries (capacity {capacity})")
            _check(rc)
            break
        out, pos = [], 0
        for t in range(steps):
            row = []
            for k in range(npop):
                c = int(counts[t, k])
                row.append(buf[pos:pos + c].copy())
                pos += c
            out.append(row)
        return out

    @property
    def time(self) -> int:
        v = C.c_int64()
        _check(lib().spice_time(self._h, C.byref(v)))
        return v.value

    @property
    def events(self) -> int:
        v = C.c_uint64()
        _check(lib().spice_events(self._h, C.byref(v)))
        return v.value

    # readback
    def spikes(self, pop: Population | int, age: int = 0) -> np.ndarray:
        pid = pop.id if isinstance(pop, Population) else int(pop)
        n = C.c_int64()
        _check(lib().spice_spike_count(self._h, pid, int(age), C.byref(n)))
        out = np.zeros(max(1, n.value), dtype=np.int32)
        _check(lib().spice_spikes(self._h, pid, int(age), out.ctypes.data, len(out), C.byref(n)))
        return out[:n.value]

    def get_state(self, pop: Population, fld: int) -> np.ndarray:
        out = np.zeros(pop.size(), dtype=np.int32 if fld == FIELD_TREF else np.float32)
        _check(lib().spice_get_state(self._h, pop.id, fld, out.ctypes.data))
        return out

    def set_state(self, pop: Population, fld: int, values):
        v = np.ascontiguousarray(values, dtype=np.int32 if fld == FIELD_TREF else np.float32)
        if v.size != pop.size():
            raise LogicError(EINVAL, "state array must have one entry per neuron")
        _check(lib().spice_set_state(self._h, pop.id, fld, v.ctypes.data))

    def synapses(self, conn: int) -> int:
        src, syn = C.c_int64(), C.c_int64()
        _check(lib().spice_conn_size(self._h, conn, C.byref(src), C.byref(syn)))
        return syn.value

    def synapse_state(self, conn: int, field: int = 0) -> np.ndarray:
        """Per-synapse state of a plastic connection (CSR order): 0 W / count, 1 x_pre, 2 x_post."""
        m = self.synapses(conn)
        out = np.zeros(max(1, m), dtype=np.float32)
        _check(lib().spice_get_synapse_state(self._h, conn, field, out.ctypes.data))
        return out[:m]

    def csr(self, conn: int):
        src, syn = C.c_int64(), C.c_int64()
        _check(lib().spice_conn_size(self._h, conn, C.byref(src), C.byref(syn)))
        off = np.zeros(src.value + 1, dtype=np.int64)
        nb = np.zeros(max(1, syn.value), dtype=np.int32)
        _check(lib().spice_get_csr(self._h, conn, off.ctypes.data, nb.ctypes.data))
        return off, nb[:syn.value]

    def csc(self, conn: int):
        """The transposed adjacency: column starts (dst_size + 1) and the sources of each target's
        synapses, ascending within a column."""
        src, syn = C.c_int64(), C.c_int64()
        _check(lib().spice_conn_size(self._h, conn, C.byref(src), C.byref(syn)))
        dst = self._conns[conn][1].size()
        off = np.zeros(dst + 1, dtype=np.int64)
        nb = np.zeros(max(1, syn.value), dtype=np.int32)
        _check(lib().spice_get_csc(self._h, conn, off.ctypes.data, nb.ctypes.data))
        return off, nb[:syn.value]

    def synapse_weights(self, conn: int) -> np.ndarray:
        """Per-synapse weights of a weighted connection, CSR order."""
        return self.synapse_state(conn, 0)

    # profiling
    def set_profiling(self, on: bool):
        _check(lib().spice_set_profiling(self._h, 1 if on else 0))

    def kernel_stats(self, kind: int):
        n, ms = C.c_int64(), C.c_double()
        _check(lib().spice_kernel_stats(self._h, kind, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def kernel_span(self, kind: int):
        """Neuron-update (kind 0) or delivery (kind 1) launches since profiling was switched on:
        (launches with a span, summed ms from the first CTA's start to the last CTA's end on the
        device timer)."""
        n, ms = C.c_int64(), C.c_double()
        _check(lib().spice_kernel_span(self._h, kind, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def launch_count(self) -> int:
        v = C.c_int64()
        _check(lib().spice_launch_count(self._h, C.byref(v)))
        return v.value

    def synchronize(self):
        _check(lib().spice_synchronize(self._h))

    def stream_handle(self) -> int:
        """The raw cudaStream_t of the net (e.g. for torch.cuda.ExternalStream)."""
        v = C.c_void_p()
        _check(lib().spice_get_stream(self._h, C.byref(v)))
        return v.value or 0


def brunel(N: int, p: float, seed: int = 1337, dt: float = 1e-4, delay: float = 15e-4, mode: int = MODE_DETERMINISTIC):
    """The Brunel network of samples/brunel.cpp:75-103 (P = N/2 Poisson, E = 0.4 N and I = 0.1 N
    LIF, six fixed_probability(p) projections) with weights scaled by 0.1/p so the mean input is
    the same at any p.  Returns (net, (P, E, I))."""
    net = snn(dt, delay, [seed])
    net.set_mode(mode)
    P = net.add_population(poisson(20.0), N // 2)
    E = net.add_population(lif(), N * 4 // 10)
    I = net.add_population(lif(), N // 10)
    we = float(np.float32((2.0 / N) * (0.1 / p)))
    wi = float(np.float32((-10.0 / N) * (0.1 / p)))
    for s, d, w in ((P, E, we), (P, I, we), (E, E, we), (E, I, we), (I, E, wi), (I, I, wi)):
        net.connect(s, d, fixed_probability(p), delay, fixed_weight(w))
    return net, (P, E, I)


class batch:
    """Many independent nets stepped together (spice_batch_* in include/spice_gb300.h): one launch
    per kernel kind and window covers every member, and full windows replay as a CUDA graph.  The
    members keep working as ordinary nets between runs, and each member's results are identical to
    running it alone.  No counterpart in the reference."""

    def __init__(self, nets: Sequence[snn]):
        self._nets = list(nets)
        arr = (C.c_void_p * max(1, len(self._nets)))(*[n._h for n in self._nets])
        h = C.c_void_p()
        _check(lib().spice_batch_create(arr, len(self._nets), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().spice_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nets(self) -> list:
        return list(self._nets)

    def run(self, steps: int):
        _check(lib().spice_batch_run(self._h, int(steps)))

    def set_tuning(self, tile_bytes: int | None = None, deliver_threads: int | None = None,
                   deliver_parts: int | None = None, deliver_algo: int | None = None,
                   overlap_sources: bool | None = None, graph_windows: int | None = None):
        """Launch shape of the batch (and of its members); results are independent of it."""
        for knob, v in ((0, tile_bytes), (1, deliver_threads), (2, deliver_parts), (3, deliver_algo),
                        (4, None if overlap_sources is None else int(bool(overlap_sources))), (5, graph_windows)):
            if v is not None:
                _check(lib().spice_batch_set_tuning(self._h, knob, int(v)))

    def set_profiling(self, on: bool):
        _check(lib().spice_batch_set_profiling(self._h, 1 if on else 0))

    def kernel_stats(self, kind: int):
        n, ms = C.c_int64(), C.c_double()
        _check(lib().spice_batch_kernel_stats(self._h, kind, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def launch_count(self) -> int:
        v = C.c_int64()
        _check(lib().spice_batch_launch_count(self._h, C.byref(v)))
        return v.value

    def synchronize(self):
        """spice_batch_run returns when its steps are done; kept for the tuner's interface."""

    def stream_handle(self) -> int:
        v = C.c_void_p()
        _check(lib().spice_batch_get_stream(self._h, C.byref(v)))
        return v.value or 0

    @property
    def events(self) -> int:
        return sum(n.events for n in self._nets)


def brunel_sweep_sizes(count: int = 256, n_min: int = 5000, n_max: int = 80000, seed: int = 4):
    """Network sizes of the batched Brunel sweep: `count` sizes drawn log-uniformly from
    [n_min, n_max] with a seeded numpy generator, rounded to multiples of 10 (so the 5:4:1
    P/E/I split is exact)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count))
    return [int(round(x / 10.0)) * 10 for x in n]


def brunel_sweep(sizes: Sequence[int], seed0: int = 1000, mode: int = MODE_DETERMINISTIC):
    """One Brunel net per size with p = 0.1 * min(1, 2e4 / N) (weights scaled by 0.1/p) and seed
    seed0 + i.  Returns a list of (net, (P, E, I))."""
    return [brunel(int(N), 0.1 * min(1.0, 20000.0 / N), seed0 + i, mode=mode) for i, N in enumerate(sizes)]


def selftest_skip_rounding(count: int = 1 << 26, seed: int = 1):
    """Runs the device self-test of the plastic trace decay's rounding (integer arithmetic against
    the double multiply) on `count` random pairs; returns (mismatches, first_a_bits, first_f)."""
    m, a, f = C.c_int64(), C.c_uint32(), C.c_double()
    _check(lib().spice_selftest_skip_rounding(int(count), int(seed), C.byref(m), C.byref(a), C.byref(f)))
    return m.value, a.value, f.value


__all__ = ["snn", "Population", "poisson", "lif", "lif_cond", "external_input", "fixed_weight", "weighted", "excitatory",
           "inhibitory", "istdp", "count_synapse", "fixed_probability", "adj_list", "brunel", "batch", "brunel_sweep", "brunel_sweep_sizes",
           "SpiceError", "LogicError", "CudaError", "MODE_DETERMINISTIC", "MODE_ATOMIC", "lib",
           "selftest_skip_rounding"]
