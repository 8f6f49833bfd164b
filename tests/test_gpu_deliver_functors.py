"""GPU: synapses whose deliver() is user code (spice2_gb300/examples/deliver_functors.cu, compiled with
nvcc here): deliver() that reads the source neuron (the reference's DeliverFromTo concept), sets a
flag or takes a maximum.  Each case is replayed here in the reference's delivery order
(snn.cpp:7-28: all populations update, then each connection in connect order delivers the spikes of
`delay - 1` steps ago, sources ascending, each along its CSR row -- synapse_population.h:88-139 --
reading the source neurons as they are after this step's update)."""
import heapq
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def functors(engine, tmp_path_factory):
    exe = tmp_path_factory.mktemp("df") / "deliver_functors"
    libdir = os.path.join(ROOT, "spice2_gb300")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++20", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "spice2_gb300", "examples", "deliver_functors.cu"),
                    "-L", libdir, "-lspice_gb300", f"-Xlinker=-rpath={libdir}", "-o", str(exe)], check=True)

    def run(*args):
        out = subprocess.run([str(exe)] + [str(a) for a in args], check=True, capture_output=True, text=True).stdout
        return json.loads(out)
    return run


def _edge_weight(s, d):
    return 1 + (s * 7919 + d * 104729) % 9


def _dijkstra(V, off, nb, w, src):
    dist = [None] * V
    heap = [(0, src)]
    while heap:
        d, u = heapq.heappop(heap)
        if dist[u] is not None:
            continue
        dist[u] = d
        for e in range(off[u], off[u + 1]):
            if dist[nb[e]] is None:
                heapq.heappush(heap, (d + w[e], nb[e]))
    return [-1 if d is None else d for d in dist]


@pytest.mark.parametrize("V,E,src,steps,seed", [(7, 0, 0, 6, 1), (2000, 9000, 3, 80, 5), (5000, 12000, 17, 40, 9)])
def test_shortest_paths_in_the_reference_order(functors, V, E, src, steps, seed):
    got = functors("sssp", V, E, src, steps, seed)
    off, nb, w = got["csr"]["off"], got["csr"]["nb"], got["w"]
    # the CSR of an adj_list holds each source's targets ascending (topology.cpp:65-71)
    for s in range(V):
        row = nb[off[s]:off[s + 1]]
        assert row == sorted(row)
        assert all(w[e] == _edge_weight(s, nb[e]) for e in range(off[s], off[s + 1]))
    INF = -1
    dist, prev, fire = [INF] * V, [-1] * V, [False] * V
    dist[src], prev[src], fire[src] = 0, src, True
    for t in range(steps):
        spikes = [i for i in range(V) if fire[i]]
        for i in spikes:
            fire[i] = False
        assert got["raster"][t] == spikes, t
        for s in spikes:  # one population: a later source reads what an earlier delivery wrote
            for e in range(off[s], off[s + 1]):
                d = nb[e]
                if dist[s] != INF and (dist[d] == INF or dist[s] + w[e] < dist[d]):
                    dist[d], prev[d], fire[d] = dist[s] + w[e], s, True
    assert got["distance"] == dist
    assert got["previous"] == prev
    assert got["fire"] == [int(f) for f in fire]
    if not any(fire):  # converged: the shortest paths
        assert dist == _dijkstra(V, off, nb, w, src)
    if E > 0:
        assert sum(d >= 0 for d in dist) > V // 2


def test_ping_pong_alternates(functors):
    got = functors("pingpong", 10000, 10)["counts"]
    assert got == [[5000, 0] if t % 2 == 0 else [0, 5000] for t in range(10)]


@pytest.mark.parametrize("NA,NB,p,steps,seed", [(400, 300, 0.05, 200, 3), (3000, 2000, 0.01, 120, 11)])
def test_relay_reads_the_source_state(functors, NA, NB, p, steps, seed):
    got = functors("relay", NA, NB, p, steps, seed)
    f32 = np.float32
    level = np.array(got["level0"], dtype=f32)
    ids = np.arange(NA)
    off0, nb0 = got["csr0"]["off"], np.array(got["csr0"]["nb"])
    off1, nb1 = got["csr1"]["off"], np.array(got["csr1"]["nb"])
    w = np.array(got["w"], dtype=f32)
    assert len(w) == len(nb0) and np.all((w >= 0) & (w < 1)) and len(np.unique(w)) > len(w) // 2
    src0 = np.repeat(np.arange(NA), np.diff(off0))
    src1 = np.repeat(np.arange(NA), np.diff(off1))
    slots0, slots1 = _columns(src0, nb0, NB), _columns(src1, nb1, NB)
    sums = np.zeros(NB, dtype=f32)
    peak = np.zeros(NB, dtype=f32)
    hits = np.zeros(NB, dtype=np.int64)
    maxsrc = np.full(NB, -1)
    history = []
    rows = np.arange(NB)
    for t in range(steps):
        level = (level + f32(0.25)).astype(f32)
        history.append((ids + t + 1) % 7 == 0)
        if t < 2:
            continue
        fired = history[t - 2]
        for r in range(slots0.shape[1]):  # each target's r-th synapse in ascending source order
            e = slots0[:, r]
            on = (e >= 0) & fired[src0[np.maximum(e, 0)]]
            j, e = rows[on], e[on]
            sums[j] = (sums[j] + (w[e] * level[src0[e]]).astype(f32)).astype(f32)
            hits[j] += 1
            maxsrc[j] = np.maximum(maxsrc[j], src0[e])
        for r in range(slots1.shape[1]):
            e = slots1[:, r]
            on = (e >= 0) & fired[src1[np.maximum(e, 0)]]
            j, e = rows[on], e[on]
            peak[j] = np.maximum(peak[j], level[src1[e]])
    assert np.array_equal(np.array(got["level"], dtype=f32), level)
    assert np.array_equal(np.array(got["hits"]), hits)
    assert np.array_equal(np.array(got["maxsrc"]), maxsrc)
    assert np.array_equal(np.array(got["sum"], dtype=f32).view(np.uint32), sums.view(np.uint32))
    assert np.array_equal(np.array(got["peak"], dtype=f32), peak)
    assert hits.sum() > 1000


def _columns(src, nb, ndst):
    """[ndst, max in-degree] synapse indices, each row one target's synapses in ascending source
    (then CSR) order, padded with -1."""
    e = np.arange(len(nb))
    order = np.lexsort((e, src, nb))
    deg = np.bincount(nb, minlength=ndst)
    out = np.full((ndst, max(int(deg.max(initial=0)), 1)), -1, dtype=np.int64)
    start = np.concatenate([[0], np.cumsum(deg)[:-1]])
    rank = np.arange(len(nb)) - np.repeat(start, deg)
    out[nb[order], rank] = order
    return out
