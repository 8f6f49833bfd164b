"""CPU test of the autotuner's host logic with a stand-in network: it times every candidate with
the sources serialised, applies the fastest delivery shape, then the fastest neuron-window variant,
and restores overlapped sources."""
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)


class FakeNet:
    def __init__(self, deliver_us, neuron_us):
        self.deliver_us, self.neuron_us = deliver_us, neuron_us
        self.shape, self.variant, self.overlap, self.calls = None, 0, True, []
        self.profiling = False

    def set_tuning(self, tile_bytes=None, deliver_threads=None, deliver_parts=None, deliver_algo=None,
                   overlap_sources=None, neuron_variant=None, launch_mode=None):
        if tile_bytes is not None:
            self.shape = (tile_bytes, deliver_threads, deliver_parts, deliver_algo)
        if overlap_sources is not None:
            self.overlap = overlap_sources
        if neuron_variant is not None:
            self.variant = neuron_variant
        self.calls.append((self.shape, self.variant, self.overlap))

    def run(self, n):
        pass

    def synchronize(self):
        pass

    def set_profiling(self, on):
        self.profiling = on

    def kernel_stats(self, kind):
        assert self.profiling
        if kind == 1:
            return 10, 10 * self.deliver_us(self.shape, self.overlap) / 1e3
        return 10, 10 * self.neuron_us(self.variant) / 1e3


def test_autotune_applies_the_fastest_shape_and_variant():
    from spice2_gb300 import autotune as at
    cands = [(4096, 64, 1, 1), (8192, 128, 1, 5), (16384, 256, 2, 8)]
    seen_overlap = []

    def deliver_us(shape, overlap):
        seen_overlap.append(overlap)
        return {cands[0]: 30.0, cands[1]: 12.0, cands[2]: 20.0}[shape]

    net = FakeNet(deliver_us, lambda v: {0: 9.0, 1: 8.0, 2: 7.0, 3: 9.5, 4: 6.5, 5: 6.9, 6: 6.6, 7: 6.7, 8: 6.8, 9: 6.55}[v])
    rep = at.autotune(net, steps=5, warm=1, candidates=cands)
    best = rep["best"]
    assert (best["tile_bytes"], best["threads"], best["parts"], best["algo"]) == cands[1]
    assert best["neuron_variant"] == 4 and abs(best["neuron_us"] - 6.5) < 1e-9
    assert net.shape == cands[1] and net.variant == 4 and net.overlap is True
    assert seen_overlap and not any(seen_overlap)  # deliveries timed with the sources serialised
    assert len(rep["results"]) == len(cands)
