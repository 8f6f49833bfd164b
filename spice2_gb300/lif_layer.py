"""Differentiable recurrent LIF layer on the GPU: the hand-written forward and adjoint kernels of
spice_lif_* (include/spice_gb300.h) wrapped in a torch.autograd.Function.  No counterpart in the
reference (its plasticity is local and online; this is gradient-based training of the same kind of
network).

    layer = RecurrentLIF(n_in=700, n_rec=1024, p_in=0.2, p_rec=0.1, seed=1)
    x_bits = poisson_input(batch=64, steps=200, n_in=700, seed=2)
    counts = layer(x_bits, steps=200)                 # [64, 1024] spike counts
    loss = ((counts[:, :128] - target) ** 2).mean()
    loss.backward()                                   # adjoint kernel, checkpoint every 20 steps

Connectivity is the engine's fixed_probability adjacency (the reference's generator, bit for bit),
weights are drawn from N(0, 1/sqrt(fan_in)) with fan_in = p * n_src, theta = 1 and
beta = exp(-dt / tau_m).  The model, its surrogate gradient and the relaxed forward used for
finite-difference checks are described at spice_lif_layer in include/spice_gb300.h.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _check, fixed_probability, fixed_weight, lib, lif, poisson, snn


def connectivity(n_in: int, n_rec: int, p_in: float, p_rec: float, seed: int):
    """CSR (offsets int64, neighbours int32) of input->recurrent and recurrent->recurrent
    fixed_probability projections, generated by the engine with the reference's seed order."""
    net = snn(1e-3, 1e-3, [seed])
    X = net.add_population(poisson(0.0), n_in)
    R = net.add_population(lif(), n_rec)
    ci = net.connect(X, R, fixed_probability(p_in), 1e-3, fixed_weight(0.0))
    cr = net.connect(R, R, fixed_probability(p_rec), 1e-3, fixed_weight(0.0))
    out = net.csr(ci), net.csr(cr)
    net.close()
    return out


def pack_bits(x: torch.Tensor) -> torch.Tensor:
    """[..., n] bool -> [..., ceil(n/32)] int32 words, bit k of word k // 32 = element k."""
    n = x.shape[-1]
    nw = (n + 31) // 32
    pad = torch.zeros(*x.shape[:-1], nw * 32 - n, dtype=torch.bool, device=x.device)
    xb = torch.cat([x, pad], dim=-1).reshape(*x.shape[:-1], nw, 32).to(torch.int64)
    w = (xb << torch.arange(32, device=x.device, dtype=torch.int64)).sum(-1)
    w = torch.where(w >= 2 ** 31, w - 2 ** 32, w)
    return w.to(torch.int32).contiguous()


def poisson_input(batch: int, steps: int, n_in: int, rate_max: float = 50.0, dt: float = 1e-3, seed: int = 0,
                  device: str = "cuda", return_dense: bool = False):
    """Poisson input spikes: per (sample, input) a rate uniform in [0, rate_max) Hz, then
    x_t = (uniform < rate * dt) for each step.  Returns the packed bits (and the bool array)."""
    g = torch.Generator(device=device).manual_seed(seed)
    rates = torch.rand(batch, 1, n_in, generator=g, device=device) * rate_max
    x = torch.rand(batch, steps, n_in, generator=g, device=device) < rates * dt
    bits = pack_bits(x)
    return (bits, x) if return_dense else bits


class _Layer:
    """Owns the C-ABI handle (device copy of the connectivity, scratch)."""

    def __init__(self, n_in, n_rec, in_csr, rec_csr):
        self.n_in, self.n = n_in, n_rec
        io, inb = [np.ascontiguousarray(a) for a in in_csr]
        ro, rnb = [np.ascontiguousarray(a) for a in rec_csr]
        h = C.c_void_p()
        _check(lib().spice_lif_layer_create(n_in, n_rec, io.ctypes.data, inb.ctypes.data, ro.ctypes.data,
                                            rnb.ctypes.data, C.byref(h)))
        self.h = h
        self.in_syn, self.rec_syn = int(io[-1]), int(ro[-1])

    def __del__(self):
        try:
            if self.h:
                lib().spice_lif_layer_destroy(self.h)
                self.h = None
        except Exception:
            pass


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev_f32(t: torch.Tensor) -> torch.Tensor:
    if not t.is_cuda or t.dtype != torch.float32:
        raise TypeError("LIF layer tensors must be float32 CUDA tensors")
    return t.contiguous()


class _LIFFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w_in, w_rec, theta, beta, layer: _Layer, x_bits, steps: int, ck: int, relaxed: bool,
                slope: float):
        B = x_bits.shape[0]
        n = layer.n
        dev = w_rec.device
        w_in, w_rec, theta, beta = (_dev_f32(t) for t in (w_in, w_rec, theta, beta))
        x_bits = x_bits.contiguous()
        nck = (steps + ck - 1) // ck + 1
        counts = torch.empty(B, n, device=dev, dtype=torch.float32)
        spikes = torch.empty(B, steps, n, device=dev, dtype=torch.float32)
        vck = torch.empty(B, nck, n, device=dev, dtype=torch.float32)
        _check(lib().spice_lif_forward(layer.h, B, steps, ck, int(relaxed), float(slope), _ptr(x_bits), _ptr(w_in),
                                       _ptr(w_rec), _ptr(theta), _ptr(beta), _ptr(counts), _ptr(spikes), _ptr(vck),
                                       _stream()))
        ctx.save_for_backward(w_in, w_rec, theta, beta, x_bits, spikes, vck)
        ctx.cfg = (layer, steps, ck, relaxed, slope)
        ctx.mark_non_differentiable(spikes)
        return counts, spikes

    @staticmethod
    def backward(ctx, g_counts, _g_spikes):
        w_in, w_rec, theta, beta, x_bits, spikes, vck = ctx.saved_tensors
        layer, steps, ck, relaxed, slope = ctx.cfg
        B = x_bits.shape[0]
        g_counts = g_counts.contiguous().to(torch.float32)
        gw_in = torch.empty_like(w_in)
        gw_rec = torch.empty_like(w_rec)
        gth = torch.empty_like(theta)
        gbe = torch.empty_like(beta)
        _check(lib().spice_lif_backward(layer.h, B, steps, ck, int(relaxed), float(slope), _ptr(x_bits), _ptr(w_in),
                                        _ptr(w_rec), _ptr(theta), _ptr(beta), _ptr(spikes), _ptr(vck),
                                        _ptr(g_counts), _ptr(gw_in), _ptr(gw_rec), _ptr(gth), _ptr(gbe), _stream()))
        return gw_in, gw_rec, gth, gbe, None, None, None, None, None, None


class RecurrentLIF(torch.nn.Module):
    """n_in Poisson-driven inputs -> n_rec recurrent LIF neurons (tau_m, threshold, reset by
    subtraction, delay 1 step), trained through the adjoint kernel."""

    def __init__(self, n_in: int = 700, n_rec: int = 1024, p_in: float = 0.2, p_rec: float = 0.1, seed: int = 1,
                 dt: float = 1e-3, tau_m: float = 20e-3, threshold: float = 1.0, slope: float = 25.0,
                 checkpoint_every: int = 20, device: str = "cuda"):
        super().__init__()
        in_csr, rec_csr = connectivity(n_in, n_rec, p_in, p_rec, seed)
        self.in_csr, self.rec_csr = in_csr, rec_csr
        self._layer = _Layer(n_in, n_rec, in_csr, rec_csr)
        g = torch.Generator(device=device).manual_seed(seed)
        s_in = 1.0 / math.sqrt(max(p_in * n_in, 1e-12))
        s_rec = 1.0 / math.sqrt(max(p_rec * n_rec, 1e-12))
        self.w_in = torch.nn.Parameter(torch.randn(self._layer.in_syn, generator=g, device=device) * s_in)
        self.w_rec = torch.nn.Parameter(torch.randn(self._layer.rec_syn, generator=g, device=device) * s_rec)
        self.theta = torch.nn.Parameter(torch.full((n_rec,), float(threshold), device=device))
        self.beta = torch.nn.Parameter(torch.full((n_rec,), math.exp(-dt / tau_m), device=device))
        self.n_in, self.n_rec = n_in, n_rec
        self.slope, self.checkpoint_every = slope, checkpoint_every

    def forward(self, x_bits: torch.Tensor, steps: int, relaxed: bool = False, return_spikes: bool = False):
        counts, spikes = _LIFFunction.apply(self.w_in, self.w_rec, self.theta, self.beta, self._layer, x_bits,
                                            int(steps), int(self.checkpoint_every), bool(relaxed), float(self.slope))
        return (counts, spikes) if return_spikes else counts


def count_loss(counts: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """MSE between the spike counts of the first target.shape[1] neurons and the target counts."""
    return ((counts[:, :target.shape[1]] - target) ** 2).mean()


def count_targets(batch: int, n_out: int = 128, high: float = 20.0, seed: int = 3, device: str = "cuda"):
    """Seeded target counts uniform in [0, high) for the first n_out neurons of each sample."""
    g = torch.Generator(device=device).manual_seed(seed)
    return torch.rand(batch, n_out, generator=g, device=device) * high


def time_step(batch: int = 64, steps: int = 200, n_in: int = 700, n_rec: int = 1024, reps: int = 10, seed: int = 1):
    """Median CUDA-event times (ms) of one forward and one backward (adjoint) call of the layer on
    the C5-sized problem, with the MSE count loss."""
    layer = RecurrentLIF(n_in=n_in, n_rec=n_rec, seed=seed)
    x_bits = poisson_input(batch, steps, n_in, seed=seed + 1)
    target = count_targets(batch)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fw, bw = [], []
    for r in range(reps + 3):
        layer.zero_grad()
        ev[0].record()
        counts = layer(x_bits, steps)
        ev[1].record()
        count_loss(counts, target).backward()
        ev[2].record()
        torch.cuda.synchronize()
        if r >= 3:
            fw.append(ev[0].elapsed_time(ev[1]))
            bw.append(ev[1].elapsed_time(ev[2]))
    fw.sort()
    bw.sort()
    return {"forward_ms": fw[len(fw) // 2], "backward_ms": bw[len(bw) // 2],
            "backward_over_forward": bw[len(bw) // 2] / fw[len(fw) // 2],
            "rate_hz": float(counts.detach().mean()) / (steps * 1e-3)}


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time the recurrent LIF layer's forward and adjoint kernels")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args()
    print(json.dumps(time_step(args.batch, args.steps, reps=args.reps)))
