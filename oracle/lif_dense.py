"""Dense FP64 PyTorch reference of the differentiable recurrent LIF layer (spice_lif_* of
include/spice_gb300.h) -- test infrastructure, the oracle of the adjoint kernels.  Not part of the
product: only tests import it.

The reference has no such model (its plasticity is local); the layer's semantics are the ones
documented at spice_lif_layer_create.  This module restates them with dense masked weight
matrices and lets torch.autograd differentiate:
  u_t = beta * v_{t-1} + x_{t-1} @ W_in + s_{t-1} @ W_rec
  s_t = H(u_t - theta) with the fast-sigmoid surrogate 1/(1 + k|x|)^2 as its derivative, or the
        relaxed g(x) = (1 + kx/(1+k|x|))/2 differentiated exactly
  v_t = u_t - theta * s_t,   counts = sum_t s_t
`forced_spikes` replaces the threshold decision of the spiking forward by a given raster (the
kernel's), so that a float64 rerun compares gradients along the same spike train: a float32 and a
float64 forward can disagree about a membrane potential within rounding of the threshold.
"""
from __future__ import annotations

import torch


def dense(off, nb, w, n_src: int, n_dst: int, dtype=torch.float64, device="cpu"):
    """Scatter per-synapse values (CSR order) into a dense [n_src, n_dst] matrix."""
    off = torch.as_tensor(off, device=device)
    nb = torch.as_tensor(nb, device=device).long()
    rows = torch.repeat_interleave(torch.arange(n_src, device=device), off[1:] - off[:-1])
    W = torch.zeros(n_src, n_dst, dtype=dtype, device=device)
    W[rows, nb] = w.to(dtype)
    return W, rows, nb


class _Spike(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, forced, slope):
        ctx.save_for_backward(x)
        ctx.slope = slope
        return forced.clone() if forced is not None else (x > 0).to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        return g / (1.0 + ctx.slope * x.abs()) ** 2, None, None


def run(in_csr, rec_csr, w_in, w_rec, theta, beta, x, steps: int, slope: float = 25.0, relaxed: bool = False,
        forced_spikes=None, grad_counts=None, dtype=torch.float64):
    """Forward (and, with grad_counts, backward of L = sum(counts * grad_counts)).
    x: [B, T, n_in] {0,1}.  Returns dict(counts, spikes, u, grads per synapse / neuron)."""
    dev = w_rec.device
    n_in = len(in_csr[0]) - 1
    n = len(rec_csr[0]) - 1
    B = x.shape[0]
    Win, ri, ci = dense(in_csr[0], in_csr[1], w_in.detach(), n_in, n, dtype, dev)
    Wrec, rr, cr = dense(rec_csr[0], rec_csr[1], w_rec.detach(), n, n, dtype, dev)
    th = theta.detach().to(dtype).clone()
    be = beta.detach().to(dtype).clone()
    for t in (Win, Wrec, th, be):
        t.requires_grad_(True)
    xd = x.to(dtype)
    v = torch.zeros(B, n, dtype=dtype, device=dev)
    s = torch.zeros(B, n, dtype=dtype, device=dev)
    counts = torch.zeros(B, n, dtype=dtype, device=dev)
    us, ss = [], []
    k = float(slope)
    for t in range(1, steps + 1):
        u = be * v + xd[:, t - 1] @ Win + s @ Wrec
        xm = u - th
        if relaxed:
            s = 0.5 * (1.0 + k * xm / (1.0 + k * xm.abs()))
        else:
            forced = None if forced_spikes is None else forced_spikes[:, t - 1].to(dtype)
            s = _Spike.apply(xm, forced, k)
        v = u - th * s
        counts = counts + s
        us.append(u.detach())
        ss.append(s.detach())
    out = {"counts": counts.detach(), "u": torch.stack(us, 1), "spikes": torch.stack(ss, 1)}
    if grad_counts is not None:
        L = (counts * grad_counts.to(dtype)).sum()
        L.backward()
        out["loss"] = float(L.detach())
        out["g_w_in"] = Win.grad[ri, ci]
        out["g_w_rec"] = Wrec.grad[rr, cr]
        out["g_theta"] = th.grad
        out["g_beta"] = be.grad
    return out


def loss_value(in_csr, rec_csr, w_in, w_rec, theta, beta, x, steps, slope, grad_counts):
    """L = sum(counts * grad_counts) of the relaxed forward, in float64 (for finite differences)."""
    with torch.no_grad():
        r = run(in_csr, rec_csr, w_in, w_rec, theta, beta, x, steps, slope, relaxed=True)
    return float((r["counts"] * grad_counts.to(torch.float64)).sum())
