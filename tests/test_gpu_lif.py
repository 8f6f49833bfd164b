"""Differentiable recurrent LIF layer: the adjoint kernels against a dense float64 PyTorch autograd
reference (oracle/lif_dense.py) and against central finite differences of the relaxed forward.
Relative error = max |g - g_ref| / max |g_ref| per parameter tensor."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-3  # relative error bound of the adjoint gradients against float64


def _rel(g, ref):
    g, ref = g.detach().double(), ref.detach().double()
    return float((g - ref).abs().max() / ref.abs().max().clamp_min(1e-300))


def _setup(B, T, seed=1, ck=20):
    from spice2_gb300.lif_layer import RecurrentLIF, poisson_input
    layer = RecurrentLIF(seed=seed, checkpoint_every=ck)
    x_bits, x = poisson_input(B, T, 700, seed=seed + 10, return_dense=True)
    g = torch.Generator(device="cuda").manual_seed(seed + 20)
    G = torch.randn(B, 1024, generator=g, device="cuda") * 0.01
    return layer, x_bits, x, G


def _grads(layer, x_bits, T, G, relaxed=False):
    layer.zero_grad()
    counts, spikes = layer(x_bits, T, relaxed=relaxed, return_spikes=True)
    counts.backward(G)
    return counts, spikes, {k: getattr(layer, k).grad.clone() for k in ("w_in", "w_rec", "theta", "beta")}


def _reference(layer, x, T, G, relaxed=False, forced=None):
    from oracle import lif_dense
    return lif_dense.run(layer.in_csr, layer.rec_csr, layer.w_in, layer.w_rec, layer.theta, layer.beta, x, T,
                         slope=layer.slope, relaxed=relaxed, forced_spikes=forced, grad_counts=G)


def _check_against_reference(layer, x_bits, x, T, G, relaxed):
    counts, spikes, g = _grads(layer, x_bits, T, G, relaxed)
    ref = _reference(layer, x, T, G, relaxed=relaxed, forced=None if relaxed else spikes)
    errs = {k: _rel(g[k], ref["g_" + k]) for k in g}
    assert all(e < TOL for e in errs.values()), errs
    if not relaxed:
        # the float64 rerun's own threshold decisions agree with the kernel's spikes
        own = (ref["u"] - layer.theta.detach().double() > 0).to(torch.float32)
        mismatch = float((own != spikes).float().mean())
        assert mismatch < 1e-4, mismatch
        assert torch.equal(counts, spikes.sum(1))
        assert float(spikes.sum()) > 0
    else:
        assert _rel(counts, ref["counts"]) < 1e-4
    return errs


def test_adjoint_spiking_matches_fp64(engine):
    layer, x_bits, x, G = _setup(4, 50)
    _check_against_reference(layer, x_bits, x, 50, G, relaxed=False)


def test_adjoint_relaxed_matches_fp64(engine):
    layer, x_bits, x, G = _setup(2, 30, seed=5)
    _check_against_reference(layer, x_bits, x, 30, G, relaxed=True)


def test_adjoint_relaxed_matches_finite_differences(engine):
    """Central differences of the float64 relaxed forward at sampled parameters (the entries with
    the largest gradients and random ones).  With slope 25 the relaxed network is stiff: at
    eps = 1e-3 the O(eps^2) truncation error of the difference quotient itself is several percent
    at the largest gradients (printed), so the check is made where the quotient has converged,
    eps = 1e-5, with the float64 forward's rounding (~1e-11 / eps) far below the bound."""
    from oracle import lif_dense
    T = 25
    layer, x_bits, x, G = _setup(2, T, seed=7)
    _, _, g = _grads(layer, x_bits, T, G, relaxed=True)
    rng = np.random.default_rng(0)
    params = {"w_in": layer.w_in, "w_rec": layer.w_rec, "theta": layer.theta, "beta": layer.beta}
    worst = {1e-3: 0.0, 1e-5: 0.0}
    for name, prm in params.items():
        top = torch.topk(g[name].abs(), 3).indices.tolist()
        idx = top + rng.integers(0, prm.numel(), size=3).tolist()
        scale = float(g[name].abs().max())
        for i in idx:
            for eps in worst:
                vals = []
                for sgn in (1.0, -1.0):
                    p = {k: v.detach().double().clone() for k, v in params.items()}
                    p[name][i] += sgn * eps
                    vals.append(lif_dense.loss_value(layer.in_csr, layer.rec_csr, p["w_in"], p["w_rec"], p["theta"],
                                                     p["beta"], x, T, layer.slope, G))
                fd = (vals[0] - vals[1]) / (2 * eps)
                err = abs(float(g[name][i]) - fd) / scale
                worst[eps] = max(worst[eps], err)
                if eps == 1e-5:
                    assert err < 2e-3, (name, i, float(g[name][i]), fd)
    print(f"finite differences, worst |g - fd| / max|g|: eps=1e-3 {worst[1e-3]:.2e}, eps=1e-5 {worst[1e-5]:.2e}")


def test_checkpointing_is_exact(engine):
    """Recomputing segments from checkpoints is exact: any segment length gives the same bits
    (20; 23, the longest whose u and s fit the CTA's shared memory at n = 1024; 7, not dividing T)."""
    layer, x_bits, x, G = _setup(3, 60, seed=3)
    _, s1, g1 = _grads(layer, x_bits, 60, G)
    layer.checkpoint_every = 23
    _, s2, g2 = _grads(layer, x_bits, 60, G)
    layer.checkpoint_every = 7
    _, s3, g3 = _grads(layer, x_bits, 60, G)
    assert torch.equal(s1, s2) and torch.equal(s1, s3)
    for k in g1:
        assert torch.equal(g1[k], g2[k]) and torch.equal(g1[k], g3[k]), k


def test_full_config_matches_fp64(engine):
    """Batch 64, 700 -> 1024, 200 steps, checkpoint every 20, MSE on the first 128 counts."""
    from spice2_gb300.lif_layer import count_loss, count_targets
    layer, x_bits, x, _ = _setup(64, 200, seed=11)
    target = count_targets(64)
    layer.zero_grad()
    counts, spikes = layer(x_bits, 200, return_spikes=True)
    loss = count_loss(counts, target)
    loss.backward()
    # dL/dcounts of the MSE, then the float64 reference along the kernel's spike train
    cc = counts.detach().clone().requires_grad_(True)
    Gc = torch.autograd.grad(count_loss(cc, target), cc)[0]
    ref = _reference(layer, x, 200, Gc, forced=spikes)
    errs = {k: _rel(getattr(layer, k).grad, ref["g_" + k]) for k in ("w_in", "w_rec", "theta", "beta")}
    print("full config relative errors", errs)
    assert all(e < TOL for e in errs.values()), errs


def test_training_lowers_the_loss(engine):
    from spice2_gb300.lif_layer import count_loss, count_targets
    layer, x_bits, x, _ = _setup(16, 100, seed=13)
    target = count_targets(16, seed=4)
    opt = torch.optim.Adam([layer.w_in, layer.w_rec, layer.theta], lr=3e-3)
    losses = []
    for _ in range(20):
        opt.zero_grad()
        loss = count_loss(layer(x_bits, 100), target)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert min(losses[-5:]) < 0.7 * losses[0], losses
