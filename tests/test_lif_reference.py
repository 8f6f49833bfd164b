"""CPU pins of the float64 LIF reference (oracle/lif_dense.py) used to check the adjoint kernels:
its autograd gradients of the relaxed forward equal central finite differences, and the input
packing used by the harness is the documented bit layout."""
import numpy as np
import torch


def _tiny(seed=0, n_in=12, n=9, p_in=0.5, p_rec=0.4):
    rng = np.random.default_rng(seed)
    def csr(ns, nd, p):
        rows = [np.sort(np.flatnonzero(rng.random(nd) < p)) for _ in range(ns)]
        off = np.zeros(ns + 1, np.int64)
        off[1:] = np.cumsum([len(r) for r in rows])
        return off, np.concatenate(rows + [np.zeros(0, int)]).astype(np.int32)
    in_csr, rec_csr = csr(n_in, n, p_in), csr(n, n, p_rec)
    g = torch.Generator().manual_seed(seed)
    w_in = torch.randn(int(in_csr[0][-1]), generator=g, dtype=torch.float64) * 0.6
    w_rec = torch.randn(int(rec_csr[0][-1]), generator=g, dtype=torch.float64) * 0.4
    theta = torch.full((n,), 1.0, dtype=torch.float64)
    beta = torch.full((n,), 0.95, dtype=torch.float64)
    x = (torch.rand(3, 15, n_in, generator=g, dtype=torch.float64) < 0.3).to(torch.float64)
    G = torch.randn(3, n, generator=g, dtype=torch.float64)
    return in_csr, rec_csr, w_in, w_rec, theta, beta, x, G


def test_dense_reference_relaxed_gradients_match_finite_differences():
    from oracle import lif_dense
    in_csr, rec_csr, w_in, w_rec, theta, beta, x, G = _tiny()
    T = 15
    r = lif_dense.run(in_csr, rec_csr, w_in, w_rec, theta, beta, x, T, slope=5.0, relaxed=True, grad_counts=G)
    params = {"w_in": w_in, "w_rec": w_rec, "theta": theta, "beta": beta}
    eps = 1e-6
    for name, prm in params.items():
        for i in range(0, prm.numel(), max(1, prm.numel() // 5)):
            vals = []
            for sgn in (1.0, -1.0):
                p = {k: v.clone() for k, v in params.items()}
                p[name][i] += sgn * eps
                vals.append(lif_dense.loss_value(in_csr, rec_csr, p["w_in"], p["w_rec"], p["theta"], p["beta"],
                                                 x, T, 5.0, G))
            fd = (vals[0] - vals[1]) / (2 * eps)
            assert abs(fd - float(r["g_" + name][i])) <= 1e-6 * max(1.0, abs(fd)), (name, i)


def test_dense_reference_spiking_forward_resets_by_subtraction():
    from oracle import lif_dense
    in_csr, rec_csr, w_in, w_rec, theta, beta, x, G = _tiny(seed=2)
    r = lif_dense.run(in_csr, rec_csr, w_in * 3, w_rec, theta, beta, x, 15)
    s, u = r["spikes"], r["u"]
    assert torch.equal(s, (u - theta > 0).to(s.dtype))
    assert float(s.sum()) > 0
    assert torch.equal(r["counts"], s.sum(1))


def test_pack_bits_layout():
    from spice2_gb300.lif_layer import pack_bits
    g = torch.Generator().manual_seed(1)
    x = torch.rand(2, 3, 70, generator=g) < 0.5
    w = pack_bits(x).numpy().astype(np.uint32)
    for b in range(2):
        for t in range(3):
            for k in range(70):
                assert bool((w[b, t, k // 32] >> (k % 32)) & 1) == bool(x[b, t, k])
