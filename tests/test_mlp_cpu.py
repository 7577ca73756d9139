"""Learned-proposal oracle and ABI surface, without a GPU.

The oracle (oracle/mlp_oracle.py) is checked against torch autograd and
torch.optim.Adam in float64, and its Metropolis-Hastings chain against exact
Boltzmann probabilities; a planted mistake (the reverse-proposal term left
out) must fail the same check.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo


def _net(rng, B=6, n=8, H=16):
    x = rng.choice([-1.0, 1.0], size=(B, n))
    w1 = rng.normal(size=(H, n)) / np.sqrt(n)
    b1 = rng.normal(size=H) * 0.1
    w2 = rng.normal(size=(n, H)) / np.sqrt(H)
    b2 = rng.normal(size=n) * 0.1
    t = (rng.random((B, n)) < 0.3).astype(float)
    rw = np.ones(B)
    rw[-1] = 0.0
    return x, w1, b1, w2, b2, t, rw


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    a = (rng.normal(size=4096) * 10.0 ** rng.integers(-5, 5, 4096)).astype(
        np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(mo.bf16(a), ref)


def test_backward_matches_torch_autograd_f64():
    rng = np.random.default_rng(1)
    x, w1, b1, w2, b2, t, rw = _net(rng)
    a1, z2 = mo.forward(x, w1, b1, w2, b2, emulate=False)
    loss, dw1, db1, dw2, db2 = mo.backward(x, a1, z2, t, rw, w2,
                                           emulate=False)
    T = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)
    W1, B1, W2, B2 = T(w1), T(b1), T(w2), T(b2)
    X = torch.tensor(x)
    Z2 = torch.relu(X @ W1.T + B1) @ W2.T + B2
    per = torch.nn.functional.binary_cross_entropy_with_logits(
        Z2, torch.tensor(t), reduction="none").sum(1)
    w = torch.tensor(rw)
    L = (per * w).sum() / w.sum()
    L.backward()
    assert abs(loss - L.item()) < 1e-12
    for mine, theirs in ((dw1, W1), (db1, B1), (dw2, W2), (db2, B2)):
        assert np.allclose(mine, theirs.grad.numpy(), rtol=1e-10, atol=1e-12)


def test_adam_matches_torch_optim_f64():
    rng = np.random.default_rng(2)
    w = rng.normal(size=50)
    m = np.zeros(50)
    v = np.zeros(50)
    P = torch.nn.Parameter(torch.tensor(w))
    opt = torch.optim.Adam([P], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    for step in range(1, 6):
        g = rng.normal(size=50)
        w, m, v = mo.adam(w, m, v, g, 1e-2, 0.9, 0.999, 1e-8, step)
        P.grad = torch.tensor(g)
        opt.step()
    assert np.allclose(w, P.detach().numpy(), rtol=1e-12, atol=1e-14)


def test_flip_mask_and_log_q():
    z = np.array([[-3.0, 0.0, 2.0, 40.0]])
    u = np.array([[0.01, 0.6, 0.5, 0.99]])
    f, lq = mo.flip_mask(z, u)
    assert f.tolist() == [[1.0, 0.0, 1.0, 1.0]]
    p = mo.sigmoid(z)
    want = np.log(p[0, 0]) + np.log(1 - p[0, 1]) + np.log(p[0, 2]) + np.log(
        p[0, 3])
    assert abs(lq[0] - want) < 1e-12
    assert abs(mo.log_q(z, f)[0] - want) < 1e-12


@pytest.mark.parametrize("problem_type", ["ising", "qubo"])
def test_mh_chain_is_exact_and_planted_mistake_is_caught(problem_type):
    rng = np.random.default_rng(1)
    n = 4
    J = np.triu(rng.choice([-1.0, 1.0], size=(n, n)), 1)
    J = J + J.T
    h = rng.choice([-1.0, 0.0, 1.0], size=n)
    W = rng.normal(size=(n, n)) * 1.5
    b = rng.normal(size=n) * 0.5 - 0.5
    net = lambda s: W @ s + b
    beta = 0.7
    p = mo.boltzmann(problem_type, J, h, beta)
    tv = {}
    for rev in (True, False):
        hist = np.zeros(2**n)
        r = np.random.default_rng(5)
        for _ in range(20):
            if problem_type == "ising":
                s0 = r.choice([-1.0, 1.0], size=n)
            else:
                s0 = r.choice([0.0, 1.0], size=n)
            out = mo.mh_chain(problem_type, J, h, beta, net, s0, 2000, r,
                              reverse_term=rev)
            hist += np.bincount(mo.state_index(out[100:], problem_type),
                                minlength=2**n)
        tv[rev] = 0.5 * np.abs(hist / hist.sum() - p).sum()
    assert tv[True] < 0.05, tv
    assert tv[False] > 0.08, tv


def test_mlp_structs_and_null_arguments():
    from pysa_gb300 import _lib
    lib = _lib.load()
    assert ctypes.sizeof(_lib.Mlp) == 4 * 4 + 28 * 8
    assert ctypes.sizeof(_lib.ProposalScratch) == 6 * 8
    assert lib.pysa_gb_mlp_forward(None, None) == -1
    assert lib.pysa_gb_mlp_backward(None, None, None, None) == -1
    assert lib.pysa_gb_mlp_adam(None, 1e-3, 0.9, 0.999, 1e-8, 1, None) == -1
    assert lib.pysa_gb_propose(None, None, None, None, None, None, 1, None,
                               0, 0, 0.0, None, None) == -1
    assert lib.pysa_gb_proposal_j_elems(2, 300, 1) < 0
    assert lib.pysa_gb_proposal_j_elems(2, 512, 2) == 2 * 2 * 512 * 512
    m = _lib.Mlp(1, 512, 1000, 128)   # hidden not a multiple of 256
    assert lib.pysa_gb_mlp_forward(ctypes.byref(m), None) == -1
    assert b"mlp" in lib.pysa_gb_last_error()
