"""CPU oracle of the learned flip proposal (numpy, float64).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA
MLP kernels (pysa_gb300/csrc/mlp.cu, gemm_tc.cu); the product package never
imports it.  The proposal has no counterpart in the reference, so this
oracle restates the mathematics directly:

  network     z2 = W2 relu(W1 x + b1) + b2, one Bernoulli flip logit per
              spin, p = sigmoid(z2)
  loss        row-weighted mean over rows of sum_j BCE(sigmoid(z2_j), f_j)
  optimiser   Adam (Kingma & Ba, ICLR 2015) with bias correction
  proposal    flip mask f_j ~ Bernoulli(p_j(s)), s' = s flipped on f;
              accept iff log u < -beta dE + log q(s|s') - log q(s'|s)
              (Metropolis-Hastings, Hastings 1970)

With `emulate=True` the tensors are rounded to BF16 where the GPU rounds them
(the operands of every GEMM), everything else stays float64, so GPU results
agree to FP32-accumulation precision.  With `emulate=False` it is the plain
float64 mathematics, which tests compare with torch autograd.
"""
from __future__ import annotations

import numpy as np


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _r(a, emulate):
    return bf16(a) if emulate else np.asarray(a, np.float64)


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def log_sigmoid(z):
    z = np.asarray(z, np.float64)
    return -(np.maximum(-z, 0.0) + np.log1p(np.exp(-np.abs(z))))


def forward(x, w1, b1, w2, b2, emulate=True):
    """x [B, n] -> (a1 [B, H], z2 [B, n])."""
    a1 = np.maximum(_r(x, emulate) @ _r(w1, emulate).T + b1, 0.0)
    z2 = _r(a1, emulate) @ _r(w2, emulate).T + b2
    return a1, z2


def backward(x, a1, z2, target, row_w, w2, emulate=True):
    """Gradients of L = sum_r w_r sum_j BCE(z2[r, j], target[r, j]) / sum w.

    Returns (loss, dw1, db1, dw2, db2)."""
    w = np.asarray(row_w, np.float64)
    ws = w.sum()
    wn = w / ws if ws > 0 else np.zeros_like(w)
    z = np.asarray(z2, np.float64)
    t = np.asarray(target, np.float64)
    bce = np.maximum(z, 0.0) - z * t + np.log1p(np.exp(-np.abs(z)))
    loss = float((wn[:, None] * bce).sum())
    dz2 = wn[:, None] * (sigmoid(z) - t)
    dw2 = _r(dz2, emulate).T @ _r(a1, emulate)
    da1 = _r(dz2, emulate) @ _r(w2, emulate)
    dz1 = da1 * (np.asarray(a1) > 0)
    dw1 = _r(dz1, emulate).T @ _r(x, emulate)
    return loss, dw1, dz1.sum(0), dw2, dz2.sum(0)


def adam(w, m, v, g, lr, beta1, beta2, eps, step):
    """One Adam step; returns new (w, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    c1 = 1 - beta1**step
    c2 = 1 - beta2**step
    return w - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def flip_shift(z, k):
    """Shift c with sum_j sigmoid(z_j + c) = k (40 bisection steps on
    [-60, 60], as the GPU does); 0 when k <= 0."""
    if k <= 0:
        return 0.0
    lo, hi = -60.0, 60.0
    z = np.asarray(z, np.float64)
    for _ in range(40):
        c = 0.5 * (lo + hi)
        if sigmoid(z + c).sum() > k:
            hi = c
        else:
            lo = c
    return 0.5 * (lo + hi)


def flip_mask(z, u):
    """f_j = u_j < sigmoid(z_j) and log q(f | z)."""
    p = sigmoid(np.asarray(z, np.float64))
    f = (np.asarray(u) < p).astype(np.float64)
    lq = np.where(f > 0, log_sigmoid(z), log_sigmoid(-np.asarray(z))).sum(-1)
    return f, lq


def log_q(z, f):
    return np.where(f > 0, log_sigmoid(z), log_sigmoid(-np.asarray(z))).sum(-1)


def energy(J, h, s):
    """E(s) = s.(J s / 2 + h)  (pysa/ising.py:32-37, pysa/qubo.py:32-37)."""
    s = np.asarray(s, np.float64)
    return float(s @ (0.5 * (np.asarray(J, np.float64) @ s) + h))


def mh_chain(problem_type, J, h, beta, net, s0, steps, rng,
             reverse_term=True):
    """Metropolis-Hastings with the learned proposal on one chain (float64,
    numpy uniforms).  net(s) -> logits z.  reverse_term=False drops
    log q(s|s') - log q(s'|s) (a wrong chain, for planted-mistake tests).
    Returns the visited states [steps, n]."""
    s = np.array(s0, np.float64)
    out = np.zeros((steps, len(s)))
    e = energy(J, h, s)
    for t in range(steps):
        z = net(s)
        f, lqf = flip_mask(z, rng.random(len(s)))
        sp = np.where(f > 0, (-s if problem_type == "ising" else 1.0 - s), s)
        lqr = log_q(net(sp), f)
        ep = energy(J, h, sp)
        la = -beta * (ep - e) + ((lqr - lqf) if reverse_term else 0.0)
        if f.sum() > 0 and (la >= 0 or np.log(rng.random()) < la):
            s, e = sp, ep
        out[t] = s
    return out


def boltzmann(problem_type, J, h, beta):
    """Exact probabilities of all 2^n states, index = sum_j bit_j 2^j with
    bit 1 = spin +1 (Ising) or 1 (QUBO)."""
    n = len(h)
    idx = np.arange(2**n)
    bits = (idx[:, None] >> np.arange(n)) & 1
    s = bits * 2.0 - 1.0 if problem_type == "ising" else bits.astype(float)
    e = np.einsum("ki,ij,kj->k", s, np.asarray(J, float), s) / 2 + s @ h
    lw = -beta * e
    p = np.exp(lw - lw.max())
    return p / p.sum()


def state_index(s, problem_type):
    bits = (np.asarray(s) > 0).astype(np.int64)
    return bits @ (1 << np.arange(bits.shape[-1]))
