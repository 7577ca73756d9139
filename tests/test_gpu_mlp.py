"""Learned flip proposal on the GPU: MLP kernels against the CPU oracle
(oracle/mlp_oracle.py), exactness of the Metropolis-Hastings move, and the
bookkeeping of accepted moves (spins, fields, energies, best state).

Tolerances: the GEMMs take BF16 operands and accumulate in FP32 while the
oracle rounds the same operands to BF16 and accumulates in FP64, so
activations agree to ~1e-6 relative; a value that lands on the other side of
a BF16 rounding boundary moves downstream results by one BF16 ulp (2^-8
relative) of that value, hence the 2e-3-of-scale bounds on logits and
gradients.
"""
import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

TAG_PROPOSAL = 4


def _sk(rng, n):
    J = np.triu(rng.choice([-1.0, 1.0], size=(n, n)), 1)
    return (J + J.T).astype(np.float32)


def _batch(ptype, Js, hs, ladder, reads, seed=0, kernel="auto"):
    from pysa_gb300 import Instance, PTBatch, pack_spins
    rng = np.random.default_rng(seed)
    b = PTBatch(ptype, [Instance(J, h, np.asarray(ladder, np.float32), reads)
                        for J, h in zip(Js, hs)], kernel=kernel)
    states = []
    for J, h in zip(Js, hs):
        n = len(h)
        R = len(ladder)
        if ptype == "ising":
            x = rng.choice([-1.0, 1.0], size=(reads * R, n))
        else:
            x = rng.choice([0.0, 1.0], size=(reads * R, n))
        states.append(pack_spins(x.astype(np.float32), ptype, b.words))
    b.set_states(np.concatenate(states))
    return b


def _perturb(prop, seed, scale=0.05):
    g = torch.Generator(device="cpu").manual_seed(seed)
    for k in ("w1", "b1", "w2", "b2"):
        t = prop.t[k]
        t.add_(scale * torch.randn(t.shape, generator=g).to(t.device))
    prop.sync()


def _scale_err(got, want):
    return np.abs(got - want).max() / max(np.abs(want).max(), 1e-30)


def test_forward_backward_adam_match_oracle():
    from pysa_gb300.proposal import LearnedProposal
    rng = np.random.default_rng(0)
    ns = [200, 256]
    b = _batch("ising", [_sk(rng, n) for n in ns],
               [np.zeros(n, np.float32) for n in ns], [0.5, 1.0], 100)
    prop = LearnedProposal(b, hidden=512, lr=1e-3, init_seed=3)
    _perturb(prop, 1)
    I, B, nn, H = prop.I, prop.B, prop.nn, prop.H
    assert (nn, H, B) == (256, 512, 128)
    x = rng.choice([-1.0, 1.0], size=(I, B, nn)).astype(np.float32)
    x[0, :, 200:] = 0.0
    tgt = (rng.random((I, B, nn)) < 0.2).astype(np.float32)
    rw = np.ones((I, B), np.float32)
    rw[:, 100:] = 0.0
    w = {k: prop.t[k].cpu().numpy().astype(np.float64)
         for k in ("w1", "b1", "w2", "b2")}
    z2 = prop.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    a1 = prop.t["a1"].cpu().numpy()
    for i in range(I):
        a1_o, z2_o = mo.forward(x[i], w["w1"][i], w["b1"][i], w["w2"][i],
                                w["b2"][i])
        assert _scale_err(a1[i], a1_o) < 5e-5
        assert _scale_err(z2[i], z2_o) < 2e-3
    loss = prop.train_step(torch.from_numpy(tgt).cuda(),
                           torch.from_numpy(rw).cuda()).cpu().numpy()
    g = {k: prop.t[k].cpu().numpy() for k in ("dw1", "db1", "dw2", "db2")}
    after = {k: prop.t[k].cpu().numpy() for k in ("w1", "b1", "w2", "b2")}
    for i in range(I):
        # oracle backward on the GPU's own activations (isolates backward)
        lo, dw1, db1, dw2, db2 = mo.backward(x[i], a1[i].astype(np.float64),
                                             z2[i].astype(np.float64), tgt[i],
                                             rw[i], w["w2"][i])
        assert abs(loss[i] - lo) < 1e-4 * abs(lo)
        assert _scale_err(g["dw1"][i], dw1) < 2e-3
        assert _scale_err(g["dw2"][i], dw2) < 2e-3
        assert _scale_err(g["db1"][i], db1) < 1e-3
        assert _scale_err(g["db2"][i], db2) < 1e-5
        # Adam on the GPU's gradients
        for k, gk in (("w1", "dw1"), ("b1", "db1"), ("w2", "dw2"),
                      ("b2", "db2")):
            wn, _, _ = mo.adam(w[k][i], 0.0, 0.0, g[gk][i].astype(np.float64),
                               1e-3, 0.9, 0.999, 1e-8, 1)
            assert np.abs(after[k][i] - wn).max() < 2e-6


def test_training_fits_a_learnable_target():
    from pysa_gb300.proposal import LearnedProposal
    rng = np.random.default_rng(1)
    n = 256
    b = _batch("ising", [_sk(rng, n)], [np.zeros(n, np.float32)], [1.0], 128)
    prop = LearnedProposal(b, hidden=512, lr=1e-2, init_seed=1)
    I, B, nn = prop.I, prop.B, prop.nn
    losses = []
    for step in range(150):
        x = rng.choice([-1.0, 1.0], size=(I, B, nn)).astype(np.float32)
        # flip spin j when spin (j + 1) % n is down: a function of the input
        tgt = (np.roll(x, -1, axis=2) < 0).astype(np.float32)
        prop.forward(torch.from_numpy(x).cuda())
        losses.append(float(prop.train_step(torch.from_numpy(tgt).cuda())[0]))
    # starts near 600 (untrained output bias flips ~2 spins); a float64
    # torch run of the same setup ends near 17
    assert losses[-1] < 0.1 * losses[0], (losses[0], losses[-1])


@pytest.mark.parametrize("target_flips", [0.0, 4.0])
def test_flip_sampling_and_log_q_match_oracle(oracle, target_flips):
    from pysa_gb300.proposal import LearnedProposal
    from pysa_gb300 import unpack_spins
    rng = np.random.default_rng(2)
    ns = [100, 256]
    b = _batch("qubo", [_sk(rng, n) for n in ns],
               [rng.integers(-2, 3, n).astype(np.float32) for n in ns],
               [0.2, 0.4, 0.8], 50)
    prop = LearnedProposal(b, hidden=256, init_seed=5, init_flips=20.0,
                           target_flips=target_flips)
    _perturb(prop, 2, 0.2)
    w = {k: prop.t[k].cpu().numpy().astype(np.float64)
         for k in ("w1", "b1", "w2", "b2")}
    spins0 = b.spins.cpu().numpy().view("<u4").copy()
    seed, rnd = 987654321, 7
    prop.propose(seed, rnd)
    torch.cuda.synchronize()
    b.check_status()
    rows = prop.rows.cpu().numpy()
    flip = prop.sc_t["flip"].cpu().numpy()
    lqf = prop.sc_t["logq_fwd"].cpu().numpy()
    lqr = prop.sc_t["logq_rev"].cpu().numpy()
    checked = 0
    nflips = []
    for i, n in enumerate(ns):
        for r in range(prop.B):
            c = rows[i, r]
            if r >= 50:
                assert c == -1
                continue
            s = unpack_spins(spins0[c][None], n, "qubo", np.float64)[0]
            x = np.zeros(prop.nn)
            x[:n] = s
            _, z = mo.forward(x[None], w["w1"][i], w["b1"][i], w["w2"][i],
                              w["b2"][i])
            z = z[0, :n]
            z = z + mo.flip_shift(z, target_flips)
            u = oracle.uniforms(seed, TAG_PROPOSAL, i, rnd, int(c), n)
            f_o = (u < mo.sigmoid(z)).astype(float)
            clear = np.abs(u - mo.sigmoid(z)) > 5e-3
            assert np.array_equal(flip[i, r, :n][clear], f_o[clear])
            assert not flip[i, r, n:].any()
            assert abs(lqf[i, r] - mo.log_q(z, flip[i, r, :n])) < 0.05
            sp = np.where(flip[i, r, :n] > 0, 1.0 - s, s)
            xp = np.zeros(prop.nn)
            xp[:n] = sp
            _, zr = mo.forward(xp[None], w["w1"][i], w["b1"][i], w["w2"][i],
                               w["b2"][i])
            zr = zr[0, :n]
            zr = zr + mo.flip_shift(zr, target_flips)
            assert abs(lqr[i, r] - mo.log_q(zr, flip[i, r, :n])) < 0.05
            nflips.append(flip[i, r].sum())
            checked += 1
    assert checked == 100
    if target_flips > 0:
        assert abs(np.mean(nflips) - target_flips) < 1.0


@pytest.mark.parametrize("ptype", ["ising", "qubo"])
def test_accepted_moves_keep_spins_fields_energies_consistent(ptype):
    from pysa_gb300.proposal import LearnedProposal
    from pysa_gb300 import unpack_spins
    rng = np.random.default_rng(3)
    ns = [300, 512]
    Js = [_sk(rng, n) for n in ns]
    hs = [rng.integers(-2, 3, n).astype(np.float32) for n in ns]
    b = _batch(ptype, Js, hs, [0.05, 0.1, 0.2], 64, kernel="plain")
    prop = LearnedProposal(b, hidden=256, init_seed=7, init_flips=3.0)
    total = 0
    for k in range(30):
        b.run(2, seed=11, graph_chunk=0)
        prop.propose(99, k)
    torch.cuda.synchronize()
    b.check_status()
    total = int(prop.accepted.sum())
    assert total > 0
    r = b.fetch()
    fields = b.fields.cpu().numpy().copy()
    e_inc = r["energies"].copy()
    from pysa_gb300 import _lib
    _lib.check(b.lib.pysa_gb_prepare(_lib.ref(b.p), _lib.ref(b.s),
                                     _lib.ref(b.ws), 1, 0, 0,
                                     b._stream.cuda_stream), "prepare")
    torch.cuda.synchronize()
    assert np.array_equal(b.energies.cpu().numpy(), e_inc)
    assert np.array_equal(b.fields.cpu().numpy(), fields)
    off = 0
    for i, n in enumerate(ns):
        C = 3 * 64
        best = unpack_spins(r["best_spins"][off:off + C], n, ptype, np.float64)
        for c in range(0, C, 7):
            e = mo.energy(Js[i], hs[i], best[c])
            assert e == r["best_energy"][off + c]
            assert r["best_energy"][off + c] <= r["energies"][off + c]
        off += C


def test_mh_move_samples_boltzmann_exactly():
    """Proposals only (no sweeps) on a 5-spin Ising system padded to a
    256-wide network: the visited-state histogram of 128 chains matches the
    exact Boltzmann law.  The network is random and strongly state-dependent,
    so q(s'|s) != q(s|s') and the reverse term matters (the same check with
    the reverse term removed fails on the CPU oracle)."""
    from pysa_gb300.proposal import LearnedProposal
    from pysa_gb300 import unpack_spins
    rng = np.random.default_rng(4)
    n, beta = 5, 0.7
    J = _sk(rng, n)
    h = rng.choice([-1.0, 0.0, 1.0], size=n).astype(np.float32)
    b = _batch("ising", [J], [h], [beta], 128, kernel="plain")
    prop = LearnedProposal(b, hidden=256, init_seed=9)
    w1 = np.zeros((1, 256, 256), np.float32)
    w1[0, :, :n] = rng.normal(size=(256, n)) * 0.6
    w2 = np.zeros((1, 256, 256), np.float32)
    w2[0, :n, :] = rng.normal(size=(n, 256)) * 0.15
    b2 = np.full((1, 256), -0.5, np.float32)
    prop.t["w1"].copy_(torch.from_numpy(w1))
    prop.t["w2"].copy_(torch.from_numpy(w2))
    prop.t["b1"].zero_()
    prop.t["b2"].copy_(torch.from_numpy(b2))
    prop.sync()
    hist = np.zeros(2**n)
    for k in range(960):
        prop.propose(2024, k)
        if k >= 40 and k % 4 == 0:
            s = unpack_spins(b.spins.cpu().numpy().view("<u4"), n, "ising",
                             np.float64)
            hist += np.bincount(mo.state_index(s, "ising"), minlength=2**n)
    torch.cuda.synchronize()
    b.check_status()
    acc = int(prop.accepted[0]) / (960 * 128)
    assert 0.05 < acc < 0.95, acc
    p = mo.boltzmann("ising", J, h, beta)
    tv = 0.5 * np.abs(hist / hist.sum() - p).sum()
    assert tv < 0.04, tv


def test_training_raises_acceptance_of_equal_size_proposals():
    """What the trained network gains: on +-1 SK instances at T = 0.3 the
    cold chains are nearly frozen, so 2-spin proposals of the untrained
    network (spins picked almost uniformly) are essentially never accepted.
    After online training on same-chain pairs the network picks spins that
    actually move at that temperature, and proposals of the same expected
    size are accepted measurably often."""
    from pysa_gb300.proposal import LearnedProposal
    rng = np.random.default_rng(6)
    I, n, R = 4, 256, 16
    lad = np.sort(1.0 / np.geomspace(0.3, 3.0, R)).astype(np.float32)
    b = _batch("ising", [_sk(rng, n) for _ in range(I)],
               [np.zeros(n, np.float32)] * I, lad, 128)
    b.run(300, seed=1)
    prop = LearnedProposal(b, hidden=512, lr=1e-3, init_seed=0,
                           target_flips=2.0)
    rnd = [0]

    def acceptance(rounds):
        a0 = prop.accepted.clone()
        for _ in range(rounds):
            b.run(10, seed=1, graph_chunk=0)
            prop.propose(5, rnd[0])
            rnd[0] += 1
        torch.cuda.synchronize()
        return float((prop.accepted - a0).sum()) / (rounds * I * 128)

    before = acceptance(30)
    for _ in range(600):
        b.run(2, seed=1, graph_chunk=0)
        prop.observe()
    after = acceptance(30)
    b.check_status()
    # measured on a GB300: 6.5e-5 before, 3.1e-3 after (47x)
    assert after >= 1e-3 and after > 5 * before, (before, after)
