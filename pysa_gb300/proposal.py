"""Learned flip proposal for the coldest replica of every read.

No counterpart in the reference: an addition on top of the parallel-tempering
loop of pysa/simulation.py:123-181.  Each instance owns an MLP
nn -> hidden -> nn (ReLU hidden layer, one Bernoulli flip logit per spin),
trained online on pairs of cold states of the same read taken `interval`
sweeps apart (target = which spins changed).  Between sweep chunks the
network proposes a multi-spin move for the coldest chain of every read and a
Metropolis-Hastings test with the reverse-proposal likelihood accepts or
rejects it, so the chain keeps exp(-beta E) as its stationary law.  An
instance whose acceptance rate stays below `min_accept` stops proposing and
runs plain sweeps only.

All compute (GEMMs on tcgen05 tensor cores, sampling, acceptance, Adam) runs
in libpysa_gb.so; this module allocates device memory and sequences calls.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import check, ref
from .engine import PTBatch, bf16_exact


def _round_up(x: int, m: int) -> int:
    return (int(x) + m - 1) // m * m


def _ptr(t: torch.Tensor | None) -> int:
    return 0 if t is None else t.data_ptr()


@dataclass
class ProposalStats:
    rounds: int = 0
    proposed: np.ndarray = field(default_factory=lambda: np.zeros(0))
    accepted: np.ndarray = field(default_factory=lambda: np.zeros(0))
    enabled: np.ndarray = field(default_factory=lambda: np.zeros(0))
    train_steps: int = 0
    loss: list = field(default_factory=list)

    @property
    def acceptance(self) -> np.ndarray:
        return self.accepted / np.maximum(self.proposed, 1)


class LearnedProposal:
    """MLP flip proposals for the coldest replica of each read of `batch`.

    hidden: width of the hidden layer (multiple of 256).
    lr, adam_betas, eps: Adam hyper-parameters.
    init_flips: expected number of flipped spins of the untrained network
        (sets the output bias).
    target_flips: when > 0, every proposal is rescaled (one logit shift per
        state, applied the same way in the reverse pass) to flip this many
        spins on average; the network then decides which spins.
    """

    def __init__(self, batch: PTBatch, hidden: int = 1024, lr: float = 1e-3,
                 adam_betas=(0.9, 0.999), eps: float = 1e-8,
                 init_seed: int = 0, init_flips: float = 2.0,
                 target_flips: float = 0.0):
        self.lib = _lib.load()
        self.target_flips = float(target_flips)
        self.b = batch
        dev = batch.device
        I = len(batch.instances)
        self.I = I
        self.nn = _round_up(max(batch.max_n, 1), 256)
        self.H = _round_up(hidden, 256)
        self.B = _round_up(int(np.max(batch.Rd)), 128)
        self.words = batch.words
        self.lr, self.adam_betas, self.eps = lr, adam_betas, eps
        self.step = 0
        nn, H, B = self.nn, self.H, self.B

        def z(*shape, dt=torch.float32):
            return torch.zeros(*shape, dtype=dt, device=dev)

        self.t = dict(
            w1=z(I, H, nn), b1=z(I, H), w2=z(I, nn, H), b2=z(I, nn),
            m1=z(I, H, nn), v1=z(I, H, nn), mb1=z(I, H), vb1=z(I, H),
            m2=z(I, nn, H), v2=z(I, nn, H), mb2=z(I, nn), vb2=z(I, nn),
            dw1=z(I, H, nn), db1=z(I, H), dw2=z(I, nn, H), db2=z(I, nn),
            w1_p=z(I, H * nn, dt=torch.int16), w2_p=z(I, nn * H, dt=torch.int16),
            w2t_p=z(I, H * nn, dt=torch.int16),
            x=z(I, B, nn), a1=z(I, B, H), z2=z(I, B, nn), dz2=z(I, B, nn),
            da1=z(I, B, H), pa=z(I, B * max(nn, H), dt=torch.int16),
            pb=z(I, B * max(nn, H), dt=torch.int16), loss=z(I))
        t = self.t
        self.m = _lib.Mlp(I, nn, H, B, *(_ptr(t[k]) for k in (
            "w1", "b1", "w2", "b2", "m1", "v1", "mb1", "vb1", "m2", "v2",
            "mb2", "vb2", "dw1", "db1", "dw2", "db2", "w1_p", "w2_p", "w2t_p",
            "x", "a1", "z2", "dz2", "da1", "pa", "pb", "loss")),
            _ptr(batch.status))
        self.sc_t = dict(flip=z(I, B, nn), delta=z(I, B, nn), jd=z(I, B, nn),
                         logq_fwd=z(I, B), logq_rev=z(I, B), de=z(I, B))
        self.sc = _lib.ProposalScratch(*(_ptr(self.sc_t[k]) for k in (
            "flip", "delta", "jd", "logq_fwd", "logq_rev", "de")))
        self.rows = z(I, B, dt=torch.int32)
        self.obs_rows = z(I, B, dt=torch.int32)
        self.enabled = torch.ones(I, dtype=torch.int32, device=dev)
        self.accepted = z(I, dt=torch.int32)
        self.snap = [z(I, B, self.words, dt=torch.int32) for _ in range(2)]
        self.have_snap = False
        self.target = z(I, B, nn)
        rw = np.zeros((I, B), np.float32)
        for i in range(I):
            rw[i, :int(batch.Rd[i])] = 1.0
        self.row_weight = torch.from_numpy(rw).to(dev)
        self.n_inst = batch._t["n"]
        # couplings as the B operand of J delta (split when not BF16-exact)
        self.terms = 1 if all(bf16_exact(np.asarray(x.J, np.float32))
                              for x in batch.instances) else 2
        ne = check(self.lib.pysa_gb_proposal_j_elems(I, nn, self.terms),
                   "proposal couplings size")
        self.j_packed = z(ne, dt=torch.int16)
        self._host = [np.ascontiguousarray(a, dtype=dt) for a, dt in (
            (batch.n, np.int32), (batch.R, np.int32), (batch.Rd, np.int32),
            (batch.chain_off, np.int64), (self._j_off(), np.int64),
            (batch.ld, np.int32))]
        self.ht = _lib.HostTables(*(a.ctypes.data for a in self._host))
        check(self.lib.pysa_gb_pack_proposal_j(
            ref(batch.p), ref(self.ht), nn, self.terms, _ptr(self.j_packed),
            self._st()), "pack proposal couplings")
        self.init_weights(init_seed, init_flips)
        self.stats = ProposalStats(
            proposed=np.zeros(I), accepted=np.zeros(I), enabled=np.ones(I, bool))

    # ------------------------------------------------------------ helpers
    def _j_off(self):
        b = self.b
        off = np.zeros(self.I, np.int64)
        acc = 0
        for i in range(self.I):
            off[i] = acc
            acc += int(b.n[i]) * int(b.ld[i])
        return off

    def _st(self):
        return self.b._stream.cuda_stream

    def init_weights(self, seed: int = 0, init_flips: float = 2.0):
        """Uniform(+-1/sqrt(fan_in)) weights and hidden biases; output bias
        logit(init_flips / n) so the untrained network flips about
        `init_flips` spins."""
        rng = np.random.default_rng(seed)
        nn, H, I = self.nn, self.H, self.I
        t = self.t
        for k, shape, fan in (("w1", (I, H, nn), nn), ("b1", (I, H), nn),
                              ("w2", (I, nn, H), H)):
            a = 1.0 / math.sqrt(fan)
            t[k].copy_(torch.from_numpy(
                rng.uniform(-a, a, size=shape).astype(np.float32)))
        b2 = np.zeros((I, nn), np.float32)
        for i in range(I):
            p0 = min(max(init_flips / max(int(self.b.n[i]), 1), 1e-6), 0.5)
            b2[i] = math.log(p0 / (1 - p0))
        t["b2"].copy_(torch.from_numpy(b2))
        for k in ("m1", "v1", "mb1", "vb1", "m2", "v2", "mb2", "vb2"):
            t[k].zero_()
        self.step = 0
        self.sync()

    def sync(self):
        check(self.lib.pysa_gb_mlp_sync_weights(ref(self.m), self._st()),
              "mlp sync")

    def forward(self, x: torch.Tensor | None = None) -> torch.Tensor:
        """Logits z2 [I, B, nn] for inputs x (default: the current x)."""
        if x is not None:
            self.t["x"].copy_(x)
        check(self.lib.pysa_gb_mlp_forward(ref(self.m), self._st()),
              "mlp forward")
        return self.t["z2"]

    def train_step(self, target: torch.Tensor | None = None,
                   row_weight: torch.Tensor | None = None) -> torch.Tensor:
        """Backward on the last forward's activations, then one Adam step.
        Returns the per-instance loss (device tensor)."""
        tg = self.target if target is None else target
        rw = self.row_weight if row_weight is None else row_weight
        check(self.lib.pysa_gb_mlp_backward(ref(self.m), _ptr(tg), _ptr(rw),
                                            self._st()), "mlp backward")
        self.step += 1
        b1, b2 = self.adam_betas
        check(self.lib.pysa_gb_mlp_adam(ref(self.m), self.lr, b1, b2, self.eps,
                                        self.step, self._st()), "mlp adam")
        return self.t["loss"]

    # --------------------------------------------------------- online loop
    def observe(self) -> bool:
        """Training data from the chains themselves: with a previous
        observation, snapshot the same chains again (the pair is their state
        then and now, target = the spins that changed) and train one step on
        it; then record the chains now holding the coldest slot for the next
        pair.  Returns whether a training step ran."""
        b = self.b
        st = self._st()
        trained = False
        if self.have_snap:
            check(self.lib.pysa_gb_snapshot(ref(b.p), ref(b.s),
                                            _ptr(self.obs_rows), self.B,
                                            _ptr(self.snap[1]), st), "snapshot")
            check(self.lib.pysa_gb_mlp_pairs(
                ref(self.m), b.ptype, _ptr(self.n_inst), _ptr(self.snap[0]),
                _ptr(self.snap[1]), self.words, _ptr(self.target), st),
                "pairs")
            self.forward()
            self.train_step()
            self.stats.train_steps += 1
            trained = True
        check(self.lib.pysa_gb_cold_rows(ref(b.p), ref(b.s), 0, self.B,
                                         _ptr(self.obs_rows), st), "cold rows")
        check(self.lib.pysa_gb_snapshot(ref(b.p), ref(b.s),
                                        _ptr(self.obs_rows), self.B,
                                        _ptr(self.snap[0]), st), "snapshot")
        self.have_snap = True
        return trained

    def propose(self, seed: int, round_: int):
        """One proposal for the coldest chain of every read of the enabled
        instances; accepted counts accumulate in self.accepted."""
        b = self.b
        st = self._st()
        check(self.lib.pysa_gb_cold_rows(ref(b.p), ref(b.s),
                                         _ptr(self.enabled), self.B,
                                         _ptr(self.rows), st), "cold rows")
        check(self.lib.pysa_gb_propose(
            ref(b.p), ref(b.s), ref(b.ws), ref(self.m), _ptr(self.rows),
            _ptr(self.j_packed), self.terms, ref(self.sc),
            seed & ((1 << 64) - 1), round_ & 0xFFFFFFFF, self.target_flips,
            _ptr(self.accepted), st), "propose")


def run_with_proposals(batch: PTBatch, prop: LearnedProposal | None,
                       num_sweeps: int, *, seed: int, interval: int = 10,
                       train_every: int | None = None,
                       train_pairs: int = 200_000, min_train_steps: int = 200,
                       check_every: int = 20, min_accept: float = 0.01,
                       use_pt: bool = True,
                       propose: bool = True) -> ProposalStats | None:
    """num_sweeps sequential PT sweeps of `batch`.  With a network: every
    `train_every` sweeps (default `interval`) one training step on the
    same-chain pairs of every read, until each instance has seen
    `train_pairs` pairs; every `interval` sweeps one learned proposal per
    read.  Once the network has had `min_train_steps` steps, every
    `check_every` proposal rounds an instance whose acceptance rate over
    those rounds is below `min_accept` stops proposing for the rest of the
    run (plain sweeps only); training stops when no instance proposes.
    Returns the proposal statistics (None without a network)."""
    if prop is None:
        batch.run(num_sweeps, seed=seed, use_pt=use_pt)
        return None
    # a chain that accepts a proposal continues on a fresh sweep stream;
    # on the shared counter-based stream its next sweeps would replay the
    # uniforms of the unmoved chain and largely undo the move
    batch.enable_stream_keys()
    interval = max(int(interval), 1)
    train_every = interval if train_every is None else max(int(train_every), 1)
    step = math.gcd(interval, train_every)
    st = prop.stats
    reads = np.asarray(batch.Rd, np.float64)
    max_steps = int(math.ceil(train_pairs / max(float(reads.min()), 1.0)))
    done = 0
    win_rounds = 0
    acc0 = prop.accepted.clone()

    def settle():
        nonlocal acc0, win_rounds
        now = prop.accepted.clone()
        acc = (now - acc0).cpu().numpy().astype(np.float64)
        acc0 = now
        st.accepted += acc
        rate = acc / np.maximum(win_rounds * reads, 1.0)
        win_rounds = 0
        return rate

    while done < int(num_sweeps):
        todo = min(step, int(num_sweeps) - done)
        batch.run(todo, seed=seed, use_pt=use_pt, graph_chunk=0,
                  final_recompute=False)
        done += todo
        if (done % train_every == 0 and st.train_steps < max_steps
                and st.enabled.any()):
            prop.observe()
        if not propose or done % interval or not st.enabled.any():
            continue
        prop.propose(seed, st.rounds)
        st.rounds += 1
        st.proposed += reads * st.enabled
        win_rounds += 1
        if win_rounds >= check_every:
            rate = settle()
            if st.train_steps >= min(min_train_steps, max_steps):
                low = st.enabled & (rate < min_accept)
                if low.any():
                    st.enabled &= ~low
                    prop.enabled.copy_(torch.from_numpy(
                        st.enabled.astype(np.int32)))
    if win_rounds:
        settle()
    if batch.tc and batch.tc_terms == 2:
        batch.recompute()
    return st
