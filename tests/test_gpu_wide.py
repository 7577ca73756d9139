"""Instances beyond the register-resident kernel: parity with the oracle.

pysa.sa.Solver accepts any square symmetric problem (pysa/sa.py:57-70).
Dense instances up to 4096 spins sweep on the register-resident plain kernel
(or the tensor cores for 64 <= n <= 2048); wider ones on k_sweep_wide, whose
fields live in global memory.  Integer couplings make every field exact, so
trajectories must equal the oracle's (the reference's dense-dot rule on the
same Philox stream) bit for bit, in both visiting orders, alone and mixed in
one batch with instances of the other kernels.  n = 3072 is the size of the
reference's own published timing (tutorials/example_ising.ipynb:562-563).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _int_qubo(rng, n):
    Q = np.triu(rng.integers(-8, 9, (n, n)), 1)
    Q = (Q + Q.T).astype(np.float32)
    return Q, rng.integers(-16, 17, n).astype(np.float32)


def _pm1(rng, n):
    P = np.triu(2 * rng.integers(0, 2, (n, n)) - 1, 1)
    return (P + P.T).astype(np.float32), np.zeros(n, np.float32)


def _batch_vs_oracle(oracle, ptype, insts, sweeps, update, seed):
    """insts: [(J, h, betas, x0 [Rd, R, n])]; one PTBatch, per-instance
    oracle runs (instance index i keys instance i's streams)."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    b = PTBatch(ptype, [Instance(J, h, bt, x0.shape[0])
                        for J, h, bt, x0 in insts])
    words = b.words
    b.set_states(np.concatenate([pack_spins(x0, ptype, words).reshape(
        -1, words) for *_, x0 in insts]), None)
    b.run(sweeps, seed=seed, update=update)
    got = b.fetch()
    for i, (J, h, bt, x0) in enumerate(insts):
        Rd, R, n = x0.shape
        c0 = int(b.chain_off[i])
        sl = slice(c0, c0 + Rd * R)
        e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                      np.float32)
        want = oracle.pt_run(ptype, J, h, bt, x0, e0,
                             np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                             seed=seed, num_sweeps=sweeps, update=update,
                             inst=i)
        sp = unpack_spins(got["spins"][sl].reshape(Rd, R, -1), n, ptype,
                          np.float32)
        assert (sp == want["spins"]).all(), (i, n, "spins")
        assert (got["energies"][sl].reshape(Rd, R) == want["energies"]).all()
        assert (got["beta_idx"][sl].reshape(Rd, R) == want["beta_idx"]).all()
        assert (got["best_energy"][sl].reshape(Rd, R) ==
                want["best_energy"]).all()
        assert (got["best_sweep"][sl].reshape(Rd, R) ==
                want["best_sweep"]).all()
        bs = unpack_spins(got["best_spins"][sl].reshape(Rd, R, -1), n, ptype,
                          np.float32)
        assert (bs == want["best_spins"]).all(), (i, n, "best spins")
    return b


@pytest.mark.parametrize("update", ["sequential", "random"])
@pytest.mark.parametrize("n,ptype", [(3072, "ising"), (6000, "qubo"),
                                     (9001, "ising")])
def test_large_instance_bit_exact(oracle, n, ptype, update):
    rng = np.random.default_rng(n)
    J, h = _int_qubo(rng, n) if ptype == "qubo" else _pm1(rng, n)
    R, Rd = 5, 3                    # 15 chains: a partial wide work item
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    if ptype == "qubo":
        x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    else:
        x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    b = _batch_vs_oracle(oracle, ptype, [(J, h, betas, x0)], 3, update,
                         seed=n + 1)
    if n > 4096:
        assert b.ws.wide_item_count == 2


def test_mixed_batch_with_wide_instance(oracle):
    """A wide, a register-resident and two tensor-core instances in one
    batch, sequential sweeps (tensor cores and plain kernels in the same
    sweep) and random sweeps."""
    rng = np.random.default_rng(5)
    insts = []
    for n, R, Rd in ((5000, 3, 2), (3000, 4, 2), (700, 6, 3), (256, 4, 5)):
        J, h = _int_qubo(rng, n)
        bt = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
        insts.append((J, h, bt, rng.integers(0, 2, (Rd, R, n)).astype(
            np.float32)))
    for update in ("sequential", "random"):
        b = _batch_vs_oracle(oracle, "qubo", insts, 4, update, seed=17)
        assert b.ws.wide_item_count == 1 and b.tc


def test_solver_n6000_float64_energies():
    """Through Solver: float64 runs report the exact f64 energies of the
    returned states, also on the wide-instance kernel."""
    from pysa_gb300 import Solver
    rng = np.random.default_rng(6)
    n = 6000
    J, _ = _pm1(rng, n)
    P = J.astype(np.float64)
    P[np.diag_indices(n)] = rng.integers(-2, 3, n)
    np.random.seed(3)
    rows = Solver(P, "ising", "float64").metropolis_update(
        num_sweeps=2, num_reads=2, num_replicas=4, min_temp=0.5,
        max_temp=3.0, update_strategy="sequential", return_dataframe=False,
        seed=9)
    h = np.diag(P)
    J64 = P - np.diag(h)
    for r in rows:
        S = np.asarray(r["states"], np.float64)
        E = np.einsum("ri,ij,rj->r", S, J64, S) / 2 + S @ h
        assert np.array_equal(np.asarray(r["energies"]), E)
        b = np.asarray(r["best_state"], np.float64)
        assert float(r["best_energy"]) == float(b @ J64 @ b / 2 + b @ h)
