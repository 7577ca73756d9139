"""Tuning knobs of the sweep: parity with the oracle under every setting.

The autotuner (PTBatch.autotune) chooses the tensor-core threshold, the
chains per tensor-core CTA and the sweeps per work unit by timing; none of
them may change a trajectory.  The replica-exchange interval is an opt-in
knob with no counterpart in the reference (pysa/simulation.py:167-168
exchanges after every sweep): with exchange_every = k the oracle exchanges
only after sweeps s with (s + 1) % k == 0, and the GPU must match it bit for
bit on the fused tensor-core path and on the plain kernel.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _qubo(rng, n):
    Q = np.triu(rng.integers(-8, 9, (n, n)), 1)
    return (Q + Q.T).astype(np.float32), rng.integers(-16, 17, n).astype(
        np.float32)


def _check(oracle, b, J, h, betas, x0, e0, seed, sweeps, **ok):
    from pysa_gb300 import unpack_spins
    Rd, R, n = x0.shape
    got = b.fetch()
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=seed, num_sweeps=sweeps, **ok)
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, "qubo", np.float32)
    assert (sp == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()


def _setup(n, R, Rd, seed, kernel):
    from pysa_gb300 import Instance, PTBatch, pack_spins
    from oracle import oracle
    rng = np.random.default_rng(seed)
    J, h = _qubo(rng, n)
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    b = PTBatch("qubo", [Instance(J, h, betas, Rd)], kernel=kernel)
    b.set_states(pack_spins(x0, "qubo", b.words), e0)
    return b, J, h, betas, x0, e0


@pytest.mark.parametrize("n,kernel", [(1024, "tc"), (200, "plain")])
@pytest.mark.parametrize("every", [2, 3])
def test_exchange_interval_bit_exact(oracle, n, kernel, every):
    b, J, h, betas, x0, e0 = _setup(n, 64 if kernel == "tc" else 8, 2,
                                    50 + every, kernel)
    if kernel == "tc":
        assert b.ws.tc_fusable == 1
    b.run(20, seed=5, graph_chunk=0, exchange_every=every)
    _check(oracle, b, J, h, betas, x0, e0, 5, 20, exchange_every=every)


@pytest.mark.parametrize("item_chains", [32, 48])
def test_fixed_chains_per_cta_bit_exact(oracle, item_chains):
    """n = 1024 (64 chains per CTA at fold 2) with R = 16: items of 32
    chains (two reads), and 48 (three reads)."""
    b, J, h, betas, x0, e0 = _setup(1024, 16, 6, 60, "tc")
    b._setup_tc(64, item_chains)
    cnt = b.ws.tc_variant_count[1]
    assert cnt == -(-6 * 16 // item_chains)
    b.run(20, seed=6, graph_chunk=0)
    _check(oracle, b, J, h, betas, x0, e0, 6, 20)


def test_autotune_report_and_unchanged_results(oracle):
    b, J, h, betas, x0, e0 = _setup(1024, 32, 8, 61, "auto")
    b.autotune(sweeps=4, candidates=(64, None), item_chains=(0, 0.5),
               unit_sweeps=(0, 4, 8))
    rep = b.autotune_report
    assert set(rep["ms_per_sweep"]["threshold"]) == {64, None}
    assert rep["choice"]["exchange_every"] == 1
    if rep["choice"]["threshold"] is not None:
        assert set(rep["ms_per_sweep"]["unit_sweeps"]) == {0, 4, 8}
        assert set(rep["ms_per_sweep"]["item_chains"]) == {0, 32}
    b.run(24, seed=7, graph_chunk=0)
    _check(oracle, b, J, h, betas, x0, e0, 7, 24)
