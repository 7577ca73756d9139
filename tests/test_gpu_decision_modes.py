"""Both decision forms of the tensor-core sweep, each forced for a whole
run, bit for bit against the CPU oracle.

A 64-spin block is decided either in rounds over the whole block (every
undecided position tested against the current fields at once; the first one
not certainly rejected is decided, an accepted flip corrects all 64 fields)
or as four sequential 16-spin sub-blocks.  The default picks per block;
pysa_gb_set_decision_mode(1 or 2) forces one form.  Both must reproduce
pysa/simulation.py:150-171 with the rule of pysa/qubo.py:40-63 /
pysa/ising.py:40-63 exactly: integer couplings make every sum exact, so the
returned arrays must be equal.  The cases cover folds 1, 2 and 4, a last
block shorter than 64 spins, work items with unused chain slots, a beta = 0
slot (every flip accepted: 64 rounds in a block), the fused exchange and both
visiting orders.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def mode():
    from pysa_gb300 import _lib
    lib = _lib.load()
    yield lambda m: _lib.check(lib.pysa_gb_set_decision_mode(m), "mode")
    _lib.check(lib.pysa_gb_set_decision_mode(0), "mode reset")


def _case(oracle, ptype, n, R, Rd, sweeps, seed, update, betas=None):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    rng = np.random.default_rng(seed)
    if ptype == "qubo":
        J = np.triu(rng.integers(-8, 9, (n, n)), 1)
        J = (J + J.T).astype(np.float32)
        h = rng.integers(-16, 17, n).astype(np.float32)
        x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    else:
        J = np.triu(2 * rng.integers(0, 2, (n, n)) - 1, 1)
        J = (J + J.T).astype(np.float32)
        h = np.zeros(n, np.float32)
        x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    if betas is None:
        betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    b = PTBatch(ptype, [Instance(J, h, betas, Rd)], kernel="tc")
    assert b.tc and b.tc_terms == 1
    b.set_states(pack_spins(x0, ptype, b.words), e0)
    b.run(sweeps, seed=seed, update=update)
    got = b.fetch()
    want = oracle.pt_run(ptype, J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=seed, num_sweeps=sweeps, update=update)
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, ptype, np.float32)
    bs = unpack_spins(got["best_spins"].reshape(Rd, R, -1), n, ptype,
                      np.float32)
    assert (sp == want["spins"]).all(), "spins"
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (bs == want["best_spins"]).all(), "best spins"


@pytest.mark.parametrize("m", [1, 2])
def test_fold2_qubo1024_fused(oracle, mode, m):
    """The headline shape: fold 2, R = 64 (exchange fused), 40 sweeps."""
    mode(m)
    _case(oracle, "qubo", 1024, 64, 2, 40, 101, "sequential")


@pytest.mark.parametrize("m", [1, 2])
def test_fold4_qubo1300(oracle, mode, m):
    mode(m)
    _case(oracle, "qubo", 1300, 32, 2, 20, 102, "sequential")


@pytest.mark.parametrize("m", [1, 2])
def test_fold1_short_last_block_unused_slots_beta0(oracle, mode, m):
    """n = 300: the last block has 44 spins; 7 reads x 6 replicas leave
    unused chain slots in the work items; one slot has beta = 0."""
    mode(m)
    betas = np.concatenate([(1.0 / np.geomspace(0.5, 8.0, 5)),
                            [0.0]]).astype(np.float32)
    _case(oracle, "qubo", 300, 6, 7, 12, 103, "sequential", betas=betas)


@pytest.mark.parametrize("m", [1, 2])
@pytest.mark.parametrize("n", [256, 700])
def test_random_order_ising_pm1(oracle, mode, m, n):
    """Random visiting order at folds 1 and 2 (fields gathered by position)."""
    mode(m)
    _case(oracle, "ising", n, 4, 3, 37, 104 + n, "random")


def test_auto_mode_long_run_matches_oracle(oracle, mode):
    """The default per-block choice over a run that starts hot (many flips:
    sub-blocks) and cools (few flips: rounds)."""
    mode(0)
    _case(oracle, "qubo", 1024, 64, 2, 150, 105, "sequential")
