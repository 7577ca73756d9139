"""CUDA path vs the CPU oracle on the same Philox stream (bit-exact on
integer couplings), and vs the reference's golden trajectories.

Every call goes through the C ABI of libpysa_gb (PTBatch -> pysa_gb_setup /
pysa_gb_prepare / pysa_gb_sweeps).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _int_qubo(rng, n, lo=-8, hi=8, dlo=-16, dhi=16):
    Q = rng.integers(lo, hi + 1, (n, n))
    Q = np.triu(Q, 1)
    Q = (Q + Q.T).astype(np.float32)
    return Q, rng.integers(dlo, dhi + 1, n).astype(np.float32)


def _pm1_ising(rng, n):
    P = rng.integers(0, 2, (n, n))
    P = np.triu(2 * P - 1, 1)
    P = (P + P.T).astype(np.float32)
    return P, np.zeros(n, np.float32)


def _run_both(oracle, ptype, J, h, betas, x0, *, seed, sweeps, update,
              use_pt=True, log_omega=False, best_global=False):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    Rd, R, n = x0.shape
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    b = PTBatch(ptype, [Instance(J, h, betas, Rd)])
    b.set_states(pack_spins(x0, ptype, b.words), None,
                 best_global=best_global)
    b.run(sweeps, seed=seed, update=update, use_pt=use_pt,
          log_omega=log_omega)
    got = b.fetch()
    want = oracle.pt_run(ptype, J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=seed, num_sweeps=sweeps, update=update,
                         use_pt=use_pt, log_omega=log_omega,
                         best_mode="global" if best_global else "replica")
    words = b.words
    got["spins_f"] = unpack_spins(got["spins"].reshape(Rd, R, words), n,
                                  ptype, np.float32)
    got["best_f"] = unpack_spins(got["best_spins"].reshape(Rd, R, words), n,
                                 ptype, np.float32)
    return got, want


def _assert_same(got, want, Rd, R):
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (got["best_f"] == want["best_spins"]).all()


# one size per kernel variant (columns per lane 1, 2, 4, ..., 128)
@pytest.mark.parametrize("n", [24, 50, 100, 200, 400, 1000, 1500, 3000])
@pytest.mark.parametrize("update", ["sequential", "random"])
def test_qubo_bit_exact_all_variants(oracle, n, update):
    rng = np.random.default_rng(n)
    J, h = _int_qubo(rng, n)
    R = 6 if n <= 1000 else 3
    Rd = 3 if n <= 1000 else 1
    sweeps = 12 if n <= 1000 else 4
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    got, want = _run_both(oracle, "qubo", J, h, betas, x0, seed=n + 1,
                          sweeps=sweeps, update=update)
    _assert_same(got, want, Rd, R)


@pytest.mark.parametrize("update", ["sequential", "random"])
def test_ising_pm1_bit_exact(oracle, update):
    rng = np.random.default_rng(5)
    n, R, Rd = 128, 32, 4
    J, h = _pm1_ising(rng, n)
    betas = (1.0 / np.geomspace(0.3, 3.0, R)).astype(np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    got, want = _run_both(oracle, "ising", J, h, betas, x0, seed=99,
                          sweeps=30, update=update)
    _assert_same(got, want, Rd, R)


def test_graph_replay_matches_direct(oracle):
    """> 2 graph chunks: sweeps replayed from a captured CUDA graph."""
    rng = np.random.default_rng(11)
    n, R, Rd = 64, 8, 4
    J, h = _int_qubo(rng, n, -3, 3, -4, 4)
    betas = (1.0 / np.geomspace(0.5, 4.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    got, want = _run_both(oracle, "qubo", J, h, betas, x0, seed=3, sweeps=150,
                          update="sequential")
    _assert_same(got, want, Rd, R)


def test_log_omega_and_global_best(oracle):
    rng = np.random.default_rng(12)
    n, R, Rd = 40, 7, 3
    J, h = _pm1_ising(rng, n)
    betas = np.append(1.0 / np.geomspace(0.5, 4.0, R - 1), 0.0).astype(
        np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    got, want = _run_both(oracle, "ising", J, h, betas, x0, seed=8, sweeps=20,
                          update="random", log_omega=True, best_global=True)
    _assert_same(got, want, Rd, R)
    np.testing.assert_allclose(got["log_omega"], want["log_omega"], rtol=0,
                               atol=1e-12)


def test_no_pt(oracle):
    rng = np.random.default_rng(13)
    J, h = _int_qubo(rng, 90)
    betas = (1.0 / np.geomspace(0.5, 8.0, 5)).astype(np.float32)
    x0 = rng.integers(0, 2, (2, 5, 90)).astype(np.float32)
    got, want = _run_both(oracle, "qubo", J, h, betas, x0, seed=21, sweeps=10,
                          update="sequential", use_pt=False)
    _assert_same(got, want, 2, 5)


def test_uneven_batch_matches_per_instance(oracle):
    """Several instances of different n in one batch (several variants)."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    rng = np.random.default_rng(14)
    sizes, R, Rd, S = [37, 130, 300, 64], 4, 2, 8
    insts, x0s = [], []
    for n in sizes:
        J, h = _int_qubo(rng, n)
        betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
        insts.append(Instance(J, h, betas, Rd))
        x0s.append(rng.integers(0, 2, (Rd, R, n)).astype(np.float32))
    b = PTBatch("qubo", insts)
    words = b.words
    allw = np.concatenate([pack_spins(x, "qubo", words).reshape(-1, words)
                           for x in x0s])
    b.set_states(allw, None)
    b.run(S, seed=77, update="random")
    got = b.fetch()
    c0 = 0
    for i, (inst, x0) in enumerate(zip(insts, x0s)):
        n = len(inst.h)
        e0 = np.array([[oracle.energy64(inst.J, inst.h, s) for s in r]
                       for r in x0], np.float32)
        want = oracle.pt_run("qubo", inst.J, inst.h, inst.ladder, x0, e0,
                             np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                             seed=77, num_sweeps=S, update="random", inst=i)
        sl = slice(c0, c0 + R * Rd)
        sp = unpack_spins(got["spins"][sl].reshape(Rd, R, words), n, "qubo",
                          np.float32)
        assert (sp == want["spins"]).all(), f"instance {i}"
        assert (got["energies"][sl].reshape(Rd, R) == want["energies"]).all()
        assert (got["beta_idx"][sl].reshape(Rd, R) == want["beta_idx"]).all()
        c0 += R * Rd


@pytest.mark.parametrize("name", ["pt_qubo_seq", "pt_qubo_rand",
                                  "pt_ising_seq", "pt_ising_rand",
                                  "pt_qubo64_nopt", "pt_ising_logz"])
def test_golden_reference_trajectories(name):
    """GPU against trajectories made by the reference's own update_spin."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    g = golden(name)
    ptype = str(g["problem_type"])
    x0 = g["init_spins"]
    Rd, R, n = x0.shape
    b = PTBatch(ptype, [Instance(g["J"], g["h"], g["betas"], Rd)])
    b.set_states(pack_spins(x0, ptype, b.words), g["init_energies"])
    b.run(int(g["sweeps"]), seed=int(g["seed"]), update=str(g["update"]),
          use_pt=bool(g["use_pt"]), log_omega=bool(g["log_omega_on"]))
    got = b.fetch()
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, ptype, np.float32)
    assert (sp == g["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == g["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == g["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == g["best_energy"]).all()
    if bool(g["log_omega_on"]):
        np.testing.assert_allclose(got["log_omega"], g["log_omega"],
                                   rtol=1e-6, atol=1e-6)
