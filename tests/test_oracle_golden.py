"""The CPU oracle reproduces the reference's own update rule (golden vectors).

The golden files were produced by tests/golden/make_golden.py, which drives
pysa.ising.update_spin / pysa.qubo.update_spin (pysa/ising.py:40-63,
pysa/qubo.py:40-63) and update_spin_ref (pysa/ising.py:66-92) with the shared
Philox stream.  Integer couplings make every comparison exact.
"""
import numpy as np
import pytest

from conftest import golden

PT_CASES = ["pt_qubo_seq", "pt_qubo_rand", "pt_ising_seq", "pt_ising_rand",
            "pt_qubo64_nopt", "pt_ising_logz"]
AIS_CASES = ["ais_ising_uniform", "ais_qubo_bernoulli", "ais_ising_bernoulli"]


def test_philox_known_answers(oracle):
    g = golden("philox")
    for row, want in zip(g["kat_in"], g["kat_out"]):
        got = oracle.philox(row[:4], row[4:])
        assert (got == want).all()
    for tag in range(4):
        got = [oracle.draw(12345, tag, 3, 7, 11, i) for i in range(64)]
        assert (np.array(got, np.uint32) == g["stream"][tag]).all()
    for s in range(4):
        assert (oracle.permutation(99, 2, s, 37) == g["perms"][s]).all()


@pytest.mark.parametrize("name", PT_CASES)
def test_pt_trajectory_matches_reference(oracle, name):
    g = golden(name)
    out = oracle.pt_run(str(g["problem_type"]), g["J"], g["h"], g["betas"],
                        g["init_spins"], g["init_energies"],
                        np.tile(np.arange(g["betas"].size, dtype=np.int32),
                                (g["init_spins"].shape[0], 1)),
                        seed=int(g["seed"]), num_sweeps=int(g["sweeps"]),
                        update=str(g["update"]), use_pt=bool(g["use_pt"]),
                        log_omega=bool(g["log_omega_on"]))
    assert (out["spins"] == g["spins"]).all()
    assert (out["energies"] == g["energies"]).all()
    assert (out["beta_idx"] == g["beta_idx"]).all()
    assert (out["best_energy"] == g["best_energy"]).all()
    assert (out["best_sweep"] == g["best_sweep"]).all()
    assert (out["best_spins"] == g["best_spins"]).all()
    if bool(g["log_omega_on"]):
        # the reference under the numba stand-in sums log-omega in f32 where
        # numba sums in f64; the oracle follows numba
        np.testing.assert_allclose(out["log_omega"], g["log_omega"],
                                   rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("name", AIS_CASES)
def test_ais_matches_reference(oracle, name):
    g = golden(name)
    samples, lw = oracle.ais_run(str(g["problem_type"]), g["J"], g["h"],
                                 g["temps"], g["init"], seed=int(g["seed"]),
                                 update=str(g["update"]), ref=str(g["ref"]),
                                 p=float(g["p"]))
    assert (samples == g["samples"]).all()
    np.testing.assert_allclose(lw, g["log_w"], rtol=1e-9, atol=1e-9)
    logz = oracle.omegas_to_partition(lw, float(g["logz0"]))
    assert abs(logz - float(g["logz"])) < 1e-9


def test_energy64_matches_reference_energy(oracle):
    g = golden("pt_qubo64_nopt")
    for s, e in zip(g["spins"].reshape(-1, g["J"].shape[0]),
                    g["energies"].reshape(-1)):
        assert oracle.energy64(g["J"], g["h"], s) == float(e)


def test_logz_exact_small(oracle):
    rng = np.random.default_rng(3)
    n = 10
    J = rng.normal(size=(n, n)).astype(np.float32)
    J = np.triu(J, 1)
    J = J + J.T
    h = rng.normal(size=n).astype(np.float32)
    for ptype, vals in (("ising", (-1.0, 1.0)), ("qubo", (0.0, 1.0))):
        grid = np.array(np.meshgrid(*[vals] * n, indexing="ij")).reshape(n, -1).T
        E = np.einsum("si,ij,sj->s", grid, J.astype(np.float64), grid) / 2 + grid @ h
        want = np.log(np.sum(np.exp(-0.7 * E)))
        assert abs(oracle.logz_exact(ptype, J, h, 0.7) - want) < 1e-9


@pytest.mark.parametrize("name", ["pt_ising_f64_seq", "pt_ising_f64_rand",
                                  "pt_qubo_f64_seq"])
def test_pt_f64_trajectory_matches_reference(oracle, name):
    """The oracle's f64 driver (float_type='float64' arithmetic) against the
    reference's update_spin run on f64 arrays with real couplings
    (tests/golden/make_golden_f64.py): same decisions, energies to 1e-12
    relative (the two f64 dots sum in different orders)."""
    g = golden(name)
    reads, R, _ = g["init_spins"].shape
    out = oracle.pt_run64(str(g["problem_type"]), g["J"], g["h"], g["betas"],
                          g["init_spins"], g["init_energies"],
                          np.tile(np.arange(R, dtype=np.int32), (reads, 1)),
                          seed=int(g["seed"]), num_sweeps=int(g["sweeps"]),
                          update=str(g["update"]))
    assert (out["spins"] == g["spins"]).all()
    assert (out["beta_idx"] == g["beta_idx"]).all()
    np.testing.assert_allclose(out["energies"], g["energies"], rtol=1e-12,
                               atol=1e-12)
