"""AIS and exact log Z on the GPU.

* Trajectories and log weights of annealed importance sampling against the
  golden vectors made with the reference's update_spin_ref / ais_sample
  (pysa/simulation.py:293-317) on the shared stream.
* Exact log Z by enumeration against the CPU oracle.
* AIS estimates of log Z for SK instances at N=24, beta=2, 200 temperatures
  against the exact value; the reference's weight-after-sweep order is
  biased upward, the standard order is not.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ais_ising_uniform", "ais_qubo_bernoulli",
                                  "ais_ising_bernoulli"])
def test_ais_matches_reference_golden(name):
    from pysa_gb300.engine import run_ais
    g = golden(name)
    samples, lw = run_ais(str(g["problem_type"]), g["J"], g["h"], g["temps"],
                          g["init"], seed=int(g["seed"]),
                          update=str(g["update"]), reference=str(g["ref"]),
                          p=float(g["p"]))
    assert np.array_equal(samples, g["samples"])
    np.testing.assert_allclose(lw, g["log_w"], rtol=1e-9, atol=1e-9)


def _sk(rng, n):
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    return (J + J.T).astype(np.float32)


def test_logz_exact_matches_oracle(oracle):
    from pysa_gb300.engine import logz_exact
    rng = np.random.default_rng(4)
    insts = []
    for n in (10, 13, 16):
        insts.append((_sk(rng, n), (0.3 * rng.normal(size=n)).astype(np.float32)))
    for ptype in ("ising", "qubo"):
        got = logz_exact(ptype, insts, beta=1.7)
        for (J, h), v in zip(insts, got):
            want = oracle.logz_exact(ptype, J, h, 1.7)
            assert abs(v - want) < 1e-9 * max(1.0, abs(want))


def test_ais_estimate_vs_exact_n24():
    from pysa_gb300 import Solver
    from pysa_gb300.engine import logz_exact
    rng = np.random.default_rng(24)
    errs_ref, errs_std = [], []
    for k in range(3):
        J = _sk(rng, 24).astype(np.float64)
        exact = logz_exact("ising", [(J, np.zeros(24))], beta=2.0)[0]
        s = Solver(J, "ising", "float32")
        np.random.seed(k)
        lz_ref, samples, w = s.annealed_importance(200, 1024, "uniform",
                                                   beta=2.0, seed=k)
        np.random.seed(k)
        lz_std, _, _ = s.annealed_importance(200, 1024, "uniform", beta=2.0,
                                             seed=k, ais_order="standard")
        assert samples.shape == (1024, 24) and abs(sum(w) - 1) < 1e-9
        errs_ref.append(lz_ref - exact)
        errs_std.append(lz_std - exact)
    # the reference's weight-after-sweep order overshoots; standard order is
    # within the sampling error of 1024 samples
    assert max(abs(e) for e in errs_std) < 0.15, errs_std
    assert min(errs_ref) > -0.1 and np.mean(errs_ref) > np.mean(errs_std)


@pytest.mark.parametrize("update", ["sequential", "random"])
def test_batched_ais_matches_oracle_per_instance(oracle, update):
    """Several instances of different n and sample counts in one launch:
    each instance i follows the oracle's ais_run with instance index i (its
    own random streams), bit for bit on integer couplings."""
    from pysa_gb300.engine import run_ais_batch
    rng = np.random.default_rng(9)
    insts = []
    for n, ns in ((12, 40), (33, 17), (7, 64)):
        J = np.triu(rng.integers(-2, 3, (n, n)), 1)
        J = (J + J.T).astype(np.float32)
        h = rng.integers(-1, 2, n).astype(np.float32)
        x0 = (2 * rng.integers(0, 2, (ns, n)) - 1).astype(np.float32)
        insts.append((0.5 * J, 0.5 * h, x0))
    temps = np.linspace(0.05, 1.0, 15).astype(np.float32)
    got = run_ais_batch("ising", insts, temps, seed=1234, update=update,
                        reference="bernoulli", p=0.3)
    for i, ((J, h, x0), (samples, lw)) in enumerate(zip(insts, got)):
        want_s, want_lw = oracle.ais_run("ising", J, h, temps, x0, seed=1234,
                                         update=update, ref="bernoulli",
                                         p=0.3, inst=i)
        assert np.array_equal(samples, want_s), f"instance {i}"
        np.testing.assert_allclose(lw, want_lw, rtol=1e-9, atol=1e-9)
