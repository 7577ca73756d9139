"""Statistical parity on real-valued couplings.

With real couplings the GPU's split-BF16 tensor-core sweep and the reference
rule differ in the last bits of every field, so trajectories part ways and
parity is statistical: the GPU path must sample the same distribution as the
reference algorithm.  Three arms run on independent random streams:

  gpu   PTBatch (tensor-core sweep, J = J_hi + J_lo in BF16, FP32
        accumulation, in-kernel recompute every 4 sweeps)
  f32   the oracle's f32 driver (the reference's float32 arithmetic,
        pysa/sa.py:204-205 with float_type='float32')
  f64   the oracle's f64 driver (float_type='float64': f64 fields,
        energies and exchange)

Statistics per arm: each read's best energy, taken as the f64 energy of its
best state (pysa/simulation.py:174-181), and each temperature slot's final
energy.  Tests, all at alpha = 0.01 (two-sided):
  * Kolmogorov-Smirnov two-sample test of the per-read best energies;
  * hit rate at a target energy, the pooled 25 % quantile of every arm's
    best energies (a target each arm reaches on a fraction of its reads;
    the instances' temperature ranges do not reach a common ground state
    in these budgets): Fisher's exact test on the hit counts;
  * mean final energy of every temperature slot: Welch's t-test, Bonferroni
    corrected over the slots.
The seeds are fixed, so the outcome is deterministic.  The arms gpu/f64
answer whether the float32 sweeps of a float_type='float64' Solver sample
the reference's float64 distribution.
"""
import os

import numpy as np
import pytest

import stat_parity as sp

# PYSA_GB_STATS_FULL=1: the C1 configuration's own sizes (400 reads, 1000
# sweeps) instead of the quick test sizes; used for the recorded note
FULL = os.environ.get("PYSA_GB_STATS_FULL") == "1"

pytestmark = pytest.mark.gpu


def _run_arms(oracle, J, betas, Rd, S, seed):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    n, R = J.shape[0], len(betas)
    h = np.zeros(n, np.float32)
    rng = np.random.default_rng(seed)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    e0 = sp.e64(J, x0.reshape(-1, n)).reshape(Rd, R)
    bidx0 = np.tile(np.arange(R, dtype=np.int32), (Rd, 1))
    out = {}
    b = PTBatch("ising", [Instance(J, h, betas, Rd)])
    assert b.tc and b.tc_terms == 2
    b.set_states(pack_spins(x0, "ising", b.words), e0.astype(np.float32))
    b.run(S, seed=seed + 1)
    g = b.fetch()
    out["gpu"] = sp.arm_stats(
        J, g["best_energy"],
        unpack_spins(g["best_spins"], n, "ising", np.float32),
        unpack_spins(g["spins"], n, "ising", np.float32).reshape(Rd, R, n),
        g["beta_idx"])
    o = oracle.pt_run("ising", J, h, betas, x0, e0.astype(np.float32), bidx0,
                      seed=seed + 2, num_sweeps=S)
    out["f32"] = sp.arm_stats(J, o["best_energy"], o["best_spins"],
                              o["spins"], o["beta_idx"])
    o = oracle.pt_run64("ising", J, h, betas, x0, e0, bidx0, seed=seed + 3,
                        num_sweeps=S)
    out["f64"] = sp.arm_stats(J, o["best_energy"], o["best_spins"],
                              o["spins"], o["beta_idx"])
    return out


def test_sk128_statistically_indistinguishable(oracle):
    """SK N=128, J ~ N(0, 1)/sqrt(N), 32 replicas on T 1.0-3.5 (the C1
    ensemble), 256 reads, 200 sweeps."""
    J = sp.sk(128, 1)
    Rd, S = (400, 1000) if FULL else (256, 200)
    sp.assert_same(sp.compare(_run_arms(
        oracle, J, sp.ladder(32, 1.0, 3.5), Rd, S, 100), "sk128"), "sk128")


def test_wishart256_statistically_indistinguishable(oracle):
    """Planted Wishart N=256, M=128 (alpha 0.5), 32 replicas on T 0.05-1.0,
    256 reads, 100 sweeps."""
    J = sp.wishart(256, 128, 2)
    Rd, S = (400, 500) if FULL else (256, 100)
    sp.assert_same(sp.compare(_run_arms(
        oracle, J, sp.ladder(32, 0.05, 1.0), Rd, S, 200), "wishart256"),
        "wishart256")
