"""Power of the statistical parity tests (tests/test_gpu_statistics.py).

The comparisons must tell a wrong sampler from a right one at the sizes the
GPU test uses.  A mistake is planted in the oracle, on the CPU: the "gpu" arm
runs the f32 oracle on a ladder whose temperatures are 10 % too high (every
beta scaled by 1/1.1), and the comparison must reject it; the same arm on
the right ladder and another stream must pass.  SK N=64 keeps the run to a
few seconds.
"""
import numpy as np

import stat_parity as sp


def _arms(oracle, J, betas, wrong_betas, Rd, S, seed):
    n, R = J.shape[0], len(betas)
    h = np.zeros(n, np.float32)
    rng = np.random.default_rng(seed)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    e0 = sp.e64(J, x0.reshape(-1, n)).reshape(Rd, R)
    b0 = np.tile(np.arange(R, dtype=np.int32), (Rd, 1))
    out = {}
    for name, lad, sd in (("gpu", wrong_betas, seed + 1),
                          ("f32", betas, seed + 2)):
        o = oracle.pt_run("ising", J, h, lad, x0, e0.astype(np.float32), b0,
                          seed=sd, num_sweeps=S)
        out[name] = sp.arm_stats(J, o["best_energy"], o["best_spins"],
                                 o["spins"], o["beta_idx"])
    o = oracle.pt_run64("ising", J, h, betas, x0, e0, b0, seed=seed + 3,
                        num_sweeps=S)
    out["f64"] = sp.arm_stats(J, o["best_energy"], o["best_spins"],
                              o["spins"], o["beta_idx"])
    return out


def test_comparison_rejects_a_planted_temperature_error(oracle):
    J = sp.sk(64, 4)
    betas = sp.ladder(16, 1.0, 3.5)
    rep = sp.compare(_arms(oracle, J, betas, (betas / 1.1).astype(np.float32),
                           256, 100, 40), "planted")
    for pair in ("gpu/f32", "gpu/f64"):
        pks, pf, pw, _, _ = rep[pair]
        assert min(pks, pf, pw) <= sp.ALPHA, pair
    sp.assert_same({"f32/f64": rep["f32/f64"]}, "planted")


def test_comparison_accepts_the_right_sampler(oracle):
    J = sp.sk(64, 4)
    betas = sp.ladder(16, 1.0, 3.5)
    sp.assert_same(sp.compare(_arms(oracle, J, betas, betas, 256, 100, 40),
                              "right"), "right")
