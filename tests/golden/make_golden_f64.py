"""Golden trajectories of the reference's float64 arithmetic.

A Solver built with float_type='float64' casts couplings, fields, states and
betas to f64 (pysa/sa.py:204-205), so the reference's update_spin
(pysa/ising.py:40-63, pysa/qubo.py:40-63) forms the field, dn and the
acceptance test in f64 and the exchange (pysa/utils.py:44-58) uses f64
energies.  This script drives the reference's own update_spin on f64 arrays
with the shared Philox stream (the sweep loops of pysa/simulation.py:41-76
and the exchange restated, as make_golden.py does for float32) and records
the trajectories; tests/test_oracle_golden.py pins the oracle's f64 driver
(oracle.pt_run64) to them.  Real-valued couplings: the decisions must agree
(a different summation order of the f64 dot changes dn only in its last
bits), the energies to 1e-12 relative.

    python tests/golden/make_golden_f64.py --reference /path/to/PySA
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from make_golden import permutation, uniforms  # noqa: E402


def hook_pt64(mod, J, h, betas, states, energies, *, seed, sweeps, update):
    """simulation_parallel in f64 with the supplied stream."""
    reads, R, n = states.shape
    states = states.copy()
    energies = energies.copy()
    bidx = np.tile(np.arange(R, dtype=np.int32), (reads, 1))
    for s in range(sweeps):
        perm = permutation(seed, 0, s, n) if update == "random" else None
        for rd in range(reads):
            bsort = np.empty_like(betas)
            for k in range(R):
                bsort[bidx[rd, k]] = betas[k]
            for k in range(R):
                u = uniforms(seed, 0, 0, s, rd * R + k, n)
                de = 0.0
                for t in range(n):
                    pos = int(perm[t]) if perm is not None else t
                    de += mod.update_spin(J, h, states[rd, k], pos, bsort[k],
                                          np.log(u[t]))
                energies[rd, k] = energies[rd, k] + de
            u = uniforms(seed, 1, 0, s, rd, max(R - 1, 1))
            for k in range(R - 1):
                k1, k2 = R - k - 1, R - k - 2
                d = ((energies[rd, bidx[rd, k1]] - energies[rd, bidx[rd, k2]])
                     * (betas[k1] - betas[k2]))
                if d >= 0 or u[k] < np.exp(d):
                    bidx[rd, k1], bidx[rd, k2] = bidx[rd, k2], bidx[rd, k1]
    return dict(spins=states, energies=energies, beta_idx=bidx)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYSA_REFERENCE"),
                    help="nasa/PySA source tree (or $PYSA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or PYSA_REFERENCE) is required")
    sys.path[:0] = [os.path.join(REPO, "oracle", "stubs"), args.reference]
    import sitecustomize  # noqa: F401
    import pysa.ising as ising
    import pysa.qubo as qubo

    rng = np.random.default_rng(20250101)
    cases = [("pt_ising_f64_seq", "ising", 24, 6, 2, 25, "sequential", 31),
             ("pt_ising_f64_rand", "ising", 24, 6, 2, 25, "random", 32),
             ("pt_qubo_f64_seq", "qubo", 20, 5, 2, 25, "sequential", 33)]
    for name, ptype, n, R, reads, sweeps, update, seed in cases:
        mod = ising if ptype == "ising" else qubo
        P = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
        P = P + P.T
        P[np.diag_indices(n)] = 0.3 * rng.normal(size=n)
        h = np.copy(np.diag(P))
        J = np.copy(P)
        np.fill_diagonal(J, 0)
        ratio = np.exp(1 / (R - 1) * np.log(3.0 / 0.3))
        betas = np.array([1 / (0.3 * ratio**k) for k in range(R)], np.float64)
        r2 = np.random.default_rng(seed)
        if ptype == "ising":
            states = (2 * r2.integers(0, 2, (reads, R, n)) - 1).astype(
                np.float64)
        else:
            states = r2.integers(0, 2, (reads, R, n)).astype(np.float64)
        energies = np.array([[mod.get_energy(J, h, s) for s in rs]
                             for rs in states], np.float64)
        out = hook_pt64(mod, J, h, betas, states, energies, seed=seed,
                        sweeps=sweeps, update=update)
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            problem_type=ptype, J=J, h=h, betas=betas,
                            init_spins=states, init_energies=energies,
                            seed=seed, sweeps=sweeps, update=update, **out)
        print(name, "done")


if __name__ == "__main__":
    main()
