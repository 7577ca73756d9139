"""Generate the golden vectors in tests/golden/ from the reference itself.

Run in a container where the nasa/PySA source tree is available (numba,
pandas and more_itertools may be absent: oracle/stubs stands in for them):

    python tests/golden/make_golden.py --reference /path/to/PySA

What it records
---------------
* philox.npz     -- Random123 Philox4x32-10 known answers plus draws of the
                    stream spec, computed here by an independent NumPy
                    implementation.
* pt_*.npz       -- parallel-tempering trajectories.  The sweep loops of
                    pysa/simulation.py:41-76 and the exchange of
                    pysa/utils.py:44-58 are restated with a SUPPLIED uniform
                    stream and permutation, and every spin attempt is made by
                    the reference's own update_spin (pysa/ising.py:40-63,
                    pysa/qubo.py:40-63); initial energies by its get_energy
                    and log-omega by its get_log_omega (pysa/ais.py:79-112).
* ais_*.npz      -- annealed importance sampling (pysa/simulation.py:293-317)
                    with the reference's update_spin_ref, ref_prob and
                    get_energy on the supplied stream.
* solver_*.npz   -- whole Solver.metropolis_update frames on problems whose
                    outcome does not depend on the sweep RNG (J = h = 0: every
                    attempt has dn = 0 and is accepted, every exchange has
                    de = 0 and swaps), pinning initial-state draws, the ladder,
                    the temps column (including its inverse-permutation order
                    when unsorted), best tracking and log_Zf.
* wishart50.npz  -- the planted Wishart N=50 instance shipped in the
                    reference's tutorials with its ground-state energy.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

# ------------------------------------------------------ independent Philox
M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox_np(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint64 arrays holding 32-bit words."""
    c = [np.asarray(x, np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k0, k1 = int(k0) & 0xFFFFFFFF, int(k1) & 0xFFFFFFFF
    for r in range(10):
        if r:
            k0 = (k0 + W0) & 0xFFFFFFFF
            k1 = (k1 + W1) & 0xFFFFFFFF
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ np.uint64(k0), lo1, hi0 ^ c[3] ^ np.uint64(k1), lo0]
    return [x.astype(np.uint32) for x in c]


def draws(seed, tag, inst, a, b, count):
    idx = np.arange(count, dtype=np.uint64)
    out = philox_np(idx >> np.uint64(2), np.full(count, a), np.full(count, b),
                    np.full(count, (inst << 4) | tag), seed & 0xFFFFFFFF,
                    seed >> 32)
    stacked = np.stack(out, axis=1)
    return stacked[np.arange(count), (idx & np.uint64(3)).astype(np.int64)]


def uniforms(seed, tag, inst, a, b, count):
    return (draws(seed, tag, inst, a, b, count).astype(np.float64) +
            0.5) * 2.0**-32


def permutation(seed, inst, sweep, n):
    p = np.arange(n, dtype=np.int32)
    if n > 1:
        x = draws(seed, 2, inst, sweep, 0, n)
    for i in range(n - 1, 0, -1):
        j = (int(x[i]) * (i + 1)) >> 32
        p[i], p[j] = p[j], p[i]
    return p


# --------------------------------------------------------- hook drivers
def hook_pt(mod, get_log_omega, J, h, betas, states, energies, *, seed,
            sweeps, update, use_pt, log_omega, inst=0):
    """simulation_parallel with the supplied stream; reads are independent."""
    reads, R, n = states.shape
    states = states.copy()
    energies = energies.copy()
    bidx = np.tile(np.arange(R, dtype=np.int32), (reads, 1))
    best_e = energies.copy()
    best_s = np.zeros((reads, R), np.int32)
    best_x = states.copy()
    lo = np.zeros((reads, sweeps))
    for s in range(sweeps):
        perm = permutation(seed, inst, s, n) if update == "random" else None
        for rd in range(reads):
            bsort = np.empty_like(betas)
            for k in range(R):
                bsort[bidx[rd, k]] = betas[k]
            for k in range(R):
                chain = rd * R + k
                u = uniforms(seed, 0, inst, s, chain, n)
                de = np.float64(0.0)  # numba types the sweep sum as f64
                for t in range(n):
                    pos = int(perm[t]) if perm is not None else t
                    # the reference's own spin update; beta passed as f64 so
                    # beta * dn is formed exactly as numba does (f64)
                    de += mod.update_spin(J, h, states[rd, k], pos,
                                          np.float64(bsort[k]), np.log(u[t]))
                energies[rd, k] = np.float32(np.float64(energies[rd, k]) + de)
                if energies[rd, k] < best_e[rd, k]:
                    best_e[rd, k] = energies[rd, k]
                    best_x[rd, k] = states[rd, k]
                    best_s[rd, k] = s
            if use_pt:
                u = uniforms(seed, 1, inst, s, rd, max(R - 1, 1))
                for k in range(R - 1):
                    k1, k2 = R - k - 1, R - k - 2
                    d = np.float32(
                        (energies[rd, bidx[rd, k1]] - energies[rd, bidx[rd, k2]])
                        * (betas[k1] - betas[k2]))
                    if d >= 0 or u[k] < np.exp(np.float64(d)):
                        bidx[rd, k1], bidx[rd, k2] = bidx[rd, k2], bidx[rd, k1]
            if log_omega:
                lo[rd, s] = get_log_omega(betas, bidx[rd], energies[rd])
    return dict(spins=states, energies=energies, beta_idx=bidx,
                best_energy=best_e, best_sweep=best_s, best_spins=best_x,
                log_omega=lo)


def hook_ais(mod, ais, J, h, temps, init, *, seed, update, ref, p, inst=0):
    """ais_sample (pysa/simulation.py:293-317) with the supplied stream."""
    if ref == "uniform":
        ref_prob = ais.uniform_ref_prob
    else:
        def ref_prob(state, pos=-1):
            return ais.bernoulli_ref_prob(state, p, pos)
    ns, n = init.shape
    samples = init.copy()
    lw = np.zeros(ns)
    perms = [permutation(seed, inst, k, n) for k in range(len(temps))
             ] if update == "random" else None
    for i in range(ns):
        state = samples[i]
        log_omega = 0.0
        beta_old = np.float32(0)
        for k, beta in enumerate(temps):
            u = uniforms(seed, 3, inst, k, i, n)
            for t in range(n):
                pos = int(perms[k][t]) if perms is not None else t
                mod.update_spin_ref(J, h, state, pos, np.float64(beta),
                                    np.log(u[t]), ref_prob)
            cur = np.float32(mod.get_energy(J, h, state))
            ref_e = -np.log(np.float64(ref_prob(state)))
            lk = np.float64(np.float32(-beta * cur)) - (1.0 - np.float64(beta)) * ref_e
            lm = np.float64(np.float32(-beta_old * cur)) - (
                1.0 - np.float64(beta_old)) * ref_e
            log_omega += lk - lm
            beta_old = beta
        lw[i] = log_omega
    return samples, lw


def geometric_betas(R, tmin, tmax):
    ratio = np.exp(1 / (R - 1) * np.log(tmax / tmin))
    return np.array([1 / (tmin * ratio**k) for k in range(R)], np.float32)


# ----------------------------------------------------------------- cases
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYSA_REFERENCE"),
                    help="nasa/PySA source tree (or $PYSA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or PYSA_REFERENCE) is required")
    sys.path[:0] = [os.path.join(REPO, "oracle", "stubs"), args.reference]
    import sitecustomize  # noqa: F401  (np.alltrue alias for NumPy 2)
    import pysa.ising as ising
    import pysa.qubo as qubo
    import pysa.ais as ais
    import pysa.simulation as simulation
    import pysa.utils as utils
    from pysa.sa import Solver

    class _SeparateSweepRng:
        """numba keeps its own generator for np.random inside jitted code, so
        the sweeps never consume the global NumPy stream that Solver's
        initial states come from; reproduce that split under the stubs."""

        def __init__(self, seed):
            self.random = np.random.RandomState(seed)

        def __getattr__(self, name):
            return getattr(np, name)

    simulation.np = _SeparateSweepRng(1)
    utils.np = _SeparateSweepRng(2)

    # Philox known answers (Random123 kat_vectors) and stream draws
    kat_in = np.array([[0, 0, 0, 0, 0, 0], [0xFFFFFFFF] * 6,
                       [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344,
                        0xa4093822, 0x299f31d0]], dtype=np.uint64)
    kat_out = np.array([[0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8],
                        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd],
                        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]],
                       dtype=np.uint32)
    for row, want in zip(kat_in, kat_out):
        got = np.array([x[()] for x in philox_np(*row)], np.uint32)
        assert (got == want).all(), (got, want)
    stream = np.stack([draws(12345, t, 3, 7, 11, 64) for t in range(4)])
    perms = np.stack([permutation(99, 2, s, 37) for s in range(4)])
    np.savez_compressed(os.path.join(HERE, "philox.npz"), kat_in=kat_in,
                        kat_out=kat_out, stream=stream, perms=perms)

    rng = np.random.default_rng(20240601)

    def qubo_int(n, lo=-8, hi=8, dlo=-16, dhi=16):
        Q = rng.integers(lo, hi + 1, (n, n))
        Q = np.triu(Q, 1)
        Q = Q + Q.T
        Q[np.diag_indices(n)] = rng.integers(dlo, dhi + 1, n)
        return Q.astype(np.float32)

    def ising_pm1(n):
        P = rng.integers(0, 2, (n, n))
        P = (P + P.T) % 2
        P = 2 * P - 1
        return P.astype(np.float32)

    cases = [
        ("pt_qubo_seq", "qubo", qubo_int(24), 4, 2, 20, "sequential", True,
         False, 11),
        ("pt_qubo_rand", "qubo", qubo_int(24), 4, 2, 20, "random", True, False,
         12),
        ("pt_ising_seq", "ising", ising_pm1(32), 6, 2, 12, "sequential", True,
         False, 13),
        ("pt_ising_rand", "ising", ising_pm1(32), 6, 2, 12, "random", True,
         False, 14),
        ("pt_qubo64_nopt", "qubo", qubo_int(64), 5, 2, 6, "sequential", False,
         False, 15),
        ("pt_ising_logz", "ising", ising_pm1(20), 5, 3, 10, "sequential", True,
         True, 16),
    ]
    for name, ptype, P, R, reads, sweeps, update, use_pt, lo, seed in cases:
        mod = ising if ptype == "ising" else qubo
        h = np.copy(np.diag(P)).astype(np.float32)
        J = np.copy(P)
        np.fill_diagonal(J, 0)
        n = len(P)
        if lo:
            betas = np.append(geometric_betas(R - 1, 0.5, 4.0), 0.0).astype(
                np.float32)
        else:
            betas = geometric_betas(R, 0.5, 4.0)
        r2 = np.random.default_rng(seed)
        if ptype == "ising":
            states = (2 * r2.integers(0, 2, (reads, R, n)) - 1).astype(np.float32)
        else:
            states = r2.integers(0, 2, (reads, R, n)).astype(np.float32)
        energies = np.array([[mod.get_energy(J, h, s) for s in rs]
                             for rs in states], np.float32)
        out = hook_pt(mod, ais.get_log_omega, J, h, betas, states, energies,
                      seed=seed, sweeps=sweeps, update=update, use_pt=use_pt,
                      log_omega=lo)
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            problem_type=ptype, J=J, h=h, betas=betas,
                            init_spins=states, init_energies=energies,
                            seed=seed, sweeps=sweeps, update=update,
                            use_pt=use_pt, log_omega_on=lo, **out)
        print(name, "done")

    ais_cases = [
        ("ais_ising_uniform", "ising", ising_pm1(10), 12, 16, "sequential",
         "uniform", 0.5, 2.0, 21),
        ("ais_qubo_bernoulli", "qubo", qubo_int(10, -3, 3, -4, 4), 10, 12,
         "random", "bernoulli", 0.3, 0.5, 22),
        ("ais_ising_bernoulli", "ising", ising_pm1(9), 8, 10, "sequential",
         "bernoulli", 0.4, 1.0, 23),
    ]
    for name, ptype, P, K, ns, update, ref, p, beta, seed in ais_cases:
        mod = ising if ptype == "ising" else qubo
        h = np.copy(np.diag(P)).astype(np.float32) * np.float32(beta)
        J = np.copy(P)
        np.fill_diagonal(J, 0)
        J = (J * np.float32(beta)).astype(np.float32)
        temps = np.array([(i + 1) / K for i in range(K)], np.float32)
        r2 = np.random.default_rng(seed)
        lo_v = -1 if ptype == "ising" else 0
        init = np.where(r2.random((ns, len(P))) < p, lo_v, 1).astype(np.float32)
        samples, lw = hook_ais(mod, ais, J, h, temps, init, seed=seed,
                               update=update, ref=ref, p=p)
        logz0 = ais.uniform_partition_fun(len(P)) if ref == "uniform" else 0.0
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            problem_type=ptype, J=J, h=h, temps=temps,
                            init=init, seed=seed, update=update, ref=ref, p=p,
                            samples=samples, log_w=lw,
                            logz=ais.omegas_to_partition(lw, logz0),
                            logz0=logz0)
        print(name, "done")

    # Solver frames that do not depend on the sweep RNG (J = h = 0)
    frames = [
        ("solver_ising_par", "ising", 7, dict(num_sweeps=3, num_reads=3,
                                              num_replicas=5, min_temp=0.5,
                                              max_temp=3.0,
                                              update_strategy="sequential",
                                              parallel=True)),
        ("solver_ising_seq_sorted", "ising", 6,
         dict(num_sweeps=4, num_reads=2, num_replicas=4, min_temp=0.3,
              max_temp=1.5, update_strategy="random", parallel=False,
              sort_output_temps=True)),
        ("solver_qubo_logz", "qubo", 5, dict(num_sweeps=2, num_reads=2,
                                             num_replicas=6, min_temp=0.4,
                                             max_temp=2.0,
                                             update_strategy="sequential",
                                             get_part_fun=True)),
        ("solver_qubo_ones", "qubo", 4, dict(num_sweeps=3, num_reads=1,
                                             num_replicas=3,
                                             initialize_strategy="ones",
                                             update_strategy="sequential")),
        ("solver_ising_r1", "ising", 8, dict(num_sweeps=2, num_reads=2,
                                             num_replicas=1,
                                             update_strategy="sequential")),
        ("solver_ising_r2_nopt", "ising", 8, dict(num_sweeps=5, num_reads=1,
                                                  num_replicas=2, use_pt=False,
                                                  update_strategy="sequential")),
    ]
    for name, ptype, n, kw in frames:
        P = np.zeros((n, n), np.float64)
        np.random.seed(4321)
        rows = Solver(P, ptype, "float32").metropolis_update(
            return_dataframe=False, **kw)
        out = {}
        for key in ("states", "energies", "best_state", "temps"):
            out[key] = np.stack([np.asarray(r[key]) for r in rows])
        out["best_energy"] = np.array([r["best_energy"] for r in rows])
        out["min_sweeps"] = np.array([r["min_sweeps"] for r in rows])
        out["num_sweeps"] = np.array([r["num_sweeps"] for r in rows])
        if "log_Zf" in rows[0]:
            out["log_Zf"] = np.array([r["log_Zf"] for r in rows])
        out["columns"] = np.array(list(rows[0].keys()))
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            problem_type=ptype, n=n, np_seed=4321,
                            kwargs=repr(kw), **out)
        print(name, "done")

    # planted Wishart fixture shipped with the reference tutorials
    tut = os.path.join(args.reference, "tutorials")
    raw = np.loadtxt(os.path.join(tut,
                                  "wishart_planting_N_50_alpha_0.50_inst_1.txt"))
    W = np.zeros((50, 50))
    for i, j, v in raw:
        W[int(i), int(j)] = v
    W = (W + W.T) / 2
    with open(os.path.join(tut, "gs_energies.txt")) as f:
        gs = float(f.read().split()[-1])
    np.savez_compressed(os.path.join(HERE, "wishart50.npz"), problem=W,
                        ground_energy_x2=gs)
    print("wishart50 done")


if __name__ == "__main__":
    main()
