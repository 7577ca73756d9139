"""Golden record of the reference's driver calls, for the binding tests.

pysa_gb300.compat replaces pysa.simulation.simulation_parallel and
simulation_sequential, the driver functions that pysa.sa.Solver picks at
pysa/sa.py:209-211 and calls at pysa/sa.py:329-332 / :349-352.  This script
runs the reference's own Solver.metropolis_update on several keyword sets
with those two functions wrapped by a recorder, and saves for every call

  * the arguments the Solver passed (problem tables, initial states and
    energies, beta_idx, betas, n_sweeps, get_part_fun, use_pt, and which
    update rule and sweep function it handed over),
  * the structure of what the reference driver returned (nesting, Python
    types, dtypes and shapes),
  * the structure of the frame rows the Solver built from it (column order,
    types, dtypes and shapes).

tests/test_gpu_binding.py replays the recorded calls through the GPU drivers
and requires the same structures, in-place updates and oracle trajectories;
tests/test_binding_cpu.py drives the reference's own Solver through the
binding where the reference source is at hand.

    python tests/golden/make_golden_binding.py --reference /path/to/PySA
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

# (name, problem type, n, generator, float_type, metropolis_update kwargs)
CASES = [
    ("qubo_par_seq", "qubo", 40, "qubo_int", "float32",
     dict(num_sweeps=15, num_reads=2, num_replicas=6, min_temp=0.5,
          max_temp=4.0, update_strategy="sequential")),
    ("ising_par_rand_sorted", "ising", 33, "pm1", "float64",
     dict(num_sweeps=12, num_reads=2, num_replicas=5, min_temp=0.3,
          max_temp=3.0, update_strategy="random", sort_output_temps=True)),
    ("ising_seq_driver", "ising", 24, "pm1", "float32",
     dict(num_sweeps=10, num_reads=2, num_replicas=4, min_temp=0.5,
          max_temp=2.0, update_strategy="sequential", parallel=False)),
    ("qubo_logz", "qubo", 20, "qubo_int", "float32",
     dict(num_sweeps=8, num_reads=2, num_replicas=6, min_temp=0.5,
          max_temp=3.0, update_strategy="sequential", get_part_fun=True,
          beta0=True)),
    ("qubo_recompute_f64", "qubo", 28, "qubo_int", "float64",
     dict(num_sweeps=9, num_reads=1, num_replicas=4, min_temp=0.5,
          max_temp=3.0, update_strategy="random", recompute_energy=True)),
    ("ising_nopt", "ising", 30, "pm1", "float32",
     dict(num_sweeps=7, num_reads=1, num_replicas=3, min_temp=0.5,
          max_temp=3.0, update_strategy="sequential", use_pt=False)),
]


def describe(x):
    """Nesting, Python type, dtype and shape of a value."""
    if isinstance(x, tuple):
        return ["tuple", [describe(v) for v in x]]
    if isinstance(x, np.ndarray):
        return ["ndarray", str(x.dtype), list(x.shape)]
    if isinstance(x, np.generic):
        return ["scalar", str(x.dtype)]
    return [type(x).__name__]


def problem(kind, n, rng):
    if kind == "qubo_int":
        Q = np.triu(rng.integers(-8, 9, (n, n)), 1)
        Q = Q + Q.T
        Q[np.diag_indices(n)] = rng.integers(-16, 17, n)
        return Q.astype(np.float64)
    P = np.triu(2 * rng.integers(0, 2, (n, n)) - 1, 1)
    P = P + P.T
    P[np.diag_indices(n)] = rng.integers(-2, 3, n)
    return P.astype(np.float64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYSA_REFERENCE"),
                    help="nasa/PySA source tree (or $PYSA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or PYSA_REFERENCE) is required")
    sys.path[:0] = [os.path.join(REPO, "oracle", "stubs"), args.reference]
    import sitecustomize  # noqa: F401
    import pysa.simulation as simulation
    import pysa.utils as utils
    from pysa.sa import Solver

    class _SeparateSweepRng:
        """numba keeps its own generator for np.random inside jitted code,
        so the sweeps never consume the global NumPy stream that the
        Solver's initial states come from; reproduce that split under the
        stubs (the recorded arguments then do not depend on the driver)."""

        def __init__(self, seed):
            self.random = np.random.RandomState(seed)

        def __getattr__(self, name):
            return getattr(np, name)

    simulation.np = _SeparateSweepRng(1)
    utils.np = _SeparateSweepRng(2)

    calls = []

    def recorder(fn, driver):
        def wrapped(update_spin, sweep, couplings, local_fields, states,
                    energies, beta_idx, betas, n_sweeps, get_part_fun=False,
                    use_pt=True):
            rec = dict(driver=driver,
                       update_spin=f"{update_spin.__module__}."
                                   f"{update_spin.__name__}",
                       sweep=f"{sweep.__module__}.{sweep.__name__}",
                       n_sweeps=int(n_sweeps), get_part_fun=bool(get_part_fun),
                       use_pt=bool(use_pt),
                       arrays=dict(couplings=np.copy(couplings),
                                   local_fields=np.copy(local_fields),
                                   states=np.copy(states),
                                   energies=np.copy(energies),
                                   beta_idx=np.copy(beta_idx),
                                   betas=np.copy(betas)),
                       arg_types=describe((couplings, local_fields, states,
                                           energies, beta_idx, betas)))
            out = fn(update_spin, sweep, couplings, local_fields, states,
                     energies, beta_idx, betas, n_sweeps, get_part_fun,
                     use_pt)
            rec["returns"] = describe(out)
            rec["in_place"] = [out[0][0] is states, out[0][1] is energies,
                               out[0][2] is beta_idx]
            calls.append(rec)
            return out
        return wrapped

    simulation.simulation_parallel = recorder(simulation.simulation_parallel,
                                              "parallel")
    simulation.simulation_sequential = recorder(
        simulation.simulation_sequential, "sequential")

    rng = np.random.default_rng(20250202)
    meta, arrays = [], {}
    for name, ptype, n, kind, ft, kw in CASES:
        P = problem(kind, n, rng)
        first = len(calls)
        np.random.seed(1234)
        rows = Solver(P, ptype, ft).metropolis_update(return_dataframe=False,
                                                      **kw)
        frame = [[k, describe(v)] for k, v in rows[0].items()]
        arrays[f"{name}__problem"] = P
        recs = []
        for c, rec in enumerate(calls[first:]):
            for k, v in rec.pop("arrays").items():
                arrays[f"{name}__{c}__{k}"] = v
            recs.append(rec)
        meta.append(dict(name=name, problem_type=ptype, float_type=ft,
                         kwargs=kw, calls=recs, frame=frame))
        print(name, len(recs), "driver calls")
    np.savez_compressed(os.path.join(HERE, "binding.npz"),
                        meta=json.dumps(meta), **arrays)


if __name__ == "__main__":
    main()
