"""The reference's own Solver driven through the binding, on the CPU.

pysa_gb300.compat.install() points pysa.simulation.simulation_parallel and
simulation_sequential at the GPU drivers.  Here the reference source tree
($PYSA_REFERENCE, imported under oracle/stubs) is at hand but no GPU is, so
compat's chain runner is swapped for the oracle on the same stream (test
infrastructure only) and the reference's unmodified Solver.metropolis_update
(pysa/sa.py:92-430) runs end to end on the six keyword sets of
tests/golden/binding.npz.  Checked: the Solver passes the driver the
recorded arguments, the frames have the recorded columns, types, dtypes and
shapes, the energies are the energies of the returned states
(pysa/ising.py:32-37), and the best state's energy is the best energy.  The
GPU half of the same calls is tests/test_gpu_binding.py.  Skipped where the
reference source is absent.
"""
import os
import sys

import numpy as np
import pytest

import binding_replay as br

REF = os.environ.get("PYSA_REFERENCE")
pytestmark = pytest.mark.skipif(
    not REF or not os.path.isdir(os.path.join(REF, "pysa")),
    reason="reference source tree not given (PYSA_REFERENCE)")

CASES = br.load()


@pytest.fixture(scope="module")
def reference():
    from conftest import ROOT
    sys.path[:0] = [os.path.join(ROOT, "oracle", "stubs"), REF]
    import sitecustomize  # noqa: F401
    import pysa.sa
    import pysa.simulation
    yield pysa
    for p in (os.path.join(ROOT, "oracle", "stubs"), REF):
        sys.path.remove(p)


def _oracle_backend(oracle):
    def run(ptype, update, J, h, betas, states, energies, n_sweeps, use_pt,
            log_omega, best_global, seed):
        R, n = states.shape
        Jf = np.asarray(J, np.float32)
        hf = np.asarray(h, np.float32)
        out = oracle.pt_run(ptype, Jf, hf, np.asarray(betas, np.float32),
                            np.asarray(states, np.float32)[None],
                            np.asarray(energies, np.float32)[None],
                            np.arange(R, dtype=np.int32)[None], seed=seed,
                            num_sweeps=n_sweeps, update=update,
                            use_pt=bool(use_pt),
                            best_mode="global" if best_global else "replica",
                            log_omega=bool(log_omega))
        return dict(spins=out["spins"][0].astype(np.float64),
                    energies=out["energies"][0], beta_idx=out["beta_idx"][0],
                    best_energy=out["best_energy"][0],
                    best_sweep=out["best_sweep"][0],
                    best_spins=out["best_spins"][0].astype(np.float64),
                    log_omega=None if out["log_omega"] is None else
                    out["log_omega"][0],
                    energy64=lambda x: np.array(
                        [oracle.energy64(Jf, hf, s) for s in x]))
    return run


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_reference_solver_through_binding(reference, oracle, case,
                                          monkeypatch):
    from pysa_gb300 import compat
    monkeypatch.setattr(compat, "_backend", _oracle_backend(oracle))
    seen = []
    real_run = compat._run

    def spy(*args):
        seen.append([np.copy(x) for x in args[2:8]])
        return real_run(*args)
    monkeypatch.setattr(compat, "_run", spy)
    originals = compat.install(reference.simulation)
    try:
        compat.set_seed(99)
        np.random.seed(1234)
        rows = reference.sa.Solver(case["problem"], case["problem_type"],
                                   case["float_type"]).metropolis_update(
                                       return_dataframe=False,
                                       **case["kwargs"])
    finally:
        compat.uninstall(reference.simulation, originals)
        compat.set_seed(None)
    assert len(seen) == len(case["calls"])
    keys = ("couplings", "local_fields", "states", "energies", "beta_idx",
            "betas")
    for got, rec in zip(seen, case["calls"]):
        for k, v in zip(keys, got):
            assert np.array_equal(v, rec["arrays"][k]), k
    assert [[k, br.describe(v)] for k, v in rows[0].items()] == case["frame"]
    solver = reference.sa.Solver(case["problem"], case["problem_type"],
                                 case["float_type"])
    for r in rows:
        for s, e in zip(r["states"], r["energies"]):
            assert float(solver.get_energy(s)) == float(e)
        assert float(solver.get_energy(r["best_state"])) == \
            float(r["best_energy"])
