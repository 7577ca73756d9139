"""The reference-side binding on the GPU: recorded driver calls replayed.

tests/golden/binding.npz holds every call the reference's own
Solver.metropolis_update made to its driver (pysa/sa.py:329-332, :349-352)
on six keyword sets -- both drivers, both visiting orders, float32 and
float64, get_part_fun with beta0, recompute_energy, use_pt=False -- with the
arguments it passed, the structure of what the reference driver returned and
the structure of the frame rows it built (tests/golden/make_golden_binding.py).

Each recorded call is replayed through pysa_gb300.compat's GPU drivers, which
must (a) return the same nesting, types, dtypes and shapes, (b) update
states, energies and beta_idx in place and return those same arrays, and
(c) produce the oracle's chains on the same stream bit for bit (integer
couplings).  Then pysa_gb300.Solver, run with the same keywords, must build
frame rows of the recorded structure.
"""
import numpy as np
import pytest

import binding_replay as br

pytestmark = pytest.mark.gpu

CASES = br.load()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_replayed_driver_calls(oracle, case):
    from pysa_gb300 import compat
    seed = 5150
    compat.set_seed(seed)
    for c, rec in enumerate(case["calls"]):
        a = {k: np.copy(v) for k, v in rec["arrays"].items()}
        driver = (compat.simulation_parallel if rec["driver"] == "parallel"
                  else compat.simulation_sequential)
        mod = rec["update_spin"].rsplit(".", 1)[0]   # pysa.ising / pysa.qubo
        sweep = rec["sweep"].rsplit(".", 1)[1]       # random_sweep / ...
        states, energies, bidx = a["states"], a["energies"], a["beta_idx"]
        out = driver(mod, sweep, a["couplings"], a["local_fields"], states,
                     energies, bidx, a["betas"], rec["n_sweeps"],
                     rec["get_part_fun"], rec["use_pt"])
        assert br.describe(out) == rec["returns"]
        assert out[0][0] is states and out[0][1] is energies and \
            out[0][2] is bidx
        want = br.oracle_expect(oracle, rec, seed + c)
        assert (states == want["spins"]).all()
        assert (energies == want["energies"]).all()
        assert (bidx == want["beta_idx"]).all()
        best_state, best_energy, best_sweeps, ns = out[1]
        assert (best_state == want["best"][0]).all()
        assert float(best_energy) == want["best"][1]
        assert int(best_sweeps) == want["best"][2] and ns == rec["n_sweeps"]
        if rec["get_part_fun"]:
            np.testing.assert_allclose(out[0][3], want["log_omega"],
                                       rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_solver_frame_structure_matches_reference(case):
    from pysa_gb300 import Solver
    np.random.seed(1234)
    rows = Solver(case["problem"], case["problem_type"],
                  case["float_type"]).metropolis_update(
                      return_dataframe=False, seed=3, **case["kwargs"])
    got = [[k, br.describe(v)] for k, v in rows[0].items()]
    assert got == case["frame"]
