"""TTS arithmetic against golden outputs of the reference's own nts,
raw_to_tts and tts_boots (tests/test_tts.py:171-277), recorded by
tests/golden/make_golden_tts.py."""
import json

import numpy as np
import pytest

from conftest import golden


def test_nts_raw_to_tts_and_bootstrap_match_reference():
    from pysa_gb300 import tts
    g = golden("tts")
    raw = json.loads(str(g["raw_json"]))
    for ptgt in (0.9, 0.99):
        key = str(ptgt).replace(".", "")
        assert np.array_equal(tts.nts(g["succ"], ptgt), g["nts_" + key])
        for set_name in (None, "s"):
            r = tts.raw_to_tts(raw, set_name=set_name, ptgt=ptgt)
            tag = key + "_" + (set_name or "all")
            for k in ("success_prob", "nts", "tts", "runtime_mean_seconds"):
                assert np.array_equal(r[k], g[f"raw_{tag}_{k}"]), (tag, k)
        r = tts.raw_to_tts(raw, ptgt=ptgt)
        np.random.seed(5)
        b = tts.tts_boots(r, 9, ptgt)
        assert np.isfinite(b).all()
        assert np.array_equal(b, g["boots_" + key])


def test_batch_tts_convention():
    from pysa_gb300 import tts
    best = np.array([[-10, -10, -9, -8], [-5, -5, -5, -5], [0, 1, 2, 3.0]])
    r = tts.batch_tts(best, [-10, -5, -1], t_batch=1.2, ptgt=0.99)
    assert r["t_run"] == 1.2 / 12
    assert np.allclose(r["success_prob"], [0.5, 1.0, 0.0])
    assert r["tts"][1] == r["t_run"]
    assert np.isclose(r["tts"][0], r["t_run"] * np.log(0.01) / np.log(0.5))
    assert np.isinf(r["tts"][2])
    assert r["solved_instances"] == 2


# ------------------------------------------------- HPO tutorial helpers
@pytest.mark.parametrize("name", ["wishart", "ising_int", "ising_sparse"])
def test_delta_e_and_temperature_range_match_reference(name):
    from pysa_gb300.tts import delta_e_ising, temperature_range
    g = golden("hpo")
    J, h = g[f"{name}_J"], g[f"{name}_h"]
    for sc in (1, 0):
        got = delta_e_ising(J, h, bool(sc))
        assert np.array_equal(np.array(got, float), g[f"{name}_{sc}"])
    hot, cold, cnt = delta_e_ising(J, h)
    assert np.allclose(temperature_range(hot, cold, cnt), g[f"{name}_range"],
                       rtol=0, atol=0)


def test_delta_e_qubo_matches_reference():
    from pysa_gb300.tts import delta_e_qubo
    g = golden("hpo")
    assert np.array_equal(np.array(delta_e_qubo(g["qubo_Q"]), float),
                          g["qubo"])


def test_tts_objective_matches_reference():
    from pysa_gb300.tts import tts_objective
    g = golden("hpo")
    got = [tts_objective(g["tts_energies"], 0.25, gs)
           for gs in (-100.0, -110.0, -90.0, -200.0)]
    assert np.array_equal(np.array(got), g["tts_objective"])
