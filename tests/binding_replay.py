"""Shared pieces of the binding tests (tests/test_gpu_binding.py,
tests/test_binding_cpu.py): the recorded reference driver calls of
tests/golden/binding.npz and the value-structure description they use."""
import json
import os

import numpy as np

from conftest import GOLDEN


def describe(x):
    """Nesting, Python type, dtype and shape of a value (the same record
    tests/golden/make_golden_binding.py writes)."""
    if isinstance(x, tuple):
        return ["tuple", [describe(v) for v in x]]
    if isinstance(x, np.ndarray):
        return ["ndarray", str(x.dtype), list(x.shape)]
    if isinstance(x, np.generic):
        return ["scalar", str(x.dtype)]
    return [type(x).__name__]


def load():
    d = np.load(os.path.join(GOLDEN, "binding.npz"), allow_pickle=False)
    meta = json.loads(str(d["meta"]))
    for case in meta:
        case["problem"] = d[case["name"] + "__problem"]
        for c, rec in enumerate(case["calls"]):
            rec["arrays"] = {k: d[f"{case['name']}__{c}__{k}"]
                             for k in ("couplings", "local_fields", "states",
                                       "energies", "beta_idx", "betas")}
    return meta


def oracle_expect(oracle, rec, seed):
    """What the GPU drivers must return for a recorded call: the oracle's
    chains on the same stream (f32 sweeps), reduced the way each reference
    driver reduces them."""
    a = rec["arrays"]
    ptype = "qubo" if rec["update_spin"].endswith("qubo.update_spin") else \
        "ising"
    update = "random" if rec["sweep"].endswith("random_sweep") else \
        "sequential"
    R, n = a["states"].shape
    glob = rec["driver"] == "sequential"
    out = oracle.pt_run(ptype, a["couplings"].astype(np.float32),
                        a["local_fields"].astype(np.float32),
                        a["betas"].astype(np.float32),
                        a["states"][None].astype(np.float32),
                        a["energies"][None].astype(np.float32),
                        np.arange(R, dtype=np.int32)[None], seed=seed,
                        num_sweeps=rec["n_sweeps"], update=update,
                        use_pt=rec["use_pt"],
                        best_mode="global" if glob else "replica",
                        log_omega=rec["get_part_fun"])
    be, bs = out["best_energy"][0], out["best_sweep"][0]
    e0 = np.float32(a["energies"][0])
    if glob:
        k = int(np.lexsort((np.arange(R), bs, be))[0])
        if not be[k] < e0:
            k = None
    else:
        k = int(np.argmin(be))
    best = (out["spins"][0][0], float(e0), 0) if k is None else \
        (out["best_spins"][0][k], float(be[k]), int(bs[k]))
    return dict(spins=out["spins"][0], energies=out["energies"][0],
                beta_idx=out["beta_idx"][0], best=best,
                log_omega=None if out["log_omega"] is None else
                out["log_omega"][0])
