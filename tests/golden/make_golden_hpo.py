"""Golden outputs of the temperature heuristics and tuning objective of the
reference's HPO tutorial.

Run where the nasa/PySA source tree is available:

    python tests/golden/make_golden_hpo.py --reference /path/to/PySA

Executes the function definitions of tutorials/hpo_demo.ipynb
(get_delta_e_ising, get_delta_e_qubo, tts_objective_fcn) and its
temperature-range formula on the Wishart N=50 fixture and on seeded random
Ising / QUBO problems, and records the results in hpo.npz.
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def notebook_functions(path):
    nb = json.load(open(path))
    env = {"np": np}
    for cell in nb["cells"]:
        code = "".join(cell["source"])
        if cell["cell_type"] == "code" and code.lstrip().startswith("def ") \
                and ("get_delta_e" in code or "tts_objective_fcn" in code):
            exec(code, env)
    return env


class Dense(np.ndarray):
    """ndarray with the .A attribute the notebook's QUBO helper reads."""
    @property
    def A(self):
        return np.asarray(self)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYSA_REFERENCE"),
                    help="nasa/PySA source tree (or $PYSA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or PYSA_REFERENCE) is required")
    env = notebook_functions(os.path.join(args.reference, "tutorials",
                                          "hpo_demo.ipynb"))
    out = {}
    W = np.load(os.path.join(HERE, "wishart50.npz"))["problem"]
    rng = np.random.default_rng(12)
    cases = {"wishart": (W, np.zeros(W.shape[0]))}
    J = np.triu(rng.integers(-3, 4, (40, 40)).astype(float), 1)
    cases["ising_int"] = (J + J.T, rng.integers(-2, 3, 40).astype(float))
    J = np.triu(rng.normal(size=(30, 30)), 1)
    J[rng.random((30, 30)) < 0.6] = 0
    cases["ising_sparse"] = (J + J.T, np.zeros(30))
    for name, (J, h) in cases.items():
        for sc in (True, False):
            hot, cold, cnt = env["get_delta_e_ising"](J, h, sc)
            out[f"{name}_{int(sc)}"] = np.array([hot, cold, cnt], float)
        hot, cold, cnt = env["get_delta_e_ising"](J, h)
        out[f"{name}_range"] = np.array([-cold / np.log(1. / 100. / cnt),
                                         -hot / np.log(50. / 100.)])
        out[f"{name}_J"], out[f"{name}_h"] = J, h
    Q = np.triu(rng.integers(-5, 6, (25, 25)).astype(float))
    Q = Q + np.triu(Q, 1).T
    out["qubo_Q"] = Q
    out["qubo"] = np.array(env["get_delta_e_qubo"](Q.view(Dense)), float)
    energies = rng.normal(-100, 5, 64)
    objs = []
    for gs in (-100.0, -110.0, -90.0, -200.0):
        with contextlib.redirect_stdout(io.StringIO()):
            objs.append(env["tts_objective_fcn"](energies, 0.25, gs))
    out["tts_energies"] = energies
    out["tts_objective"] = np.array(objs)
    np.savez_compressed(os.path.join(HERE, "hpo.npz"), **out)
    print("hpo done", sorted(out))


if __name__ == "__main__":
    main()
