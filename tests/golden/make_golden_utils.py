"""Golden outputs of the reference's problem ingestion.

Run where the nasa/PySA source tree is available:

    python tests/golden/make_golden_utils.py --reference /path/to/PySA

Calls pysa.utils.get_problem_matrix (pysa/utils.py:61-89, with oracle/stubs
standing in for numba and more_itertools) on seeded interaction lists with
unsorted, gapped and mixed-sign labels and records the matrices, and the
lattice adjacency of tutorials/ising_tutorial.py:175-189 for two shapes, in
utils.npz.
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def lists(rng):
    out = []
    for k, nvar in enumerate((5, 12, 30)):
        labels = rng.choice(np.arange(-50, 200), nvar, replace=False)
        pairs = set()
        inst = []
        for _ in range(3 * nvar):
            a, b = rng.choice(labels, 2, replace=k == 2)
            key = tuple(sorted((int(a), int(b))))
            if key in pairs:
                continue
            pairs.add(key)
            inst.append((int(a), int(b), float(rng.integers(-9, 10))))
        out.append(inst)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYSA_REFERENCE"),
                    help="nasa/PySA source tree (or $PYSA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or PYSA_REFERENCE) is required")
    sys.path[:0] = [os.path.join(REPO, "oracle", "stubs"), args.reference]
    import sitecustomize  # noqa: F401
    from pysa import utils as ref_utils
    spec = importlib.util.spec_from_file_location(
        "ref_ising_tutorial",
        os.path.join(args.reference, "tutorials", "ising_tutorial.py"))
    out = {}
    rng = np.random.default_rng(31)
    for k, inst in enumerate(lists(rng)):
        out[f"inst{k}"] = np.array(inst, np.float64)
        out[f"problem{k}"] = ref_utils.get_problem_matrix(inst)
    try:
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        for m, n in ((3, 4), (5, 5)):
            out[f"lattice_{m}x{n}"] = mod.Ising2DwithPySA.matrix_to_adjacency(
                np.zeros((m, n)))
    except Exception as e:  # the tutorial module needs matplotlib
        print("lattice skipped:", e)
    np.savez_compressed(os.path.join(HERE, "utils.npz"), **out)
    print("utils done", sorted(out))


if __name__ == "__main__":
    main()
