"""Golden vectors for the TTS arithmetic, from the reference's own functions.

Run where the nasa/PySA source tree is available:

    python tests/golden/make_golden_tts.py --reference /path/to/PySA

Imports nts, raw_to_tts and tts_boots from the reference's
tests/test_tts.py (with oracle/stubs standing in for numba / pandas) and
records their outputs on seeded synthetic benchmark records in tts.npz.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def records(rng, ninst=7, nrep=41):
    out = []
    for i in range(ninst):
        p = [0.2, 0.25, 0.3, 0.7, 0.995, 1.0, 0.5][i % 7]
        gap = np.where(rng.random(nrep) < p, 0.0,
                       rng.integers(1, 9, nrep).astype(float))
        out.append({"set": "s" if i % 3 else "t", "instance_idx": i,
                    "runs_attempted": nrep,
                    "runs_solved": int((gap <= 0).sum()),
                    "runtime_seconds": list(rng.uniform(0.1, 2.0, nrep)),
                    "energy_gap": list(gap)})
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
    spec = importlib.util.spec_from_file_location(
        "ref_test_tts", os.path.join(args.reference, "tests", "test_tts.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(77)
    succ = rng.random((5, 33)) < np.array([0, 0.01, 0.2, 0.9, 1.0])[:, None]
    raw = records(rng)
    out = {"succ": succ, "raw_json": json.dumps(raw)}
    for ptgt in (0.9, 0.99):
        key = str(ptgt).replace(".", "")
        out["nts_" + key] = mod.nts(succ, ptgt)
        for set_name in (None, "s"):
            r = mod.raw_to_tts(raw, set_name=set_name, ptgt=ptgt)
            tag = key + "_" + (set_name or "all")
            for k in ("success_prob", "nts", "tts", "runtime_mean_seconds"):
                out[f"raw_{tag}_{k}"] = r[k]
        r = mod.raw_to_tts(raw, ptgt=ptgt)
        np.random.seed(5)
        out["boots_" + key] = mod.tts_boots(r, 9, ptgt)
    np.savez_compressed(os.path.join(HERE, "tts.npz"), **out)
    print("tts done")


if __name__ == "__main__":
    main()
