"""Time-to-solution statistics on solver output.

Restates the benchmark arithmetic of the reference's TTS test
(tests/test_tts.py:171-277): the number of independent runs needed to reach
the target with probability ptgt, its product with the mean runtime, and a
bootstrap of the ptgt-quantile over instances.  Plus `batch_tts`, which
applies the same rule to a GPU batch whose reads run concurrently.
"""
from __future__ import annotations

import warnings

import numpy as np


def nts(success_arr, ptgt: float = 0.99) -> np.ndarray:
    """Runs to solution along the last axis (tests/test_tts.py:171-192):
    ln(1 - ptgt) / ln(1 - p_s); 1 when p_s >= ptgt, inf when p_s == 0."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        s = np.asarray(success_arr)
        ps = np.sum(s, axis=-1) / s.shape[-1]
        out = np.where(ps < ptgt, np.log(1.0 - ptgt) / np.log(1.0 - ps), 1.0)
        return np.where(ps > 0.0, out, np.inf)


def raw_to_tts(raw_data, set_name=None, gap_key: str = "energy_gap",
               ptgt: float = 0.99) -> dict:
    """Per-instance success probability, NTS and TTS from benchmark records
    (list of dicts with instance_idx, runs_attempted, runs_solved,
    runtime_seconds, <gap_key>), as tests/test_tts.py:195-254."""
    rows = [r for r in raw_data if set_name is None or r["set"] == set_name]
    idx = np.asarray([r["instance_idx"] for r in rows])
    attempted = np.asarray([r["runs_attempted"] for r in rows])
    solved = np.asarray([r["runs_solved"] for r in rows])
    runtime = np.stack([np.asarray(r["runtime_seconds"]) for r in rows], 0)
    mean_rt = runtime.mean(axis=1)
    gap = np.stack([np.asarray(r[gap_key]) for r in rows], 0)
    success = gap <= 0.0
    for i in range(len(attempted)):
        if attempted[i] != success.shape[1] or solved[i] != success[i].sum():
            raise ValueError(f"record {i}: run counts do not match its gaps")
    n = nts(success, ptgt)
    return {"set": set_name, "ptgt": ptgt, "instance_idx": idx,
            "runs_attempted": attempted, "runs_solved": solved,
            "runtime_seconds": runtime, "runtime_mean_seconds": mean_rt,
            gap_key: gap, "success_prob": success.sum(1) / attempted,
            "nts": n, "tts": n * mean_rt}


def tts_boots(bench_tts: dict, nboots: int = 20, ptgt: float = 0.99,
              rng=None, gap_key: str = "energy_gap") -> np.ndarray:
    """Bootstrap samples of the ptgt-quantile over instances of the
    per-instance TTS, resampling each instance's runs with replacement
    (tests/test_tts.py:257-277).  rng: a numpy Generator/RandomState, or
    None for the global numpy stream (as the reference does)."""
    choice = (rng or np.random).choice
    gap = np.asarray(bench_tts[gap_key])
    mean_rt = np.asarray(bench_tts["runtime_mean_seconds"])
    ninst, nrep = gap.shape
    out = []
    for _ in range(nboots):
        t = []
        for j in range(ninst):
            reps = choice(np.arange(nrep), nrep)
            t.append(mean_rt[j] * nts(gap[j, reps] <= 0, ptgt))
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out.append(np.quantile(t, ptgt))
    return np.asarray(out)


def batch_tts(best_energy, target, t_batch: float, ptgt: float = 0.99,
              atol: float = 1e-6) -> dict:
    """TTS of a GPU batch: best_energy [I, Rd] (per read), target [I];
    every read of every instance ran concurrently in t_batch seconds, so the
    cost of one run is t_batch / (I * Rd).  Success: best <= target + atol."""
    be = np.asarray(best_energy, np.float64)
    tg = np.asarray(target, np.float64)[:, None]
    success = be <= tg + atol
    I, Rd = be.shape
    t_run = float(t_batch) / (I * Rd)
    n = nts(success, ptgt)
    tts = n * t_run
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        med = float(np.median(tts))
    return {"success_prob": success.mean(1), "nts": n, "t_run": t_run,
            "tts": tts, "tts_median": med,
            "solved_instances": int(np.isfinite(tts).sum())}


# ------------------------------------------------------------ HPO helpers
# The temperature heuristics and objective of the reference's hyperparameter
# tutorial (tutorials/hpo_demo.ipynb, cells "get_delta_e_ising",
# "get_delta_e_qubo", the temperature range cell and "tts_objective_fcn").

def delta_e_ising(J, h, scaling_correction: bool = True):
    """(dE_hot, dE_cold, count_min) of an Ising problem with symmetric J and
    field vector h: dE_hot = 2 max_i (sum_j |J_ij| + |h_i|), the largest
    single-flip energy change; dE_cold = 2 min of the nonzero |J_ij|, |h_i|,
    the smallest; count_min = how many spins have that smallest coupling as
    their own smallest nonzero term (their |h_i| if nonzero, else their
    smallest |J_ij|), or 1 without the scaling correction."""
    J = np.asarray(J.toarray() if hasattr(J, "toarray") else J, np.float64)
    h = np.asarray(h, np.float64).reshape(-1)
    aJ, ah = np.abs(J), np.abs(h)
    de_hot = 2.0 * float(np.max(aJ.sum(axis=1) + ah))
    smallest = min(float(aJ[aJ != 0].min(initial=np.inf)),
                   float(ah[ah != 0].min(initial=np.inf)))
    row_min = np.where(aJ != 0, aJ, np.inf).min(axis=1)
    own = np.where(ah != 0, ah, row_min)
    count = int(np.sum(np.minimum(row_min, own) == smallest)) \
        if scaling_correction else 1
    return de_hot, 2.0 * smallest, count


def delta_e_qubo(Q):
    """delta_e_ising of the Ising form of a symmetric QUBO matrix Q
    (x = (s + 1) / 2): J = offdiag(Q) / 4, h = (1^T Q) / 2."""
    Q = np.asarray(Q.toarray() if hasattr(Q, "toarray") else Q, np.float64)
    J = (Q - np.diag(np.diag(Q))) / 4.0
    h = np.ones(Q.shape[0]) @ Q / 2.0
    return delta_e_ising(J, h)


def temperature_range(de_hot: float, de_cold: float, count_min: int = 1,
                      p_hot: float = 0.5, p_cold: float = 0.01):
    """(min_temp, max_temp) at which the smallest move is accepted with
    probability p_cold / count_min and the largest with p_hot:
    T = -dE / log(p)."""
    max_temp = -de_hot / np.log(p_hot)
    min_temp = -de_cold / np.log(p_cold / count_min)
    return float(min_temp), float(max_temp)


def tts_objective(energies, mean_runtime: float, gs_energy: float,
                  s: float = 0.99, opt_gap: float = 0.05,
                  fail_value: float = 1e10) -> float:
    """Time to solution for tuning: success = energy within opt_gap of the
    ground-state energy (E <= E_gs (1 - opt_gap)); mean_runtime when the
    success rate reaches s, fail_value when it is 0, else
    mean_runtime ln(1 - s) / ln(1 - p)."""
    p = float(np.mean(np.asarray(energies) <= gs_energy * (1.0 - opt_gap)))
    if p == 0.0:
        return float(fail_value)
    if p >= s:
        return float(mean_runtime)
    return float(mean_runtime * np.log(1.0 - s) / np.log(1.0 - p))
