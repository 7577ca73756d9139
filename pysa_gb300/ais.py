"""Partition-function helpers of pysa.ais (pysa/ais.py), same names.

The per-sweep log-omega of a PT run and the per-sample AIS log weights are
produced on the GPU (libpysa_gb); these are the small host-side reductions and
the reference distributions used to start an anneal.
"""
from __future__ import annotations

from typing import List

import numpy as np

Vector = List[float]


def get_log_omega(betas, beta_idx, energies) -> float:
    """AIS log weight of one sorted ladder (pysa/ais.py:79-112)."""
    betas = np.asarray(betas)
    _sort = np.argsort(betas, kind="stable")
    cur_betas = betas[_sort]
    cur_energies = np.asarray(energies)[np.asarray(beta_idx)[_sort]]
    if cur_betas[0] != 0:
        raise ValueError(
            '''Calculating the Partition Function requires a zero beta.  The most likely solution is that when you are calling metrpolis_update you need to include np.inf in your temperature list (if using user defined temperatures) or use the beta0 = True option (if using min_temp and max_temp).'''
        )
    log_omega = 0.0
    beta_old = cur_betas.dtype.type(0)
    for r in range(1, len(betas)):
        beta, energy = cur_betas[r], cur_energies[r]
        log_omega += float((-beta * energy) - (-beta_old * energy))
        beta_old = beta
    return log_omega


def omegas_to_partition(log_omegas, logZ0: float) -> float:
    """log-mean-exp of the weights plus log Z0 (pysa/ais.py:115-131)."""
    lw = np.asarray(log_omegas, dtype=np.float64)
    smax = lw.max()
    expsum = np.sum(np.exp(lw - smax))
    # np.float64, the type the reference returns (a frame's log_Zf column)
    return np.float64(smax - np.log(len(lw)) + logZ0 + np.log(expsum))


def combine_logZf(solution) -> float:
    """Combine the per-read log_Zf of a frame (pysa/ais.py:59-76)."""
    col = solution['log_Zf']
    log_Zf = np.asarray(col.to_numpy() if hasattr(col, "to_numpy") else col,
                        dtype=np.float64)
    smax = log_Zf.max()
    return np.float64(smax - np.log(len(log_Zf)) +
                      np.log(np.sum(np.exp(log_Zf - smax))))


def partition_function_post(solution) -> float:
    """log Z from the temps/energies columns of a frame (pysa/ais.py:29-56).

    The reference calls get_log_omega with two of its three arguments and
    always raises; here the columns are already aligned (temps[k] is the
    temperature of energies[k]), so the identity slot map is passed.
    """
    states = solution["states"]
    n = len(states[0][0])
    temps = solution["temps"]
    energies = solution["energies"]
    log_omegas = []
    for s in range(len(temps)):
        cur_temps = np.asarray(temps[s])
        with np.errstate(divide="ignore"):
            cur_betas = 1 / cur_temps
        log_omegas.append(
            get_log_omega(cur_betas, np.arange(len(cur_betas)),
                          np.asarray(energies[s])))
    return omegas_to_partition(np.array(log_omegas), n * np.log(2))


# ----------------------------------------------- "uniform" (pysa/ais.py:137-169)
def uniform_prob_initialization(n: int, problem_type: str, initial_args=None):
    if problem_type == "qubo":
        state = np.random.randint(2, size=n)
    elif problem_type == "ising":
        state = 2 * np.random.randint(2, size=n) - 1
    else:
        raise ValueError(f"problem_type=='{problem_type}' not supported.")
    return np.array(state)


def uniform_ref_prob(state: Vector, pos: int = None):
    return 1


def uniform_partition_fun(n: int):
    return n * np.log(2)


# --------------------------------------------- "bernoulli" (pysa/ais.py:175-226)
def bernoulli_prob_initialization(n: int, problem_type: str,
                                  initial_args=(0.5,)):
    p = initial_args[0]
    if problem_type == "qubo":
        state = [np.random.binomial(1, 1 - p) for i in range(n)]
    elif problem_type == "ising":
        state = [2 * np.random.binomial(1, 1 - p) - 1 for i in range(n)]
    else:
        raise ValueError(f"problem_type=='{problem_type}' not supported.")
    return np.array(state)


def bernoulli_ref_prob(state: Vector, p: float, pos: int = -1):
    state = np.asarray(state)
    bits = (state == 1).astype(np.int64)
    if 0 <= pos < len(state):
        bits[pos] = 1 - bits[pos]
    c = int(bits.sum())
    n = len(state)
    return (p**(n - c)) * ((1 - p)**c)


def bernoulli_partition_fun(n: int):
    return 0
