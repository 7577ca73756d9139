"""The reference's driver functions on the GPU.

Drop-in replacements for pysa.simulation.simulation_parallel and
simulation_sequential (pysa/simulation.py:123-236): the functions that
pysa/sa.py:209-211 picks and calls at pysa/sa.py:329-332 and :349-352 as

    simulation(update_spin, sweep, couplings, local_fields, states,
               energies, beta_idx, betas, n_sweeps, get_part_fun, use_pt)

A code base that keeps the reference's own Solver binds the GPU path with
install(pysa.simulation): the Solver's argument checks, temperature ladder,
initial states and energies, optional recompute and output frame then run
unchanged, and every sweep, exchange, best-tracking step and log-omega runs
in libpysa_gb (through PTBatch and the C ABI).

Kept from the reference:
  * states [R, n], energies [R] and beta_idx [R] are updated in place and
    returned, with their dtypes;
  * the return value ((states, energies, beta_idx, log_omegas),
    (best_state, best_energy, best_sweeps, n_sweeps)), log_omegas a float64
    array of n_sweeps (zeros without get_part_fun);
  * best tracking: per replica with strict < then the first argmin
    (simulation_parallel, pysa/simulation.py:150-181); the earliest global
    strict improvement over replica 0's initial energy
    (simulation_sequential, pysa/simulation.py:203-236), whose best_state
    stays a view of states[0] when nothing improves on it;
  * the ValueError of get_log_omega (pysa/ais.py:94-97) when get_part_fun is
    set without a beta = 0 slot.
`update_spin` and `sweep` name the problem type and visiting order: the
reference's own functions (pysa.ising.update_spin, pysa.qubo.update_spin,
pysa.simulation.random_sweep, pysa.simulation.sequential_sweep, matched by
module and name) or the strings 'ising' / 'qubo', 'random' / 'sequential'.

Different, by design: the random stream is Philox keyed by a seed (fresh
entropy per call unless set_seed() fixed one), random order shares one
visiting order per sweep across the replicas, and the sweeps compute in
float32; float64 arrays receive the exact f64 energies of the returned
states.
"""
from __future__ import annotations

import secrets

import numpy as np

from .engine import Instance, PTBatch, pack_spins, unpack_spins

_seed = None
_calls = 0


def set_seed(seed: int | None):
    """Fix the stream: call k after this uses seed + k (None: fresh entropy
    on every call)."""
    global _seed, _calls
    _seed = None if seed is None else int(seed)
    _calls = 0


def _next_seed() -> int:
    global _calls
    if _seed is None:
        return secrets.randbits(63)
    s = _seed + _calls
    _calls += 1
    return s


def _problem_type(update_spin) -> str:
    if isinstance(update_spin, str):
        name = update_spin
    else:  # numba dispatchers keep the jitted function as py_func
        f = getattr(update_spin, "py_func", update_spin)
        name = getattr(f, "__module__", "") or ""
    if name.endswith("qubo"):
        return "qubo"
    if name.endswith("ising"):
        return "ising"
    raise ValueError(f"update_spin {update_spin!r} is neither the ising nor "
                     "the qubo update rule")


def _update(sweep) -> str:
    if isinstance(sweep, str):
        name = sweep
    else:
        name = getattr(getattr(sweep, "py_func", sweep), "__name__", "")
    if name in ("random", "random_sweep"):
        return "random"
    if name in ("sequential", "sequential_sweep"):
        return "sequential"
    raise ValueError(f"sweep {sweep!r} is neither random_sweep nor "
                     "sequential_sweep")


def _gpu_chains(ptype, update, J, h, betas, states, energies, n_sweeps,
                use_pt, log_omega, best_global, seed):
    """The R chains of one read on the GPU (PTBatch over the C ABI).
    Returns final spins, f32 energies, beta_idx, per-chain best energy,
    sweep and spins, the log-omega row (or None) and a function giving the
    exact f64 energies of float states."""
    R, n = states.shape
    b = PTBatch(ptype, [Instance(np.asarray(J, np.float32),
                                 np.asarray(h, np.float32),
                                 np.asarray(betas, np.float32), 1)])
    b.set_states(pack_spins(states, ptype, b.words),
                 np.asarray(energies, np.float32), best_global=best_global)
    b.run(n_sweeps, seed=seed, update=update, use_pt=bool(use_pt),
          log_omega=bool(log_omega))
    r = b.fetch()

    def energy64(x):
        import torch
        w = torch.from_numpy(pack_spins(np.atleast_2d(x), ptype,
                                        b.words).view(np.int32)).to(b.device)
        return b.energy64(0, np.asarray(J, np.float64).T,
                          np.asarray(h, np.float64), w)

    return dict(spins=unpack_spins(r["spins"][:R], n, ptype, np.float64),
                energies=r["energies"][:R], beta_idx=r["beta_idx"][:R],
                best_energy=r["best_energy"][:R],
                best_sweep=r["best_sweep"][:R],
                best_spins=unpack_spins(r["best_spins"][:R], n, ptype,
                                        np.float64),
                log_omega=r["log_omega"][0] if log_omega else None,
                energy64=energy64)


# the chains' runner: the GPU; tests swap in a CPU stand-in to drive the
# reference's own Solver through this module where no GPU is present
_backend = _gpu_chains


def _run(update_spin, sweep, couplings, local_fields, states, energies,
         beta_idx, betas, n_sweeps, get_part_fun, use_pt, best_global):
    ptype, update = _problem_type(update_spin), _update(sweep)
    betas = np.asarray(betas)
    if get_part_fun and np.sort(betas.astype(np.float64))[0] != 0:
        raise ValueError(
            "Calculating the Partition Function requires a zero beta.")
    R, n = states.shape
    n_sweeps = int(n_sweeps)
    # pysa/sa.py:326 and :346 pass beta_idx = arange(R)
    if not np.array_equal(np.asarray(beta_idx), np.arange(R)):
        raise ValueError("beta_idx must start as arange(num_replicas)")
    edt = np.asarray(energies).dtype
    e_init0 = edt.type(np.asarray(energies)[0]) if R else edt.type(0)
    r = _backend(ptype, update, couplings, local_fields, betas, states,
                 energies, n_sweeps, use_pt, get_part_fun, best_global,
                 _next_seed())
    be, bs = r["best_energy"], r["best_sweep"]
    if best_global:  # earliest (sweep, replica) strict improvement
        k = int(np.lexsort((np.arange(R), bs, be))[0]) if R else 0
        improved = R > 0 and be[k] < np.float32(e_init0)
    else:            # first argmin of the per-replica bests
        k = int(np.argmin(be)) if R else 0
        improved = True
    E, best_e = r["energies"].astype(np.float64), float(be[k]) if R else 0.0
    if edt == np.float64 and R:
        # the sweeps ran in float32: exact f64 energies of the states
        e64 = r["energy64"](np.concatenate([r["spins"],
                                            r["best_spins"][k:k + 1]]))
        E, best_e = e64[:R], float(e64[R])
    states[...] = r["spins"].astype(states.dtype)
    energies[...] = E.astype(edt)
    beta_idx[...] = r["beta_idx"].astype(np.asarray(beta_idx).dtype)
    lo = (np.asarray(r["log_omega"], np.float64) if get_part_fun
          else np.zeros(n_sweeps))
    if best_global and not improved:
        # pysa/simulation.py:204-206: replica 0's initial energy and a view
        # of states[0]
        best = (states[0], e_init0, 0, n_sweeps)
    elif best_global:
        best = (r["best_spins"][k].astype(states.dtype), edt.type(best_e),
                int(bs[k]), n_sweeps)
    else:
        best = (r["best_spins"][k].astype(states.dtype), edt.type(best_e),
                np.int32(bs[k]), n_sweeps)
    return (states, energies, beta_idx, lo), best


def simulation_parallel(update_spin, sweep, couplings, local_fields, states,
                        energies, beta_idx, betas, n_sweeps,
                        get_part_fun=False, use_pt=True):
    """pysa/simulation.py:123-181 on the GPU (per-replica best)."""
    return _run(update_spin, sweep, couplings, local_fields, states, energies,
                beta_idx, betas, n_sweeps, get_part_fun, use_pt, False)


def simulation_sequential(update_spin, sweep, couplings, local_fields, states,
                          energies, beta_idx, betas, n_sweeps,
                          get_part_fun=False, use_pt=True):
    """pysa/simulation.py:184-236 on the GPU (global best)."""
    return _run(update_spin, sweep, couplings, local_fields, states, energies,
                beta_idx, betas, n_sweeps, get_part_fun, use_pt, True)


def install(simulation_module):
    """Point the reference's driver names at the GPU drivers; returns the
    originals (pass them to uninstall)."""
    old = (simulation_module.simulation_parallel,
           simulation_module.simulation_sequential)
    simulation_module.simulation_parallel = simulation_parallel
    simulation_module.simulation_sequential = simulation_sequential
    return old


def uninstall(simulation_module, originals):
    (simulation_module.simulation_parallel,
     simulation_module.simulation_sequential) = originals
