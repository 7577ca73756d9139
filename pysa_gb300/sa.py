"""Drop-in `Solver` for pysa.sa.Solver, running on the GB300 kernels.

Host logic follows pysa/sa.py line for line (argument checks and their
errors, temperature ladder, initial-state draws from NumPy's global RNG,
output frame); the simulation itself -- every sweep, exchange, best
tracking, log-omega and energy recompute -- runs in libpysa_gb on the GPU.

Differences from the reference, all deliberate:
  * The sweep random stream is Philox keyed by (instance, read, replica,
    sweep, spin) from `seed` (new keyword; fresh entropy when None) instead of
    numba's Mersenne Twister, so runs are reproducible given `seed`.
  * With update_strategy='random' all chains of an instance share the
    per-sweep visiting order (the reference draws one per replica).
  * All reads run concurrently; 'runtime (us)' and 'init_time (us)' are the
    batch times divided by num_reads.
  * Sweeps compute in float32 whatever float_type is; float_type sets the
    output dtypes (pysa/sa.py:204-205 casts the problem the same way).  With
    float_type='float64' the returned energies and best energies are the
    exact (f64) energies of the returned states.
  * num_sweeps < 1 raises ValueError (the reference fails with
    UnboundLocalError at pysa/simulation.py:181).
"""
from __future__ import annotations

import secrets
from concurrent.futures import ThreadPoolExecutor
from time import time
from typing import Any, List

import numpy as np

from . import ais as _ais
from . import tts as _tts
from .engine import Instance, PTBatch, pack_spins, run_ais, unpack_spins

Vector = List[float]


class ResultFrame(list):
    """Rows of metropolis_update when pandas is not installed.

    A list of row dicts with column access by key or attribute
    (frame['best_energy'], frame.best_energy) returning NumPy arrays.
    """

    def __getitem__(self, key):
        if isinstance(key, str):
            col = [r[key] for r in self]
            try:
                return np.asarray(col)
            except ValueError:
                return np.asarray(col, dtype=object)
        return list.__getitem__(self, key)

    def __getattr__(self, key):
        if self and key in self[0]:
            return self[key]
        raise AttributeError(key)


def _frame(rows):
    try:
        import pandas as pd
    except ImportError:
        return ResultFrame(rows)
    return pd.DataFrame(rows)


class Solver(object):
    """pysa.sa.Solver on the GPU (pysa/sa.py:35-553)."""

    def __init__(self, problem, problem_type: str, float_type: Any = 'float32'):
        # pysa/sa.py:43-48
        if problem_type == 'qubo':
            pass
        elif problem_type == 'ising':
            pass
        else:
            raise ValueError(f"problem_type='{problem_type}' not supported.")
        self.problem_type = problem_type
        self.n_vars = len(problem)
        self.float_type = float_type
        problem = np.asarray(problem)
        # pysa/sa.py:60-65
        if problem.shape != (self.n_vars, self.n_vars):
            raise ValueError("Problem must be a square matrix.")
        if not np.allclose(problem, problem.T):
            raise ValueError("Problem must be a symmetric matrix.")
        # pysa/sa.py:68-70
        self.local_fields = np.copy(np.diag(problem))
        self.couplings = np.copy(problem)
        np.fill_diagonal(self.couplings, 0)
        self._dev64 = None

    # ------------------------------------------------------------ energy
    def _energies64(self, states: np.ndarray) -> np.ndarray:
        """f64 energies of [k, n] states on the GPU (pysa/ising.py:32-37)."""
        import torch
        from . import _lib
        from ._lib import check
        lib = _lib.load()
        dev = torch.device("cuda")
        if self._dev64 is None:
            J = torch.from_numpy(np.ascontiguousarray(
                self.couplings.astype(np.float64).T)).to(dev)
            h = torch.from_numpy(np.ascontiguousarray(
                self.local_fields.astype(np.float64))).to(dev)
            self._dev64 = (J, h)
        J, h = self._dev64
        st = np.atleast_2d(np.asarray(states))
        words = (self.n_vars + 31) // 32
        w = torch.from_numpy(pack_spins(st, self.problem_type,
                                        words).view(np.int32)).to(dev)
        out = torch.empty(st.shape[0], dtype=torch.float64, device=dev)
        ptype = _lib.ISING if self.problem_type == 'ising' else _lib.QUBO
        check(lib.pysa_gb_energy64(ptype, self.n_vars, self.n_vars,
                                   J.data_ptr(), h.data_ptr(), w.data_ptr(),
                                   words, st.shape[0], out.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream),
              "energy64")
        return out.cpu().numpy()

    def get_energy(self, conf: Vector, dtype: Any = None):
        """Energy of one configuration (pysa/sa.py:72-83)."""
        if dtype is None:
            dtype = self.couplings.dtype
        conf = np.asarray(conf).astype(dtype)
        return np.dtype(dtype).type(self._energies64(conf[None])[0])

    # ---------------------------------------------------- metropolis
    def metropolis_update_async(self, **kwargs):
        kwargs['send_background'] = False
        return self.metropolis_update(**kwargs)

    def metropolis_update(self,
                          num_sweeps: int,
                          num_reads: int = 1,
                          num_replicas: int = None,
                          temps: np.ndarray = None,
                          min_temp: float = 0.3,
                          max_temp: float = 1.5,
                          update_strategy: str = 'random',
                          initialize_strategy: str = 'random',
                          init_energies: List[float] = None,
                          recompute_energy: bool = False,
                          sort_output_temps: bool = False,
                          return_dataframe: bool = True,
                          parallel: bool = True,
                          use_pt: bool = True,
                          send_background: bool = False,
                          verbose: bool = False,
                          get_part_fun: bool = False,
                          beta0: bool = False,
                          seed: int = None,
                          sparse=None):
        """Parallel-tempering Metropolis run (pysa/sa.py:92-430).

        Returns one row per read with the reference's columns: 'states',
        'energies', 'best_state', 'best_energy', 'temps', ['log_Zf'],
        'num_sweeps', 'min_sweeps', 'init_time (us)', 'runtime (us)',
        'problem_type', 'float_type'.  `seed` keys the GPU random stream;
        `sparse` (None, True or 'auto') sends the sweeps to the sparse-row
        kernel, whose cost per attempt follows the row's nonzero couplings.
        min_temp / max_temp may be 'auto': the temperature range of the
        reference's HPO tutorial (pysa_gb300.tts.temperature_range).
        """
        if send_background:  # pysa/sa.py:140-142
            kw = dict(locals())
            kw.pop('self')
            return ThreadPoolExecutor(max_workers=1).submit(
                self.metropolis_update_async, **kw)

        # pysa/sa.py:145-161
        if temps is not None:
            if num_replicas and len(temps) != num_replicas:
                raise ValueError("len('temps') != 'num_replicas'.")
            else:
                num_replicas = len(temps)
        if type(initialize_strategy) != str:
            if num_replicas and len(initialize_strategy) != num_replicas:
                raise ValueError(
                    "len('initialize_strategy') != 'num_replicas'.")
            else:
                num_replicas = len(initialize_strategy)
            if init_energies is not None and len(init_energies) != num_replicas:
                raise ValueError("len('init_energies') != 'num_replicas'.")
        if get_part_fun:
            beta0 = True
        if min_temp == "auto" or max_temp == "auto":
            # the HPO tutorial's range: the largest single-flip change
            # accepted half the time at max_temp, the smallest one 1 % of
            # the time (over its multiplicity) at min_temp
            if self.problem_type == "qubo":
                hot, cold, cnt = _tts.delta_e_qubo(
                    self.couplings + np.diag(self.local_fields))
            else:
                hot, cold, cnt = _tts.delta_e_ising(self.couplings,
                                                    self.local_fields)
            lo, hi = _tts.temperature_range(hot, cold, cnt)
            min_temp = lo if min_temp == "auto" else min_temp
            max_temp = hi if max_temp == "auto" else max_temp
        # ladder, pysa/sa.py:167-201
        if temps is None:
            if not num_replicas:
                num_replicas = 4
            if num_replicas == 1:
                betas = np.array([1 / min_temp], dtype=self.float_type)
            elif num_replicas == 2:
                betas = np.array([1 / min_temp, 1 / max_temp],
                                 dtype=self.float_type)
            elif num_replicas > 2:
                if beta0:
                    _ratio = np.exp(1 / (num_replicas - 2) *
                                    np.log(max_temp / min_temp))
                    betas = np.array([
                        1 / (min_temp * _ratio**k)
                        for k in range(num_replicas - 1)
                    ], dtype=self.float_type)
                    betas = np.append(betas, 0.0)
                else:
                    _ratio = np.exp(1 / (num_replicas - 1) *
                                    np.log(max_temp / min_temp))
                    betas = np.array([
                        1 / (min_temp * _ratio**k) for k in range(num_replicas)
                    ], dtype=self.float_type)
        else:
            if beta0:
                if np.inf not in temps:
                    raise ValueError("get_part_fun = True or beta0 = True \
                    require the temps array to include np.inf")
            betas = 1 / np.array(temps, dtype=self.float_type)

        couplings = self.couplings.astype(self.float_type)
        local_fields = self.local_fields.astype(self.float_type)
        R, N = int(num_replicas), self.n_vars

        # initial states, pysa/sa.py:214-313 (NumPy global RNG, per read)
        energies_given = None
        draw_small = None  # random: the read's values as small integers
        if type(initialize_strategy) == str:
            if initialize_strategy == 'random':
                if self.problem_type == 'qubo':
                    def draw():
                        return np.random.randint(2, size=(R, N)).astype(
                            self.float_type)

                    def draw_small():
                        return np.random.randint(2, size=(R, N))
                elif self.problem_type == 'ising':
                    def draw():
                        return 2 * np.random.randint(2, size=(R, N)).astype(
                            self.float_type) - 1

                    def draw_small():
                        return 2 * np.random.randint(2, size=(R, N)) - 1
                else:
                    raise ValueError(
                        f"self.problem_type=='{self.problem_type}' not supported.")
            elif initialize_strategy == 'zeros' and self.problem_type == 'qubo':
                def draw():
                    return np.zeros((R, N), dtype=self.float_type)
                energies_given = np.zeros(R, dtype=self.float_type)
            elif initialize_strategy == 'ones':
                def draw():
                    return np.ones((R, N), dtype=self.float_type)
                energies_given = np.ones(R, dtype=self.float_type) * (
                    np.sum(couplings) / 2 + np.sum(local_fields))
            else:
                raise ValueError(
                    f"initialize_strategy='{initialize_strategy}' not recognized.")
        else:
            try:
                given = np.copy(initialize_strategy).astype(self.float_type)
                if given.shape != (R, N):
                    raise ValueError
                if init_energies is None:
                    energies_given = self._energies64(given).astype(
                        self.float_type)
                else:
                    energies_given = np.copy(init_energies).astype(
                        self.float_type)
            except Exception:
                raise ValueError("Cannot initialize system.")

            def draw():
                return given

        if update_strategy not in ('random', 'sequential'):
            raise ValueError(
                f"update_strategy='{update_strategy}' not recognized.")
        if int(num_sweeps) < 1:
            raise ValueError("num_sweeps must be >= 1.")
        if get_part_fun and np.sort(np.asarray(betas, np.float64))[0] != 0:
            raise ValueError(
                '''Calculating the Partition Function requires a zero beta.  The most likely solution is that when you are calling metrpolis_update you need to include np.inf in your temperature list (if using user defined temperatures) or use the beta0 = True option (if using min_temp and max_temp).'''
            )
        if seed is None:
            seed = secrets.randbits(64)

        # ------------------------------------------------- GPU run
        t0 = time()
        Rd = int(num_reads)
        if Rd and draw_small is not None:
            # the same NumPy RNG calls, read after read, with the values
            # (0/1 or +-1) written straight into one int8 array: no float
            # copies on the host and a quarter of the bytes to the device,
            # where they become float32 exactly
            states0 = np.empty((Rd, R, N), np.int8)
            for r in range(Rd):
                states0[r] = draw_small()
        elif Rd:
            states0 = np.stack([draw() for _ in range(Rd)])
        else:
            states0 = np.zeros((0, R, N), self.float_type)
        batch = PTBatch(self.problem_type, [
            Instance(np.asarray(couplings, np.float32),
                     np.asarray(local_fields, np.float32),
                     np.asarray(betas, np.float32), Rd)
        ], sparse=sparse)
        words = batch.words
        e0 = None if energies_given is None else np.tile(
            np.asarray(energies_given, np.float32), Rd)
        if Rd:
            # the states travel as float32 and are packed on the device
            import torch
            batch.set_states_device(
                torch.from_numpy(np.ascontiguousarray(
                    states0.reshape(Rd * R, N),
                    dtype=np.int8 if states0.dtype == np.int8
                    else np.float32)),
                None if e0 is None else torch.from_numpy(e0),
                best_global=not parallel)
        else:
            batch.set_states(pack_spins(states0, self.problem_type, words),
                             e0, best_global=not parallel)
        init_e = None
        if not parallel:
            import torch
            torch.cuda.synchronize()
            init_e = batch.energies.cpu().numpy().reshape(Rd, R).copy()
        t1 = time()
        batch.run(int(num_sweeps), seed=int(seed), update=update_strategy,
                  use_pt=bool(use_pt), log_omega=bool(get_part_fun))
        # final states unpacked on the device, copied as float32
        states_dev = batch.unpack_device() if Rd else None
        res = batch.fetch()
        t2 = time()
        init_us = int((t1 - t0) * 1e6 / max(Rd, 1))
        run_us = int((t2 - t1) * 1e6 / max(Rd, 1))

        if Rd:
            out_states_all = states_dev.cpu().numpy().reshape(Rd, R, N).astype(
                self.float_type, copy=False)
        else:
            out_states_all = np.zeros((0, R, N), self.float_type)
        energies = res['energies'].reshape(Rd, R).astype(self.float_type)
        bidx = res['beta_idx'].reshape(Rd, R).astype(np.int64)
        be = res['best_energy'].reshape(Rd, R)
        bs = res['best_sweep'].reshape(Rd, R)
        bsp = res['best_spins'].reshape(Rd, R, words)

        best_states, best_energies, best_sweeps = [], [], []
        for r in range(Rd):
            if parallel:  # pysa/simulation.py:174-177
                k = int(np.argmin(be[r]))
                best_states.append(
                    unpack_spins(bsp[r, k], N, self.problem_type,
                                 self.float_type))
                best_energies.append(np.dtype(self.float_type).type(be[r, k]))
                best_sweeps.append(np.int32(bs[r, k]))
            else:  # pysa/simulation.py:204-225, strict < in (sweep, replica)
                order = np.lexsort((np.arange(R), bs[r], be[r]))
                k = int(order[0])
                if init_e[r, 0] <= be[r, k]:
                    # best stays the initial energy of replica 0 while the
                    # state is a view of replica 0 (pysa/simulation.py:204)
                    best_states.append(out_states_all[r, 0])
                    best_energies.append(
                        np.dtype(self.float_type).type(init_e[r, 0]))
                    best_sweeps.append(0)
                else:
                    best_states.append(
                        unpack_spins(bsp[r, k], N, self.problem_type,
                                     self.float_type))
                    best_energies.append(
                        np.dtype(self.float_type).type(be[r, k]))
                    best_sweeps.append(int(bs[r, k]))

        if not recompute_energy and np.dtype(self.float_type) == np.float64:
            # the sweeps ran in float32; a float64 run reports the exact
            # energies of its states, as the reference's float64 sweeps do
            allst = np.concatenate([out_states_all.reshape(-1, N),
                                    np.stack(best_states)]) if Rd else None
            e64 = self._energies64(allst) if Rd else np.zeros(0)
            energies = e64[:Rd * R].reshape(Rd, R)
            best_energies = [np.float64(x) for x in e64[Rd * R:]]
        if recompute_energy:  # pysa/sa.py:372-377 (original dtype)
            dt = self.couplings.dtype
            allst = np.concatenate([out_states_all.reshape(-1, N),
                                    np.stack(best_states)]) if Rd else None
            e64 = self._energies64(allst) if Rd else np.zeros(0)
            energies = e64[:Rd * R].reshape(Rd, R).astype(dt)
            best_energies = [dt.type(x) for x in e64[Rd * R:]]

        rows = []
        for r in range(Rd):
            out_states = out_states_all[r]
            out_energies = energies[r]
            if sort_output_temps:  # pysa/sa.py:380-387
                out_betas = betas
                out_states = out_states[bidx[r]]
                out_energies = out_energies[bidx[r]]
            else:
                out_betas = betas[bidx[r]]
            with np.errstate(divide='ignore'):
                out_temps = np.divide(1, out_betas)
            row = {
                'states': out_states,
                'energies': out_energies,
                'best_state': best_states[r],
                'best_energy': best_energies[r],
                'temps': out_temps,
            }
            if get_part_fun:
                row['log_Zf'] = _ais.omegas_to_partition(
                    res['log_omega'][r], self.n_vars * np.log(2))
            row.update({
                'num_sweeps': int(num_sweeps),
                'min_sweeps': best_sweeps[r],
                'init_time (us)': init_us,
                'runtime (us)': run_us,
                'problem_type': self.problem_type,
                'float_type': self.float_type
            })
            rows.append(row)
        return _frame(rows) if return_dataframe else rows

    # ------------------------------------------------------------- AIS
    def annealed_importance(self,
                            num_temps: int,
                            num_samps: int,
                            reference_prob: "str",
                            update_strategy: str = 'random',
                            reference_args=None,
                            beta: float = 1.0,
                            parallel: bool = True,
                            seed: int = None,
                            ais_order: str = 'reference'):
        """Annealed importance sampling estimate of log Z (pysa/sa.py:432-553).

        Returns (logZf, samples [num_samps, n], normalised weights list).
        ais_order='reference' weights each step after its sweep, as
        pysa/simulation.py:305-316 does; 'standard' weights before the sweep
        (the unbiased AIS ordering).
        """
        if reference_prob == "uniform":
            logZ0 = _ais.uniform_partition_fun(self.n_vars)
            p = 0.5

            def init():
                return _ais.uniform_prob_initialization(
                    self.n_vars, self.problem_type, None)
        elif reference_prob == "bernoulli":
            logZ0 = _ais.bernoulli_partition_fun(self.n_vars)
            p = float(reference_args[0])

            def init():
                return _ais.bernoulli_prob_initialization(
                    self.n_vars, self.problem_type, reference_args)
        else:
            raise ValueError("Reference Probability not recognized.")
        if update_strategy not in ('random', 'sequential'):
            raise ValueError(
                f"update_strategy='{update_strategy}' not recognized.")
        if ais_order not in ('reference', 'standard'):
            raise ValueError(f"ais_order='{ais_order}' not recognized.")
        temps = np.array([(i + 1) / num_temps for i in range(num_temps)],
                         dtype=self.float_type)
        couplings = beta * self.couplings.astype(self.float_type)
        local_fields = beta * self.local_fields.astype(self.float_type)
        initial = np.array([init().astype(self.float_type)
                            for _ in range(num_samps)])
        if seed is None:
            seed = secrets.randbits(64)
        samples, log_omegas = run_ais(
            self.problem_type, couplings, local_fields, temps, initial,
            seed=int(seed), update=update_strategy, reference=reference_prob,
            p=p, order=ais_order)
        samples = samples.astype(self.float_type)
        logZf = _ais.omegas_to_partition(np.array(log_omegas), logZ0)
        lomax = log_omegas.max()
        normalization = np.sum(np.exp(log_omegas - lomax))
        omegas = [np.exp(log_omegas[i] - lomax) / normalization
                  for i in range(num_samps)]
        return logZf, samples, omegas
