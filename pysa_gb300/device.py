"""Device-resident parallel tempering: problems, chains and results that stay
in GPU memory between calls.

`DeviceSolver` is the torch-facing form of `pysa.sa.Solver.metropolis_update`
(pysa/sa.py:92-430) for callers whose problem and states already live on the
GPU and change every call, the RBM negative phase of
tutorials/rbm_pysa.py:111-140 being the reference's own example: there the
dense QUBO is rebuilt, copied to the host, solved, and the states copied back
every training step.  Here the problem is split into couplings and fields on
the device (`pysa_gb_load_problem`), the states are packed and unpacked on the
device (`pysa_gb_pack`, `pysa_gb_unpack`), the sweeps run in the same kernels
as `Solver`, and the result is a dict of device tensors.  Given the same seed,
states and problem, the chains equal `Solver.metropolis_update`'s bit for bit.

Resume: `initialize_strategy=None` continues the chains where the previous
call stopped (states, energies, temperature slots, best states and the sweep
counter of the random stream), so two calls of k sweeps equal one of 2k.
Passing states instead restarts the temperature slots at 0..R-1, as feeding a
frame's states back into the reference does (pysa/sa.py:325).
"""
from __future__ import annotations

import secrets

import numpy as np
import torch

from ._lib import check, ref
from .engine import Instance, PTBatch, _ptr


def ladder(num_replicas: int, min_temp: float, max_temp: float,
           beta0: bool = False, float_type: str = "float32") -> np.ndarray:
    """The geometric inverse-temperature ladder of pysa/sa.py:167-201."""
    R = int(num_replicas)
    if R == 1:
        return np.array([1 / min_temp], dtype=float_type)
    if R == 2:
        return np.array([1 / min_temp, 1 / max_temp], dtype=float_type)
    if beta0:
        ratio = np.exp(1 / (R - 2) * np.log(max_temp / min_temp))
        b = np.array([1 / (min_temp * ratio**k) for k in range(R - 1)],
                     dtype=float_type)
        return np.append(b, 0.0).astype(float_type)
    ratio = np.exp(1 / (R - 1) * np.log(max_temp / min_temp))
    return np.array([1 / (min_temp * ratio**k) for k in range(R)],
                    dtype=float_type)


class DeviceSolver:
    """Parallel tempering on one problem of size n whose couplings, chains and
    results stay on the GPU.

    problem_type: 'ising' or 'qubo'; num_replicas x num_reads chains; the
    ladder is built as metropolis_update builds it from min_temp / max_temp
    (or given as temps).  kernel: as PTBatch ('auto' puts 64 <= n <= 2048 on
    the tensor cores).
    """

    def __init__(self, problem_type: str, n: int, *, num_replicas: int,
                 num_reads: int = 1, min_temp: float = 1.0,
                 max_temp: float = 3.5, temps=None, beta0: bool = False,
                 kernel: str = "auto", device=None):
        if problem_type not in ("ising", "qubo"):
            raise ValueError(f"problem_type='{problem_type}' not supported.")
        if temps is not None:
            betas = 1 / np.asarray(temps, dtype=np.float32)
        else:
            betas = ladder(num_replicas, min_temp, max_temp, beta0)
        self.problem_type = problem_type
        self.n = int(n)
        self.R = len(betas)
        self.Rd = int(num_reads)
        self.betas = np.asarray(betas, np.float32)
        z = np.zeros((self.n, self.n), np.float32)
        self.batch = PTBatch(problem_type, [
            Instance(z, np.zeros(self.n, np.float32), self.betas, self.Rd)
        ], device=device, kernel="auto" if kernel == "autotune" else kernel,
                             tc_terms=2)
        self.device = self.batch.device
        self._betas_d = torch.from_numpy(self.betas).to(self.device)
        self._P = None
        self._started = False

    # ------------------------------------------------------------- problem
    def set_problem(self, problem: torch.Tensor, check_symmetric: bool = True):
        """Dense symmetric [n, n] problem on the device (couplings off the
        diagonal, local fields on it, pysa/sa.py:66-69).  The symmetry check
        of pysa/sa.py:63-65 runs on the device."""
        P = torch.as_tensor(problem).detach().to(self.device)
        if P.shape != (self.n, self.n):
            raise ValueError("Problem must be a square matrix.")
        if check_symmetric and not bool(torch.allclose(P, P.T)):
            raise ValueError("Problem must be a symmetric matrix.")
        P32 = P.to(torch.float32).contiguous()
        self.batch.load_problem(0, P32)
        self._P = P32

    def _energies64(self, x: torch.Tensor) -> torch.Tensor:
        """f64 energies of device states [k, n] (pysa/qubo.py:32-37) from the
        loaded couplings, as Solver computes them for given initial states
        (its f64 copy of the same f32 values, same order)."""
        b = self.batch
        words = torch.empty(x.shape[0], b.words, dtype=torch.int32,
                            device=self.device)
        st = b._stream.cuda_stream
        check(b.lib.pysa_gb_pack(b.ptype, self.n, _ptr(x), self.n, x.shape[0],
                                 _ptr(words), b.words, st), "pack")
        out = torch.empty(x.shape[0], dtype=torch.float64, device=self.device)
        check(b.lib.pysa_gb_energy64_tables(ref(b.p), ref(b._ht), 0,
                                            _ptr(words), b.words, x.shape[0],
                                            _ptr(out), st), "energy64")
        return out

    # -------------------------------------------------------------- sweeps
    def metropolis_update(self, num_sweeps: int, *, initialize_strategy=None,
                          init_energies=None,
                          update_strategy: str = "sequential",
                          use_pt: bool = True, parallel: bool = True,
                          sort_output_temps: bool = False,
                          seed: int | None = None) -> dict:
        """num_sweeps sweeps; initialize_strategy: device states [R, n] (the
        same for every read, as pysa/sa.py:303-309) or [num_reads, R, n], or
        None to continue the current chains.  Returns device tensors with
        the frame's columns: 'states' [Rd, R, n], 'energies' [Rd, R],
        'best_state' [Rd, n], 'best_energy' [Rd], 'temps' [Rd, R],
        'min_sweeps' [Rd], plus 'num_sweeps'."""
        if self._P is None:
            raise ValueError("set_problem() first")
        if update_strategy not in ("random", "sequential"):
            raise ValueError(
                f"update_strategy='{update_strategy}' not recognized.")
        if int(num_sweeps) < 1:
            raise ValueError("num_sweeps must be >= 1.")
        b = self.batch
        R, Rd, n = self.R, self.Rd, self.n
        if initialize_strategy is not None:
            x = torch.as_tensor(initialize_strategy).detach().to(
                device=self.device, dtype=torch.float32)
            if x.shape == (R, n):
                x = x.unsqueeze(0).expand(Rd, R, n)
            if x.shape != (Rd, R, n):
                raise ValueError("Cannot initialize system.")
            x = x.reshape(Rd * R, n).contiguous()
            if init_energies is None:
                e = self._energies64(x).to(torch.float32)
            else:
                e = torch.as_tensor(init_energies).to(
                    device=self.device, dtype=torch.float32).reshape(-1)
                if e.numel() == R:
                    e = e.repeat(Rd)
            b.set_states_device(x, e, best_global=not parallel)
            self._init_e = e.reshape(Rd, R).clone()
            self._started = True
        elif not self._started:
            raise ValueError("first call needs initialize_strategy")
        if seed is None:
            seed = secrets.randbits(64)
        b.run(int(num_sweeps), seed=int(seed), update=update_strategy,
              use_pt=bool(use_pt))
        return self._results(parallel, sort_output_temps, int(num_sweeps))

    def _results(self, parallel: bool, sort_output_temps: bool,
                 num_sweeps: int) -> dict:
        b = self.batch
        R, Rd, n = self.R, self.Rd, self.n
        states = b.unpack_device().reshape(Rd, R, n)
        energies = b.energies.reshape(Rd, R).clone()
        bidx = b.beta_idx.reshape(Rd, R).to(torch.int64)
        be = b.best_energy.reshape(Rd, R)
        bs = b.best_sweep.reshape(Rd, R)
        if parallel:  # pysa/simulation.py:174-177 (first minimum)
            k = torch.argmin(be, dim=1)
        else:  # pysa/simulation.py:204-225: earliest (sweep, replica)
            emin = be.min(dim=1, keepdim=True).values
            cand = torch.where(be == emin, bs.to(torch.int64),
                               torch.iinfo(torch.int64).max)
            smin = cand.min(dim=1, keepdim=True).values
            idx = torch.arange(R, device=self.device).expand(Rd, R)
            k = torch.where(cand == smin, idx, R).min(dim=1).values
        rows = torch.arange(Rd, device=self.device)
        best_words = b.best_spins.reshape(Rd, R, -1)[rows, k]
        best_state = b.unpack_device(best_words).reshape(Rd, n)
        best_energy = be[rows, k].clone()
        min_sweeps = bs[rows, k].clone()
        if not parallel:
            # best stays replica 0's initial energy (and its state view,
            # pysa/simulation.py:204) unless a sweep went strictly lower
            keep = self._init_e[:, 0] <= best_energy
            best_state = torch.where(keep[:, None], states[:, 0], best_state)
            best_energy = torch.where(keep, self._init_e[:, 0], best_energy)
            min_sweeps = torch.where(keep, torch.zeros_like(min_sweeps),
                                     min_sweeps)
        if sort_output_temps:  # pysa/sa.py:380-387
            out_states = torch.gather(
                states, 1, bidx[:, :, None].expand(Rd, R, n))
            out_energies = torch.gather(energies, 1, bidx)
            out_betas = self._betas_d.expand(Rd, R)
        else:
            out_states, out_energies = states, energies
            out_betas = self._betas_d[bidx]
        return {
            "states": out_states,
            "energies": out_energies,
            "best_state": best_state,
            "best_energy": best_energy,
            "temps": 1.0 / out_betas,
            "num_sweeps": num_sweeps,
            "min_sweeps": min_sweeps.to(torch.int32),
        }

    def check_status(self):
        """Raise if a kernel reported an error (synchronises)."""
        torch.cuda.synchronize(self.device)
        self.batch.check_status()
