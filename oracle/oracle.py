"""Python face of the CPU oracle (oracle/pt_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product package never
imports this module.

Every function here restates a reference routine (file:line inside nasa/PySA)
on the shared counter-based random stream, so that its output can be compared
bit for bit with the CUDA path on integer couplings:

  pt_run          simulation_parallel / simulation_sequential + utils.pt
                  (pysa/simulation.py:123-236, pysa/utils.py:26-58)
  pt_run64        the same in f64 (float_type='float64', pysa/sa.py:204-205)
  ais_run         ais_sample + update_spin_ref (pysa/simulation.py:293-317,
                  pysa/ising.py:66-92, pysa/qubo.py:66-92)
  energy64        get_energy (pysa/ising.py:32-37) in f64
  omegas_to_partition  pysa/ais.py:115-131
  logz_exact      exact log Z by Gray-code enumeration (no reference
                  counterpart; the value AIS estimates)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
# the same source built tuned for the host CPU (oracle/Makefile); only the
# timed CPU-baseline legs select it, the tests use the parity build
_TIMED_PATH = os.path.join(_HERE, "_build", "liboracle_timed.so")
_lib = None
_libs: dict = {}
_variant = "parity"

TAG_SWEEP, TAG_PT, TAG_PERM, TAG_AIS = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed); returns
    the path of the selected build (see use_build)."""
    src = os.path.getmtime(os.path.join(_HERE, "pt_oracle.c"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src
                    for p in (_LIB_PATH, _TIMED_PATH)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _TIMED_PATH if _variant == "timed" else _LIB_PATH


def use_build(variant: str) -> None:
    """'parity' (default; generic target) or 'timed' (tuned for the host
    CPU, same arithmetic): the build every later call goes to."""
    global _variant, _lib
    if variant not in ("parity", "timed"):
        raise ValueError(variant)
    _variant = variant
    _lib = _libs.get(variant)


class _PtArgs(ctypes.Structure):
    _fields_ = [("problem_type", ctypes.c_int32), ("n", ctypes.c_int32),
                ("ld", ctypes.c_int32), ("replicas", ctypes.c_int32),
                ("reads", ctypes.c_int32), ("inst", ctypes.c_int32),
                ("update", ctypes.c_int32), ("use_pt", ctypes.c_int32),
                ("best_mode", ctypes.c_int32), ("log_omega", ctypes.c_int32),
                ("exchange_every", ctypes.c_int32),
                ("seed", ctypes.c_uint64)]


class _PtState(ctypes.Structure):
    _fields_ = [("spins", ctypes.c_void_p), ("energies", ctypes.c_void_p),
                ("beta_idx", ctypes.c_void_p),
                ("best_energy", ctypes.c_void_p),
                ("best_sweep", ctypes.c_void_p),
                ("best_spins", ctypes.c_void_p),
                ("log_omega", ctypes.c_void_p),
                ("lo_stride", ctypes.c_int32)]


class _PtState64(ctypes.Structure):
    _fields_ = [("spins", ctypes.c_void_p), ("energies", ctypes.c_void_p),
                ("beta_idx", ctypes.c_void_p),
                ("best_energy", ctypes.c_void_p),
                ("best_sweep", ctypes.c_void_p),
                ("best_spins", ctypes.c_void_p)]


class _AisArgs(ctypes.Structure):
    _fields_ = [("problem_type", ctypes.c_int32), ("n", ctypes.c_int32),
                ("ld", ctypes.c_int32), ("num_temps", ctypes.c_int32),
                ("samples", ctypes.c_int32), ("inst", ctypes.c_int32),
                ("update", ctypes.c_int32), ("ref", ctypes.c_int32),
                ("order", ctypes.c_int32), ("p", ctypes.c_double),
                ("seed", ctypes.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        _lib = _libs[_variant] = ctypes.CDLL(build())
        P = ctypes.c_void_p
        _lib.orc_philox.argtypes = [P, P, P]
        _lib.orc_draw.argtypes = [ctypes.c_uint64] + [ctypes.c_uint32] * 5
        _lib.orc_draw.restype = ctypes.c_uint32
        _lib.orc_permutation.argtypes = [
            ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, P
        ]
        _lib.orc_energy64.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P]
        _lib.orc_energy64.restype = ctypes.c_double
        _lib.orc_pt_run.argtypes = [
            ctypes.POINTER(_PtArgs), P, P, P, P,
            ctypes.POINTER(_PtState), ctypes.c_int64, ctypes.c_int32,
            ctypes.c_int
        ]
        _lib.orc_pt_run.restype = ctypes.c_int
        _lib.orc_pt_run64.argtypes = [
            ctypes.POINTER(_PtArgs), P, P, P, ctypes.POINTER(_PtState64),
            ctypes.c_int64, ctypes.c_int32, ctypes.c_int
        ]
        _lib.orc_pt_run64.restype = ctypes.c_int
        _lib.orc_ais_run.argtypes = [
            ctypes.POINTER(_AisArgs), P, P, P, P, P, ctypes.c_int
        ]
        _lib.orc_ais_run.restype = ctypes.c_int
        _lib.orc_omegas_to_partition.argtypes = [P, ctypes.c_int64,
                                                 ctypes.c_double]
        _lib.orc_omegas_to_partition.restype = ctypes.c_double
        _lib.orc_logz_exact.argtypes = [ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, P, P, ctypes.c_double]
        _lib.orc_logz_exact.restype = ctypes.c_double
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# ------------------------------------------------------------------ streams
def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(out))
    return out


def draw(seed, tag, inst, a, b, idx) -> int:
    return int(lib().orc_draw(seed, tag, inst, a, b, idx))


def permutation(seed: int, inst: int, sweep: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.int32)
    lib().orc_permutation(seed, inst, sweep, n, _p(out))
    return out


def uniforms(seed, tag, inst, a, b, count) -> np.ndarray:
    """u = (x + 0.5) 2^-32 for draws idx = 0..count-1 (f64, exact)."""
    xs = np.array([draw(seed, tag, inst, a, b, i) for i in range(count)],
                  dtype=np.float64)
    return (xs + 0.5) * 2.0**-32


# ------------------------------------------------------------------- energy
def energy64(J: np.ndarray, h: np.ndarray, s: np.ndarray) -> float:
    J = np.ascontiguousarray(J, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    s = np.ascontiguousarray(s, np.float32)
    n = J.shape[0]
    return float(lib().orc_energy64(n, J.shape[1], _p(J), _p(h), _p(s)))


# ---------------------------------------------------------------- PT driver
def pt_run(problem_type: str,
           J: np.ndarray,
           h: np.ndarray,
           betas: np.ndarray,
           spins: np.ndarray,
           energies: np.ndarray,
           beta_idx: np.ndarray,
           *,
           seed: int,
           num_sweeps: int,
           first_sweep: int = 0,
           update: str = "sequential",
           use_pt: bool = True,
           best_mode: str = "replica",
           best: tuple | None = None,
           log_omega: bool = False,
           inst: int = 0,
           nthreads: int = 0,
           exchange_every: int = 1):
    """Run the oracle PT driver in place-free form.

    spins: [reads, R, n] float32 (+-1 or 0/1); energies [reads, R] float32;
    beta_idx [reads, R] int32 slot -> replica.  Returns a dict with the final
    spins, energies, beta_idx, per-chain best (energy, sweep, spins) and the
    per-read log-omega rows (or None).
    """
    J = np.ascontiguousarray(J, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    betas = np.ascontiguousarray(betas, np.float32)
    reads, R, n = spins.shape
    sp = np.ascontiguousarray(spins, np.float32).copy()
    en = np.ascontiguousarray(energies, np.float32).copy()
    bi = np.ascontiguousarray(beta_idx, np.int32).copy()
    if best is None:
        if best_mode == "replica":
            be, bs, bsp = en.copy(), np.zeros_like(bi), sp.copy()
        else:
            be = np.full_like(en, np.inf)
            bs, bsp = np.zeros_like(bi), sp.copy()
    else:
        be, bs, bsp = (np.ascontiguousarray(x).copy() for x in best)
    stride = first_sweep + num_sweeps
    lo = np.zeros((reads, stride), np.float64)
    sorted_slots = np.argsort(betas, kind="stable").astype(np.int32)
    args = _PtArgs(0 if problem_type == "ising" else 1, n, J.shape[1], R,
                   reads, inst, 1 if update == "random" else 0, int(use_pt),
                   0 if best_mode == "replica" else 1, int(log_omega),
                   int(exchange_every), seed & ((1 << 64) - 1))
    st = _PtState(sp.ctypes.data, en.ctypes.data, bi.ctypes.data,
                  be.ctypes.data, bs.ctypes.data, bsp.ctypes.data,
                  lo.ctypes.data, stride)
    rc = lib().orc_pt_run(ctypes.byref(args), _p(J), _p(h), _p(betas),
                          _p(sorted_slots), ctypes.byref(st), first_sweep,
                          num_sweeps, nthreads)
    if rc != 0:
        raise MemoryError("oracle pt_run failed")
    return dict(spins=sp,
                energies=en,
                beta_idx=bi,
                best_energy=be,
                best_sweep=bs,
                best_spins=bsp,
                log_omega=lo[:, first_sweep:] if log_omega else None)


def pt_run64(problem_type: str,
             J: np.ndarray,
             h: np.ndarray,
             betas: np.ndarray,
             spins: np.ndarray,
             energies: np.ndarray,
             beta_idx: np.ndarray,
             *,
             seed: int,
             num_sweeps: int,
             first_sweep: int = 0,
             update: str = "sequential",
             use_pt: bool = True,
             inst: int = 0,
             nthreads: int = 0,
             exchange_every: int = 1):
    """The PT driver in f64 throughout: the reference's arithmetic for a
    Solver built with float_type='float64' (pysa/sa.py:204-205).  Same
    stream and arguments as pt_run (per-replica best); arrays in f64."""
    J = np.ascontiguousarray(J, np.float64)
    h = np.ascontiguousarray(h, np.float64)
    betas = np.ascontiguousarray(betas, np.float64)
    reads, R, n = spins.shape
    sp = np.ascontiguousarray(spins, np.float64).copy()
    en = np.ascontiguousarray(energies, np.float64).copy()
    bi = np.ascontiguousarray(beta_idx, np.int32).copy()
    be, bs, bsp = en.copy(), np.zeros_like(bi), sp.copy()
    args = _PtArgs(0 if problem_type == "ising" else 1, n, J.shape[1], R,
                   reads, inst, 1 if update == "random" else 0, int(use_pt),
                   0, 0, int(exchange_every), seed & ((1 << 64) - 1))
    st = _PtState64(sp.ctypes.data, en.ctypes.data, bi.ctypes.data,
                    be.ctypes.data, bs.ctypes.data, bsp.ctypes.data)
    rc = lib().orc_pt_run64(ctypes.byref(args), _p(J), _p(h), _p(betas),
                            ctypes.byref(st), first_sweep, num_sweeps,
                            nthreads)
    if rc != 0:
        raise MemoryError("oracle pt_run64 failed")
    return dict(spins=sp, energies=en, beta_idx=bi, best_energy=be,
                best_sweep=bs, best_spins=bsp)


# ---------------------------------------------------------------------- AIS
def ais_run(problem_type: str,
            J: np.ndarray,
            h: np.ndarray,
            temps: np.ndarray,
            init: np.ndarray,
            *,
            seed: int,
            update: str = "sequential",
            ref: str = "uniform",
            p: float = 0.5,
            order: str = "reference",
            inst: int = 0,
            nthreads: int = 0):
    """ais_sample over every row of init; J, h already scaled by beta."""
    J = np.ascontiguousarray(J, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    temps = np.ascontiguousarray(temps, np.float32)
    s = np.ascontiguousarray(init, np.float32).copy()
    ns, n = s.shape
    lw = np.zeros(ns, np.float64)
    args = _AisArgs(0 if problem_type == "ising" else 1, n, J.shape[1],
                    len(temps), ns, inst, 1 if update == "random" else 0,
                    0 if ref == "uniform" else 1,
                    0 if order == "reference" else 1, p,
                    seed & ((1 << 64) - 1))
    rc = lib().orc_ais_run(ctypes.byref(args), _p(J), _p(h), _p(temps), _p(s),
                           _p(lw), nthreads)
    if rc != 0:
        raise MemoryError("oracle ais_run failed")
    return s, lw


def omegas_to_partition(log_w: np.ndarray, logz0: float) -> float:
    lw = np.ascontiguousarray(log_w, np.float64)
    return float(lib().orc_omegas_to_partition(_p(lw), len(lw), logz0))


def logz_exact(problem_type: str, J: np.ndarray, h: np.ndarray,
               beta: float = 1.0) -> float:
    J = np.ascontiguousarray(J, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    return float(lib().orc_logz_exact(0 if problem_type == "ising" else 1,
                                      J.shape[0], J.shape[1], _p(J), _p(h),
                                      beta))
