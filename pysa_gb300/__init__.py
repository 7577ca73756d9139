"""pysa_gb300 -- GB300-native parallel-tempering simulated annealing.

Drop-in for nasa/PySA's hot path: `Solver(problem, problem_type,
float_type).metropolis_update(...)` and `.annealed_importance(...)`, with the
sweeps, replica exchange and log-omega running as sm_103a CUDA kernels in
libpysa_gb.so (C ABI: include/pysa_gb.h).
"""
from . import ais
from .engine import Instance, PTBatch, pack_spins, unpack_spins
from .sa import ResultFrame, Solver

__all__ = ["Solver", "ResultFrame", "ais", "PTBatch", "Instance",
           "pack_spins", "unpack_spins"]
