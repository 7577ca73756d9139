"""ctypes binding of libpysa_gb.so (the C ABI in include/pysa_gb.h).

The structures below mirror the header field for field.  Loading fails
loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpysa_gb.so")

ISING, QUBO = 0, 1
SEQUENTIAL, RANDOM = 0, 1
ERR_TIMEOUT = -4

P = ctypes.c_void_p
I32, I64, U64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64
F32 = ctypes.c_float


class Problems(ctypes.Structure):
    _fields_ = [("problem_type", I32), ("num_instances", I32), ("max_n", I32),
                ("words", I32), ("num_chains", I64), ("num_reads", I64),
                ("n", P), ("replicas", P), ("reads", P), ("j_off", P),
                ("ld", P), ("h_off", P), ("chain_off", P), ("read_off", P),
                ("ladder_off", P), ("read_inst", P), ("J", P), ("h", P),
                ("ladder", P), ("ladder_sorted", P), ("csr_row_off", P),
                ("csr_ent_off", P), ("csr_rows", P), ("csr_col", P),
                ("csr_val", P), ("csr_width", I32), ("pad_", I32)]


class State(ctypes.Structure):
    _fields_ = [("spins", P), ("energies", P), ("beta_idx", P),
                ("chain_beta", P), ("best_energy", P), ("best_sweep", P),
                ("best_spins", P), ("log_omega", P), ("sweep_counter", P),
                ("status", P), ("ticket", P), ("stream_key", P)]


class Workspace(ctypes.Structure):
    _fields_ = [("fields", P), ("field_ld", I32), ("perm_slots", I32),
                ("perm", P), ("packed_j", P), ("packed_j_elems", I64),
                ("items", P), ("num_items", I32),
                ("variant_start", I32 * 8), ("variant_count", I32 * 8),
                ("tc_b", P), ("tc_b_elems", I64), ("tc_diag", P),
                ("tc_diag_elems", I64), ("tc_items", P),
                ("tc_num_items", I32), ("tc_terms", I32), ("tc_enabled", I32),
                ("tc_variant_start", I32 * 3), ("tc_variant_count", I32 * 3),
                ("tc_min_n", I32), ("tc_inst", P), ("plain_live", I32),
                ("tc_fusable", I32), ("tc_sched", P), ("tc_unit_sweeps", I32),
                ("tc_launch_sweeps", I32), ("tc_b_rand", P),
                ("tc_diag_rand", P), ("tc_inst_off", P),
                ("tc_rand_slots", I32), ("csr_item_start", I32),
                ("csr_item_count", I32), ("csr_width", I32),
                ("csr_chains", I32), ("wide_item_start", I32),
                ("wide_item_count", I32), ("tc_item_chains", I32),
                ("tc_uniform", I32), ("tc_fp8", I32)]


class HostTables(ctypes.Structure):
    _fields_ = [("n", P), ("replicas", P), ("reads", P), ("chain_off", P),
                ("j_off", P), ("ld", P), ("sparse", P)]


class Options(ctypes.Structure):
    _fields_ = [("seed", U64), ("update", I32), ("use_pt", I32),
                ("log_omega_stride", I32), ("best_global", I32),
                ("phases", I32), ("recompute_every", I32),
                ("exchange_every", I32), ("pad_", I32)]


class Mlp(ctypes.Structure):
    _fields_ = [("num_instances", I32), ("n", I32), ("hidden", I32),
                ("batch", I32)] + [(k, P) for k in (
                    "w1", "b1", "w2", "b2", "m1", "v1", "mb1", "vb1", "m2",
                    "v2", "mb2", "vb2", "dw1", "db1", "dw2", "db2", "w1_p",
                    "w2_p", "w2t_p", "x", "a1", "z2", "dz2", "da1", "pa", "pb",
                    "loss", "status")]


class ProposalScratch(ctypes.Structure):
    _fields_ = [(k, P) for k in ("flip", "delta", "jd", "logq_fwd",
                                 "logq_rev", "de")]


class AisOptions(ctypes.Structure):
    _fields_ = [("seed", U64), ("update", I32), ("reference", I32),
                ("order", I32), ("num_temps", I32), ("p", ctypes.c_double),
                ("max_samples", I32), ("pad_", I32)]


_lib = None


class LibraryError(RuntimeError):
    pass


def load() -> ctypes.CDLL:
    """Load the CUDA library; build it first when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    sig = {
        "pysa_gb_abi_version": ([], ctypes.c_int),
        "pysa_gb_set_trace": ([P], ctypes.c_int),
        "pysa_gb_set_unit_wait_limit": ([U64], ctypes.c_int),
        "pysa_gb_set_decision_mode": ([ctypes.c_int32], ctypes.c_int),
        "pysa_gb_set_block_round_limit": ([ctypes.c_int32], ctypes.c_int),
        "pysa_gb_set_tc_max_ctas": ([ctypes.c_int32], ctypes.c_int),
        "pysa_gb_tc_wrap_piece": ([ctypes.c_int32] * 5 + [P], ctypes.c_int),
        "pysa_gb_last_error": ([], ctypes.c_char_p),
        "pysa_gb_workspace_bytes": ([I32, P, P], ctypes.c_int),
        "pysa_gb_setup": ([P, P, P, P], ctypes.c_int),
        "pysa_gb_tc_workspace": ([I32, P, I32, I32, P], ctypes.c_int),
        "pysa_gb_tc_setup": ([P, P, P, P], ctypes.c_int),
        "pysa_gb_prepare": ([P, P, P, I32, I32, I32, P], ctypes.c_int),
        "pysa_gb_sweeps": ([P, P, P, P, I32, P], ctypes.c_int),
        "pysa_gb_sweeps_noalloc": ([P, P, P, P, I32, I32, P], ctypes.c_int),
        "pysa_gb_energy64": ([I32, I32, I32, P, P, P, I32, I64, P, P],
                             ctypes.c_int),
        "pysa_gb_unpack": ([I32, I32, P, I32, I64, P, I32, P], ctypes.c_int),
        "pysa_gb_pack": ([I32, I32, P, I32, I64, P, I32, P], ctypes.c_int),
        "pysa_gb_energy64_tables": ([P, P, I32, P, I32, I64, P, P],
                                    ctypes.c_int),
        "pysa_gb_load_problem": ([P, P, I32, P, I32, P], ctypes.c_int),
        "pysa_gb_ais": ([P, P, P, P, P, P, P], ctypes.c_int),
        "pysa_gb_logz_parts": ([I32, I32], I64),
        "pysa_gb_logz_exact": ([P, ctypes.c_double, P, P, P], ctypes.c_int),
        "pysa_gb_mlp_sync_weights": ([P, P], ctypes.c_int),
        "pysa_gb_mlp_forward": ([P, P], ctypes.c_int),
        "pysa_gb_mlp_backward": ([P, P, P, P], ctypes.c_int),
        "pysa_gb_mlp_adam": ([P, F32, F32, F32, F32, I32, P], ctypes.c_int),
        "pysa_gb_mlp_pairs": ([P, I32, P, P, P, I32, P, P], ctypes.c_int),
        "pysa_gb_cold_rows": ([P, P, P, I32, P, P], ctypes.c_int),
        "pysa_gb_snapshot": ([P, P, P, I32, P, P], ctypes.c_int),
        "pysa_gb_proposal_j_elems": ([I32, I32, I32], I64),
        "pysa_gb_pack_proposal_j": ([P, P, I32, I32, P, P], ctypes.c_int),
        "pysa_gb_propose": ([P, P, P, P, P, P, I32, P, U64, ctypes.c_uint32,
                             F32, P, P], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if lib.pysa_gb_abi_version() != 2:
        raise LibraryError("libpysa_gb ABI version mismatch")
    _lib = lib
    return lib


def check(rc: int, what: str) -> int:
    if rc < 0:
        msg = load().pysa_gb_last_error().decode(errors="replace")
        raise LibraryError(f"{what} failed ({rc}): {msg}")
    return rc


def ref(s: ctypes.Structure):
    return ctypes.byref(s)
