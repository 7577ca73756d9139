"""C-ABI library and host logic, without a GPU (no compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden


def _header_functions():
    src = open(os.path.join(ROOT, "include", "pysa_gb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pysa_gb_\w+)\s*\(", src)))


def test_library_exports_every_header_symbol():
    from pysa_gb300 import _lib
    lib = _lib.load()
    names = _header_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
    assert lib.pysa_gb_abi_version() == 2


def test_struct_sizes_match_header_layout():
    from pysa_gb300 import _lib
    assert ctypes.sizeof(_lib.Problems) == 4 * 4 + 2 * 8 + 19 * 8 + 2 * 4
    assert ctypes.sizeof(_lib.State) == 12 * 8
    assert ctypes.sizeof(_lib.Options) == 8 + 8 * 4
    assert ctypes.sizeof(_lib.AisOptions) == 8 + 4 * 4 + 8 + 2 * 4


def _tables(n, R, Rd):
    from pysa_gb300 import _lib
    arrs = [np.asarray(n, np.int32), np.asarray(R, np.int32),
            np.asarray(Rd, np.int32)]
    return arrs, _lib.HostTables(*(a.ctypes.data for a in arrs), 0, 0, 0, 0)


def test_workspace_plan_host_only():
    from pysa_gb300 import _lib
    lib = _lib.load()
    arrs, ht = _tables([100, 1024, 3000], [8, 64, 4], [3, 2, 1])
    out = (ctypes.c_int64 * 3)()
    items = lib.pysa_gb_workspace_bytes(3, ctypes.byref(ht), out)
    # 24 chains / 64 per block + 128 / 32 + 4 / 8
    assert items == 1 + 4 + 1
    assert out[2] == 4096
    assert out[1] == items * 8


@pytest.mark.parametrize("bad", [([0], [4], [1]), ([70000], [4], [1]),
                                 ([10], [0], [1]), ([10], [600], [1])])
def test_workspace_rejects_bad_sizes(bad):
    from pysa_gb300 import _lib
    lib = _lib.load()
    arrs, ht = _tables(*bad)
    out = (ctypes.c_int64 * 3)()
    assert lib.pysa_gb_workspace_bytes(1, ctypes.byref(ht), out) < 0
    assert lib.pysa_gb_last_error()


def test_workspace_plan_wide_instances():
    """Dense instances above 4096 spins take the wide-instance sweep: eight
    chains per work item, no packed couplings, fields as wide as n."""
    from pysa_gb300 import _lib
    lib = _lib.load()
    arrs, ht = _tables([6000, 100, 65536], [5, 8, 2], [3, 2, 1])
    out = (ctypes.c_int64 * 3)()
    items = lib.pysa_gb_workspace_bytes(3, ctypes.byref(ht), out)
    assert items == 2 + 1 + 1          # 15 / 8, 16 / 64, 2 / 8
    assert out[0] == 100 * 32 * 4       # packed rows of the n = 100 instance
    assert out[2] == 65536


def test_null_arguments_rejected_without_gpu():
    from pysa_gb300 import _lib
    lib = _lib.load()
    assert lib.pysa_gb_sweeps(None, None, None, None, 1, None) == -1
    assert lib.pysa_gb_prepare(None, None, None, 1, 1, 0, None) == -1
    assert lib.pysa_gb_ais(None, None, None, None, None, None, None) == -1
    assert lib.pysa_gb_logz_parts(1, 40) == -1


def test_decision_mode_setter_validates_without_gpu():
    """pysa_gb_set_decision_mode takes 0 (per block), 1 (block rounds) or 2
    (sequential sub-blocks) and rejects anything else with an error."""
    from pysa_gb300 import _lib
    lib = _lib.load()
    for bad in (-1, 3, 7):
        assert lib.pysa_gb_set_decision_mode(bad) == -1
        assert b"decision mode" in lib.pysa_gb_last_error()
    for good in (1, 2, 0):
        assert lib.pysa_gb_set_decision_mode(good) == 0


def test_schedule_knobs_validate_without_gpu():
    """pysa_gb_set_block_round_limit takes 0..64 and pysa_gb_set_tc_max_ctas
    any count >= 0 (0: one CTA per SM); both reject the rest."""
    from pysa_gb300 import _lib
    lib = _lib.load()
    for bad in (-1, 65):
        assert lib.pysa_gb_set_block_round_limit(bad) == -1
        assert b"round limit" in lib.pysa_gb_last_error()
    assert lib.pysa_gb_set_tc_max_ctas(-2) == -1
    assert b"max CTAs" in lib.pysa_gb_last_error()
    for good in (0, 64, 12):
        assert lib.pysa_gb_set_block_round_limit(good) == 0
    assert lib.pysa_gb_set_tc_max_ctas(5) == 0
    assert lib.pysa_gb_set_tc_max_ctas(0) == 0


def _wrap_plan(lib, items, sweeps, ctas):
    out = (ctypes.c_int32 * 3)()
    plan = []
    for k in range(ctas):
        pieces = []
        j = 0
        while True:
            r = lib.pysa_gb_tc_wrap_piece(items, sweeps, ctas, k, j, out)
            assert r in (0, 1)
            if r == 0:
                break
            pieces.append((out[0], out[1], out[2]))
            j += 1
        plan.append(pieces)
    return plan


@pytest.mark.parametrize("items,sweeps,ctas", [
    (256, 20, 152), (256, 128, 152), (3, 136, 2), (7, 128, 3), (7, 9, 3),
    (5, 1, 5), (152, 5, 152), (1000, 13, 152), (153, 128, 152), (2, 7, 1)])
def test_wrap_schedule_covers_every_item_sweep_in_order(items, sweeps, ctas):
    """The kernel's wrap-around split (host copy of the same code): every
    (item, sweep) is run exactly once; each CTA runs at most one head (the
    first sweeps of an item, first) and one tail (the last sweeps of an
    item, last) around whole items; the CTA holding a tail is the next one
    after the CTA holding that item's head, whose head is its first piece
    and ends, at one time unit per item-sweep, no later than the tail
    starts; shares differ by at most one item-sweep."""
    from pysa_gb300 import _lib
    lib = _lib.load()
    plan = _wrap_plan(lib, items, sweeps, ctas)
    seen = np.zeros((items, sweeps), np.int32)
    where = {}
    for k, pieces in enumerate(plan):
        t = 0
        for j, (it, sb, sl) in enumerate(pieces):
            assert 0 <= it < items and sl >= 1 and sb + sl <= sweeps
            seen[it, sb:sb + sl] += 1
            where.setdefault(it, []).append((sb, sl, k, j, t))
            if sb > 0:
                assert j == len(pieces) - 1, "a tail runs last"
            if sl < sweeps and sb == 0:
                assert j == 0, "a head runs first"
            t += sl
    assert (seen == 1).all()
    sizes = [sum(p[2] for p in pieces) for pieces in plan]
    assert max(sizes) - min(sizes) <= 1
    for it, parts in where.items():
        parts.sort()
        if len(parts) == 1:
            assert parts[0][:2] == (0, sweeps)
            continue
        assert len(parts) == 2
        (hb, hl, hk, hj, ht), (tb, tl, tk, tj, tt) = parts
        assert hb == 0 and tb == hl and tb + tl == sweeps
        assert tk == hk + 1 and hj == 0
        assert ht + hl <= tt, "the head ends before the tail starts"


def test_wrap_schedule_rejects_bad_arguments():
    from pysa_gb300 import _lib
    lib = _lib.load()
    out = (ctypes.c_int32 * 3)()
    assert lib.pysa_gb_tc_wrap_piece(3, 10, 4, 0, 0, out) == -1  # ctas > items
    assert lib.pysa_gb_tc_wrap_piece(4, 10, 4, 4, 0, out) == -1  # share out
    assert lib.pysa_gb_tc_wrap_piece(4, 0, 4, 0, 0, out) == -1


def test_e4m3_exactness_matches_torch_conversion():
    """The host check that selects FP8 E4M3 tiles agrees with a round trip
    through torch's float8_e4m3fn on integers, subnormals, the largest
    finite value and values just outside each range."""
    import torch
    from pysa_gb300.engine import e4m3_exact
    rng = np.random.default_rng(3)
    vals = np.concatenate([
        np.arange(-20, 21), [448, 480, 464, 2 ** -9, 3 * 2 ** -9, 2 ** -10,
                             2 ** -6, 1.0625, 1.125, 0.3, 1e-3],
        rng.normal(size=300) * 8, rng.integers(-16, 17, 50) / 8.0,
    ]).astype(np.float32)
    for v in vals:
        a = np.array([v], np.float32)
        want = bool((torch.from_numpy(a).to(torch.float8_e4m3fn)
                     .to(torch.float32).numpy() == a).all())
        assert e4m3_exact(a) == want, v
    assert e4m3_exact(np.triu(rng.integers(-16, 17, (64, 64)), 1)
                      .astype(np.float32))
    assert not e4m3_exact(np.array([[0.0, np.inf]], np.float32))


def test_pack_unpack_roundtrip():
    from pysa_gb300.engine import pack_spins, unpack_spins
    rng = np.random.default_rng(0)
    for n in (1, 31, 32, 33, 100, 1024, 1025):
        words = (n + 31) // 32
        x = (2 * rng.integers(0, 2, (3, 2, n)) - 1).astype(np.float32)
        w = pack_spins(x, "ising", words)
        assert w.shape == (3, 2, words)
        assert (unpack_spins(w, n, "ising", np.float32) == x).all()
        q = rng.integers(0, 2, (4, n)).astype(np.float64)
        assert (unpack_spins(pack_spins(q, "qubo", words), n, "qubo",
                             np.float64) == q).all()
        # bit j of word j // 32 holds spin j
        j = n - 1
        e = np.zeros((1, n))
        e[0, j] = 1
        assert pack_spins(e, "qubo", words)[0, j // 32] == 1 << (j % 32)


def test_solver_argument_errors_match_reference():
    from pysa_gb300 import Solver
    P = np.zeros((4, 4))
    with pytest.raises(ValueError):
        Solver(P, "spin")
    with pytest.raises(ValueError):
        Solver(np.zeros((4, 3)), "ising")
    with pytest.raises(ValueError):
        Solver(np.triu(np.ones((4, 4)), 1), "ising")
    s = Solver(P, "ising")
    with pytest.raises(ValueError):
        s.metropolis_update(num_sweeps=2, num_replicas=3, temps=[1, 2])
    with pytest.raises(ValueError):
        s.metropolis_update(num_sweeps=2, initialize_strategy="zeros")
    with pytest.raises(ValueError):
        s.metropolis_update(num_sweeps=2, update_strategy="spiral")
    with pytest.raises(ValueError):
        s.metropolis_update(num_sweeps=2, temps=[1.0, 2.0], beta0=True)
    with pytest.raises(ValueError):
        s.metropolis_update(num_sweeps=2, num_replicas=2,
                            initialize_strategy=np.ones((3, 4)))
    with pytest.raises(ValueError):
        s.annealed_importance(4, 4, "gaussian")


def test_ais_host_helpers_match_reference_formulas():
    from pysa_gb300 import ais
    lw = np.array([0.3, -1.2, 2.5])
    want = lw.max() - np.log(3) + 5.0 + np.log(np.exp(lw - lw.max()).sum())
    assert abs(ais.omegas_to_partition(lw, 5.0) - want) < 1e-12
    st = np.array([1, -1, -1, 1])
    p = 0.3
    # flipping bit 1 (-1 -> +1) raises the count of ones from 2 to 3
    assert abs(ais.bernoulli_ref_prob(st, p, 1) - p**1 * (1 - p)**3) < 1e-15
    assert abs(ais.bernoulli_ref_prob(st, p) - p**2 * (1 - p)**2) < 1e-15
    g = golden("pt_ising_logz")
    lo = ais.get_log_omega(g["betas"], g["beta_idx"][0], g["energies"][0])
    assert np.isfinite(lo)
