"""Device-resident parallel-tempering batch over the C ABI.

`PTBatch` owns the device buffers of a batch of dense instances (uneven sizes
allowed), their chains (instance x read x replica) and the workspace, and
drives libpysa_gb: set-up (coupling packing, work list), preparation (local
fields and energies in f64), sweeps with replica exchange (optionally replayed
from a captured CUDA graph) and read-back.  PyTorch only provides device
memory and the stream.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import check, ref


def pack_spins(states: np.ndarray, problem_type: str, words: int) -> np.ndarray:
    """[..., n] float (+-1 or 0/1) -> [..., words] uint32 bit-packed."""
    st = np.asarray(states)
    bits = (st > 0) if problem_type == "ising" else (st != 0)
    flat = bits.reshape(-1, st.shape[-1])
    by = np.packbits(flat, axis=1, bitorder="little")
    out = np.zeros((flat.shape[0], words * 4), np.uint8)
    out[:, :by.shape[1]] = by
    return out.view("<u4").reshape(st.shape[:-1] + (words,))


def unpack_spins(words_arr: np.ndarray, n: int, problem_type: str,
                 dtype) -> np.ndarray:
    """[..., words] uint32 -> [..., n] values +-1 (Ising) or 0/1 (QUBO)."""
    w = np.ascontiguousarray(words_arr, dtype="<u4")
    by = w.view(np.uint8).reshape(w.shape[:-1] + (w.shape[-1] * 4,))
    bits = np.unpackbits(by, axis=-1, bitorder="little")[..., :n]
    if problem_type == "ising":
        return (2 * bits.astype(np.int8) - 1).astype(dtype)
    return bits.astype(dtype)


def _dense(J) -> np.ndarray:
    return J.toarray() if hasattr(J, "toarray") else np.asarray(J)


def bf16_exact(a: np.ndarray) -> bool:
    """True when every value is exactly representable in bfloat16."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32)
    return bool(np.all((u & 0xFFFF) == 0))


def e4m3_exact(a: np.ndarray) -> bool:
    """True when every value is exactly representable in FP8 E4M3 (four
    exponent bits, bias 7, three mantissa bits, largest finite 448): zero,
    multiples of 2^-9 below 2^-6, and above it values whose float32
    mantissa keeps only its top three bits."""
    x = np.abs(np.ascontiguousarray(a, np.float32))
    if not np.all(np.isfinite(x)) or x.max(initial=0.0) > 448.0:
        return False
    small = x < 2.0 ** -6
    sub_ok = np.all(np.mod(x[small] * 2.0 ** 9, 1.0) == 0.0)
    u = x[~small].view(np.uint32)
    return bool(sub_ok and np.all((u & 0xFFFFF) == 0))


def csr_tables(J: np.ndarray):
    """Sparse-row tables of a dense coupling matrix, as the sparse-row sweep
    reads them: row i of J^T (the row every kernel reads for spin i) keeps
    its nonzero entries grouped by column % 8, ascending column inside a
    group.  Returns rows [n, 9] int32 (group starts and the row end), col
    int32 and val float32."""
    if hasattr(J, "tocoo"):  # scipy.sparse: never densified
        T = J.T.tocoo()
        n = T.shape[0]
        keep = T.data != 0
        r = T.row[keep].astype(np.int64)
        c = T.col[keep].astype(np.int64)
        v = T.data[keep].astype(np.float32)
        g = c & 7
        order = np.lexsort((c, g, r))
        r, c, g, v = r[order], c[order], g[order], v[order]
    else:
        Jt = np.ascontiguousarray(np.asarray(J, np.float32).T)
        n = Jt.shape[0]
        r, c = np.nonzero(Jt)
        g = c & 7
        order = np.lexsort((c, g, r))
        r, c, g = r[order], c[order], g[order]
        v = Jt[r, c].astype(np.float32)
    cnt = np.zeros(8 * n, np.int64)
    np.add.at(cnt, 8 * r + g, 1)
    starts = np.concatenate([[0], np.cumsum(cnt)])
    rows = starts[8 * np.arange(n)[:, None] + np.arange(9)[None, :]]
    return rows.astype(np.int32), c.astype(np.int32), v


def csr_records(J: np.ndarray, width: int):
    """Fixed-width sparse rows: row i of J^T as `width` entries in the order
    of csr_tables (grouped by column % 8), bit 31 of the column set on the
    last entry of each group, padding entries (column i, value 0) flagged
    last.  Returns col [n, width] int32 and val [n, width] float32."""
    rows, col, val = csr_tables(J)
    n = rows.shape[0]
    deg = (rows[:, 8] - rows[:, 0]).astype(np.int64)
    if n and deg.max() > width:
        raise ValueError("a row has more entries than the record width")
    k = np.arange(width)[None, :]
    live = k < deg[:, None]
    e = np.where(live, rows[:, :1].astype(np.int64) + k, 0)
    c = np.where(live, col[e] if len(col) else 0,
                 np.arange(n)[:, None]).astype(np.int64)
    v = np.where(live, val[e] if len(val) else 0.0, 0.0).astype(np.float32)
    nxt_live = np.concatenate([live[:, 1:], np.zeros((n, 1), bool)], axis=1)
    nxt_grp = np.concatenate([c[:, 1:] & 7, np.full((n, 1), -1)], axis=1)
    last = ~live | ~nxt_live | (nxt_grp != (c & 7))
    c = c | (last.astype(np.int64) << 31)
    return (c & 0xFFFFFFFF).astype(np.uint32).view(np.int32), v


def mean_degree(J) -> float:
    """Nonzero couplings per row (dense array or scipy.sparse matrix)."""
    if hasattr(J, "tocoo"):
        return float(J.count_nonzero()) / max(J.shape[0], 1)
    J = np.asarray(J)
    return float(np.count_nonzero(J)) / max(J.shape[0], 1)


def max_degree(J) -> int:
    """Most nonzero couplings in a column (dense or scipy.sparse)."""
    if hasattr(J, "tocoo"):
        T = J.tocsc()
        T.eliminate_zeros()
        return int(np.diff(T.indptr).max(initial=0))
    return int(np.count_nonzero(J, axis=0).max(initial=0))


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr() if t is not None and t.numel() > 0 else 0


@dataclass
class Instance:
    J: np.ndarray       # [n, n] couplings, zero diagonal; a scipy.sparse
    #                     matrix is taken as is for sparse-row instances
    #                     (never densified), densified otherwise
    h: np.ndarray       # [n]
    ladder: np.ndarray  # [R] betas in slot order
    reads: int


class PTBatch:

    def __init__(self, problem_type: str, instances: list[Instance],
                 device: torch.device | str | None = None,
                 perm_slots: int = 1, kernel: str = "auto",
                 tc_terms: int | None = None, sparse=None,
                 tc_fp8: bool = False):
        """kernel: 'plain' (CUDA-core sweep for every instance), 'tc'
        (tensor-core blocked sweep for every instance, sequential order,
        64 <= n <= 2048), 'auto' (tensor cores for the instances with
        64 <= n <= 2048, the plain kernel for the rest, in the same sweep)
        or 'autotune' ('auto' until autotune() picks the threshold by
        timing; run() calls it on first use).  tc_terms sizes the
        tensor-core tiles for 1 or 2 BF16 terms (default: 1 when every J is
        exactly BF16); load_problem() needs room for 2 when later couplings
        may not be.  sparse: instances that sweep on the sparse-row kernel
        (field of spin i from row i's nonzero couplings, O(degree) per
        attempt): None / False for none, True for all, 'auto' for those
        whose mean degree is at most max(8, n / 64), or one bool per
        instance.  tc_fp8: tensor-core tiles in FP8 E4M3 when every dense
        J is exact in E4M3 and one BF16 term suffices (BF16 otherwise); the
        results are the same either way."""
        if not torch.cuda.is_available():
            raise RuntimeError(
                "pysa_gb300 needs a CUDA GPU: the sweeps run only as "
                "sm_103a kernels (no CPU path)")
        self.lib = _lib.load()
        self._tc_terms_req = tc_terms
        self._tc_fp8_req = tc_fp8
        self.device = torch.device(device or "cuda")
        self.problem_type = problem_type
        self.ptype = _lib.ISING if problem_type == "ising" else _lib.QUBO
        I = len(instances)
        self.instances = instances
        # sparse-row instances and their tables
        if sparse is None or sparse is False:
            flags = [False] * I
        elif sparse is True:
            flags = [True] * I
        elif sparse == "auto":
            flags = [mean_degree(x.J) <= max(8.0, len(x.h) / 64)
                     for x in instances]
        else:
            flags = [bool(f) for f in sparse]
            if len(flags) != I:
                raise ValueError("sparse: one flag per instance")
        n = np.array([len(x.h) for x in instances], np.int32)
        R = np.array([len(x.ladder) for x in instances], np.int32)
        Rd = np.array([x.reads for x in instances], np.int32)
        ld = ((n + 3) // 4 * 4).astype(np.int32)
        j_off = np.zeros(I, np.int64)
        h_off = np.zeros(I, np.int64)
        chain_off = np.zeros(I, np.int64)
        read_off = np.zeros(I, np.int64)
        ladder_off = np.zeros(I, np.int64)
        jt, ht, lt, ls = 0, 0, 0, 0
        ct, rt = 0, 0
        for i in range(I):
            j_off[i], h_off[i], ladder_off[i] = jt, ht, lt
            chain_off[i], read_off[i] = ct, rt
            if not flags[i]:  # sparse instances keep no dense couplings
                jt += int(n[i]) * int(ld[i])
            ht += int(n[i])
            lt += int(R[i])
            ct += int(R[i]) * int(Rd[i])
            rt += int(Rd[i])
        self.n, self.R, self.Rd, self.ld = n, R, Rd, ld
        self.chain_off, self.read_off = chain_off, read_off
        self.num_chains, self.num_reads = ct, rt
        self.max_n = int(n.max()) if I else 1
        self.words = (self.max_n + 31) // 32
        Jcat = np.zeros(max(jt, 1), np.float32)
        hcat = np.zeros(max(ht, 1), np.float32)
        lad = np.zeros(max(lt, 1), np.float32)
        lsort = np.zeros(max(lt, 1), np.int32)
        for i, x in enumerate(instances):
            ni, li = int(n[i]), int(ld[i])
            if not flags[i]:
                blk = np.zeros((ni, li), np.float32)
                # transposed: row j = change of every field when spin j flips
                blk[:, :ni] = np.asarray(_dense(x.J), np.float32).T
                Jcat[j_off[i]:j_off[i] + ni * li] = blk.ravel()
            hcat[h_off[i]:h_off[i] + ni] = np.asarray(x.h, np.float32)
            lad[ladder_off[i]:ladder_off[i] + R[i]] = x.ladder
            lsort[ladder_off[i]:ladder_off[i] + R[i]] = np.argsort(
                np.asarray(x.ladder, np.float32), kind="stable")
        read_inst = np.repeat(np.arange(I, dtype=np.int32), Rd)
        dev = self.device
        # sparse-row instances and their tables (flags above)
        self.sparse = np.asarray(flags, np.int32) if I else np.zeros(
            1, np.int32)
        row_off = np.full(max(I, 1), -1, np.int64)
        ent_off = np.zeros(max(I, 1), np.int64)
        rows_l, col_l, val_l = [], [], []
        nr, ne = 0, 0
        # fixed records when every sparse row has at most 32 entries
        maxdeg = max([max_degree(x.J)
                      for i, x in enumerate(instances) if flags[i]] or [0])
        self.csr_width = next((w for w in (4, 8, 16, 32) if maxdeg <= w), 0)
        for i, x in enumerate(instances):
            if not flags[i]:
                continue
            row_off[i], ent_off[i] = nr, ne
            if self.csr_width:
                cc, vv = csr_records(x.J, self.csr_width)
                col_l.append(cc.ravel())
                val_l.append(vv.ravel())
                nr += cc.shape[0]
                ne += cc.size
            else:
                rw, cc, vv = csr_tables(x.J)
                rows_l.append(rw)
                col_l.append(cc)
                val_l.append(vv)
                nr += rw.shape[0]
                ne += cc.shape[0]
        self.has_sparse = any(flags)

        def T(a):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

        self._t = dict(n=T(n), R=T(R), Rd=T(Rd), ld=T(ld), j_off=T(j_off),
                       h_off=T(h_off), chain_off=T(chain_off),
                       read_off=T(read_off), ladder_off=T(ladder_off),
                       read_inst=T(read_inst if rt else np.zeros(1, np.int32)),
                       J=T(Jcat), h=T(hcat), ladder=T(lad), lsort=T(lsort))
        if self.has_sparse:
            self._t.update(
                csr_row_off=T(row_off), csr_ent_off=T(ent_off),
                csr_rows=T(np.concatenate(rows_l) if rows_l else
                           np.zeros(9, np.int32)),
                csr_col=T(np.concatenate(col_l) if ne else
                          np.zeros(1, np.int32)),
                csr_val=T(np.concatenate(val_l) if ne else
                          np.zeros(1, np.float32)))
        t = self._t
        self.p = _lib.Problems(
            self.ptype, I, self.max_n, self.words, ct, rt, _ptr(t["n"]),
            _ptr(t["R"]), _ptr(t["Rd"]), _ptr(t["j_off"]), _ptr(t["ld"]),
            _ptr(t["h_off"]), _ptr(t["chain_off"]), _ptr(t["read_off"]),
            _ptr(t["ladder_off"]), _ptr(t["read_inst"]), _ptr(t["J"]),
            _ptr(t["h"]), _ptr(t["ladder"]), _ptr(t["lsort"]))
        if self.has_sparse:
            for k in ("csr_row_off", "csr_ent_off", "csr_rows", "csr_col",
                      "csr_val"):
                setattr(self.p, k, _ptr(t[k]))
            self.p.csr_width = self.csr_width
        C, W = max(ct, 1), self.words
        z = lambda *s, dt: torch.zeros(*s, dtype=dt, device=dev)  # noqa: E731
        self.spins = z(C, W, dt=torch.int32)
        self.energies = z(C, dt=torch.float32)
        self.beta_idx = z(C, dt=torch.int32)
        self.chain_beta = z(C, dt=torch.float32)
        self.best_energy = z(C, dt=torch.float32)
        self.best_sweep = z(C, dt=torch.int32)
        self.best_spins = z(C, W, dt=torch.int32)
        self.sweep_counter = z(1, dt=torch.int64)
        self.status = z(1, dt=torch.int32)
        self.ticket = z(1, dt=torch.int32)
        self.log_omega = None
        self.s = _lib.State(_ptr(self.spins), _ptr(self.energies),
                            _ptr(self.beta_idx), _ptr(self.chain_beta),
                            _ptr(self.best_energy), _ptr(self.best_sweep),
                            _ptr(self.best_spins), 0, _ptr(self.sweep_counter),
                            _ptr(self.status), _ptr(self.ticket))
        # workspace
        self._host = (n, R, Rd, chain_off, j_off, ld, self.sparse)
        ht_ = _lib.HostTables(*(a.ctypes.data for a in self._host))
        need = (ctypes.c_int64 * 3)()
        items = check(self.lib.pysa_gb_workspace_bytes(I, ref(ht_), need),
                      "workspace sizing")
        self.field_ld = int(need[2])
        self.fields = z(C, self.field_ld, dt=torch.float32)
        self.packed_j = z(max(int(need[0]), 1), dt=torch.float32)
        self.items = z(max(int(need[1]), 8), dt=torch.int32)
        self.perm_slots = max(int(perm_slots), 1)
        self.perm = z(self.perm_slots * I * self.max_n, dt=torch.int32)
        self.ws = _lib.Workspace(_ptr(self.fields), self.field_ld,
                                 self.perm_slots, _ptr(self.perm),
                                 _ptr(self.packed_j), int(need[0]),
                                 _ptr(self.items), max(items, 1))
        self.ws.csr_width = self.csr_width
        self._stream = torch.cuda.current_stream(dev)
        check(self.lib.pysa_gb_setup(ref(self.p), ref(ht_), ref(self.ws),
                                     self._stream.cuda_stream), "setup")
        self._graphs = {}
        self._ht = ht_
        self.tc = False
        self.tc_min_n = None
        dense_tc = (n >= 64) & (n <= 2048) & (self.sparse[:I] == 0)
        if kernel == "tc":
            dense = self.sparse[:I] == 0
            if I and dense.any() and (n[dense].min() < 64 or
                                      n[dense].max() > 2048):
                raise ValueError("kernel='tc' needs 64 <= n <= 2048 for "
                                 "every dense instance")
            if dense_tc.any():
                self._setup_tc(64)
        elif kernel in ("auto", "autotune"):
            if I and dense_tc.any():
                self._setup_tc(64)
        elif kernel != "plain":
            raise ValueError(f"unknown kernel {kernel!r}")
        self.autotune_pending = kernel == "autotune"

    def _setup_tc(self, min_n: int | None, item_chains: int | None = None):
        """Select the tensor-core sweep for instances with
        min_n <= n <= 2048 (None: plain kernel for every instance).
        item_chains: chains per tensor-core work item (0: automatic; None:
        keep the current choice)."""
        I = len(self.instances)
        if min_n is None:
            self.ws.tc_enabled = 0
            self.tc = False
            self.tc_min_n = None
            return
        ht_ = self._ht
        if not hasattr(self, "tc_b"):
            # sized once for the widest selection (every instance >= 64)
            terms = 1 if all(bf16_exact(_dense(x.J)) for i, x in
                             enumerate(self.instances)
                             if not self.sparse[i]) else 2
            if self._tc_terms_req is not None:
                terms = max(terms, int(self._tc_terms_req))
            tneed = (ctypes.c_int64 * 3)()
            titems = check(self.lib.pysa_gb_tc_workspace(
                I, ref(ht_), terms, 64, tneed), "tc sizing")
            z = lambda k, dt: torch.zeros(k, dtype=dt, device=self.device)
            self.tc_b = z(max(int(tneed[0]), 1), torch.int16)
            self.tc_diag = z(max(int(tneed[1]), 1), torch.float32)
            self.tc_items = z(max(int(tneed[2]), 8), torch.int32)
            self.tc_inst = z(max(I, 1), torch.int32)
            self.tc_sched = z(2 + max(titems, 1), torch.int32)
            self.ws.tc_b = _ptr(self.tc_b)
            self.ws.tc_b_elems = int(tneed[0])
            self.ws.tc_diag = _ptr(self.tc_diag)
            self.ws.tc_diag_elems = int(tneed[1])
            self.ws.tc_items = _ptr(self.tc_items)
            self.ws.tc_num_items = max(titems, 1)
            self.ws.tc_inst = _ptr(self.tc_inst)
            self.ws.tc_sched = _ptr(self.tc_sched)
            self.ws.tc_terms = terms
            self.tc_terms = terms
            self._tc_terms_cap = terms
            fp8 = bool(self._tc_fp8_req) and terms == 1 and all(
                e4m3_exact(_dense(x.J)) for i, x in enumerate(self.instances)
                if not self.sparse[i])
            self.ws.tc_fp8 = int(fp8)
            self.tc_fp8 = fp8
        self.ws.tc_min_n = int(min_n)
        if item_chains is not None:
            self.ws.tc_item_chains = int(item_chains)
        check(self.lib.pysa_gb_tc_setup(ref(self.p), ref(ht_), ref(self.ws),
                                        self._stream.cuda_stream), "tc setup")
        self._graphs = {}
        self.tc = True
        self.tc_min_n = int(min_n)

    def _setup_random_tc(self, budget_bytes: int = 2 << 30,
                         max_slots: int = 16):
        """Buffers for random-order sweeps on the tensor cores: the tiles and
        diagonal blocks repacked in each sweep's visiting order, for up to
        `max_slots` sweeps at a time within `budget_bytes`, and as many
        visiting-order slots.  Done once per batch."""
        if self.ws.tc_rand_slots > 0:
            return
        per = 2 * int(self.ws.tc_b_elems) + 4 * int(self.ws.tc_diag_elems)
        slots = int(max(1, min(max_slots, budget_bytes // max(per, 1))))
        z = lambda k, dt: torch.zeros(k, dtype=dt, device=self.device)
        I = len(self.instances)
        self.tc_b_rand = z(max(slots * int(self.ws.tc_b_elems), 1),
                           torch.int16)
        self.tc_diag_rand = z(max(slots * int(self.ws.tc_diag_elems), 1),
                              torch.float32)
        self.tc_inst_off = z(2 * max(I, 1), torch.int64)
        if self.perm_slots < slots:
            self.perm_slots = slots
            self.perm = z(self.perm_slots * I * self.max_n, torch.int32)
            self.ws.perm = _ptr(self.perm)
            self.ws.perm_slots = self.perm_slots
        self.ws.tc_b_rand = _ptr(self.tc_b_rand)
        self.ws.tc_diag_rand = _ptr(self.tc_diag_rand)
        self.ws.tc_inst_off = _ptr(self.tc_inst_off)
        # re-run the set-up so it writes the per-instance offsets
        self._setup_tc(self.tc_min_n)
        self.ws.tc_rand_slots = slots

    def autotune(self, sweeps: int = 8,
                 candidates=(64, 256, 512, 1024, None),
                 item_chains=(0, 0.5, 0.25), unit_sweeps=(0, 4, 16),
                 exchange_every=(1,), seed: int = 1) -> dict:
        """Pick the tuning knobs of the sweep by timing them on the current
        chains (CUDA events; a coordinate search, one knob at a time, each
        starting from the best of the previous ones):

          candidates      tensor-core threshold: instances with n >= it
                          take the tensor-core sweep, the rest the plain
                          kernel (None: plain only)
          item_chains     chains per tensor-core CTA: 0 automatic, or a
                          fraction of a CTA's full tensor memory (128 / F)
          unit_sweeps     sweeps per work unit of the persistent kernel
                          (0: chosen per launch)
          exchange_every  replica-exchange interval; only (1,), every
                          sweep as the reference does, unless the caller
                          opts in to others

        The chains are restored afterwards, so results do not depend on the
        tuning.  Returns {candidate threshold: ms per sweep} for the first
        knob (the threshold); every timing and the choice are kept in
        self.autotune_report."""
        self.autotune_pending = False
        keep = [self.spins, self.energies, self.beta_idx, self.chain_beta,
                self.best_energy, self.best_sweep, self.best_spins,
                self.sweep_counter, self.status, self.ticket, self.fields]
        saved = [t.clone() for t in keep]
        n = np.asarray(self.n)
        st = self._stream

        def timed(k):
            self.run(k, seed=seed, graph_chunk=0, final_recompute=False,
                     exchange_every=self._xe)     # warm-up, attributes
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            self.run(k, seed=seed, graph_chunk=0, final_recompute=False,
                     exchange_every=self._xe)
            b.record(st)
            b.synchronize()
            for t, v in zip(keep, saved):
                t.copy_(v)
            return a.elapsed_time(b) / k

        report = {"threshold": {}, "item_chains": {}, "unit_sweeps": {},
                  "exchange_every": {}}
        self._xe = 1
        for c in candidates:
            if c is not None and not ((n >= max(c, 64)) & (n <= 2048)).any():
                continue
            self._setup_tc(c, 0)
            self.ws.tc_unit_sweeps = 0
            report["threshold"][c] = timed(sweeps)
        best_c = min(report["threshold"], key=report["threshold"].get)
        best = {"threshold": best_c, "item_chains": 0, "unit_sweeps": 0,
                "exchange_every": 1}
        if best_c is not None:
            self._setup_tc(best_c, 0)
            full = int(128 / (1 if n.max() <= 512 else
                              2 if n.max() <= 1024 else 4))
            for f in item_chains:
                ic = 0 if not f else max(int(full * f), 1)
                if ic in report["item_chains"]:
                    continue
                self._setup_tc(best_c, ic)
                report["item_chains"][ic] = timed(sweeps)
            best["item_chains"] = min(report["item_chains"],
                                      key=report["item_chains"].get)
            self._setup_tc(best_c, best["item_chains"])
            for u in unit_sweeps:
                self.ws.tc_unit_sweeps = int(u)
                report["unit_sweeps"][u] = timed(max(sweeps, 2 * int(u)))
            best["unit_sweeps"] = min(report["unit_sweeps"],
                                      key=report["unit_sweeps"].get)
            self.ws.tc_unit_sweeps = int(best["unit_sweeps"])
        for xe in exchange_every:
            self._xe = int(xe)
            report["exchange_every"][int(xe)] = timed(sweeps)
        best["exchange_every"] = min(report["exchange_every"],
                                     key=report["exchange_every"].get)
        self._xe = best["exchange_every"]
        if best_c is None:
            self._setup_tc(None)
        torch.cuda.synchronize(self.device)
        self.autotune_pending = False
        self.autotune_ms = report["threshold"]
        self.autotune_report = {"choice": best, "ms_per_sweep": report}
        return report["threshold"]

    def enable_stream_keys(self):
        """Per-chain sweep-stream keys (all 0: the plain streams); accepted
        proposals (pysa_gb_propose) advance their chain's key so its later
        sweeps draw fresh uniforms.  Done once per batch."""
        if getattr(self, "stream_key", None) is None:
            self.stream_key = torch.zeros(max(self.num_chains, 1),
                                          dtype=torch.int32,
                                          device=self.device)
            self.s.stream_key = _ptr(self.stream_key)

    # ---------------------------------------------- device-resident inputs
    def load_problem(self, inst: int, P: torch.Tensor):
        """Couplings and fields of instance `inst` from a dense symmetric
        problem matrix in device memory, split on the device as
        pysa/sa.py:66-69 does; the kernels' packed copies of J are rebuilt
        on the device.  Only the BF16- and E4M3-exactness flags of P (a
        byte each) come to the host."""
        n = int(self.n[inst])
        P = P.detach().to(device=self.device, dtype=torch.float32)
        if P.shape != (n, n):
            raise ValueError(f"problem must be {n} x {n}")
        P = P.contiguous()
        st = self._stream.cuda_stream
        check(self.lib.pysa_gb_load_problem(ref(self.p), ref(self._ht),
                                            int(inst), _ptr(P), n, st),
              "load_problem")
        check(self.lib.pysa_gb_setup(ref(self.p), ref(self._ht),
                                     ref(self.ws), st), "setup")
        if self.tc:
            exact = bool((P.to(torch.bfloat16).to(torch.float32) == P).all())
            terms = 1 if exact else 2
            if terms > self._tc_terms_cap:
                raise ValueError("couplings are not exact in BF16: build "
                                 "the batch with tc_terms=2")
            self.ws.tc_terms = terms
            self.tc_terms = terms
            # E4M3 tiles only while every instance's couplings stay exact
            # (checked on the device: one more byte to the host)
            fp8 = bool(self.tc_fp8 and terms == 1 and bool(
                (P.to(torch.float8_e4m3fn).to(torch.float32) == P).all()))
            self.ws.tc_fp8 = int(fp8)
            self.tc_fp8 = fp8
            check(self.lib.pysa_gb_tc_setup(ref(self.p), ref(self._ht),
                                            ref(self.ws), st), "tc setup")
        self._graphs = {}
        self._P_keep = P  # alive until the stream has read it

    def set_states_device(self, states: torch.Tensor, energies=None,
                          best_global: bool = False):
        """Chains from device float states [num_chains, n] (+-1 or 0/1) of a
        batch whose instances share n, packed on the device; energies
        [num_chains] (device or host) or None to compute them with the
        fields.  Temperature slots restart at 0..R-1 (pysa/sa.py:325)."""
        n = int(self.n[0]) if len(self.n) else 0
        if len(self.n) and (self.n != n).any():
            raise ValueError("set_states_device needs one n for the batch")
        # to the device in the caller's dtype (int8 states move a quarter of
        # float32's bytes), float32 there
        x = states.detach().to(device=self.device).to(torch.float32)
        x = x.reshape(self.num_chains, n).contiguous()
        st = self._stream.cuda_stream
        check(self.lib.pysa_gb_pack(self.ptype, n, _ptr(x), n,
                                    self.num_chains, _ptr(self.spins),
                                    self.words, st), "pack")
        if energies is not None:
            self.energies.copy_(torch.as_tensor(energies).reshape(-1).to(
                device=self.device, dtype=torch.float32))
        if not hasattr(self, "_bidx0"):
            self._bidx0 = torch.from_numpy(np.concatenate([
                np.tile(np.arange(self.R[i], dtype=np.int32), self.Rd[i])
                for i in range(len(self.instances))
            ]) if self.num_chains else np.zeros(1, np.int32)).to(self.device)
        self.beta_idx.copy_(self._bidx0)
        self.sweep_counter.zero_()
        self.status.zero_()
        self.ticket.zero_()
        self.best_global = bool(best_global)
        self._x_keep = x
        check(self.lib.pysa_gb_prepare(ref(self.p), ref(self.s), ref(self.ws),
                                       int(energies is None), 1,
                                       int(best_global), st), "prepare")

    def unpack_device(self, spins_words: torch.Tensor | None = None,
                      dtype=torch.float32) -> torch.Tensor:
        """Bit-packed device chains (default: the current ones) as device
        floats [rows, n] (+-1 or 0/1), unpacked on the device."""
        w = self.spins if spins_words is None else spins_words
        n = int(self.n[0])
        out = torch.empty(w.shape[0], n, dtype=torch.float32,
                          device=self.device)
        check(self.lib.pysa_gb_unpack(self.ptype, n, _ptr(w), self.words,
                                      w.shape[0], _ptr(out), n,
                                      self._stream.cuda_stream), "unpack")
        return out if dtype == torch.float32 else out.to(dtype)

    # ------------------------------------------------------------ states
    def set_states(self, spins_words: np.ndarray, energies=None,
                   best_global: bool = False):
        """Load chains ([C, words] uint32) and optional energies [C]; then
        compute local fields (and energies when not given) on the GPU."""
        st = self._stream.cuda_stream
        w = np.ascontiguousarray(spins_words, "<u4").reshape(self.num_chains,
                                                            self.words)
        self.spins.copy_(torch.from_numpy(w.view(np.int32)))
        if energies is not None:
            self.energies.copy_(torch.from_numpy(
                np.ascontiguousarray(energies, np.float32).reshape(-1)))
        bidx = np.concatenate([
            np.tile(np.arange(self.R[i], dtype=np.int32), self.Rd[i])
            for i in range(len(self.instances))
        ]) if self.num_chains else np.zeros(1, np.int32)
        self.beta_idx.copy_(torch.from_numpy(bidx))
        self.sweep_counter.zero_()
        self.status.zero_()
        self.ticket.zero_()
        self.best_global = bool(best_global)
        check(self.lib.pysa_gb_prepare(ref(self.p), ref(self.s), ref(self.ws),
                                       int(energies is None), 1,
                                       int(best_global), st), "prepare")

    # ------------------------------------------------------------ sweeps
    def run(self, num_sweeps: int, *, seed: int, update: str = "sequential",
            use_pt: bool = True, log_omega: bool = False,
            graph_chunk: int = 128, recompute_every: int | None = None,
            final_recompute: bool = True, exchange_every: int | None = None):
        """Sweeps with exchange.  recompute_every: the tensor-core path
        rebuilds fields and energies from the spins every that many sweeps
        (default 4 when J is not exact in BF16, never otherwise); with
        final_recompute the returned energies are then recomputed once more
        at the end (callers chaining many short runs can skip it and call
        recompute() once).  exchange_every: replica exchange after every
        sweep (1, the reference's schedule) or only after every k-th (an
        opt-in knob; None: the autotuner's choice, else 1)."""
        if self.autotune_pending and update == "sequential" and num_sweeps:
            self.autotune()
        if update == "random" and self.tc and num_sweeps:
            self._setup_random_tc()
        if recompute_every is None:
            recompute_every = 4 if (self.tc and self.tc_terms == 2) else 0
        upd = _lib.RANDOM if update == "random" else _lib.SEQUENTIAL
        stride = int(num_sweeps) if log_omega else 0
        if log_omega:
            self.log_omega = torch.zeros(max(self.num_reads, 1), max(stride, 1),
                                         dtype=torch.float64,
                                         device=self.device)
            self.s.log_omega = _ptr(self.log_omega)
        else:
            self.s.log_omega = 0
        if exchange_every is None:
            exchange_every = getattr(self, "_xe", 1)
        opts = _lib.Options(seed & ((1 << 64) - 1), upd, int(use_pt), stride,
                            int(self.best_global), 0, int(recompute_every),
                            int(exchange_every))
        st = self._stream.cuda_stream
        # first call with zero sweeps sets kernel attributes outside capture
        check(self.lib.pysa_gb_sweeps(ref(self.p), ref(self.s), ref(self.ws),
                                      ref(opts), 0, st), "sweeps")
        remaining = int(num_sweeps)
        chunk = int(graph_chunk)
        if chunk > 1 and remaining >= 2 * chunk:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                cs = torch.cuda.current_stream(self.device).cuda_stream
                check(self.lib.pysa_gb_sweeps(ref(self.p), ref(self.s),
                                              ref(self.ws), ref(opts), chunk,
                                              cs), "sweeps (capture)")
            for _ in range(remaining // chunk):
                g.replay()
            remaining %= chunk
            self._graphs["last"] = g  # keep alive until the stream drains
        if remaining:
            check(self.lib.pysa_gb_sweeps(ref(self.p), ref(self.s),
                                          ref(self.ws), ref(opts), remaining,
                                          st), "sweeps")
        if (final_recompute and recompute_every and self.tc and
                (upd == _lib.SEQUENTIAL or self.ws.tc_rand_slots > 0)):
            self.recompute()

    def recompute(self):
        """Fields and energies of every chain from its spins (f32 partial
        sums accumulated in f64); best_* untouched."""
        check(self.lib.pysa_gb_prepare(ref(self.p), ref(self.s), ref(self.ws),
                                       1, 0, int(self.best_global),
                                       self._stream.cuda_stream),
              "recompute")

    def check_status(self):
        code = int(self.status.item())
        if code != 0:
            what = {-4: "a bounded wait ran out",
                    -6: "energy drift: the accumulated energies left their "
                        "recomputed values (non-finite or badly scaled "
                        "couplings)"}.get(code, "device error")
            raise _lib.LibraryError(f"device reported status {code} ({what})")

    # --------------------------------------------------------- read back
    def fetch(self) -> dict:
        torch.cuda.synchronize(self.device)
        self.check_status()
        out = dict(
            spins=self.spins.cpu().numpy().view("<u4"),
            energies=self.energies.cpu().numpy(),
            beta_idx=self.beta_idx.cpu().numpy(),
            best_energy=self.best_energy.cpu().numpy(),
            best_sweep=self.best_sweep.cpu().numpy(),
            best_spins=self.best_spins.cpu().numpy().view("<u4"),
        )
        if self.log_omega is not None:
            out["log_omega"] = self.log_omega.cpu().numpy()
        return out

    def energy64(self, inst: int, J64: np.ndarray, h64: np.ndarray,
                 spins_words: torch.Tensor) -> np.ndarray:
        """f64 energies of device bit-packed states with f64 couplings."""
        n = int(self.n[inst])
        Jd = torch.from_numpy(np.ascontiguousarray(J64, np.float64)).to(
            self.device)
        hd = torch.from_numpy(np.ascontiguousarray(h64, np.float64)).to(
            self.device)
        cnt = spins_words.shape[0]
        out = torch.empty(cnt, dtype=torch.float64, device=self.device)
        check(self.lib.pysa_gb_energy64(self.ptype, n, n, _ptr(Jd), _ptr(hd),
                                        _ptr(spins_words), self.words, cnt,
                                        _ptr(out), self._stream.cuda_stream),
              "energy64")
        return out.cpu().numpy()


# ---------------------------------------------------------------- AIS
def run_ais(problem_type: str, J: np.ndarray, h: np.ndarray,
            temps: np.ndarray, init_states: np.ndarray, *, seed: int,
            update: str = "sequential", reference: str = "uniform",
            p: float = 0.5, order: str = "reference"):
    """Annealed importance sampling on the GPU (pysa/simulation.py:293-317).

    J, h already scaled by the target beta; init_states [Ns, n] (+-1 or
    0/1).  Returns (samples [Ns, n] float32, log weights [Ns] float64).
    """
    return run_ais_batch(problem_type, [(J, h, init_states)], temps,
                         seed=seed, update=update, reference=reference, p=p,
                         order=order)[0]


def run_ais_batch(problem_type: str, instances: list, temps: np.ndarray, *,
                  seed: int, update: str = "sequential",
                  reference: str = "uniform", p: float = 0.5,
                  order: str = "reference"):
    """AIS of many instances in one launch on one temperature schedule.

    instances: [(J, h, init_states [Ns_i, n_i])], couplings already scaled
    by the target beta.  Instance i uses the random streams of instance
    index i, so a one-instance call gives the same result as index 0 of a
    batch.  Returns [(samples [Ns_i, n_i] float32, log weights [Ns_i])].
    """
    temps = np.asarray(temps, np.float32)
    insts = [Instance(np.asarray(J, np.float32), np.asarray(h, np.float32),
                      np.ones(1, np.float32), int(x0.shape[0]))
             for J, h, x0 in instances]
    batch = PTBatch(problem_type, insts, perm_slots=max(len(temps), 1),
                    kernel="plain")
    words = batch.words
    ns_all = {int(np.asarray(x0).shape[1]) for _, _, x0 in instances}
    if len(ns_all) == 1:  # one packing call for the whole batch
        packed = pack_spins(np.concatenate(
            [np.asarray(x0) for _, _, x0 in instances]), problem_type, words)
    else:
        packed = np.concatenate([
            pack_spins(np.asarray(x0), problem_type, words)
            for _, _, x0 in instances])
    batch.set_states(packed, None)
    temps_d = torch.from_numpy(temps).to(batch.device)
    C = max(batch.num_chains, 1)
    log_w = torch.zeros(C, dtype=torch.float64, device=batch.device)
    max_samples = max(int(x0.shape[0]) for _, _, x0 in instances)
    opts = _lib.AisOptions(int(seed) & ((1 << 64) - 1),
                           _lib.RANDOM if update == "random" else
                           _lib.SEQUENTIAL,
                           0 if reference == "uniform" else 1,
                           0 if order == "reference" else 1, len(temps),
                           float(p), max_samples, 0)
    check(batch.lib.pysa_gb_ais(ref(batch.p), ref(batch.s), ref(batch.ws),
                                ref(opts), temps_d.data_ptr(),
                                log_w.data_ptr(), batch._stream.cuda_stream),
          "ais")
    torch.cuda.synchronize(batch.device)
    batch.check_status()
    spins = batch.spins.cpu().numpy().view("<u4")
    lw = log_w.cpu().numpy()
    # one unpacking call when every instance has the same n
    every = (unpack_spins(spins, next(iter(ns_all)), problem_type, np.float32)
             if len(ns_all) == 1 else None)
    out = []
    for i, (_, _, x0) in enumerate(instances):
        ns, n = np.asarray(x0).shape
        c0 = int(batch.chain_off[i])
        smp = (every[c0:c0 + ns] if every is not None else
               unpack_spins(spins[c0:c0 + ns], n, problem_type, np.float32))
        out.append((smp, lw[c0:c0 + ns]))
    return out


def logz_exact(problem_type: str, instances: list, beta: float = 1.0):
    """log sum_s exp(-beta E(s)) of each (J, h) by enumeration on the GPU
    in f64 (n <= 34)."""
    lib = _lib.load()
    insts = [Instance(np.asarray(J, np.float32), np.asarray(h, np.float32),
                      np.ones(1, np.float32), 0) for J, h in instances]
    batch = PTBatch(problem_type, insts, kernel="plain")
    parts = int(lib.pysa_gb_logz_parts(len(insts), batch.max_n))
    if parts < 0:
        raise ValueError("exact log Z supports 1 <= n <= 34")
    pm = torch.empty(parts, dtype=torch.float64, device=batch.device)
    ps = torch.empty(parts, dtype=torch.float64, device=batch.device)
    check(lib.pysa_gb_logz_exact(ref(batch.p), float(beta), pm.data_ptr(),
                                 ps.data_ptr(), batch._stream.cuda_stream),
          "logz")
    m = pm.cpu().numpy().reshape(len(insts), -1)
    sm = ps.cpu().numpy().reshape(len(insts), -1)
    out = []
    for mi, si in zip(m, sm):
        ok = np.isfinite(mi)
        top = mi[ok].max()
        out.append(float(top + np.log(np.sum(si[ok] * np.exp(mi[ok] - top)))))
    return np.array(out)
