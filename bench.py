"""Benchmark of the PT Metropolis hot path (one JSON line on rank 0).

Workload (default): dense integer QUBO, N=1024, Q_ij uniform in [-8, 8]
symmetric, diagonal uniform in [-16, 16], float32; 64 replicas on a geometric
ladder T = 0.5 .. 8.0; 256 reads (16384 chains); sequential sweeps with a
replica exchange after every sweep.  Seeded synthetic instance.

A step is one sweep of every chain followed by the exchange.  `value` is
spin-flip attempts/s with all state resident in HBM, timed on the device with
CUDA events around each step; L2 is flushed (256 MB write) before every step.
`e2e` is the same metric through the public API (Solver.metropolis_update,
2000 sweeps) with host inputs and outputs, timed on the host.

--impl reference times the CPU restatement of the reference's algorithm
(dense dot per attempt, OpenMP over chains) on the same instance.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "qubo1024": dict(kind="qubo", n=1024, replicas=64, reads=256, tmin=0.5,
                     tmax=8.0, sweeps=2000, update="sequential"),
    "qubo1024_random": dict(kind="qubo", n=1024, replicas=64, reads=256,
                            tmin=0.5, tmax=8.0, sweeps=2000, update="random"),
    "sk128": dict(kind="sk", n=128, replicas=32, reads=100, tmin=1.0,
                  tmax=3.5, sweeps=1000, update="sequential"),
    # 500 uneven SK instances in one batch (autotuned kernel split)
    "sk_batch500": dict(kind="sk_batch", instances=500, nmin=64, nmax=1536,
                        replicas=32, reads=100, tmin=1.0, tmax=3.5,
                        sweeps=1000, update="sequential"),
    # planted Wishart N=2048 (real couplings: split-BF16 tensor-core path)
    "wishart2048": dict(kind="wishart", n=2048, m=1024, replicas=64,
                        reads=128, tmin=0.02, tmax=2.0, sweeps=5000,
                        update="sequential"),
    # AIS on 64 SK instances N=24 against exact enumeration of 2^24 states
    "sk24_ais": dict(kind="ais", instances=64, n=24, temps=200, beta=2.0,
                     samples=1024, update="sequential"),
    # learned proposal vs plain PT, TTS(99%) (not an attempts/s line)
    "lattice64_sparse": dict(kind="lattice", side=64, replicas=40,
                             reads=100, tmin=1.0, tmax=3.5),
    "rbm_mnist": dict(kind="rbm", visible=784, hidden=128, state_size=100,
                      steps=1, tmin=1.0, tmax=1.0, parallel=False),
    "sk512_tts": dict(kind="pm1", n=512, replicas=64, reads=32, tmin=0.3,
                      tmax=3.0, instances=64, budgets=(25000, 100000),
                      target_sweeps=100000, target_reads=4, plain_check=200,
                      target_flips=2.0, update="sequential"),
}


def planted_wishart(n, m, rng):
    """Planted Wishart ensemble: J = (1/n) sum_mu w_mu w_mu^T with every
    w_mu orthogonal to a random +-1 planted state t, zero diagonal, h = 0.
    With E = s.J s / 2, E(s) = (1/2n) sum_mu [(w_mu.s)^2 - ||w_mu||^2], so t
    is a ground state: E_gs = -(1/2n) sum_mu ||w_mu||^2.  Returns
    (J, t, E_gs)."""
    t = rng.choice([-1.0, 1.0], size=n)
    W = rng.normal(size=(m, n))
    W -= np.outer(W @ t / n, t)          # project out t
    J = (W.T @ W) / n
    np.fill_diagonal(J, 0.0)
    e_gs = float(t @ J @ t / 2)
    return J.astype(np.float32), t, e_gs


def make_instance(w: dict, seed: int = 2024):
    rng = np.random.default_rng(seed)
    n = w["n"]
    if w["kind"] == "wishart":
        J, _, _ = planted_wishart(n, w["m"], rng)
        return "ising", J
    if w["kind"] == "qubo":
        Q = rng.integers(-8, 9, (n, n))
        Q = np.triu(Q, 1)
        Q = Q + Q.T
        Q[np.diag_indices(n)] = rng.integers(-16, 17, n)
        return "qubo", Q.astype(np.float32)
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    return "ising", (J + J.T).astype(np.float32)


def ladder(w):
    R = w["replicas"]
    ratio = np.exp(1 / (R - 1) * np.log(w["tmax"] / w["tmin"]))
    return np.array([1 / (w["tmin"] * ratio**k) for k in range(R)],
                    np.float32)


class ClockSampler:
    """nvidia-smi samples around and during the timed region.

    A timed region of a few milliseconds ends before `nvidia-smi -lms`
    prints its first line, so entering waits (up to 10 s) for a first sample
    and leaving waits for one taken after the region ended; the summary keeps
    the samples from the last one before the region to the first one after
    it.  When the looping form prints nothing, single queries are polled
    instead.  Only reads clocks; changes no setting."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []   # (time, line)
        self.mode = None
        self._stop = threading.Event()
        self._got = threading.Event()
        self.t_in = self.t_out = None

    def _cmd(self, loop):
        c = ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
             "--format=csv,noheader,nounits"]
        return c + (["-lms", "100"] if loop else [])

    def _add(self, line):
        line = line.strip()
        if len(line.split(",")) >= 9:
            self.lines.append((time.perf_counter(), line))
            self._got.set()

    def _read(self):
        for line in self.proc.stdout:
            self._add(line)
            if self._stop.is_set():
                break

    def _poll(self):
        while not self._stop.is_set():
            try:
                r = subprocess.run(self._cmd(False), capture_output=True,
                                   text=True, timeout=5)
                for line in r.stdout.splitlines():
                    self._add(line)
            except (OSError, subprocess.TimeoutExpired):
                return
            self._stop.wait(0.1)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(self._cmd(True),
                                         stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.mode = "loop"
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            if not self._got.wait(5.0):
                self._end_proc()
                self.mode = "poll"
                self.t = threading.Thread(target=self._poll, daemon=True)
                self.t.start()
                self._got.wait(5.0)
        except (OSError, FileNotFoundError):
            self.proc, self.mode = None, None
        self.t_in = time.perf_counter()
        return self

    def _end_proc(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.proc = None

    def __exit__(self, *a):
        self.t_out = time.perf_counter()
        if self.mode:
            deadline = self.t_out + 5.0
            while time.perf_counter() < deadline and not any(
                    t > self.t_out for t, _ in self.lines):
                time.sleep(0.02)
        self._stop.set()
        self._end_proc()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        lines = self.lines
        if self.t_in is not None and self.t_out is not None and lines:
            before = [k for k, (t, _) in enumerate(lines) if t <= self.t_in]
            after = [k for k, (t, _) in enumerate(lines) if t >= self.t_out]
            lo = before[-1] if before else 0
            hi = after[0] if after else len(lines) - 1
            lines = lines[lo:hi + 1]
        inside = sum(1 for t, _ in lines
                     if self.t_in is not None and self.t_out is not None and
                     self.t_in < t < self.t_out)
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0, "mode": self.mode}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm),
                "samples_inside": inside, "mode": self.mode,
                "window": "last sample before the timed region to the first "
                          "after it"}


def field_errors(batch, J, h, ptype):
    """Max errors of the device's FP32 local fields and energies against an
    FP64 recomputation from the device's own spins."""
    import torch
    from pysa_gb300 import unpack_spins
    n = len(h)
    sp = unpack_spins(batch.spins.cpu().numpy().view("<u4"), n, ptype,
                      np.float64)
    S = torch.from_numpy(sp).cuda()
    J64 = torch.from_numpy(np.asarray(J, np.float64)).cuda()
    h64 = torch.from_numpy(np.asarray(h, np.float64)).cuda()
    H = S @ J64.T + h64
    E = (S * (0.5 * (S @ J64.T) + h64)).sum(1)
    Hg = batch.fields[:, :n].double()
    Eg = batch.energies.double()
    return {"field_max_abs_err": float((Hg - H).abs().max()),
            "field_max_rel_err": float((Hg - H).abs().max() / H.abs().max()),
            "energy_max_rel_err": float(((Eg - E).abs() / E.abs().clamp_min(
                1e-30)).max()),
            "energy_err_of_scale": float((Eg - E).abs().max() /
                                         E.abs().max())}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def _timed_oracle():
    """The oracle's tuned build (oracle/Makefile: same source and arithmetic
    as the parity build, compiled for the host CPU) for the timed CPU legs."""
    from oracle import oracle
    oracle.use_build("timed")
    oracle.build()
    return oracle


def cpu_reference(w, ptype, P, reads, sweeps, nthreads=0):
    """Oracle (CPU restatement, OpenMP over chains) on `reads` reads."""
    oracle = _timed_oracle()
    h = np.diag(P).astype(np.float32).copy()
    J = P.copy()
    np.fill_diagonal(J, 0)
    R, n = w["replicas"], w["n"]
    rng = np.random.default_rng(5)
    if ptype == "qubo":
        x0 = rng.integers(0, 2, (reads, R, n)).astype(np.float32)
    else:
        x0 = (2 * rng.integers(0, 2, (reads, R, n)) - 1).astype(np.float32)
    e0 = np.zeros((reads, R), np.float32)
    bidx = np.tile(np.arange(R, dtype=np.int32), (reads, 1))
    t0 = time.perf_counter()
    oracle.pt_run(ptype, J, h, ladder(w), x0, e0, bidx, seed=1,
                  num_sweeps=sweeps, update=w["update"], nthreads=nthreads)
    dt = time.perf_counter() - t0
    return reads * R * n * sweeps / dt, dt


def _median_tts_boot(success, t_run, rng, nboot=400, ptgt=0.99):
    """Bootstrap of the median over instances of TTS(ptgt): each instance's
    reads resampled with replacement (as tests/test_tts.py:257-277 does for
    its quantile).  success [I, Rd] bool; t_run seconds per read."""
    from pysa_gb300.tts import nts
    I, Rd = success.shape
    out = np.empty(nboot)
    for b in range(nboot):
        idx = rng.integers(0, Rd, (I, Rd))
        t = nts(np.take_along_axis(success, idx, axis=1), ptgt) * t_run
        out[b] = np.median(t)
    return out


def run_tts_workload(args, w, rank, world):
    """TTS(99 %) on seeded +-1 SK instances (J_ij = +-1 symmetric, zero
    diagonal), three arms:

      plain          the plain CUDA-core PT sweep (k_sweep_plain)
      split_bf16     the blocked split-BF16 tensor-core PT sweep (k_sweep_tc)
      learned        split_bf16 plus the learned flip proposal

    Target energy per instance: the best energy of a target_sweeps plain PT
    run (target_reads reads, its own seed).  Each arm runs every budget S
    from the same random states; one run = one read, all I x Rd reads run
    concurrently, so t_run = wall time / (I Rd) and TTS = t_run ln(0.01) /
    ln(1 - p_s), p_s = fraction of reads whose best reaches the target.
    +-1 couplings are exact in BF16, so the tensor-core sweep's trajectories
    equal the plain kernel's bit for bit on the same stream: the plain arm
    is run for plain_check sweeps, its chains compared with the split_bf16
    arm's after as many sweeps (must be identical), its wall time per sweep
    measured there, and its TTS at budget S formed from that time and the
    split_bf16 arm's success rates.  The target run uses the tensor-core
    sweep for the same reason.  CIs: bootstrap of the median TTS over
    instances (reads resampled per instance), and of the ratio of two arms'
    medians; the learned arm's time includes its training and proposals."""
    if rank != 0:
        return 0
    import torch
    from pysa_gb300 import Instance, PTBatch, pack_spins
    from pysa_gb300.proposal import LearnedProposal, run_with_proposals
    from pysa_gb300.tts import nts
    I, n, R, Rd = w["instances"], w["n"], w["replicas"], w["reads"]
    rng = np.random.default_rng(2024)
    Js = []
    for _ in range(I):
        J = np.triu(rng.choice([-1.0, 1.0], size=(n, n)), 1)
        Js.append((J + J.T).astype(np.float32))
    h0 = np.zeros(n, np.float32)
    lad = np.sort(ladder(w)).astype(np.float32)

    def fresh(reads, kernel="tc", seed_states=7):
        x0 = (2 * np.random.default_rng(seed_states).integers(
            0, 2, (I * reads * R, n)) - 1).astype(np.float32)
        b = PTBatch("ising", [Instance(J, h0, lad, reads) for J in Js],
                    kernel=kernel)
        b.set_states(pack_spins(x0, "ising", b.words))
        torch.cuda.synchronize()
        return b

    def per_read_best(b, reads):
        return b.best_energy.view(I, reads, R).min(dim=2).values.cpu().numpy()

    sampler = ClockSampler(0)
    with sampler:
        # target: best of a target_sweeps run
        b = fresh(w["target_reads"], seed_states=8)
        t0 = time.perf_counter()
        b.run(w["target_sweeps"], seed=11)
        torch.cuda.synchronize()
        t_target = time.perf_counter() - t0
        b.check_status()
        target = per_read_best(b, w["target_reads"]).min(axis=1)
        del b
        # plain arm: identical trajectories to split_bf16, timed per sweep
        K = w["plain_check"]
        bp = fresh(Rd, kernel="plain")
        bp.run(1, seed=13)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bp.run(K - 1, seed=13)
        torch.cuda.synchronize()
        t_plain_sweep = (time.perf_counter() - t0) / (K - 1)
        bs_ = fresh(Rd)
        bs_.run(K, seed=13)
        torch.cuda.synchronize()
        same = bool(torch.equal(bp.spins, bs_.spins) and
                    torch.equal(bp.best_energy, bs_.best_energy) and
                    torch.equal(bp.beta_idx, bs_.beta_idx))
        if not same:
            raise AssertionError("plain and tensor-core sweeps diverged")
        del bp, bs_
        arms = {"split_bf16": {}, "learned": {}}
        stats = {}
        for S in w["budgets"]:
            b = fresh(Rd)
            t0 = time.perf_counter()
            b.run(S, seed=13)
            torch.cuda.synchronize()
            arms["split_bf16"][S] = (time.perf_counter() - t0,
                                     per_read_best(b, Rd))
            b.check_status()
            del b
            b = fresh(Rd)
            prop = LearnedProposal(b, hidden=1024, lr=1e-3, init_seed=3,
                                   target_flips=w["target_flips"])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = run_with_proposals(b, prop, S, seed=13, interval=10,
                                    train_every=5, train_pairs=200_000,
                                    min_train_steps=200, min_accept=0.01)
            torch.cuda.synchronize()
            arms["learned"][S] = (time.perf_counter() - t0,
                                  per_read_best(b, Rd))
            b.check_status()
            stats[S] = {"rounds": st.rounds, "train_steps": st.train_steps,
                        "acceptance_mean": float(st.acceptance.mean()),
                        "accepted_moves": int(st.accepted.sum()),
                        "enabled_instances_at_end": int(st.enabled.sum())}
            del b, prop
    rb = np.random.default_rng(99)
    tg = target[:, None] + 1e-6
    out = {}
    boots = {}
    for S in w["budgets"]:
        t_split, best_split = arms["split_bf16"][S]
        t_learn, best_learn = arms["learned"][S]
        succ = {"split_bf16": best_split <= tg, "learned": best_learn <= tg}
        succ["plain"] = succ["split_bf16"]   # identical trajectories
        t_run = {"split_bf16": t_split / (I * Rd),
                 "learned": t_learn / (I * Rd),
                 "plain": t_plain_sweep * S / (I * Rd)}
        row = {}
        for arm in ("plain", "split_bf16", "learned"):
            tts = nts(succ[arm]) * t_run[arm]
            bt = _median_tts_boot(succ[arm], t_run[arm], rb)
            boots[(arm, S)] = bt
            fin = bt[np.isfinite(bt)]
            row[arm] = {
                "seconds": t_run[arm] * I * Rd,
                "p_success_mean": float(succ[arm].mean()),
                "instances_with_success": int(succ[arm].any(axis=1).sum()),
                "tts99_median_s": float(np.median(tts)),
                "tts99_median_ci95_s": ([float(np.quantile(bt, 0.025)),
                                         float(np.quantile(bt, 0.975))]
                                        if len(fin) == len(bt) else None)}
        for a, b_ in (("plain", "learned"), ("split_bf16", "learned"),
                      ("plain", "split_bf16")):
            ra = boots[(a, S)] / boots[(b_, S)]
            ok = np.isfinite(ra)
            row[f"ratio_{a}_over_{b_}"] = {
                "median": float(np.median(ra[ok])) if ok.any() else None,
                "ci95": [float(np.quantile(ra[ok], 0.025)),
                         float(np.quantile(ra[ok], 0.975))]
                if ok.sum() == len(ra) else None}
        out[str(S)] = row
    bestS = min(w["budgets"],
                key=lambda S: out[str(S)]["learned"]["tts99_median_s"])
    line = {
        "metric": "tts99_median_s",
        "value": out[str(bestS)]["learned"]["tts99_median_s"],
        "unit": "s", "n_gpus": 1, "steps": len(w["budgets"]), "warmup": 0,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 sweeps; bf16/f32 network", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "instances": I, "n": n,
                   "replicas": R, "reads": Rd, "tmin": w["tmin"],
                   "tmax": w["tmax"], "budgets": list(w["budgets"]),
                   "target": f"best of a {w['target_sweeps']}-sweep plain "
                             f"PT run, {w['target_reads']} reads",
                   "target_seconds": t_target,
                   "plain_arm": f"same trajectories as split_bf16 (checked "
                                f"over {K} sweeps), {t_plain_sweep * 1e3:.3f}"
                                f" ms per sweep",
                   "network": "512-1024-512 per instance, target "
                              f"{w['target_flips']} flips, propose every "
                              "10 sweeps, train every 5 (2e5 pairs max), off "
                              "below 1% acceptance after 200 training steps"},
        "best_budget_sweeps": bestS, "budgets": out,
        "proposal_stats": {str(k): v for k, v in stats.items()},
        "clocks": sampler.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_batch_workload(args, w, rank, world):
    """Many uneven SK instances in one batch (kernel split autotuned):
    spin-flip attempts/s of whole sweeps (all instances) + exchange."""
    import torch
    from pysa_gb300 import Instance, PTBatch, pack_spins
    from pysa_gb300 import _lib
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    I, R, Rd = w["instances"], w["replicas"], w["reads"]
    rng = np.random.default_rng(4242)
    sizes = rng.integers(w["nmin"], w["nmax"] + 1, I)
    lad = ladder(w)
    insts = []
    for n in sizes:
        J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
        insts.append(Instance((J + J.T).astype(np.float32),
                              np.zeros(n, np.float32), lad, Rd))
    t0 = time.perf_counter()
    batch = PTBatch("ising", insts, kernel="autotune")
    srng = np.random.default_rng(9 + rank)
    words = batch.words
    x0 = np.concatenate([
        pack_spins((2 * srng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32),
                   "ising", words).reshape(-1, words) for n in sizes])
    batch.set_states(x0, None)
    tune = batch.autotune()
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    attempts = float(R * Rd * sizes.sum())
    batch.run(args.warmup, seed=3, graph_chunk=0, final_recompute=False)
    st = torch.cuda.current_stream()
    # timed: the K sweeps in one call, as the API runs them (every instance
    # on the tensor cores: persistent launches of up to 128 sweeps with the
    # exchange fused).  The batch's couplings (1.6 GB) and fields (5 GB)
    # are far larger than L2, so no flush between sweeps.
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(
        enable_timing=True)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    with sampler:
        a.record(st)
        batch.run(args.steps, seed=3, graph_chunk=0, final_recompute=False)
        b.record(st)
        torch.cuda.synchronize()
    batch.check_status()
    total_s = a.elapsed_time(b) / 1e3
    ms = [1e3 * total_s / args.steps]
    if dist:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    value = attempts * args.steps * world / total_s
    # for comparison: one sweep per call (one launch per fold per sweep,
    # fields through HBM every sweep), L2 flushed before each
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32,
                        device="cuda")
    ev1 = [(torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(float(k))
        a1, b1 = ev1[k]
        a1.record(st)
        batch.run(1, seed=3, graph_chunk=0, final_recompute=False)
        b1.record(st)
    torch.cuda.synchronize()
    one_sweep = attempts * args.steps / (
        sum(x.elapsed_time(y) for x, y in ev1) / 1e3)
    # graph-captured chunks (the production path), one timing
    g0 = time.perf_counter()
    batch.run(128, seed=3, graph_chunk=64)
    torch.cuda.synchronize()
    graph_rate = attempts * 128 / (time.perf_counter() - g0)
    # end to end: host states in, sweeps, best energies out
    e2e = None
    if not args.no_e2e:
        se = args.e2e_sweeps or 200
        t0 = time.perf_counter()
        batch.set_states(x0, None)
        batch.run(se, seed=4)
        best = batch.best_energy.cpu().numpy()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": attempts * se / e2e_s, "unit": "attempts/s",
               "h2d_bytes_per_step": int(x0.nbytes / se),
               "d2h_bytes_per_step": int(best.nbytes / se),
               "seconds": e2e_s, "sweeps": se,
               "includes": "state upload, field set-up, sweeps (graph "
                           "chunks of 64), final recompute, best energies "
                           "download"}
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        oracle = _timed_oracle()
        k = int(np.argsort(sizes)[len(sizes) // 2])   # median-size instance
        n = int(sizes[k])
        xs = (2 * srng.integers(0, 2, (8, R, n)) - 1).astype(np.float32)
        e0 = np.zeros((8, R), np.float32)
        bidx = np.tile(np.arange(R, dtype=np.int32), (8, 1))
        t1 = time.perf_counter()
        oracle.pt_run("ising", insts[k].J, insts[k].h, lad, xs, e0, bidx,
                      seed=1, num_sweeps=20)
        dt = time.perf_counter() - t1
        cpu = {"value": 8 * R * n * 20 / dt, "unit": "attempts/s",
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"median-size instance (n={n}), 8 reads x {R} "
                         f"replicas x 20 sweeps ({dt:.1f} s)"}
    # launches in the timed call: per fold with instances, one persistent
    # kernel and its schedule reset per launch of up to 128 sweeps (fused
    # path); else per sweep the fold kernels, the plain variants and the
    # exchange
    folds = int(sum(1 for v in range(3) if batch.ws.tc_variant_count[v] > 0))
    if batch.tc_min_n is not None and all(int(x) >= batch.tc_min_n
                                          for x in sizes):
        gpu_launches = folds * -(-args.steps // 128)
    else:
        gpu_launches = args.steps * (folds + 3 + 1)
    if rank == 0:
        hbm, bf16, kind = measured_peaks()
        print(json.dumps({
            "metric": "spin_flip_attempts_per_s", "value": value,
            "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(ms)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "instances": I,
                       "n_min": int(sizes.min()), "n_max": int(sizes.max()),
                       "n_sum": int(sizes.sum()), "replicas": R, "reads": Rd,
                       "chains": int(I * R * Rd),
                       "l2": "inputs larger than L2 (couplings 1.6 GB, "
                             "fields 5 GB); the K sweeps in one call",
                       "kernel_split": {"tc_min_n": batch.tc_min_n,
                                        "autotune_ms_per_sweep":
                                            {str(k): v for k, v in tune.items()}},
                       "setup_s": setup_s},
            "graph_chunk64_value": graph_rate,
            "one_sweep_launches_value": one_sweep,
            "roofline": None, "clocks": sampler.summary(), "e2e": e2e,
            "cpu_baseline": cpu,
            "gpu_launches": gpu_launches}), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_ais_workload(args, w, rank, world):
    """AIS log Z (Solver.annealed_importance, uniform reference, beta = 2)
    of SK instances against exact enumeration of all 2^n states."""
    if rank != 0:
        return 0
    import torch
    from pysa_gb300 import Solver
    from pysa_gb300.engine import logz_exact
    I, n = w["instances"], w["n"]
    rng = np.random.default_rng(24)
    probs = []
    for _ in range(I):
        J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
        probs.append(J + J.T)
    t0 = time.perf_counter()
    exact = logz_exact("ising", [(P.astype(np.float32), np.zeros(n, np.float32))
                                 for P in probs], beta=w["beta"])
    torch.cuda.synchronize()
    t_exact = time.perf_counter() - t0
    out = {}
    for order in ("reference", "standard"):
        est = []
        np.random.seed(1)
        Solver(probs[0], "ising", "float32").annealed_importance(
            4, 16, "uniform", beta=w["beta"], seed=0, ais_order=order)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i, P in enumerate(probs):
            lz = Solver(P, "ising", "float32").annealed_importance(
                w["temps"], w["samples"], "uniform", beta=w["beta"],
                seed=100 + i, ais_order=order)[0]
            est.append(lz)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        err = np.asarray(est) - exact
        out[order] = {"seconds": dt, "mean_err": float(err.mean()),
                      "max_abs_err": float(np.abs(err).max()),
                      "attempts_per_s":
                          I * w["samples"] * w["temps"] * n / dt}
    # all instances in one launch (engine.run_ais_batch), same estimator:
    # log Z = omegas_to_partition(log w, n log 2)
    from pysa_gb300.engine import run_ais_batch
    from pysa_gb300.ais import omegas_to_partition
    temps = np.array([(i + 1) / w["temps"] for i in range(w["temps"])],
                     np.float32)
    srng = np.random.default_rng(77)
    batch_in = [((w["beta"] * P).astype(np.float32), np.zeros(n, np.float32),
                 (2 * srng.integers(0, 2, (w["samples"], n)) - 1
                  ).astype(np.float32)) for P in probs]
    run_ais_batch("ising", batch_in[:2], temps[:4], seed=0)  # warm-up
    torch.cuda.synchronize()
    bt = []
    for rep in range(3):
        t0 = time.perf_counter()
        res = run_ais_batch("ising", batch_in, temps, seed=500 + rep,
                            update="sequential")
        bt.append(time.perf_counter() - t0)
    est = [omegas_to_partition(lw, n * np.log(2.0)) for _, lw in res]
    err = np.asarray(est) - exact
    attempts = I * w["samples"] * w["temps"] * n
    out["batched_reference_order"] = {
        "seconds": min(bt), "attempts_per_s": attempts / min(bt),
        "mean_err": float(err.mean()), "max_abs_err": float(np.abs(err).max()),
        "includes": "state upload, field set-up, the AIS launch, samples and "
                    "weights download (host buffers in and out)"}
    print(json.dumps({
        "metric": "ais_attempts_per_s",
        "value": out["batched_reference_order"]["attempts_per_s"],
        "unit": "attempts/s",
        "n_gpus": 1, "steps": I, "warmup": 1, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 weights)",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "instances": I, "n": n,
                   "temps": w["temps"], "samples": w["samples"],
                   "beta": w["beta"], "reference": "uniform"},
        "ais": out,
        "exact": {"seconds": t_exact,
                  "states_per_s": I * 2.0**n / t_exact,
                  "logz_mean": float(np.mean(exact))},
        "e2e": {"value": out["batched_reference_order"]["attempts_per_s"],
                "unit": "attempts/s", "h2d_bytes_per_step": I * (
                    n * n * 4 + w["samples"] * 4 * ((n + 31) // 32)),
                "d2h_bytes_per_step": I * w["samples"] * (
                    4 * ((n + 31) // 32) + 8),
                "per_instance_solver": out["reference"]["attempts_per_s"]}}),
        flush=True)
    return 0


def run_rbm_workload(args, w, rank, world):
    """RBM negative phase (tutorials/rbm_pysa.py:111-140 at the MNIST
    tutorial's sizes): persistent-state updates per second through
    RBM_PySA.update_states_with_pysa (problem, states and results on the
    device), beside the reference's recipe on the same kernels (QUBO built
    on the host, Solver, states copied back).  W moves a little before every
    update, as an optimiser step would."""
    if rank != 0:
        return 0
    import torch
    from pysa_gb300 import Solver
    from pysa_gb300.rbm import RBM_PySA
    V, H, S = w["visible"], w["hidden"], w["state_size"]
    n = V + H
    torch.manual_seed(7)
    m = RBM_PySA(V, H, state_size=S, steps=w["steps"], parallel=w["parallel"],
                 min_temp=w["tmin"], max_temp=w["tmax"], seed=11)
    g = torch.Generator(device="cuda").manual_seed(5)
    m.v_state = (torch.rand(S, V, device="cuda", generator=g) > 0.5).float()
    m.h_state = (torch.rand(S, H, device="cuda", generator=g) > 0.5).float()

    def nudge():
        with torch.no_grad():
            m.W.add_(1e-3 * torch.randn(V, H, device="cuda", generator=g))

    def host_recipe(seed):
        W = m.W.detach().cpu().numpy()
        vb = m.v_bias.detach().cpu().numpy()
        hb = m.h_bias.detach().cpu().numpy()
        problem = np.zeros((n, n), np.float32)
        problem[:V, V:] = W
        problem[V:, :V] = W.T
        problem += np.diag(np.concatenate([vb, hb]).squeeze())
        x0 = torch.cat([m.v_state, m.h_state], 1).cpu().numpy()
        res = Solver(-problem, "qubo", "float32").metropolis_update(
            num_sweeps=w["steps"], num_reads=1, num_replicas=S,
            update_strategy="sequential", min_temp=w["tmin"],
            max_temp=w["tmax"], initialize_strategy=x0,
            parallel=w["parallel"], seed=seed, return_dataframe=False)
        st = torch.from_numpy(res[0]["states"]).cuda()
        m.v_state, m.h_state = torch.split(st, V, dim=1)

    for i in range(args.warmup):
        nudge()
        m.update_states_with_pysa(seed=i)
    torch.cuda.synchronize()
    K = max(1, min(args.steps, 500))
    t0 = time.perf_counter()
    for i in range(K):
        nudge()
        m.update_states_with_pysa(seed=1000 + i)
    torch.cuda.synchronize()
    dt_dev = (time.perf_counter() - t0) / K
    m.negative_phase().item()
    for i in range(args.warmup):
        nudge()
        host_recipe(i)
    torch.cuda.synchronize()
    Kh = max(1, min(K, 100))
    t0 = time.perf_counter()
    for i in range(Kh):
        nudge()
        host_recipe(2000 + i)
    torch.cuda.synchronize()
    dt_host = (time.perf_counter() - t0) / Kh
    attempts = S * n * w["steps"]
    print(json.dumps({
        "metric": "rbm_negative_phase_updates_per_s", "value": 1.0 / dt_dev,
        "unit": "updates/s", "n_gpus": 1, "steps": K,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt_dev,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; W ~ N(0, 1) as the "
        "reference initialises it)",
        "config": {"workload": args.workload, **w, "n": n},
        "attempts_per_s": attempts / dt_dev,
        "host_round_trip": {
            "ms_per_step": 1e3 * dt_host, "updates_per_s": 1.0 / dt_host,
            "what": "reference recipe on the same kernels: QUBO assembled "
                    "in NumPy, Solver.metropolis_update, states copied back"},
        "e2e": {"value": 1.0 / dt_dev, "unit": "updates/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 1,
                "note": "inputs and outputs are device tensors; one byte "
                        "(the BF16-exactness flag of the new couplings) "
                        "reaches the host per update"}}), flush=True)
    return 0


def run_lattice_workload(args, w, rank, world):
    """2-D Ising lattice of the reference's tutorial
    (tutorials/ising_tutorial.py:175-242: open-boundary nearest-neighbour
    couplings -1, no field, `ones` start, sequential sweeps) at 64 x 64 =
    4096 spins: attempts/s of the sparse-row sweep, beside the dense plain
    sweep on the same chains, and end to end through Solver."""
    if rank != 0:
        return 0
    import torch
    from pysa_gb300 import Instance, PTBatch, Solver, pack_spins
    from pysa_gb300 import _lib
    from pysa_gb300._lib import check, ref
    from pysa_gb300.utils import lattice_adjacency
    L = w["side"]
    n, R, Rd = L * L, w["replicas"], w["reads"]
    P = -lattice_adjacency(L, L)
    J = P.astype(np.float32)
    h = np.zeros(n, np.float32)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    out = {}
    for name, kw in (("sparse", dict(sparse=True)),
                     ("dense_plain", dict(kernel="plain"))):
        b = PTBatch("ising", [Instance(J, h, ladder(w), Rd)], **kw)
        b.set_states(pack_spins(np.ones((Rd, R, n), np.float32), "ising",
                                b.words), None)
        st = torch.cuda.current_stream().cuda_stream
        o = _lib.Options(3, _lib.SEQUENTIAL, 1, 0, 0, 0, 0)
        steps = args.steps if name == "sparse" else max(3, args.steps // 10)
        for _ in range(args.warmup):
            check(b.lib.pysa_gb_sweeps(ref(b.p), ref(b.s), ref(b.ws), ref(o),
                                       1, st), "sweep")
        ev = []
        torch.cuda.synchronize()
        for k in range(steps):
            flush.fill_(float(k))  # L2 flush (256 MB), untimed
            e0, e1 = (torch.cuda.Event(enable_timing=True),
                      torch.cuda.Event(enable_timing=True))
            e0.record()
            check(b.lib.pysa_gb_sweeps(ref(b.p), ref(b.s), ref(b.ws), ref(o),
                                       1, st), "sweep")
            e1.record()
            ev.append((e0, e1))
        torch.cuda.synchronize()
        b.check_status()
        ms = sum(a.elapsed_time(c) for a, c in ev) / steps
        out[name] = {"ms_per_sweep": ms, "attempts_per_s": Rd * R * n / ms
                     * 1e3, "sweeps": steps,
                     "best_energy": float(b.best_energy.min().item())}
    # end to end: Solver with host buffers, sparse rows chosen by 'auto'
    sv = Solver(P, "ising", "float32")
    sv.metropolis_update(num_sweeps=2, num_reads=Rd, num_replicas=R,
                         min_temp=w["tmin"], max_temp=w["tmax"],
                         initialize_strategy="ones", sparse="auto", seed=1)
    torch.cuda.synchronize()
    e2e_sweeps = 200
    t0 = time.perf_counter()
    fr = sv.metropolis_update(num_sweeps=e2e_sweeps, num_reads=Rd,
                              num_replicas=R, min_temp=w["tmin"],
                              max_temp=w["tmax"], initialize_strategy="ones",
                              sparse="auto", seed=2, return_dataframe=False)
    dt = time.perf_counter() - t0
    words = (n + 31) // 32
    print(json.dumps({
        "metric": "spin_flip_attempts_per_s",
        "value": out["sparse"]["attempts_per_s"], "unit": "attempts/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": out["sparse"]["ms_per_sweep"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "the tutorial's lattice (deterministic)",
        "config": {"workload": args.workload, **w, "n": n,
                   "l2": "flushed (256 MB write) before every timed sweep"},
        "kernels": out,
        "e2e": {"value": Rd * R * n * e2e_sweeps / dt, "unit": "attempts/s",
                "h2d_bytes_per_step": n * n * 4 + Rd * R * words * 4,
                "d2h_bytes_per_step": Rd * R * (2 * words * 4 + 16),
                "sweeps_per_call": e2e_sweeps, "seconds": dt,
                "best_energy_min": float(min(r["best_energy"] for r in fr))},
        "gpu_launches": 2 * args.steps}), flush=True)
    return 0


def _reference_sample(w):
    """(ptype, P, description) of the instance the reference arm times."""
    if w["kind"] == "sk_batch":
        rng = np.random.default_rng(4242)
        sizes = rng.integers(w["nmin"], w["nmax"] + 1, w["instances"])
        n = int(np.sort(sizes)[len(sizes) // 2])
        w2 = dict(w, kind="sk", n=n)
        ptype, P = make_instance(w2)
        return ptype, P, w2, f"median-size instance of the batch (n={n})"
    if w["kind"] == "lattice":
        from pysa_gb300.utils import lattice_adjacency
        L = w["side"]
        return ("ising", -lattice_adjacency(L, L).astype(np.float32),
                dict(w, n=L * L), f"the {L} x {L} lattice")
    ptype, P = make_instance(w)
    return ptype, P, w, "the workload's instance"


def run_reference_ais(args, w, rank, world):
    """Oracle AIS (restatement of pysa/simulation.py:293-317) on one SK
    instance of the workload, all host threads over samples."""
    if rank != 0:
        return 0
    oracle = _timed_oracle()
    n = w["n"]
    rng = np.random.default_rng(24)
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    J = (w["beta"] * (J + J.T)).astype(np.float32)
    h = np.zeros(n, np.float32)
    temps = np.linspace(0.0, 1.0, w["temps"]).astype(np.float32)
    ns = 256
    times = []
    for k in range(args.warmup + args.steps):
        x0 = (2 * np.random.default_rng(k).integers(0, 2, (ns, n)) - 1
              ).astype(np.float32)
        t0 = time.perf_counter()
        oracle.ais_run("ising", J, h, temps, x0, seed=k, update="sequential",
                       ref="uniform", order="reference")
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = ns * w["temps"] * n * len(times) / sum(times)
    cores = os.cpu_count() or 1
    print(json.dumps({
        "impl": "reference", "metric": "ais_attempts_per_s", "value": value,
        "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 weights)",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, **{k: w[k] for k in w}},
        "cpu_baseline": {"value": value, "unit": "attempts/s", "cores": cores,
                         "kind": "port",
                         "sample": f"one instance, {ns} samples x "
                                   f"{w['temps']} temperatures per step"},
        "e2e": {"value": value, "unit": "attempts/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)
    return 0


def workload_config(name, w, n, R, Rd):
    """`config` of a single-instance workload's line; both arms print the
    same dict so that their lines describe the same job."""
    return {"workload": name, "n": n, "replicas": R, "reads": Rd,
            "chains": Rd * R, "update": w["update"],
            "exchange": "every sweep", "problem": w["kind"],
            "l2": "GPU arm: flushed (256 MB write) before every timed call "
                  "(a call is one sweep and its exchange, or a fused launch "
                  "of up to 128 sweeps whose fields stay in tensor memory); "
                  "reference arm: host cores, no flush"}


def run_reference_arm(args, w, rank, world):
    """The reference's algorithm on the host cores (the oracle's tuned
    build, all threads over chains), on real chains of the workload: a step
    is `per_step` sweeps of `reads` reads (all the workload's reads when one
    sweep of them takes at most about a second), state carried from step to
    step as pysa/simulation.py:150-171 carries it, so no step repeats the
    set-up of its predecessor.  Sized from the warm-up steps so that a step
    takes about a second."""
    if rank != 0:
        return 0
    if w["kind"] == "ais":
        return run_reference_ais(args, w, rank, world)
    oracle = _timed_oracle()
    name = args.workload
    single = w["kind"] in ("qubo", "sk", "wishart")
    ptype, P, w, what = _reference_sample(w)
    cores = os.cpu_count() or 1
    h = np.diag(P).astype(np.float32).copy()
    J = P.copy()
    np.fill_diagonal(J, 0)
    R, n, Rd = w["replicas"], w["n"], w["reads"]
    update = w.get("update", "sequential")
    betas = ladder(w)

    def chains(reads):
        """Seeded random states and their energies s.(J s / 2 + h)."""
        rng = np.random.default_rng(5)
        x = rng.integers(0, 2, (reads, R, n)).astype(np.float32)
        if ptype != "qubo":
            x = 2 * x - 1
        x64 = x.reshape(-1, n).astype(np.float64)
        e = (x64 * (0.5 * (x64 @ J.astype(np.float64)) + h)).sum(1)
        return x, e.reshape(reads, R).astype(np.float32)

    # calibration: one sweep of 4 reads
    x, _ = chains(4)
    t0 = time.perf_counter()
    oracle.pt_run(ptype, J, h, betas, x, np.zeros((4, R), np.float32),
                  np.tile(np.arange(R, dtype=np.int32), (4, 1)), seed=1,
                  num_sweeps=1, update=update)
    per_read = (time.perf_counter() - t0) / 4
    # all the workload's reads unless one sweep of them would take over
    # about 3 s (4 reads overestimate the per-read time: few chains per
    # thread); sweeps per step rescaled after every warm-up step
    reads = int(min(Rd, max(4, 3.0 // max(per_read, 1e-9))))
    per_step = 1
    x, e = chains(reads)
    st = dict(spins=x, energies=e,
              beta_idx=np.tile(np.arange(R, dtype=np.int32), (reads, 1)))
    best = None
    times = []
    sweep = 0
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        out = oracle.pt_run(ptype, J, h, betas, st["spins"], st["energies"],
                            st["beta_idx"], seed=1, num_sweeps=per_step,
                            first_sweep=sweep, update=update, best=best)
        dt = time.perf_counter() - t0
        sweep += per_step
        st = out
        best = (out["best_energy"], out["best_sweep"], out["best_spins"])
        if k < args.warmup:
            per_step = int(max(1, round(per_step / max(dt, 1e-9))))
        if k >= args.warmup:
            times.append(dt)
    attempts_per_step = reads * R * n * per_step
    value = attempts_per_step * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": "spin_flip_attempts_per_s",
        "value": value, "unit": "attempts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": (workload_config(name, w, n, R, Rd)
                   if single else
                   {"workload": name, **{k: w[k] for k in w}}),
        "cpu_baseline": {
            "value": value, "unit": "attempts/s", "cores": cores,
            "kind": "port",
            "sample": f"{what}: {reads} of {Rd} reads x {R} replicas, "
                      f"{per_step} sweeps (each with its exchange) per timed "
                      f"step, chains carried across steps; the oracle's "
                      "C restatement of the reference's dense-dot rule in its "
                      "build tuned for this CPU, OpenMP over chains (numba is "
                      "not installed)"},
        "e2e": {"value": value, "unit": "attempts/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="qubo1024", choices=list(WORKLOADS))
    ap.add_argument("--kernel", default="auto",
                    choices=["auto", "tc", "plain", "autotune"],
                    help="sweep kernel of the single-instance workloads")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-sweeps", type=int, default=None)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if w["kind"] == "rbm":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable":
                                  "the reference's RBM caller runs "
                                  "pysa.sa.Solver, which needs numba (absent "
                                  "here); its host recipe is timed on the "
                                  "GPU arm's line instead"}))
            return 0
        return run_rbm_workload(args, w, rank, world)
    if w["kind"] == "lattice" and args.impl != "reference":
        return run_lattice_workload(args, w, rank, world)
    if w["kind"] in ("sk_batch", "ais") and args.impl != "reference":
        fn = run_batch_workload if w["kind"] == "sk_batch" else run_ais_workload
        return fn(args, w, rank, world)
    if args.workload.endswith("_tts"):
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable":
                                  "TTS workload compares two GPU arms; the "
                                  "reference has no learned proposal"}))
            return 0
        return run_tts_workload(args, w, rank, world)
    if args.impl == "reference":
        return run_reference_arm(args, w, rank, world)

    import torch
    from pysa_gb300 import Instance, PTBatch, Solver, pack_spins
    from pysa_gb300 import _lib
    from pysa_gb300._lib import check, ref

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ptype, P = make_instance(w)
    h = np.diag(P).astype(np.float32).copy()
    J = P.copy()
    np.fill_diagonal(J, 0)
    R, Rd, n = w["replicas"], w["reads"], w["n"]
    batch = PTBatch(ptype, [Instance(J, h, ladder(w), Rd)], kernel=args.kernel)
    if args.kernel == "autotune":
        batch.set_states(pack_spins(
            np.zeros((Rd, R, n), np.float32), ptype, batch.words), None)
        batch.autotune()
    use_tc = batch.tc
    if use_tc and w["update"] == "random":
        batch._setup_random_tc()   # tiles repacked in each sweep's order
    rng = np.random.default_rng(100 + rank)
    if ptype == "qubo":
        x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    else:
        x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    batch.set_states(pack_spins(x0, ptype, batch.words), None)
    upd = _lib.RANDOM if w["update"] == "random" else _lib.SEQUENTIAL
    seed = 7 + rank

    rc_every = 4 if (use_tc and batch.tc_terms == 2) else 0

    def opts(phases):
        return _lib.Options(seed, upd, 1, 0, 0, phases, rc_every)

    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    lib = batch.lib
    o_all, o_sweep, o_x = opts(3), opts(1), opts(2)
    check(lib.pysa_gb_sweeps(ref(batch.p), ref(batch.s), ref(batch.ws),
                             ref(o_all), 0, st), "sweeps")
    for _ in range(args.warmup):
        check(lib.pysa_gb_sweeps(ref(batch.p), ref(batch.s), ref(batch.ws),
                                 ref(o_all), 1, st), "sweeps")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32,
                        device="cuda")
    # With every instance on the tensor cores and R dividing the chains per
    # CTA, a launch runs several sweeps with the exchange fused in and the
    # fields resident in tensor memory: time launches of 128 sweeps (the
    # library's launch size; L2 flushed before each).  Otherwise time each
    # sweep and its exchange.
    fused = bool(use_tc and batch.ws.plain_live == 0 and batch.ws.tc_fusable)
    chunk = 128 if fused else 1
    iters = []
    done = 0
    while done < args.steps:
        iters.append(min(chunk, args.steps - done))
        done += iters[-1]
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in iters]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    with sampler:
        torch.cuda.synchronize()
        for k, cnt in enumerate(iters):
            flush.fill_(float(k))  # L2 flush (256 MB > 129 MB L2), untimed
            a, b, c = ev[k]
            a.record(stream)
            if fused:
                check(lib.pysa_gb_sweeps(ref(batch.p), ref(batch.s),
                                         ref(batch.ws), ref(o_all), cnt, st),
                      "sweeps")
                b.record(stream)
            else:
                check(lib.pysa_gb_sweeps(ref(batch.p), ref(batch.s),
                                         ref(batch.ws), ref(o_sweep), 1, st),
                      "sweep")
                b.record(stream)
                check(lib.pysa_gb_sweeps(ref(batch.p), ref(batch.s),
                                         ref(batch.ws), ref(o_x), 1, st),
                      "exchange")
            c.record(stream)
        torch.cuda.synchronize()
    batch.check_status()
    accuracy = None
    if w["kind"] == "wishart":
        accuracy = field_errors(batch, J, h, ptype)
        # the energies a run returns: recomputed from the spins at its end
        batch.recompute()
        accuracy["returned_energy_err_of_scale"] = field_errors(
            batch, J, h, ptype)["energy_err_of_scale"]
        _, t_pl, e_gs = planted_wishart(n, w["m"], np.random.default_rng(2024))
        rbest = batch.best_energy.view(Rd, R).min(dim=1).values.cpu().numpy()
        accuracy.update({
            "planted_energy": e_gs,
            "best_energy": float(rbest.min()),
            "reads_at_planted": int((rbest <= e_gs + 1e-5 * abs(e_gs)).sum()),
            "sweeps_run": args.warmup + args.steps,
            "block_b": 64,
            "note": "fields and energies after the last timed sweep, "
                    "accumulated since the last in-kernel recompute (every "
                    "4 sweeps, compensated f32 sums); per-chain relative "
                    "(energy_max_rel_err) and relative to the largest |E| "
                    "(energy_err_of_scale); returned_*: after the final "
                    "recompute a run ends with"})
    # per-sweep kernel time (fused launches include their exchange)
    sweep_ms = [a.elapsed_time(b) / cnt for (a, b, _), cnt in zip(ev, iters)]
    step_ms = [a.elapsed_time(c) / cnt for (a, _, c), cnt in zip(ev, iters)]
    total_s = sum(a.elapsed_time(c) for a, _, c in ev) / 1e3
    if dist:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    attempts_per_step = Rd * R * n
    value = attempts_per_step * args.steps * world / total_s

    # plain CUDA-core sweep on the same chains, for comparison
    plain = None
    if use_tc:
        pb = PTBatch(ptype, [Instance(J, h, ladder(w), Rd)], kernel="plain")
        pb.set_states(pack_spins(x0, ptype, pb.words), None)
        po = _lib.Options(seed, upd, 1, 0, 0, 1, 0)
        for _ in range(3):
            check(lib.pysa_gb_sweeps(ref(pb.p), ref(pb.s), ref(pb.ws),
                                     ref(po), 1, st), "plain warm-up")
        pk = min(args.steps, 30)
        pev = [(torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True)) for _ in range(pk)]
        for a_, b_ in pev:
            flush.fill_(1.0)
            a_.record(stream)
            check(lib.pysa_gb_sweeps(ref(pb.p), ref(pb.s), ref(pb.ws),
                                     ref(po), 1, st), "plain sweep")
            b_.record(stream)
        torch.cuda.synchronize()
        pms = float(np.mean([a_.elapsed_time(b_) for a_, b_ in pev]))
        plain = {"kernel": "k_sweep_plain<32,4,8,8>", "sweep_ms": pms,
                 "value": Rd * R * n / (pms / 1e3), "unit": "attempts/s",
                 "steps": pk}
        del pb

    C = Rd * R
    sweep_s = np.mean(sweep_ms) / 1e3
    hbm, bf16, peak_kind = measured_peaks()
    if use_tc:
        # algorithmic tensor work of one sweep launch: the rank-64 field
        # updates H += A B over every block, 2 C n^2 FLOP per BF16 term
        terms = batch.tc_terms
        alg = 2.0 * C * n * n * terms
        fold = 1 if n <= 512 else (2 if n <= 1024 else 4)
        fp8 = bool(getattr(batch, "tc_fp8", False))
        # E4M3 tiles run kind::f8f6f4 MMAs: no measured FP8 peak exists, so
        # the denominator is twice the measured BF16 one (the nominal dense
        # FP8 : BF16 ratio, 4.5 : 2.25 PFLOP/s)
        peak = 2.0 * bf16 if fp8 else bf16
        roof = {"bound": "tensor", "achieved": alg / sweep_s / 1e12,
                "peak": peak, "unit": "TFLOP/s",
                "frac": alg / sweep_s / 1e12 / peak, "traffic": None,
                "peak_source": peak_kind + (
                    " (2 x bf16 burst: nominal fp8/bf16 ratio)" if fp8
                    else " (bf16 burst)"),
                "kernel": f"k_sweep_tc<{fold}{', e4m3' if fp8 else ''}>",
                "tile_format": "e4m3" if fp8 else "bf16", "bf16_terms": terms,
                "issued_flop_per_launch": alg * fold,
                "alg_flop_per_launch": alg, "sweep_ms": sweep_s * 1e3}
        tp = os.path.join(ROOT, "profiles",
                          f"sweep_tc_{args.workload}_traffic.json")
    else:
        # algorithmic bytes of one launch: fields read+write, spins
        # read+write, J once
        alg_bytes = C * (2 * 4 * n + 2 * 4 * batch.words + 16) + 4 * n * n
        roof = {"bound": "hbm", "achieved": alg_bytes / sweep_s / 1e9,
                "peak": hbm, "unit": "GB/s",
                "frac": alg_bytes / sweep_s / 1e9 / hbm, "traffic": None,
                "peak_source": peak_kind, "kernel": "k_sweep_plain<32,4,8,8>",
                "alg_bytes_per_launch": int(alg_bytes),
                "sweep_ms": sweep_s * 1e3}
        tp = os.path.join(ROOT, "profiles",
                          f"sweep_plain_{args.workload}_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
            # per sweep, like `achieved` (one ncu capture of a 32-sweep launch)
            roof["traffic"] = tj.get("bytes_per_sweep", tj.get("bytes_per_launch"))

    # end to end through the public API (host buffers in and out)
    e2e = None
    if not args.no_e2e:
        sweeps_e2e = args.e2e_sweeps or w["sweeps"]
        solver = Solver(P.astype(np.float64), ptype, "float32")
        kw = dict(num_sweeps=sweeps_e2e, num_reads=Rd, num_replicas=R,
                  min_temp=w["tmin"], max_temp=w["tmax"],
                  update_strategy=w["update"], return_dataframe=False)
        np.random.seed(rank)
        solver.metropolis_update(**dict(kw, num_sweeps=2), seed=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rows = solver.metropolis_update(**kw, seed=2)
        e2e_s = time.perf_counter() - t0
        words = batch.words
        # couplings, fields, ladder, int8 initial states (made float32 and
        # packed on the device); float32 final states, spin words of the
        # best states, per-chain energies, slots, best energies and sweeps
        h2d = 4 * n * n + 4 * n + 4 * R + C * n
        d2h = C * (n * 4 + words * 4 * 2 + 4 * 4)
        # the returned energies must be the energies of the returned states
        # (f64 recomputation, pysa/qubo.py:32-37; exact for integer QUBO)
        Jd = torch.from_numpy(J.astype(np.float64)).cuda()
        hd = torch.from_numpy(h.astype(np.float64)).cuda()
        S = torch.from_numpy(np.stack([r["states"] for r in rows]).reshape(
            -1, n).astype(np.float64)).cuda()
        Ef = (S * (0.5 * (S @ Jd) + hd)).sum(1).cpu().numpy()
        Eg = np.concatenate([r["energies"] for r in rows]).astype(np.float64)
        e_err = float(np.max(np.abs(Eg - Ef)) / max(np.abs(Ef).max(), 1.0))
        tol = 0.0 if w["kind"] == "qubo" else 1e-5
        if e_err > tol:
            raise AssertionError(f"e2e: returned energies differ from the "
                                 f"returned states' energies ({e_err:.3e})")
        del S, Jd, hd
        # a step is one sweep: the call's copies amortised over its sweeps
        e2e = {"value": Rd * R * n * sweeps_e2e / e2e_s, "unit": "attempts/s",
               "h2d_bytes_per_step": int(h2d // sweeps_e2e),
               "d2h_bytes_per_step": int(d2h // sweeps_e2e),
               "h2d_bytes_per_call": int(h2d), "d2h_bytes_per_call": int(d2h),
               "sweeps_per_call": sweeps_e2e, "seconds": e2e_s,
               "best_energy_min": float(min(r["best_energy"] for r in rows)),
               "energy_check": {"max_err_of_scale": e_err, "tolerance": tol,
                                "against": "f64 energies of the returned "
                                           "states"}}

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        reads_cpu = 16
        rate, dt = cpu_reference(w, ptype, P, reads_cpu, 2)
        # size the sample to about 15 s of CPU work
        sweeps_cpu = max(2, int(2 * 15.0 / max(dt, 1e-3)))
        rate, dt = cpu_reference(w, ptype, P, reads_cpu, sweeps_cpu)
        cpu = {"value": rate, "unit": "attempts/s",
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{reads_cpu} reads x {R} replicas x {sweeps_cpu} "
                         f"sweeps of the same instance ({dt:.1f} s); C "
                         "restatement of the reference's dense-dot update, "
                         "OpenMP over chains"}

    if rank == 0:
        line = {
            "metric": "spin_flip_attempts_per_s", "value": value,
            "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(args.workload, w, n, R, Rd),
            "timing": {"l2": ("flushed (256 MB write) before every timed "
                              "call of up to %d sweeps; fields stay in "
                              "tensor memory within a launch" % chunk)
                             if fused else
                             "flushed (256 MB write) before every step",
                       "sweeps_per_call": iters,
                       "kernel_choice": args.kernel,
                       "tc_min_n": batch.tc_min_n,
                       "kernel": ("persistent tensor-core blocked sweep "
                                  "(tcgen05, %s%s)" %
                                  ("E4M3 tiles" if getattr(batch, "tc_fp8",
                                                           False)
                                   else "split-BF16",
                                   ", exchange fused" if fused else ""))
                                 if use_tc else
                                 "plain local-field sweep (CUDA cores)"},
            "roofline": roof,
            "plain_gpu": plain,
            "accuracy": accuracy,
            "clocks": sampler.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            # fused: one persistent launch per chunk of up to 128 sweeps, or
            # in random order per group of tc_rand_slots sweeps a visiting-
            # order kernel, a repack kernel and the sweep launch
            "gpu_launches": ((sum(3 * -(-c // int(batch.ws.tc_rand_slots))
                                  for c in iters) if upd else len(iters))
                             if fused else
                             2 * args.steps + (args.steps if upd else 0)),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
