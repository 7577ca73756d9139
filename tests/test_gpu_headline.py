"""The exact code path of the headline measurement, bit for bit against the
CPU oracle.

The dense-QUBO workload (n = 1024, Q_ij integers in [-8, 8], diagonal in
[-16, 16], 64 replicas on a geometric 0.5-8.0 temperature ladder) runs on the
persistent tensor-core sweep at fold 2 (64 chains per CTA).  R = 64 divides
the chains per CTA, so the replica exchange runs inside the kernel and one
launch covers up to 128 sweeps.  Work items of one instance size split a
launch's item-sweeps evenly over the CTAs (wrap-around units: a CTA runs the
first sweeps of one item, whole items, then the last sweeps of an item whose
first sweeps another CTA ran); with the unit length fixed by the caller,
CTAs take fixed-length units from a queue instead.  These tests drive that
path under three schedules -- one CTA per item, wrap-around units split over
two CTAs, fixed 8-sweep units -- with fused exchange, unit and launch
boundaries, runs whose length is not a multiple of 8, and CUDA-graph
replays, and compare every returned array with the oracle
(pysa/simulation.py:150-171, pysa/qubo.py:40-63, pysa/utils.py:44-58 on the
shared Philox stream).  Integer couplings make every product and sum exact,
so equality is required.  The same at fold 4 (n = 1300, 32 chains per CTA,
R = 32) and fold 1.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHEDULES = ["per_item", "wrap2", "fixed8"]
# tile formats: integer couplings |J| <= 16 are exact in FP8 E4M3 (the
# default for them) and in BF16
FORMATS = ["e4m3", "bf16"]


@pytest.fixture
def schedule_knobs():
    """Applies a schedule to a batch; puts the process-wide CTA cap back."""
    from pysa_gb300 import _lib
    lib = _lib.load()

    def apply(b, schedule):
        if schedule == "fixed8":
            b.ws.tc_unit_sweeps = 8
        _lib.check(lib.pysa_gb_set_tc_max_ctas(
            2 if schedule == "wrap2" else 0), "max ctas")
    yield apply
    _lib.check(lib.pysa_gb_set_tc_max_ctas(0), "max ctas reset")


def _qubo(rng, n):
    Q = np.triu(rng.integers(-8, 9, (n, n)), 1)
    Q = (Q + Q.T).astype(np.float32)
    return Q, rng.integers(-16, 17, n).astype(np.float32)


def _ising_pm1(rng, n):
    P = np.triu(2 * rng.integers(0, 2, (n, n)) - 1, 1)
    return (P + P.T).astype(np.float32), np.zeros(n, np.float32)


def _check_equal(got, want, Rd, R, n, ptype):
    from pysa_gb300 import unpack_spins
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, ptype, np.float32)
    bs = unpack_spins(got["best_spins"].reshape(Rd, R, -1), n, ptype,
                      np.float32)
    assert (sp == want["spins"]).all(), "spins"
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (bs == want["best_spins"]).all(), "best spins"


def _fused_batch(ptype, J, h, betas, Rd, fold, fmt="e4m3"):
    from pysa_gb300 import Instance, PTBatch
    b = PTBatch(ptype, [Instance(J, h, betas, Rd)], kernel="tc",
                tc_fp8=fmt == "e4m3")
    assert b.tc_fp8 == (fmt == "e4m3") and b.ws.tc_fp8 == b.tc_fp8
    # the path under test: every instance on the tensor cores at this fold,
    # exchange fused into the kernel
    v = {1: 0, 2: 1, 4: 2}[fold]
    assert b.tc and b.tc_terms == 1
    assert b.ws.tc_variant_count[v] > 0
    assert sum(b.ws.tc_variant_count[k] for k in range(3)) == \
        b.ws.tc_variant_count[v]
    assert b.ws.tc_fusable == 1 and b.ws.plain_live == 0
    return b


def _run_vs_oracle(oracle, ptype, n, R, Rd, tmin, tmax, plan, seed,
                   fold, graph_chunk=128, knobs=None, schedule="per_item",
                   fmt="e4m3"):
    """plan: the sweep counts of consecutive run() calls on one batch (each
    call continues the previous one's chains, as Solver resumes)."""
    from pysa_gb300 import pack_spins
    rng = np.random.default_rng(seed)
    J, h = _qubo(rng, n) if ptype == "qubo" else _ising_pm1(rng, n)
    betas = (1.0 / np.geomspace(tmin, tmax, R)).astype(np.float32)
    if ptype == "qubo":
        x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    else:
        x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    b = _fused_batch(ptype, J, h, betas, Rd, fold, fmt)
    if knobs is not None:
        knobs(b, schedule)
    if schedule != "fixed8":
        assert b.ws.tc_uniform & (1 << {1: 0, 2: 1, 4: 2}[fold])
    b.set_states(pack_spins(x0, ptype, b.words), e0)
    bidx = np.tile(np.arange(R, dtype=np.int32), (Rd, 1))
    state = (x0, e0, bidx, None)
    done = 0
    for sweeps in plan:
        b.run(sweeps, seed=seed, graph_chunk=graph_chunk)
        got = b.fetch()
        sp, en, bi, best = state
        want = oracle.pt_run(ptype, J, h, betas, sp, en, bi, seed=seed,
                             num_sweeps=sweeps, first_sweep=done, best=best)
        _check_equal(got, want, Rd, R, n, ptype)
        state = (want["spins"], want["energies"], want["beta_idx"],
                 (want["best_energy"], want["best_sweep"],
                  want["best_spins"]))
        done += sweeps
    assert int(b.sweep_counter.item()) == done


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("plan", [(136,), (20,), (20, 13, 1)])
def test_headline_qubo1024_fold2_fused_bit_exact(oracle, schedule_knobs,
                                                 plan, schedule, fmt):
    """136 sweeps: a 128-sweep launch, then an 8-sweep one (fixed8: sixteen
    8-sweep units, then one; wrap2: three items over two CTAs, the middle
    item split at sweep 64, then at sweep 4).  20 and 20 + 13 + 1: runs
    whose length is not a multiple of 8, resumed across calls."""
    _run_vs_oracle(oracle, "qubo", 1024, 64, 3, 0.5, 8.0, plan, seed=11,
                   fold=2, knobs=schedule_knobs, schedule=schedule, fmt=fmt)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_headline_qubo1024_fold2_graph_replay_bit_exact(oracle, schedule_knobs,
                                                        schedule):
    """300 sweeps as run() issues them for long runs: two replays of a
    captured 128-sweep graph, then 44 sweeps issued directly."""
    _run_vs_oracle(oracle, "qubo", 1024, 64, 3, 0.5, 8.0, (300,), seed=12,
                   fold=2, knobs=schedule_knobs, schedule=schedule)


@pytest.mark.parametrize("fmt", FORMATS)
def test_headline_ising_pm1_fold2_fused_bit_exact(oracle, fmt):
    _run_vs_oracle(oracle, "ising", 1000, 64, 2, 0.3, 3.0, (136,), seed=13,
                   fold=2, fmt=fmt)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("plan", [(136,), (20,)])
def test_fold4_qubo1300_fused_bit_exact(oracle, schedule_knobs, plan,
                                        schedule, fmt):
    _run_vs_oracle(oracle, "qubo", 1300, 32, 3, 0.5, 8.0, plan, seed=14,
                   fold=4, knobs=schedule_knobs, schedule=schedule, fmt=fmt)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_fold1_qubo512_fused_bit_exact(oracle, schedule_knobs, schedule,
                                       fmt):
    _run_vs_oracle(oracle, "qubo", 512, 32, 4, 0.5, 8.0, (136,), seed=15,
                   fold=1, knobs=schedule_knobs, schedule=schedule, fmt=fmt)


def test_wrap_split_many_items_bit_exact(oracle, schedule_knobs):
    """Seven items over three CTAs, run lengths 128 and 9: the first CTA
    runs the head of item 2 and items 0-1, the second the head of item 4,
    item 3 and the tail of item 2, the third items 5-6 and the tail of
    item 4."""
    from pysa_gb300 import _lib
    _lib.check(_lib.load().pysa_gb_set_tc_max_ctas(3), "max ctas")
    _run_vs_oracle(oracle, "qubo", 1024, 64, 7, 0.5, 8.0, (137,), seed=16,
                   fold=2)
