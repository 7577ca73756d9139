"""Tensor-core blocked sweep (k_sweep_tc): parity with the CPU oracle.

Integer couplings are exact in BF16 and every FP32 sum stays below 2^24, so
trajectories must match the oracle (the reference's dense-dot rule on the same
Philox stream) bit for bit.  Real couplings take the split J_hi + J_lo path;
their energies are checked against an FP64 recomputation of the returned
states with the tolerance the split-BF16 path promises (1e-5 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _int_qubo(rng, n):
    Q = rng.integers(-8, 9, (n, n))
    Q = np.triu(Q, 1)
    Q = (Q + Q.T).astype(np.float32)
    return Q, rng.integers(-16, 17, n).astype(np.float32)


def _run(ptype, J, h, betas, x0, *, seed, sweeps, kernel, update="sequential",
         energies=None, **run_kw):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    Rd, R, n = x0.shape
    b = PTBatch(ptype, [Instance(J, h, betas, Rd)], kernel=kernel)
    assert b.tc == (kernel == "tc")
    b.set_states(pack_spins(x0, ptype, b.words), energies)
    b.run(sweeps, seed=seed, update=update, **run_kw)
    got = b.fetch()
    got["spins_f"] = unpack_spins(got["spins"].reshape(Rd, R, -1), n, ptype,
                                  np.float32)
    got["best_f"] = unpack_spins(got["best_spins"].reshape(Rd, R, -1), n,
                                 ptype, np.float32)
    got["batch"] = b
    return got


@pytest.mark.parametrize("n", [64, 100, 256, 300, 512, 700, 1024, 1300, 2048])
def test_tc_qubo_bit_exact_vs_oracle(oracle, n):
    rng = np.random.default_rng(1000 + n)
    J, h = _int_qubo(rng, n)
    R = 6 if n <= 1024 else 4
    Rd = 7 if n <= 512 else 3  # chain counts not multiples of 128 / F
    sweeps = 6 if n <= 1024 else 3
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    got = _run("qubo", J, h, betas, x0, seed=n, sweeps=sweeps, kernel="tc")
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=n, num_sweeps=sweeps)
    assert got["batch"].tc_terms == 1
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (got["best_f"] == want["best_spins"]).all()


def test_tc_matches_plain_kernel_ising_pm1():
    rng = np.random.default_rng(3)
    n, R, Rd = 512, 16, 9
    P = rng.integers(0, 2, (n, n))
    P = np.triu(2 * P - 1, 1)
    J = (P + P.T).astype(np.float32)
    h = np.zeros(n, np.float32)
    betas = (1.0 / np.geomspace(0.3, 3.0, R)).astype(np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    a = _run("ising", J, h, betas, x0, seed=5, sweeps=20, kernel="tc")
    b = _run("ising", J, h, betas, x0, seed=5, sweeps=20, kernel="plain")
    for k in ("spins", "energies", "beta_idx", "best_energy", "best_sweep",
              "best_spins"):
        assert (a[k] == b[k]).all(), k


@pytest.mark.parametrize("ptype,n", [("qubo", 256), ("ising", 320),
                                     ("qubo", 1500)])
def test_tc_extreme_betas_bit_exact_vs_oracle(oracle, ptype, n):
    """beta = 0 (every flip accepted), tiny and very large betas: the
    threshold form of the decision must agree with the f64 rule there."""
    rng = np.random.default_rng(77 + n)
    if ptype == "qubo":
        J, h = _int_qubo(rng, n)
        x0 = rng.integers(0, 2, (3, 6, n)).astype(np.float32)
    else:
        P = np.triu(2 * rng.integers(0, 2, (n, n)) - 1, 1)
        J = (P + P.T).astype(np.float32)
        h = rng.integers(-2, 3, n).astype(np.float32)
        x0 = (2 * rng.integers(0, 2, (3, 6, n)) - 1).astype(np.float32)
    betas = np.array([0.0, 1e-3, 0.05, 1.0, 8.0, 40.0], np.float32)
    Rd, R = x0.shape[:2]
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    got = _run(ptype, J, h, betas, x0, seed=9, sweeps=5, kernel="tc")
    want = oracle.pt_run(ptype, J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=9, num_sweeps=5)
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()


@pytest.mark.parametrize("n", [320, 1024])
def test_tc_split_bf16_energy_error(oracle, n):
    """Real couplings: J = J_hi + J_lo; energies within 1e-5 relative of an
    FP64 recomputation of the returned states; fields within 1e-5 of the
    FP64 fields."""
    rng = np.random.default_rng(n)
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    J = (J + J.T).astype(np.float32)
    h = (0.1 * rng.normal(size=n)).astype(np.float32)
    R, Rd = 8, 4
    betas = (1.0 / np.geomspace(0.2, 2.0, R)).astype(np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    got = _run("ising", J, h, betas, x0, seed=9, sweeps=200, kernel="tc")
    assert got["batch"].tc_terms == 2
    E = got["energies"].reshape(-1)
    S = got["spins_f"].reshape(-1, n)
    ref = np.array([oracle.energy64(J, h, s) for s in S])
    scale = np.abs(ref).max()
    fields = got["batch"].fields.cpu().numpy()[:len(S), :n]
    f64 = S.astype(np.float64) @ J.astype(np.float64) + h
    e_err = np.max(np.abs(E - ref)) / scale
    f_err = np.max(np.abs(fields - f64)) / np.abs(f64).max()
    print(f"n={n}: energy rel err {e_err:.3e}, field rel err {f_err:.3e}")
    assert e_err <= 1e-5
    assert f_err <= 1e-5


@pytest.mark.parametrize("n", [320, 1024, 2048])
def test_tc_split_bf16_drift_between_recomputes(oracle, n):
    """Three sweeps after the last in-kernel recompute (one every 4 sweeps,
    the default, none at the end) the accumulated energies and the fields
    stay within 2e-5 relative of FP64 from the same spins (measured up to
    8e-6 and 1.1e-5 at n = 2048; every 8 sweeps gave 1.1e-5 energies at
    n = 1024 after seven).  Returned energies are recomputed at the end and
    meet 1e-5 (test_tc_split_bf16_energy_error)."""
    rng = np.random.default_rng(7 * n)
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    J = (J + J.T).astype(np.float32)
    h = (0.1 * rng.normal(size=n)).astype(np.float32)
    R, Rd = 8, 4
    betas = (1.0 / np.geomspace(0.2, 2.0, R)).astype(np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    got = _run("ising", J, h, betas, x0, seed=5, sweeps=199, kernel="tc",
               recompute_every=4, final_recompute=False)
    assert got["batch"].tc_terms == 2
    E = got["energies"].reshape(-1)
    S = got["spins_f"].reshape(-1, n)
    ref = np.array([oracle.energy64(J, h, s) for s in S])
    fields = got["batch"].fields.cpu().numpy()[:len(S), :n]
    f64 = S.astype(np.float64) @ J.astype(np.float64) + h
    e_err = np.max(np.abs(E - ref)) / np.abs(ref).max()
    f_err = np.max(np.abs(fields - f64)) / np.abs(f64).max()
    print(f"n={n}: after 3 sweeps of drift: energy rel err {e_err:.3e}, "
          f"field rel err {f_err:.3e}")
    assert e_err <= 2e-5
    assert f_err <= 2e-5


@pytest.mark.parametrize("every", [1, 3])
def test_tc_recompute_keeps_integer_trajectory(oracle, every):
    """The in-kernel recompute pass rebuilds the same exact fields and
    energies on integer couplings: the trajectory stays bit-exact."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    rng = np.random.default_rng(31)
    n, R, Rd, S = 768, 6, 5, 7
    J, h = _int_qubo(rng, n)
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    b = PTBatch("qubo", [Instance(J, h, betas, Rd)], kernel="tc")
    b.set_states(pack_spins(x0, "qubo", b.words), None)
    b.run(S, seed=4, recompute_every=every)
    got = b.fetch()
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=4, num_sweeps=S)
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, "qubo", np.float32)
    assert (sp == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()


@pytest.mark.parametrize("kernel", ["auto", "autotune"])
def test_mixed_tc_and_plain_batch_bit_exact(oracle, kernel):
    """One batch where instances with n >= 64 take the tensor-core sweep
    and the others the plain kernel in the same sweep (kernel='auto'), or
    whatever split the autotuner picks: every instance must still follow
    the oracle bit for bit, and tuning must not change the chains."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    rng = np.random.default_rng(31)
    sizes, R, Rd, S = [100, 300, 40, 700, 1300], 4, 3, 12
    insts, x0s = [], []
    for n in sizes:
        J, h = _int_qubo(rng, n)
        betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
        insts.append(Instance(J, h, betas, Rd))
        x0s.append(rng.integers(0, 2, (Rd, R, n)).astype(np.float32))
    b = PTBatch("qubo", insts, kernel=kernel)
    assert b.tc and b.tc_min_n == 64
    words = b.words
    b.set_states(np.concatenate([pack_spins(x, "qubo", words).reshape(-1, words)
                                 for x in x0s]), None)
    b.run(S, seed=5)
    if kernel == "autotune":
        assert set(b.autotune_ms) >= {64, 256, None}
    got = b.fetch()
    c0 = 0
    for i, (inst, x0) in enumerate(zip(insts, x0s)):
        n = len(inst.h)
        e0 = np.array([[oracle.energy64(inst.J, inst.h, s) for s in r]
                       for r in x0], np.float32)
        want = oracle.pt_run("qubo", inst.J, inst.h, inst.ladder, x0, e0,
                             np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                             seed=5, num_sweeps=S, inst=i)
        sl = slice(c0, c0 + R * Rd)
        sp = unpack_spins(got["spins"][sl].reshape(Rd, R, words), n, "qubo",
                          np.float32)
        assert (sp == want["spins"]).all(), f"instance {i} (n={n})"
        assert (got["energies"][sl].reshape(Rd, R) == want["energies"]).all()
        assert (got["best_energy"][sl].reshape(Rd, R)
                == want["best_energy"]).all()
        c0 += R * Rd


@pytest.mark.parametrize("n,R", [(100, 4), (300, 3), (700, 4), (1300, 4),
                                 (1300, 3)])
def test_tc_random_order_bit_exact_vs_oracle(oracle, n, R):
    """Random visiting order on the tensor cores (tiles repacked in each
    sweep's shared permutation): same trajectories as the oracle's random
    sweep, over more sweeps than the repacked-tile slots hold.  R = 4 divides
    the chains per CTA (exchange inside the kernel); R = 3 does not (one
    launch per sweep and a separate exchange)."""
    rng = np.random.default_rng(2000 + n + R)
    J, h = _int_qubo(rng, n)
    Rd, sweeps = 3, 37
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    got = _run("qubo", J, h, betas, x0, seed=n + R, sweeps=sweeps,
               kernel="tc", update="random")
    b = got["batch"]
    assert b.ws.tc_rand_slots >= 1 and b.ws.tc_rand_slots < sweeps
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=n + R, num_sweeps=sweeps, update="random")
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (got["best_f"] == want["best_spins"]).all()


def test_tc_random_order_mixed_batch_matches_plain():
    """Random order in a batch whose small instance stays on the plain
    kernel: both kernels follow the same permutations and streams."""
    from pysa_gb300 import Instance, PTBatch, pack_spins
    rng = np.random.default_rng(77)
    sizes, R, Rd = [40, 260, 600], 4, 2
    insts, x0s = [], []
    for n in sizes:
        J, h = _int_qubo(rng, n)
        insts.append(Instance(J, h, (1.0 / np.geomspace(0.5, 8.0, R)
                                     ).astype(np.float32), Rd))
        x0s.append(rng.integers(0, 2, (Rd, R, n)).astype(np.float32))
    out = {}
    for kernel in ("auto", "plain"):
        b = PTBatch("qubo", insts, kernel=kernel)
        w = b.words
        b.set_states(np.concatenate([pack_spins(x, "qubo", w).reshape(-1, w)
                                     for x in x0s]), None)
        b.run(21, seed=3, update="random")
        out[kernel] = b.fetch()
    assert b.tc is False
    for k in ("spins", "energies", "beta_idx", "best_energy", "best_sweep",
              "best_spins"):
        assert (out["auto"][k] == out["plain"][k]).all(), k


def test_energy_drift_is_reported_not_hidden():
    """A non-finite coupling makes the in-kernel recompute disagree with the
    accumulated energies: the status word says so and the host raises (no
    fault, no hang: NaN arithmetic only)."""
    from pysa_gb300 import Instance, PTBatch, pack_spins
    from pysa_gb300._lib import LibraryError
    rng = np.random.default_rng(4)
    n, R, Rd = 128, 4, 2
    J = np.triu(rng.normal(size=(n, n)), 1)
    J = (J + J.T).astype(np.float32)
    J[3, 7] = J[7, 3] = np.nan
    b = PTBatch("ising", [Instance(J, np.zeros(n, np.float32),
                                   np.ones(R, np.float32), Rd)], kernel="tc")
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    b.set_states(pack_spins(x0, "ising", b.words),
                 np.zeros(Rd * R, np.float32))
    b.run(8, seed=1, recompute_every=4)
    with pytest.raises(LibraryError, match="drift"):
        b.fetch()


@pytest.mark.parametrize("kernel,sparse", [("tc", None), ("plain", None),
                                           ("plain", True)])
def test_stream_keys_zero_is_the_plain_stream(kernel, sparse):
    """All-zero per-chain stream keys reproduce the keyless run; a nonzero
    key changes that chain only (every sweep kernel)."""
    from pysa_gb300 import Instance, PTBatch, pack_spins
    rng = np.random.default_rng(8)
    n, R, Rd = 200, 4, 3
    J, h = _int_qubo(rng, n)
    J[np.abs(J) < 7] = 0  # sparse enough for the sparse-row kernel
    betas = (1.0 / np.geomspace(0.5, 4.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)

    def go(keys):
        b = PTBatch("qubo", [Instance(J, h, betas, Rd)], kernel=kernel,
                    sparse=sparse)
        b.set_states(pack_spins(x0, "qubo", b.words), None)
        if keys is not None:
            b.enable_stream_keys()
            b.stream_key.copy_(keys)
        b.run(5, seed=3, use_pt=False)
        return b.fetch()["spins"]

    import torch
    base = go(None)
    zero = go(torch.zeros(R * Rd, dtype=torch.int32))
    assert (base == zero).all()
    k = torch.zeros(R * Rd, dtype=torch.int32)
    k[5] = 1
    moved = go(k)
    diff = (moved != base).any(axis=1)
    assert diff[5] and diff.sum() == 1


@pytest.mark.parametrize("R,Rd", [(4, 800), (32, 100)])
def test_tc_fold4_many_items_bit_exact_vs_oracle(oracle, R, Rd):
    """Fold 4 (n = 1300, 32 chains per CTA) with hundreds of work items, so
    that CTAs run several units one after another (one launch per sweep
    when R = 4, fused multi-sweep units when R = 32): trajectories must
    still equal the oracle's."""
    rng = np.random.default_rng(4400 + R)
    n = 1300
    J, h = _int_qubo(rng, n)
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    got = _run("qubo", J, h, betas, x0, seed=7, sweeps=6, kernel="tc",
               energies=e0)
    assert got["batch"].ws.tc_variant_count[2] >= 100
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=7, num_sweeps=6)
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()


def test_tc_fold4_split_bf16_many_items(oracle):
    """Real couplings at fold 4 (n = 1300, J = J_hi + J_lo, in-kernel
    recompute every 4 sweeps) with more work items than SMs, so CTAs run
    several units and a recompute follows blocks whose MMAs may still be
    in flight: no drift is reported and the returned energies stay within
    1e-5 relative of an FP64 recomputation."""
    rng = np.random.default_rng(4500)
    n, R, Rd = 1300, 4, 1300
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    J = (J + J.T).astype(np.float32)
    h = (0.1 * rng.normal(size=n)).astype(np.float32)
    betas = (1.0 / np.geomspace(0.2, 2.0, R)).astype(np.float32)
    x0 = (2 * rng.integers(0, 2, (Rd, R, n)) - 1).astype(np.float32)
    got = _run("ising", J, h, betas, x0, seed=3, sweeps=13, kernel="tc")
    b = got["batch"]
    assert b.tc_terms == 2 and b.ws.tc_variant_count[2] > 152
    S = got["spins_f"].reshape(-1, n).astype(np.float64)
    E64 = np.einsum("ri,ij,rj->r", S, J.astype(np.float64), S) / 2 + S @ h
    err = np.max(np.abs(got["energies"] - E64)) / np.abs(E64).max()
    assert err <= 1e-5, err
