"""Sparse-row sweep (k_sweep_csr): the field of spin i is the oracle's
fixed-order f32 dot over row i with its zero terms left out, so trajectories
equal the oracle's bit for bit for any couplings, not only integer ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sparse_problem(rng, n, degree, ptype, integer=False):
    J = np.zeros((n, n), np.float32)
    for i in range(n):
        nb = rng.choice(n, degree // 2, replace=False)
        J[i, nb] = (rng.integers(-3, 4, len(nb)) if integer else
                    rng.normal(size=len(nb))).astype(np.float32)
    J = np.triu(J, 1)
    J = (J + J.T).astype(np.float32)
    h = (rng.normal(size=n) if ptype == "ising" or not integer else
         rng.integers(-4, 5, n)).astype(np.float32)
    return J, h


def _states(rng, ptype, shape):
    x = rng.integers(0, 2, shape).astype(np.float32)
    return 2 * x - 1 if ptype == "ising" else x


def _run(ptype, J, h, betas, x0, e0, *, seed, sweeps, update, sparse=None,
         kernel="auto"):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    Rd, R, n = x0.shape
    b = PTBatch(ptype, [Instance(J, h, betas, Rd)], sparse=sparse,
                kernel=kernel, perm_slots=4)
    b.set_states(pack_spins(x0, ptype, b.words), e0.reshape(-1))
    b.run(sweeps, seed=seed, update=update)
    r = b.fetch()
    r["spins_f"] = unpack_spins(r["spins"].reshape(Rd, R, -1), n, ptype,
                                np.float32)
    r["best_f"] = unpack_spins(r["best_spins"].reshape(Rd, R, -1), n, ptype,
                               np.float32)
    r["batch"] = b
    return r


@pytest.mark.parametrize("ptype,n,degree,update", [
    ("ising", 50, 6, "sequential"), ("qubo", 300, 8, "sequential"),
    ("ising", 1000, 4, "random"), ("qubo", 77, 10, "random"),
    ("ising", 4096, 4, "sequential")])
def test_sparse_float_couplings_bit_exact_vs_oracle(oracle, ptype, n, degree,
                                                    update):
    rng = np.random.default_rng(n + degree)
    J, h = _sparse_problem(rng, n, degree, ptype)
    R, Rd = 5, 3 if n < 4096 else 1
    sweeps = 5 if n < 4096 else 2
    betas = (1.0 / np.geomspace(0.3, 3.0, R)).astype(np.float32)
    x0 = _states(rng, ptype, (Rd, R, n))
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    got = _run(ptype, J, h, betas, x0, e0, seed=n, sweeps=sweeps,
               update=update, sparse=True)
    assert got["batch"].has_sparse and not got["batch"].tc
    want = oracle.pt_run(ptype, J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=n, num_sweeps=sweeps, update=update)
    assert (got["spins_f"] == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
    assert (got["best_energy"].reshape(Rd, R) == want["best_energy"]).all()
    assert (got["best_sweep"].reshape(Rd, R) == want["best_sweep"]).all()
    assert (got["best_f"] == want["best_spins"]).all()


def test_lattice_sparse_equals_dense_kernels():
    """Integer couplings: the sparse-row, plain and tensor-core sweeps all
    follow the same trajectory (the 2-D lattice of the Ising tutorial)."""
    from pysa_gb300.utils import lattice_adjacency
    rng = np.random.default_rng(3)
    L = 20
    J = (-lattice_adjacency(L, L)).astype(np.float32)
    h = rng.integers(-1, 2, L * L).astype(np.float32)
    R, Rd = 8, 4
    betas = (1.0 / np.geomspace(1.0, 3.5, R)).astype(np.float32)
    x0 = _states(rng, "ising", (Rd, R, L * L))
    from pysa_gb300.engine import Instance, PTBatch, pack_spins
    b = PTBatch("ising", [Instance(J, h, betas, Rd)], kernel="plain")
    b.set_states(pack_spins(x0, "ising", b.words), None)
    b.energies.cpu()
    e0 = b.energies.cpu().numpy()
    res = {}
    for name, kw in (("sparse", dict(sparse=True)),
                     ("plain", dict(kernel="plain")),
                     ("tc", dict(kernel="tc"))):
        res[name] = _run("ising", J, h, betas, x0, e0, seed=5, sweeps=12,
                         update="sequential", **kw)
    for k in ("spins", "energies", "beta_idx", "best_energy", "best_sweep",
              "best_spins"):
        assert (res["sparse"][k] == res["plain"][k]).all(), k
        assert (res["sparse"][k] == res["tc"][k]).all(), k


def test_mixed_dense_and_sparse_batch(oracle):
    """Sparse, tensor-core and plain instances in one batch each follow the
    oracle's trajectory on their own random streams."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    rng = np.random.default_rng(9)
    sizes = [(120, True), (300, False), (40, False), (500, True)]
    insts, x0s, e0s = [], [], []
    R, Rd = 4, 2
    betas = (1.0 / np.geomspace(0.5, 4.0, R)).astype(np.float32)
    for n, sp in sizes:
        J, h = _sparse_problem(rng, n, 6, "qubo", integer=True)
        insts.append(Instance(J, h, betas, Rd))
        x = _states(rng, "qubo", (Rd, R, n))
        x0s.append(x)
        e0s.append(np.array([[oracle.energy64(J, h, s) for s in r]
                             for r in x], np.float32))
    b = PTBatch("qubo", insts, sparse=[s for _, s in sizes])
    assert b.tc
    words = b.words
    b.set_states(np.concatenate([pack_spins(x, "qubo", words).reshape(
        -1, words) for x in x0s]), np.concatenate([e.reshape(-1)
                                                    for e in e0s]))
    b.run(6, seed=11)
    r = b.fetch()
    for k, (n, sp) in enumerate(sizes):
        want = oracle.pt_run("qubo", insts[k].J, insts[k].h, betas, x0s[k],
                             e0s[k], np.tile(np.arange(R, dtype=np.int32),
                                             (Rd, 1)),
                             seed=11, num_sweeps=6, inst=k)
        c0 = int(b.chain_off[k])
        got = unpack_spins(r["spins"][c0:c0 + R * Rd].reshape(Rd, R, -1), n,
                           "qubo", np.float32)
        assert (got == want["spins"]).all(), k
        assert (r["energies"][c0:c0 + R * Rd].reshape(Rd, R) ==
                want["energies"]).all(), k


def test_sparse_log_omega_and_solver_auto():
    """Solver on the Ising tutorial's lattice problem: sparse='auto' picks
    the sparse-row sweep and matches the dense run; log_Zf needs beta = 0."""
    from pysa_gb300 import Solver
    from pysa_gb300.utils import lattice_adjacency
    P = -lattice_adjacency(16, 16)
    s = Solver(P, "ising", "float32")
    kw = dict(num_sweeps=20, num_reads=3, num_replicas=6, min_temp=1.0,
              max_temp=3.5, initialize_strategy="ones", sort_output_temps=True,
              get_part_fun=True, seed=4, return_dataframe=False)
    a = s.metropolis_update(sparse="auto", **kw)
    b = s.metropolis_update(sparse=None, **kw)
    for ra, rb in zip(a, b):
        assert (ra["states"] == rb["states"]).all()
        assert ra["best_energy"] == rb["best_energy"]
        assert ra["log_Zf"] == rb["log_Zf"]


def test_sparse_storage_prepare_and_energies_from_rows(oracle):
    """Sparse instances keep no dense couplings on the device: their fields
    and energies (pysa_gb_prepare) and their f64 energies
    (pysa_gb_energy64_tables) come from the stored rows, equal to the
    oracle's f64 energies for integer couplings.  n = 9216 (a 96 x 96
    lattice with integer couplings) also takes the sparse sweep past the
    register-resident kernel's 4096 spins, in both orders."""
    import torch
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins, _lib
    from pysa_gb300._lib import check, ref
    from pysa_gb300.utils import lattice_adjacency
    rng = np.random.default_rng(12)
    L = 96
    A = lattice_adjacency(L, L, sparse=True).tocoo()
    w = rng.integers(-3, 4, A.nnz)
    upper = A.row < A.col
    import scipy.sparse as sps
    U = sps.coo_matrix((w[upper], (A.row[upper], A.col[upper])),
                       shape=A.shape)
    Jsp = (U + U.T).tocsr().astype(np.float32)
    n = L * L
    h = rng.integers(-2, 3, n).astype(np.float32)
    R, Rd = 4, 2
    betas = (1.0 / np.geomspace(0.5, 3.0, R)).astype(np.float32)
    x0 = _states(rng, "ising", (Rd, R, n))
    Jd = Jsp.toarray()
    e0 = np.array([[oracle.energy64(Jd, h, s) for s in r] for r in x0])
    for update in ("sequential", "random"):
        b = PTBatch("ising", [Instance(Jsp, h, betas, Rd)], sparse=True,
                    perm_slots=2)
        assert b._t["J"].numel() == 1      # no dense couplings stored
        b.set_states(pack_spins(x0, "ising", b.words), None)
        got_e0 = b.energies.cpu().numpy().reshape(Rd, R)
        assert np.array_equal(got_e0, e0.astype(np.float32))
        b.run(2, seed=21, update=update)
        r = b.fetch()
        want = oracle.pt_run("ising", Jd, h, betas, x0,
                             e0.astype(np.float32),
                             np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                             seed=21, num_sweeps=2, update=update)
        sp = unpack_spins(r["spins"].reshape(Rd, R, -1), n, "ising",
                          np.float32)
        assert (sp == want["spins"]).all(), update
        assert (r["energies"].reshape(Rd, R) == want["energies"]).all()
        # f64 energies of the returned states from the stored rows
        out = torch.empty(Rd * R, dtype=torch.float64, device=b.device)
        check(_lib.load().pysa_gb_energy64_tables(
            ref(b.p), ref(b._ht), 0, b.spins.data_ptr(), b.words, Rd * R,
            out.data_ptr(), b._stream.cuda_stream), "energy64_tables")
        e64 = np.array([oracle.energy64(Jd, h, s)
                        for s in want["spins"].reshape(-1, n)])
        assert np.array_equal(out.cpu().numpy(), e64)


def test_lattice128_sparse_storage():
    """The 128 x 128 lattice (16 384 spins) of the Ising tutorial's kind
    runs from a scipy.sparse problem without any dense copy: returned
    energies equal the exact energies of the returned states, and each
    chain's best energy is its best state's energy."""
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins
    from pysa_gb300.utils import lattice_adjacency
    L = 128
    J = (-lattice_adjacency(L, L, sparse=True)).astype(np.float32)
    n = L * L
    h = np.zeros(n, np.float32)
    R, Rd = 8, 4
    betas = (1.0 / np.geomspace(1.0, 3.5, R)).astype(np.float32)
    rng = np.random.default_rng(13)
    x0 = _states(rng, "ising", (Rd, R, n))
    for update in ("sequential", "random"):
        b = PTBatch("ising", [Instance(J, h, betas, Rd)], sparse=True,
                    perm_slots=2)
        assert b._t["J"].numel() == 1
        b.set_states(pack_spins(x0, "ising", b.words), None)
        b.run(5, seed=3, update=update)
        r = b.fetch()
        S = unpack_spins(r["spins"], n, "ising", np.float64)
        E = np.einsum("ri,ri->r", S, (J @ S.T).T) / 2 + S @ h
        assert np.array_equal(r["energies"].astype(np.float64), E)
        B = unpack_spins(r["best_spins"], n, "ising", np.float64)
        Eb = np.einsum("ri,ri->r", B, (J @ B.T).T) / 2 + B @ h
        assert np.array_equal(r["best_energy"].astype(np.float64), Eb)
