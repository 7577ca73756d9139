"""Device-resident path (DeviceSolver, RBM_PySA): inputs and results that stay
on the GPU must give the chains `Solver` gives on the same seed, states and
problem, bit for bit, and the oracle's on integer couplings."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym(rng, n, integer=True):
    if integer:
        P = rng.integers(-8, 9, (n, n)).astype(np.float32)
    else:
        P = rng.normal(size=(n, n)).astype(np.float32)
    return np.triu(P) + np.triu(P, 1).T


def _states(rng, ptype, shape):
    x = rng.integers(0, 2, shape).astype(np.float32)
    return 2 * x - 1 if ptype == "ising" else x


@pytest.mark.parametrize("ptype,n", [("qubo", 37), ("ising", 100),
                                     ("qubo", 300)])
def test_pack_matches_host_packing(ptype, n):
    import torch
    from pysa_gb300 import pack_spins
    from pysa_gb300 import _lib
    rng = np.random.default_rng(n)
    x = _states(rng, ptype, (23, n))
    words = (n + 31) // 32
    out = torch.zeros(23, words, dtype=torch.int32, device="cuda")
    xd = torch.from_numpy(x).cuda()
    lib = _lib.load()
    pt = _lib.ISING if ptype == "ising" else _lib.QUBO
    _lib.check(lib.pysa_gb_pack(pt, n, xd.data_ptr(), n, 23, out.data_ptr(),
                                words, torch.cuda.current_stream().cuda_stream),
               "pack")
    want = pack_spins(x, ptype, words).view(np.int32)
    assert (out.cpu().numpy() == want).all()


def test_load_problem_splits_like_solver():
    import torch
    from pysa_gb300 import Instance, PTBatch
    rng = np.random.default_rng(5)
    n = 70
    P = _sym(rng, n, integer=False)
    b = PTBatch("qubo", [Instance(np.zeros((n, n), np.float32),
                                  np.zeros(n, np.float32),
                                  np.ones(3, np.float32), 2)],
                kernel="plain")
    b.load_problem(0, torch.from_numpy(P).cuda())
    torch.cuda.synchronize()
    ld = int(b.ld[0])
    Jt = b._t["J"].cpu().numpy()[:n * ld].reshape(n, ld)
    J = P.copy()
    np.fill_diagonal(J, 0)
    assert (Jt[:, :n] == J.T).all() and (Jt[:, n:] == 0).all()
    assert (b._t["h"].cpu().numpy()[:n] == np.diag(P)).all()


@pytest.mark.parametrize("ptype,n,R,Rd,parallel,sort_t,upd", [
    ("qubo", 40, 5, 3, True, False, "sequential"),
    ("ising", 200, 8, 2, False, False, "sequential"),
    ("qubo", 200, 8, 2, True, True, "random"),
    ("ising", 100, 6, 4, True, False, "random"),
])
def test_device_solver_matches_solver(ptype, n, R, Rd, parallel, sort_t, upd):
    import torch
    from pysa_gb300 import Solver
    from pysa_gb300.device import DeviceSolver
    rng = np.random.default_rng(n + R)
    P = _sym(rng, n, integer=(ptype == "qubo"))
    x0 = _states(rng, ptype, (R, n))
    want = Solver(P, ptype, "float32").metropolis_update(
        num_sweeps=7, num_reads=Rd, num_replicas=R, min_temp=0.5,
        max_temp=4.0, initialize_strategy=x0, update_strategy=upd,
        parallel=parallel, sort_output_temps=sort_t, seed=99,
        return_dataframe=False)
    ds = DeviceSolver(ptype, n, num_replicas=R, num_reads=Rd, min_temp=0.5,
                      max_temp=4.0)
    ds.set_problem(torch.from_numpy(P).cuda())
    got = ds.metropolis_update(7, initialize_strategy=torch.from_numpy(x0)
                               .cuda(), update_strategy=upd,
                               parallel=parallel, sort_output_temps=sort_t,
                               seed=99)
    ds.check_status()
    for r in range(Rd):
        w = want[r]
        assert (got["states"][r].cpu().numpy() == w["states"]).all()
        assert (got["energies"][r].cpu().numpy() == w["energies"]).all()
        assert (got["best_state"][r].cpu().numpy() == w["best_state"]).all()
        assert got["best_energy"][r].item() == w["best_energy"]
        assert got["min_sweeps"][r].item() == w["min_sweeps"]
        assert np.array_equal(got["temps"][r].cpu().numpy(), w["temps"])


def test_device_solver_resume_equals_one_run():
    import torch
    from pysa_gb300.device import DeviceSolver
    rng = np.random.default_rng(8)
    n, R, Rd = 150, 6, 3
    P = torch.from_numpy(_sym(rng, n)).cuda()
    x0 = torch.from_numpy(_states(rng, "qubo", (R, n))).cuda()
    one = DeviceSolver("qubo", n, num_replicas=R, num_reads=Rd)
    one.set_problem(P)
    a = one.metropolis_update(10, initialize_strategy=x0, seed=3)
    two = DeviceSolver("qubo", n, num_replicas=R, num_reads=Rd)
    two.set_problem(P)
    two.metropolis_update(4, initialize_strategy=x0, seed=3)
    b = two.metropolis_update(6, seed=3)
    for k in ("states", "energies", "best_state", "best_energy", "temps",
              "min_sweeps"):
        assert torch.equal(a[k], b[k]), k


def test_device_solver_bit_exact_vs_oracle(oracle):
    import torch
    from pysa_gb300.device import DeviceSolver, ladder
    rng = np.random.default_rng(21)
    n, R, Rd = 96, 5, 2
    P = _sym(rng, n)
    J, h = P.copy(), np.diag(P).copy()
    np.fill_diagonal(J, 0)
    x0 = _states(rng, "qubo", (Rd, R, n))
    betas = ladder(R, 0.5, 4.0)
    e0 = np.array([[oracle.energy64(J, h, s) for s in r] for r in x0],
                  np.float32)
    ds = DeviceSolver("qubo", n, num_replicas=R, num_reads=Rd, min_temp=0.5,
                      max_temp=4.0)
    ds.set_problem(torch.from_numpy(P).cuda())
    got = ds.metropolis_update(6, initialize_strategy=torch.from_numpy(x0)
                               .cuda(), seed=17)
    want = oracle.pt_run("qubo", J, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=17, num_sweeps=6)
    assert (got["states"].cpu().numpy() == want["spins"]).all()
    assert (got["energies"].cpu().numpy() == want["energies"]).all()


@pytest.mark.parametrize("parallel", [True, False])
def test_rbm_negative_phase_matches_reference_path(parallel):
    """One update of the persistent states equals the reference's recipe
    (host QUBO, Solver, states back) on the same seed."""
    import torch
    from pysa_gb300 import Solver
    from pysa_gb300.rbm import RBM_PySA
    torch.manual_seed(0)
    V, H, S = 60, 20, 12
    m = RBM_PySA(V, H, state_size=S, steps=3, parallel=parallel,
                 min_temp=1.0, max_temp=2.0)
    g = torch.Generator().manual_seed(1)
    m.v_state = (torch.rand(S, V, generator=g) > 0.5).float().cuda()
    m.h_state = (torch.rand(S, H, generator=g) > 0.5).float().cuda()
    with torch.no_grad():
        m.v_bias.copy_(torch.randn(V, 1))
        m.h_bias.copy_(torch.randn(H, 1))
    # the reference's construction, on the host
    W = m.W.detach().cpu().numpy()
    vb = m.v_bias.detach().cpu().numpy()
    hb = m.h_bias.detach().cpu().numpy()
    problem = np.zeros((V + H, V + H), np.float32)
    problem[:V, V:] = W
    problem[V:, :V] = W.T
    problem += np.diag(np.concatenate([vb, hb]).squeeze())
    x0 = torch.cat([m.v_state, m.h_state], dim=1).cpu().numpy()
    want = Solver(-problem, "qubo", "float32").metropolis_update(
        num_sweeps=3, num_reads=1, num_replicas=S, update_strategy="sequential",
        min_temp=1.0, max_temp=2.0, initialize_strategy=x0, parallel=parallel,
        seed=1234, return_dataframe=False)[0]["states"]
    m.update_states_with_pysa(seed=1234)
    got = torch.cat([m.v_state, m.h_state], dim=1)
    assert got.is_cuda
    assert (got.cpu().numpy() == want).all()
    # the training-side methods run on the device states
    x = (torch.rand(8, V, device="cuda") > 0.5).float()
    assert torch.isfinite(m.log_prob(x)).all()
