"""The bounded-wait timeout path of the tensor-core sweep, exercised safely.

Every wait inside k_sweep_tc is bounded; when one runs out the kernel writes
PYSA_GB_ERR_TIMEOUT to the status word, lets the work already in flight land,
frees its tensor memory and returns, and the host raises.  This test makes a
wait run out on purpose without faulting anything: the wait for a work
item's previous unit happens at a unit's start, when the CTA has nothing in
flight, and pysa_gb_set_unit_wait_limit shrinks its bound to a few
microseconds.  One work item run for 128 sweeps in one launch with the unit
length fixed at 8 sweeps is split into sixteen units taken by as many CTAs
at once, so the CTAs holding units 1 and later must wait for unit 0
(hundreds of microseconds) and give up.  The
batch and the context must stay usable: the next run, with the default
bound, matches the oracle bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_unit_wait_timeout_reported_and_batch_reusable(oracle):
    from pysa_gb300 import Instance, PTBatch, pack_spins, unpack_spins, _lib
    rng = np.random.default_rng(21)
    n, R, Rd = 1024, 64, 1          # 64 chains: one fold-2 work item
    Q = np.triu(rng.integers(-8, 9, (n, n)), 1)
    Q = (Q + Q.T).astype(np.float32)
    h = rng.integers(-16, 17, n).astype(np.float32)
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)
    b = PTBatch("qubo", [Instance(Q, h, betas, Rd)], kernel="tc")
    assert b.ws.tc_fusable == 1 and b.ws.plain_live == 0
    lib = _lib.load()
    b.ws.tc_unit_sweeps = 8                     # fixed units from the queue
    b.set_states(pack_spins(x0, "qubo", b.words), None)
    try:
        lib.pysa_gb_set_unit_wait_limit(2000)   # 2 us
        b.run(128, seed=3, graph_chunk=0)
        with pytest.raises(_lib.LibraryError, match="status -4"):
            b.fetch()
    finally:
        lib.pysa_gb_set_unit_wait_limit(0)      # back to one second
    # same batch, fresh state, default bound: a normal run
    e0 = np.array([[oracle.energy64(Q, h, s) for s in r] for r in x0],
                  np.float32)
    b.set_states(pack_spins(x0, "qubo", b.words), e0)
    b.run(24, seed=3, graph_chunk=0)
    got = b.fetch()
    want = oracle.pt_run("qubo", Q, h, betas, x0, e0,
                         np.tile(np.arange(R, dtype=np.int32), (Rd, 1)),
                         seed=3, num_sweeps=24)
    sp = unpack_spins(got["spins"].reshape(Rd, R, -1), n, "qubo", np.float32)
    assert (sp == want["spins"]).all()
    assert (got["energies"].reshape(Rd, R) == want["energies"]).all()
    assert (got["beta_idx"].reshape(Rd, R) == want["beta_idx"]).all()
