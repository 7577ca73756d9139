"""pysa_gb_sweeps_noalloc against the workspace entry points, through the C ABI.

pysa_gb_sweeps_noalloc serves callers that cannot allocate device memory
themselves -- for example a plugin running inside a host application whose
GPU memory all belongs to the host's own pool, or a loop that cannot afford
the device synchronisation cudaMalloc implies.  It keeps its scratch (local
fields, visiting orders, packed couplings, work list) in a fixed array owned
by the library, so its results must equal those of pysa_gb_prepare +
pysa_gb_sweeps with a caller-allocated workspace.  Integer couplings make the
comparison exact.  Two calls are made in a row, the second continuing the
first, so the shared array is reused with the previous call's contents in it.
This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _qubo(rng, n):
    Q = rng.integers(-8, 9, (n, n))
    Q = np.triu(Q, 1)
    return (Q + Q.T).astype(np.float32), rng.integers(-16, 17, n).astype(
        np.float32)


# (n, replicas, reads) per instance.  The mixed batch spans three plain-kernel
# variants with uneven reads and replicas, so the device-built work list's
# per-variant starts and the packed-coupling offsets summed across instances
# of different variants are both exercised.
BATCHES = {
    "one": [(200, 8, 12)],
    "mixed": [(20, 3, 5), (1500, 6, 3), (200, 8, 7), (33, 5, 2),
              (1100, 4, 4), (200, 2, 9)],
}


@pytest.mark.parametrize("batch", sorted(BATCHES))
@pytest.mark.parametrize("update", ["sequential", "random"])
def test_noalloc_matches_workspace_entry_points(update, batch):
    import torch
    from pysa_gb300 import Instance, PTBatch, pack_spins, _lib
    from pysa_gb300._lib import check, ref

    rng = np.random.default_rng(77)
    S, seed = 9, 4242
    insts, x0 = [], []
    for n, R, Rd in BATCHES[batch]:
        Q, h = _qubo(rng, n)
        betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
        insts.append(Instance(Q, h, betas, Rd))
        x0.append(rng.integers(0, 2, (Rd * R, n)).astype(np.float32))

    # regular path: caller-allocated workspace
    base = PTBatch("qubo", insts, kernel="plain")
    words = base.words
    packed = np.concatenate([pack_spins(x, "qubo", words) for x in x0])
    base.set_states(packed, None)
    if batch == "mixed":
        assert sum(1 for c in base.ws.variant_count if c > 0) >= 3

    # allocation-free path: only the problem tables and the chain state of
    # this batch are used (its own workspace is never touched)
    na = PTBatch("qubo", insts, kernel="plain")
    na.spins.copy_(torch.from_numpy(packed.view(np.int32)))
    na.beta_idx.copy_(torch.from_numpy(np.concatenate([
        np.tile(np.arange(R, dtype=np.int32), Rd)
        for _, R, Rd in BATCHES[batch]])))
    na.sweep_counter.zero_()
    na.status.zero_()
    na.ticket.zero_()
    host = _lib.HostTables(*(a.ctypes.data for a in na._host))
    upd = _lib.RANDOM if update == "random" else _lib.SEQUENTIAL
    opts = _lib.Options(seed, upd, 1, 0, 0, 0, 0)
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream

    for call in range(2):
        base.run(S, seed=seed, update=update, graph_chunk=0)
        want = base.fetch()
        check(lib.pysa_gb_sweeps_noalloc(ref(na.p), ref(na.s), ref(host),
                                         ref(opts), 1 if call == 0 else 0, S,
                                         stream), "sweeps_noalloc")
        got = na.fetch()
        for key in ("spins", "energies", "beta_idx", "best_energy",
                    "best_sweep", "best_spins"):
            assert np.array_equal(got[key], want[key]), (call, key)
        assert int(na.sweep_counter.item()) == (call + 1) * S


def test_noalloc_rejects_sparse_instances():
    """A sparse-row instance needs the sparse kernel's tables, which the
    fixed array has no room for: refused before anything is enqueued."""
    import torch
    from pysa_gb300 import Instance, PTBatch, _lib
    from pysa_gb300._lib import ref

    rng = np.random.default_rng(5)
    n = 64
    J = np.zeros((n, n), np.float32)
    i = np.arange(n - 1)
    J[i, i + 1] = J[i + 1, i] = -1.0
    Q, h = _qubo(rng, 100)
    betas = np.ones(4, np.float32)
    b = PTBatch("ising", [Instance(J, np.zeros(n, np.float32), betas, 2),
                          Instance(Q, h, betas, 2)],
                kernel="plain", sparse=[True, False])
    host = _lib.HostTables(*(a.ctypes.data for a in b._host))
    opts = _lib.Options(1, _lib.SEQUENTIAL, 1, 0, 0, 0, 0)
    before = b.spins.clone()
    rc = _lib.load().pysa_gb_sweeps_noalloc(
        ref(b.p), ref(b.s), ref(host), ref(opts), 1, 3,
        torch.cuda.current_stream().cuda_stream)
    assert rc == -1  # PYSA_GB_ERR_ARG
    assert b"sparse" in _lib.load().pysa_gb_last_error()
    torch.cuda.synchronize()
    assert torch.equal(b.spins, before)
    assert int(b.sweep_counter.item()) == 0
