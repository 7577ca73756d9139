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


@pytest.mark.parametrize("update", ["sequential", "random"])
def test_noalloc_matches_workspace_entry_points(update):
    import torch
    from pysa_gb300 import Instance, PTBatch, pack_spins, _lib
    from pysa_gb300._lib import check, ref

    rng = np.random.default_rng(77)
    n, R, Rd, S, seed = 200, 8, 12, 9, 4242
    Q = rng.integers(-8, 9, (n, n))
    Q = np.triu(Q, 1)
    Q = (Q + Q.T).astype(np.float32)
    h = rng.integers(-16, 17, n).astype(np.float32)
    betas = (1.0 / np.geomspace(0.5, 8.0, R)).astype(np.float32)
    x0 = rng.integers(0, 2, (Rd, R, n)).astype(np.float32)

    # regular path: caller-allocated workspace
    base = PTBatch("qubo", [Instance(Q, h, betas, Rd)], kernel="plain")
    words = base.words
    packed = pack_spins(x0, "qubo", words).reshape(-1, words)
    base.set_states(packed, None)

    # allocation-free path: only the problem tables and the chain state of
    # this batch are used (its own workspace is never touched)
    na = PTBatch("qubo", [Instance(Q, h, betas, Rd)], kernel="plain")
    na.spins.copy_(torch.from_numpy(packed.view(np.int32)))
    na.beta_idx.copy_(torch.from_numpy(
        np.tile(np.arange(R, dtype=np.int32), Rd)))
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
