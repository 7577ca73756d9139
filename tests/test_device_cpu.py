"""Host-side pieces of the device-resident path: the temperature ladder, the
RBM's QUBO and the refusal to run without a GPU."""
import numpy as np
import pytest


@pytest.mark.parametrize("R,tmin,tmax,beta0", [(1, 0.5, 2.0, False),
                                               (2, 0.5, 2.0, False),
                                               (7, 0.3, 3.0, False),
                                               (7, 0.3, 3.0, True),
                                               (100, 1.0, 1.0, False)])
def test_ladder_is_the_solvers(R, tmin, tmax, beta0):
    from pysa_gb300.device import ladder
    got = ladder(R, tmin, tmax, beta0)
    # pysa/sa.py:167-201: geometric in temperature from tmin, optional 0
    if R == 1:
        want = [1 / tmin]
    elif R == 2:
        want = [1 / tmin, 1 / tmax]
    elif beta0:
        r = np.exp(np.log(tmax / tmin) / (R - 2))
        want = [1 / (tmin * r**k) for k in range(R - 1)] + [0.0]
    else:
        r = np.exp(np.log(tmax / tmin) / (R - 1))
        want = [1 / (tmin * r**k) for k in range(R)]
    assert got.dtype == np.float32
    assert np.array_equal(got, np.asarray(want, np.float32))


def test_rbm_problem_is_the_references_qubo():
    import torch
    from pysa_gb300.rbm import rbm_problem
    g = torch.Generator().manual_seed(3)
    V, H = 9, 5
    W = torch.randn(V, H, generator=g)
    vb, hb = torch.randn(V, 1, generator=g), torch.randn(H, 1, generator=g)
    P = rbm_problem(W, vb, hb).numpy()
    want = np.zeros((V + H, V + H), np.float32)
    want[:V, V:] = W.numpy()
    want[V:, :V] = W.numpy().T
    want += np.diag(np.concatenate([vb.numpy(), hb.numpy()]).squeeze())
    assert np.array_equal(P, -want)
    assert np.array_equal(P, P.T)


def test_rbm_refuses_cpu_device():
    from pysa_gb300.rbm import RBM_PySA
    with pytest.raises(RuntimeError):
        RBM_PySA(4, 3, state_size=2, device="cpu")
