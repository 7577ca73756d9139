"""Restricted Boltzmann machine whose negative phase runs parallel tempering
on the GPU without leaving it (the consumer of tutorials/rbm_pysa.py).

`RBM_PySA` keeps the reference class's constructor, attributes and methods
(tutorials/rbm_pysa.py:22-221): weights W [V, H], biases v_bias [V, 1] and
h_bias [H, 1], persistent states v_state [S, V] and h_state [S, H], and
`update_states_with_pysa()` for the negative phase.  The reference builds the
(V+H)-spin QUBO on the host and round-trips problem and states through NumPy
every step (tutorials/rbm_pysa.py:111-140); here the QUBO is assembled on the
device, split by `pysa_gb_load_problem`, swept by the same kernels as
`Solver`, and the new states stay device tensors.  Same problem, same update:
num_reads = 1, num_replicas = state_size, sequential order, the min_temp /
max_temp ladder, the current states as the initial ones.
"""
from __future__ import annotations

import numpy as np
import torch

from .device import DeviceSolver

td = torch.distributions


def rbm_problem(W: torch.Tensor, v_bias: torch.Tensor,
                h_bias: torch.Tensor) -> torch.Tensor:
    """The QUBO the reference hands to Solver: minus the symmetric block
    matrix [[diag(v_bias), W], [W^T, diag(h_bias)]]
    (tutorials/rbm_pysa.py:113-121), assembled on W's device."""
    V, H = W.shape
    P = torch.zeros(V + H, V + H, dtype=torch.float32, device=W.device)
    P[:V, V:] = W
    P[V:, :V] = W.t()
    P += torch.diag(torch.cat([v_bias, h_bias], dim=0).reshape(-1))
    return -P


class RBM_PySA(torch.nn.Module):
    """RBM trained with a parallel-tempering negative phase on the GPU.

    visible_dim, hidden_dim: unit counts; state_size: persistent chains
    (the replicas of the PT run); steps: sweeps per update; kwargs: min_temp
    (1.0), max_temp (3.5), parallel (True), as in the reference, plus seed
    (keys the GPU random stream; drawn from the OS when absent).
    """

    def __init__(self, visible_dim, hidden_dim, state_size=100, steps=1,
                 device=None, **kwargs):
        super().__init__()
        self.visible_dim = visible_dim
        self.hidden_dim = hidden_dim
        self.state_size = state_size
        self.steps = steps
        self.min_temp = kwargs.get("min_temp", 1.0)
        self.max_temp = kwargs.get("max_temp", 3.5)
        self.parallel = kwargs.get("parallel", True)
        self.float_type = "float32"
        if device is None:
            device = "cuda"
        if torch.device(device).type != "cuda":
            raise RuntimeError("RBM_PySA runs its negative phase on a CUDA "
                               "GPU (no CPU path)")
        self.device = device
        self._rng = np.random.default_rng(kwargs.get("seed"))
        self.W = torch.nn.Parameter(
            torch.randn(visible_dim, hidden_dim, device=device))
        self.v_bias = torch.nn.Parameter(
            torch.zeros(visible_dim, 1, device=device))
        self.h_bias = torch.nn.Parameter(
            torch.zeros(hidden_dim, 1, device=device))
        self.v_state = torch.zeros(state_size, visible_dim, device=device)
        self.h_state = torch.zeros(state_size, hidden_dim, device=device)
        self._solver = None

    def v2h(self, v):
        """Sample hidden units given visible units [batch, V]."""
        logits = torch.nn.functional.linear(v, self.W.t(), self.h_bias.t())
        return td.Bernoulli(logits=logits).sample()

    def h2v(self, h):
        """Sample visible units given hidden units [batch, H]."""
        logits = torch.nn.functional.linear(h, self.W, self.v_bias.t())
        return td.Bernoulli(logits=logits).sample()

    def update_states_with_pysa(self, seed: int | None = None):
        """One negative-phase update of the persistent states: `steps`
        sweeps of parallel tempering over the RBM's QUBO, on the device."""
        n = self.visible_dim + self.hidden_dim
        if self._solver is None:
            self._solver = DeviceSolver(
                "qubo", n, num_replicas=self.state_size, num_reads=1,
                min_temp=self.min_temp, max_temp=self.max_temp,
                device=self.W.device)
        with torch.no_grad():
            self._solver.set_problem(
                rbm_problem(self.W, self.v_bias, self.h_bias),
                check_symmetric=False)
            x0 = torch.cat([self.v_state, self.h_state], dim=1)
            if seed is None:
                seed = int(self._rng.integers(0, 2**63))
            res = self._solver.metropolis_update(
                self.steps, initialize_strategy=x0,
                update_strategy="sequential", parallel=self.parallel,
                seed=seed)
            states = res["states"][0].to(self.W.device)
        self.v_state, self.h_state = torch.split(states, self.visible_dim,
                                                 dim=1)

    def _energy(self, v, h):
        """Energy -(v.b_v + h.b_h + v W h) of visible / hidden pairs."""
        return -(torch.matmul(v, self.v_bias) + torch.matmul(h, self.h_bias) +
                 torch.sum(torch.matmul(v, self.W) * h, dim=1, keepdim=True))

    def energy(self, v):
        """Energy of v with hidden units sampled from v."""
        return self._energy(v, self.v2h(v))

    def log_prob(self, v):
        """Negative of (positive phase - negative phase)."""
        return -(self.positive_phase(v) - self.negative_phase())

    def positive_phase(self, v):
        return torch.mean(self.energy(v), dim=-1)

    def negative_phase(self):
        return torch.mean(self._energy(self.v_state, self.h_state))

    def forward(self, x):
        """Reconstruction h2v(v2h(x))."""
        return self.h2v(self.v2h(x))
