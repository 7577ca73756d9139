"""Problem ingestion: interaction lists, coupling-triplet files and 2-D
lattices to the dense symmetric matrices `Solver` takes.

* `get_problem_matrix` -- pysa/utils.py:61-89: an interaction list
  [(x, y, J), ...] over arbitrary hashable-and-sortable variable labels to a
  dense matrix over the sorted labels.  The reference's duplicate warning
  calls an unimported `warn` (pysa/utils.py:71); here it is
  warnings.warn.  As in the reference the last of a duplicated coupling is
  the one kept.
* `read_triplets` / `problem_from_triplets` -- the `i j J` text files of
  planted-instance generators (the Wishart instance of the reference's
  tutorials), assembled as its HPO tutorial does: duplicates summed, then
  (M + M^T) / 2.
* `lattice_adjacency` -- the open-boundary nearest-neighbour adjacency of an
  m x n lattice (tutorials/ising_tutorial.py:175-189).
"""
from __future__ import annotations

import warnings
from collections import Counter

import numpy as np


def get_problem_matrix(instance) -> np.ndarray:
    """Dense symmetric problem from [(x, y, J), ...]; x == y entries are
    local fields on the diagonal."""
    instance = list(instance)
    if instance and set(Counter(tuple(sorted(x[:2])) for x in instance)
                        .values()) != {1}:
        warnings.warn("Duplicated couplings are ignored.")
    labels = sorted(set(v for x in instance for v in x[:2]))
    index = {v: i for i, v in enumerate(labels)}
    problem = np.zeros((len(labels), len(labels)))
    for x, y, J in instance:
        a, b = index[x], index[y]
        problem[b][a] = problem[a][b] = J
    return problem


def read_triplets(path):
    """(rows int64, cols int64, vals float64) of a whitespace-separated
    `i j J` file (comment lines starting with '#' skipped)."""
    data = np.loadtxt(path, comments="#", ndmin=2)
    return (data[:, 0].astype(np.int64), data[:, 1].astype(np.int64),
            data[:, 2].astype(np.float64))


def problem_from_triplets(rows, cols, vals, n: int | None = None):
    """Dense symmetric matrix (M + M^T) / 2 with M[i, j] = sum of the vals at
    (i, j); n defaults to the largest index + 1."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    if n is None:
        n = int(max(rows.max(initial=-1), cols.max(initial=-1))) + 1
    M = np.zeros((n, n))
    np.add.at(M, (rows, cols), np.asarray(vals, np.float64))
    return (M + M.T) / 2.0


def lattice_adjacency(m: int, n: int, sparse: bool = False):
    """Adjacency of the m x n lattice with open boundaries, site (i, j) at
    index i * n + j: a dense array, or with sparse=True a scipy.sparse CSR
    matrix (for lattices whose dense form would not fit in host memory)."""
    idx = np.arange(m * n).reshape(m, n)
    if sparse:
        import scipy.sparse as sps
        r = np.concatenate([idx[1:, :].ravel(), idx[:-1, :].ravel(),
                            idx[:, 1:].ravel(), idx[:, :-1].ravel()])
        c = np.concatenate([idx[:-1, :].ravel(), idx[1:, :].ravel(),
                            idx[:, :-1].ravel(), idx[:, 1:].ravel()])
        return sps.csr_matrix((np.ones(len(r)), (r, c)), shape=(m * n, m * n))
    A = np.zeros((m * n, m * n))
    A[idx[1:, :].ravel(), idx[:-1, :].ravel()] = 1
    A[idx[:-1, :].ravel(), idx[1:, :].ravel()] = 1
    A[idx[:, 1:].ravel(), idx[:, :-1].ravel()] = 1
    A[idx[:, :-1].ravel(), idx[:, 1:].ravel()] = 1
    return A
