"""Problem ingestion against the reference's own outputs (golden vectors from
tests/golden/make_golden_utils.py) and the Wishart fixture."""
import warnings

import numpy as np
import pytest

from conftest import golden


@pytest.mark.parametrize("k", [0, 1, 2])
def test_get_problem_matrix_matches_reference(k):
    from pysa_gb300.utils import get_problem_matrix
    g = golden("utils")
    inst = [(int(a), int(b), float(J)) for a, b, J in g[f"inst{k}"]]
    assert np.array_equal(get_problem_matrix(inst), g[f"problem{k}"])


def test_get_problem_matrix_warns_on_duplicates():
    from pysa_gb300.utils import get_problem_matrix
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        P = get_problem_matrix([(0, 1, 2.0), (1, 0, 5.0), (1, 2, 1.0)])
    assert any("Duplicated" in str(x.message) for x in w)
    assert P[0, 1] == P[1, 0] == 5.0  # the last one is kept


@pytest.mark.parametrize("m,n", [(3, 4), (5, 5)])
def test_lattice_adjacency_matches_reference(m, n):
    from pysa_gb300.utils import lattice_adjacency
    assert np.array_equal(lattice_adjacency(m, n),
                          golden("utils")[f"lattice_{m}x{n}"])


def test_triplet_file_gives_the_wishart_problem(tmp_path):
    from pysa_gb300.utils import problem_from_triplets, read_triplets
    P = golden("wishart50")["problem"]
    i, j = np.triu_indices(P.shape[0], 1)
    keep = P[i, j] != 0
    path = tmp_path / "w.txt"
    with open(path, "w") as f:
        for a, b, v in zip(i[keep], j[keep], 2 * P[i, j][keep]):
            f.write(f"{a}\t{b}\t{v:.1f}\n")
    r, c, v = read_triplets(path)
    assert np.array_equal(problem_from_triplets(r, c, v, P.shape[0]), P)


def test_csr_tables_group_rows_by_column_residue():
    from pysa_gb300.engine import csr_tables
    rng = np.random.default_rng(4)
    n = 37
    J = rng.integers(-3, 4, (n, n)).astype(np.float32)
    J[rng.random((n, n)) < 0.7] = 0
    J = np.triu(J, 1)
    J = J + J.T
    rows, col, val = csr_tables(J)
    assert rows.shape == (n, 9) and rows[0, 0] == 0
    assert rows[-1, 8] == len(col) == np.count_nonzero(J)
    for i in range(n):
        for g in range(8):
            cs = col[rows[i, g]:rows[i, g + 1]]
            assert (cs % 8 == g).all() and (np.diff(cs) > 0).all()
            assert (val[rows[i, g]:rows[i, g + 1]] == J.T[i, cs]).all()
        assert rows[i, 8] == (rows[i + 1, 0] if i + 1 < n else len(col))
