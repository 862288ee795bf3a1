"""The oracle's smoothSolver + GaussSeidel (foam's smoother, restated) on the
CPU: agreement with a direct solve in all three arithmetic orders, a known
answer, and the sweep-counting iteration controls."""
import numpy as np
import scipy.sparse.linalg as sla

from conftest import oracle_matrix
from multiregionfoam_gb300 import cases


def test_gauss_seidel_matches_direct_solve(oracle_mod):
    for s in (cases.cht_system(10, 9, 8, 4, seed=1, form="coupled", k_range=(0.1, 50.0)),
              cases.convdiff_system(10, 9, 8, seed=2)):
        A = oracle_matrix(oracle_mod, s)
        xs = sla.spsolve(A.to_scipy().tocsc(), s.b)
        for mode in ("literal", "fused", "mirror"):
            x, p = A.smooth(s.b, s.x0, tol=1e-11, max_iter=50000, mode=mode)
            assert p["converged"] and p["final_residual"] < 1e-11
            assert np.abs(x - xs).max() <= 1e-8 * np.abs(xs).max()


def test_gauss_seidel_diagonal_known_answer(oracle_mod):
    """A diagonal matrix: one sweep gives x = b / diag (correctly rounded), so
    the residual is rounding only."""
    n = 40
    lower = np.arange(n - 1, dtype=np.int32)
    rng = np.random.default_rng(1)
    d, b = rng.uniform(1, 3, n), rng.uniform(-1, 1, n)
    A = oracle_mod.OracleMatrix(n, lower, lower + 1, d, np.zeros(n - 1))
    x, p = A.smooth(b, np.zeros(n), tol=1e-14)
    assert p["n_iter"] == 1 and p["final_residual"] < 1e-15 and np.array_equal(x, b / d)


def test_gauss_seidel_counts_sweeps(oracle_mod):
    s = cases.convdiff_system(8, 8, 8, seed=3)
    A = oracle_matrix(oracle_mod, s)
    _, p = A.smooth(s.b, s.x0, tol=1e-30, max_iter=7, n_sweeps=3)
    assert p["n_iter"] == 9 and not p["converged"]       # 3 + 3 + 3: the first count >= 7
    _, p = A.smooth(s.b, s.x0, tol=1e-30, max_iter=6, n_sweeps=2)
    assert p["n_iter"] == 6
