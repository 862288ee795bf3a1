"""The oracle's GAMG restatement (oracle/gamg_oracle.py) on the CPU:
convergence to the direct solution in foam's and the GPU's arithmetic, far
fewer iterations than Gauss-Seidel alone, and the one-level case."""
import numpy as np
import scipy.sparse.linalg as sla

import gamg_oracle as G
from conftest import oracle_matrix
from multiregionfoam_gb300 import cases


def test_gamg_matches_direct_solve(oracle_mod):
    for s in (cases.cht_system(10, 9, 8, 4, seed=1, form="global", k_range=(0.1, 50.0)),
              cases.convdiff_system(10, 9, 8, seed=2)):
        A = oracle_matrix(oracle_mod, s)
        xs = sla.spsolve(A.to_scipy().tocsc(), s.b)
        g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
        assert len(g.levels) >= 3 and g.levels[-1]["n"] <= 10
        for mode in ("literal", "mirror"):
            x, p = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-11,
                           max_iter=500, mode=mode)
            assert p["converged"] and p["final_residual"] < 1e-11
            assert np.abs(x - xs).max() <= 1e-8 * np.abs(xs).max()
        _, pg = A.smooth(s.b, s.x0, tol=1e-11, max_iter=50000, mode="mirror")
        assert p["n_iter"] * 5 < pg["n_iter"]


def test_gamg_single_level_is_a_direct_solve(oracle_mod):
    s = cases.convdiff_system(2, 2, 2, seed=3)          # 8 cells <= nCellsInCoarsestLevel
    g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
    assert g.levels == []
    x, p = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-12, mode="mirror")
    assert p["n_iter"] == 1 and p["final_residual"] < 1e-12
