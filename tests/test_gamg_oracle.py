"""The oracle's GAMG restatement (oracle/gamg_oracle.py) on the CPU:
foam's pairwise agglomeration on a hand-worked chain, convergence to the
direct solution in foam's and the GPU's arithmetic, scaleCorrection's effect,
far fewer iterations than Gauss-Seidel alone, and the one-level case."""
import numpy as np
import scipy.sparse.linalg as sla

import gamg_oracle as G
from conftest import oracle_matrix
from multiregionfoam_gb300 import cases


def test_pairing_known_answer():
    # chain 0-1-2-3-4, weights 1 2 3 1: cell 0 pairs with 1 (its only face);
    # cell 2 pairs with 3 (3 > 2 and cell 1 is taken); cell 4 has no free
    # neighbour and joins 3's group; then the numbering is reversed
    lower = np.array([0, 1, 2, 3])
    upper = np.array([1, 2, 3, 4])
    agg, nc = G.agglomerate(5, lower, upper, np.array([1.0, 2.0, 3.0, 1.0]))
    assert nc == 2 and agg.tolist() == [1, 1, 0, 0, 0]
    lo_c, up_c, restrict = G.agglomerate_addressing(agg, nc, lower, upper)
    assert lo_c.tolist() == [0] and up_c.tolist() == [1]
    assert restrict.tolist() == [-2, 0, -1, -1]          # faces inside cells: -(cell + 1)
    # coefficients: diag sums the members then each interior face's upper +
    # lower; face 1 runs from coarse cell 1 to 0, so its upper and lower swap
    level = {"n": nc, "agg": agg, "restrict": restrict, "lower": lo_c, "fine_lower": lower}
    d, u, l_ = G.coarse_coeffs(level, np.arange(1.0, 6.0), np.array([-1.0, -2.0, -3.0, -4.0]),
                               np.array([-10.0, -20.0, -30.0, -40.0]))
    assert d.tolist() == [3 + 4 + 5 - 33 - 44, 1 + 2 - 11] and u.tolist() == [-20.0] and l_.tolist() == [-2.0]
    # a single cell without faces is a group of its own, numbered after the pairs
    agg, nc = G.agglomerate(3, np.array([0]), np.array([2]), np.array([1.0]))
    assert nc == 2 and agg.tolist() == [1, 0, 1]
    # faceAreaPair weights: |Sf| / sqrt(|Sf|) scaled by (1, 1.01, 1.02) per axis
    w = G.face_area_weights(np.array([[4.0, 0, 0], [0, 4.0, 0], [0, 0, 4.0]]))
    assert np.allclose(w, [2.0, 2.02, 2.04], rtol=0, atol=1e-15)


def test_gamg_matches_direct_solve(oracle_mod):
    for s in (cases.cht_system(10, 9, 8, 4, seed=1, form="global", k_range=(0.1, 50.0)),
              cases.convdiff_system(10, 9, 8, seed=2)):
        A = oracle_matrix(oracle_mod, s)
        xs = sla.spsolve(A.to_scipy().tocsc(), s.b)
        g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
        assert len(g.levels) >= 3 and g.levels[-1]["n"] >= 10 and g.levels[-2]["n"] > g.levels[-1]["n"]
        for mode in ("literal", "mirror"):
            x, p = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-11,
                           max_iter=500, mode=mode)
            assert p["converged"] and p["final_residual"] < 1e-11
            assert np.abs(x - xs).max() <= 1e-8 * np.abs(xs).max()
        _, q = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-11,
                       max_iter=500, mode="mirror", scale=False)
        assert q["converged"] and q["n_iter"] > p["n_iter"]
        _, pg = A.smooth(s.b, s.x0, tol=1e-11, max_iter=50000, mode="mirror")
        assert p["n_iter"] * 5 < pg["n_iter"]


def test_gamg_single_level_is_a_direct_solve(oracle_mod):
    s = cases.convdiff_system(2, 2, 2, seed=3)          # 8 cells < nCellsInCoarsestLevel
    g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
    assert g.levels == []
    x, p = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-12, mode="mirror")
    assert p["n_iter"] == 1 and p["final_residual"] < 1e-12
