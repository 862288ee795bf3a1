"""The oracle's BiCGStab (foam-extend's "BiCGStab" solver name, the reference
tutorials' monolithic coupled solver) on the CPU: known answers, agreement
with a direct solve in all three arithmetic orders, and the iteration
controls.  The oracle restates the published method (van der Vorst 1992) with
foam's residual normalisation; foam-extend's own source is not available
here, so its exact operation order is unpinned."""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

from conftest import oracle_matrix
from multiregionfoam_gb300 import cases

SYSTEMS = {
    "cht": lambda: cases.cht_system(12, 10, 9, 5, seed=1, form="global", k_range=(0.1, 50.0)),
    "chtc": lambda: cases.cht_system(12, 10, 9, 5, seed=1, form="coupled", k_range=(0.1, 50.0)),
    "cd": lambda: cases.convdiff_system(12, 11, 10, seed=2),
}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_bicgstab_matches_direct_solve(oracle_mod, name):
    s = SYSTEMS[name]()
    A = oracle_matrix(oracle_mod, s)
    xs = sla.spsolve(A.to_scipy().tocsc(), s.b)
    for pc in (("DIC" if s.symmetric else "DILU"), "diagonal", "none"):
        for mode in ("literal", "fused", "mirror"):
            if mode == "mirror":
                x, p = A.solve_mirror(s.b, s.x0, "BiCGStab", pc, tol=1e-11)
            else:
                x, p = A.solve(s.b, s.x0, "BiCGStab", pc, tol=1e-11, fused=mode == "fused")
            assert p["converged"] and not p["singular"] and p["final_residual"] < 1e-11, (pc, mode, p)
            # the reported residual is the foam residual of the returned x
            true_r = np.abs(s.b - A.amul(x)).sum() / A.norm_factor(s.x0, s.b)
            assert abs(true_r - p["final_residual"]) < 1e-12, (pc, mode)
            assert np.abs(x - xs).max() <= 1e-8 * np.abs(xs).max(), (pc, mode)


def test_bicgstab_fewer_iterations_with_stronger_preconditioner(oracle_mod):
    s = SYSTEMS["cd"]()
    A = oracle_matrix(oracle_mod, s)
    its = [A.solve(s.b, s.x0, "BiCGStab", pc, tol=1e-9)[1]["n_iter"] for pc in ("DILU", "diagonal", "none")]
    assert its[0] < its[1] <= its[2], its


def test_bicgstab_identity_half_step(oracle_mod):
    """A = I: alpha = 1, s = 0 after the first half step, x = b in one iteration."""
    n = 50
    lower = np.arange(n - 1, dtype=np.int32)
    upper = lower + 1
    rng = np.random.default_rng(0)
    b = rng.uniform(-1, 1, n)
    A = oracle_mod.OracleMatrix(n, lower, upper, np.ones(n), np.zeros(n - 1))
    for mode in ("literal", "mirror"):
        if mode == "mirror":
            x, p = A.solve_mirror(b, np.zeros(n), "BiCGStab", "DIC", tol=1e-12)
        else:
            x, p = A.solve(b, np.zeros(n), "BiCGStab", "DIC", tol=1e-12)
        assert p["n_iter"] == 1 and p["converged"] and p["final_residual"] == 0.0
        assert np.array_equal(x, b)


def test_bicgstab_iteration_controls(oracle_mod):
    s = SYSTEMS["cht"]()
    A = oracle_matrix(oracle_mod, s)
    _, p = A.solve(s.b, s.x0, "BiCGStab", "DIC", tol=1e-30, max_iter=4)
    assert p["n_iter"] == 4 and not p["converged"]
    xs, _ = A.solve(s.b, s.x0, "BiCGStab", "DIC", tol=1e-13)
    x, p = A.solve(s.b, xs, "BiCGStab", "DIC", tol=1e-6)
    assert p["n_iter"] == 0 and np.array_equal(x, xs)
    _, p = A.solve(s.b, xs, "BiCGStab", "DIC", tol=1e-6, min_iter=2)
    assert p["n_iter"] == 2
