"""smoothSolver + GaussSeidel on the GPU (MRG_SOLVER_SMOOTH; foam's
smoothSolver, the tutorials' fluid U solver): foam's cell-order sweep run
sync-free over the level plan, bit-identical to the oracle's GPU-order mirror
(solution, initial / final residual, iteration count), and within 1e-10 of
the oracle's foam-order arithmetic (its residual is lduMatrix::residual's
order, the GPU's b - A x)."""
import numpy as np
import pytest

from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu

SMALL = {
    "cht": lambda: cases.cht_system(14, 12, 10, 6, seed=1, form="global", k_range=(0.1, 50.0)),
    "chtc": lambda: cases.cht_system(14, 12, 10, 6, seed=1, form="coupled", k_range=(0.1, 50.0)),
    "cd": lambda: cases.convdiff_system(14, 13, 12, seed=2),
}


@pytest.mark.parametrize("name,n_sweeps", [("cht", 1), ("chtc", 1), ("cd", 1), ("cd", 3)])
def test_smooth_gs_bitexact_vs_mirror(mrg, ctx, oracle_mod, name, n_sweeps):
    s = SMALL[name]()
    A = oracle_matrix(oracle_mod, s)
    tol = 1e-8
    xm, pm = A.smooth(s.b, s.x0, tol=tol, max_iter=20000, n_sweeps=n_sweeps, mode="mirror")
    xo, po = A.smooth(s.b, s.x0, tol=tol, max_iter=20000, n_sweeps=n_sweeps, mode="literal")
    m = gpu_mesh(mrg, ctx, s)
    xg, pg = m.solve(s.b, s.x0, tol=tol, max_iter=20000, solver="smoothSolver", n_sweeps=n_sweeps)
    m.close()
    assert np.array_equal(xg, xm)
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"], pg["converged"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"], pm["converged"])
    assert pg["converged"]
    assert abs(pg["n_iter"] - po["n_iter"]) <= n_sweeps
    assert abs(pg["initial_residual"] - po["initial_residual"]) <= 1e-10 * po["initial_residual"]
    assert np.abs(xg - xo).max() <= 10 * tol * np.abs(xo).max()


@pytest.mark.parametrize("name,smoother", [("chtc", "DIC"), ("chtc", "DICGaussSeidel"), ("cd", "DILU"),
                                           ("cd", "DILUGaussSeidel")])
def test_smooth_factor_smoothers_bitexact(mrg, ctx, oracle_mod, name, smoother):
    """DIC / DILU smoothers (psi += M^-1 (b - A psi)) and their Gauss-Seidel
    combinations, bit-identical to the mirror."""
    s = SMALL[name]()
    A = oracle_matrix(oracle_mod, s)
    xm, pm = A.smooth(s.b, s.x0, tol=1e-8, max_iter=20000, mode="mirror", smoother=smoother, n_sweeps=2)
    xo, po = A.smooth(s.b, s.x0, tol=1e-8, max_iter=20000, mode="literal", smoother=smoother, n_sweeps=2)
    m = gpu_mesh(mrg, ctx, s)
    xg, pg = m.solve(s.b, s.x0, tol=1e-8, max_iter=20000, solver="smoothSolver", smoother=smoother, n_sweeps=2)
    m.close()
    assert np.array_equal(xg, xm)
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"])
    assert pg["converged"] and abs(pg["n_iter"] - po["n_iter"]) <= 2
    assert np.abs(xg - xo).max() <= 1e-7 * np.abs(xo).max()


def test_smooth_gs_controls(mrg, ctx, oracle_mod):
    s = SMALL["cd"]()
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    try:
        x, p = m.solve(s.b, s.x0, tol=1e-30, max_iter=7, solver="smoothSolver", n_sweeps=3)
        xm, pm = A.smooth(s.b, s.x0, tol=1e-30, max_iter=7, n_sweeps=3, mode="mirror")
        assert p["n_iter"] == pm["n_iter"] == 9 and np.array_equal(x, xm)
        with pytest.raises(mrg.MrgError, match="FP64"):
            m.solve(s.b, s.x0, solver="smoothSolver", precision="mixed")
        with pytest.raises(mrg.MrgError, match="FP64"):
            m.solve(s.b, s.x0, solver="smoothSolver", ordering="colour")
    finally:
        m.close()


def test_smooth_gs_batch_equals_alone(mrg, ctx):
    sys_ = [SMALL["cd"](), SMALL["cht"](), cases.convdiff_system(9, 8, 7, seed=5)]
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    alone = [m.solve(s.b, s.x0, tol=1e-7, max_iter=20000, solver="smoothSolver") for m, s in zip(meshes, sys_)]
    b = mrg.Batch(ctx, meshes)
    xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-7, max_iter=20000, solver="smoothSolver")
    for (xa, pa), xb, pb in zip(alone, xs, perfs):
        assert np.array_equal(xa, xb) and pa["n_iter"] == pb["n_iter"]
    b.close()
    for m in meshes:
        m.close()
