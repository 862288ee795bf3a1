"""CPU tests: pin the oracle (no GPU needed).

The reference's tests pin no solver numbers (its only test asserts that a
tutorial ran to "completed"), so the oracle is pinned by known-answer tests,
an independent scipy cross-check, the reference's own self-checks
(directMap conformity, GGI face-centre round trip) and committed fixtures.
"""
import numpy as np

from multiregionfoam_gb300.cases import jittered_faces  # noqa: F401  (other tests import it from here)
import pytest
import scipy.sparse.linalg as spl

from conftest import oracle_matrix
from multiregionfoam_gb300 import cases


def test_identity_one_iteration(oracle_mod):
    n = 50
    A = oracle_mod.OracleMatrix(n, np.zeros(0, np.int32), np.zeros(0, np.int32), np.ones(n), np.zeros(0))
    b = np.arange(n, dtype=float) + 1.0
    x, p = A.solve(b, np.zeros(n), "PCG", "DIC", tol=1e-12)
    assert p["n_iter"] == 1 and p["converged"]
    assert np.array_equal(x, b)


def test_laplace_1d_known_solution(oracle_mod):
    s = cases.laplace_1d(200, (1.0, 3.0))
    A = oracle_matrix(oracle_mod, s)
    x, p = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-14)
    assert p["converged"]
    np.testing.assert_allclose(x, s.meta["x_exact"], rtol=0, atol=1e-11)
    # DIC on a tridiagonal matrix is the exact Cholesky factor: one iteration.
    assert p["n_iter"] == 1


@pytest.mark.parametrize("form", ["global", "coupled"])
def test_pcg_matches_scipy(oracle_mod, form):
    s = cases.cht_system(14, 12, 10, 6, seed=3, form=form, k_range=(0.1, 50.0))
    A = oracle_matrix(oracle_mod, s)
    x, p = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-12)
    assert p["converged"]
    xs = spl.spsolve(A.to_scipy().tocsc(), s.b)
    assert np.abs(x - xs).max() / np.abs(xs).max() < 1e-10
    # scipy's own CG (unpreconditioned) reaches the same solution
    xc, info = spl.cg(A.to_scipy(), s.b, x0=s.x0, rtol=1e-13, maxiter=20000)
    assert info == 0
    assert np.abs(xc - xs).max() / np.abs(xs).max() < 1e-9


def test_pbicg_dilu_matches_scipy(oracle_mod):
    s = cases.convdiff_system(12, 11, 10, seed=4)
    assert not s.symmetric
    A = oracle_matrix(oracle_mod, s)
    x, p = A.solve(s.b, s.x0, "PBiCG", "DILU", tol=1e-12)
    assert p["converged"]
    xs = spl.spsolve(A.to_scipy().tocsc(), s.b)
    assert np.abs(x - xs).max() / np.abs(xs).max() < 1e-9


def test_amul_matches_scipy_and_forms_agree(oracle_mod):
    g = cases.cht_system(9, 8, 7, 4, seed=2, form="global")
    c = cases.cht_system(9, 8, 7, 4, seed=2, form="coupled")
    Ag, Ac = oracle_matrix(oracle_mod, g), oracle_matrix(oracle_mod, c)
    x = np.random.default_rng(0).standard_normal(g.n)
    np.testing.assert_allclose(Ag.amul(x), Ag.to_scipy() @ x, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(Ag.amul(x), Ac.amul(x), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(Ag.sumA(), np.asarray(Ag.to_scipy().sum(axis=1)).ravel(), atol=1e-14)
    np.testing.assert_allclose(Ag.sumA(), Ac.sumA(), atol=1e-15)


def test_tmul_is_transpose(oracle_mod):
    s = cases.convdiff_system(7, 6, 5, seed=1)
    A = oracle_matrix(oracle_mod, s)
    x = np.random.default_rng(1).standard_normal(s.n)
    np.testing.assert_allclose(A.tmul(x), A.to_scipy().T @ x, rtol=1e-13, atol=1e-13)


def test_dic_is_incomplete_cholesky(oracle_mod):
    # (D+L) D^-1 (D+U) applied to the preconditioned vector gives r back
    s = cases.cht_system(6, 5, 4, 3, seed=5)
    A = oracle_matrix(oracle_mod, s)
    rD = A.factor("DIC")
    r = np.random.default_rng(2).standard_normal(s.n)
    w = A.precondition("DIC", r)
    import scipy.sparse as sp
    Lm = sp.coo_matrix((s.upper_c, (s.upper, s.lower)), shape=(s.n, s.n)).tocsr()
    D = sp.diags(1.0 / rD)
    M = (D + Lm) @ sp.diags(rD) @ (D + Lm.T)
    np.testing.assert_allclose(M @ w, r, rtol=1e-10, atol=1e-10)


def test_fused_and_literal_modes_agree(oracle_mod):
    s = cases.c1()
    A = oracle_matrix(oracle_mod, s)
    x1, p1 = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-8)
    x2, p2 = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-8, fused=True)
    assert p1["n_iter"] == p2["n_iter"]
    assert np.abs(x1 - x2).max() / np.abs(x1).max() < 1e-12


def test_c1_reaches_tolerance(oracle_mod):
    s = cases.c1()
    A = oracle_matrix(oracle_mod, s)
    x, p = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-8)
    assert p["converged"] and p["final_residual"] < 1e-8
    # the recursively updated residual tracks the true one (normFactor of x0)
    true_res = np.abs(s.b - A.amul(x)).sum() / A.norm_factor(s.x0, s.b)
    assert abs(true_res - p["final_residual"]) < 1e-10


def test_maxiter_and_miniter(oracle_mod):
    s = cases.cht_system(8, 8, 8, 4, seed=1)
    A = oracle_matrix(oracle_mod, s)
    _, p = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-30, max_iter=3)
    assert p["n_iter"] == 3 and not p["converged"]
    xs, _ = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-12)
    _, p = A.solve(s.b, xs, "PCG", "DIC", tol=1e-6)
    assert p["n_iter"] == 0 and p["converged"]
    _, p = A.solve(s.b, xs, "PCG", "DIC", tol=1e-6, min_iter=2)
    assert p["n_iter"] == 2


def test_golden_regression(oracle_mod, golden_small):
    from conftest import golden_system
    g = golden_small
    for name in ("cht", "chtc", "cd"):
        s = golden_system(g, name)
        A = oracle_matrix(oracle_mod, s)
        x = g[f"{name}_x"]
        assert np.array_equal(A.amul(x), g[f"{name}_amul"]), name
        assert np.array_equal(A.tmul(x), g[f"{name}_tmul"]), name
        assert np.array_equal(A.sumA(), g[f"{name}_sumA"]), name
        kind = "DIC" if s.symmetric else "DILU"
        assert np.array_equal(A.factor(kind), g[f"{name}_rD"]), name
        assert np.array_equal(A.precondition(kind, x), g[f"{name}_prec"]), name
        solver = "PCG" if s.symmetric else "PBiCG"
        xs, p = A.solve(s.b, s.x0, solver, kind, tol=1e-10)
        assert np.array_equal(xs, g[f"{name}_sol"]), name
        assert [p["initial_residual"], p["final_residual"], p["n_iter"]] == g[f"{name}_perf"].tolist()


def test_mirror_mode_close_to_foam_order(oracle_mod, golden_small):
    """The GPU-order mirror differs from foam's sequential sums only by rounding."""
    from conftest import golden_system
    for name in ("cht", "chtc", "cd"):
        s = golden_system(golden_small, name)
        A = oracle_matrix(oracle_mod, s)
        solver, kind = ("PCG", "DIC") if s.symmetric else ("PBiCG", "DILU")
        x1, p1 = A.solve(s.b, s.x0, solver, kind, tol=1e-10)
        x2, p2 = A.solve_mirror(s.b, s.x0, solver, kind, tol=1e-10)
        assert p1["n_iter"] == p2["n_iter"]
        assert np.abs(x1 - x2).max() <= 1e-12 * np.abs(x1).max()
        assert abs(p1["final_residual"] - p2["final_residual"]) <= 1e-12 * p1["initial_residual"]


def test_real_mesh_directmap_and_solve(oracle_mod, fohp):
    # the reference's tutorial meshes: directMap finds a conformal pairing
    tol = 1e-3 * min(float(fohp["solid_iface_min_edge"]), float(fohp["fluid_iface_min_edge"]))
    m = cases.direct_map(fohp["solid_iface_centres"], fohp["fluid_iface_centres"], tol)
    assert sorted(m.tolist()) == list(range(200))
    # the case generator's hash-grid search gives the literal N^2 search's map
    assert np.array_equal(m, oracle_mod.direct_map(fohp["fluid_iface_centres"], fohp["solid_iface_centres"], tol))
    # the reference's self-check: mapping face centres A->B is exact when conformal
    np.testing.assert_allclose(fohp["solid_iface_centres"][m], fohp["fluid_iface_centres"], atol=tol)
    g = cases.flow_over_heated_plate(fohp, form="global")
    c = cases.flow_over_heated_plate(fohp, form="coupled")
    Ag, Ac = oracle_matrix(oracle_mod, g), oracle_matrix(oracle_mod, c)
    x = np.random.default_rng(3).standard_normal(g.n)
    np.testing.assert_allclose(Ag.amul(x), Ac.amul(x), rtol=1e-13, atol=1e-12)
    xg, pg = Ag.solve(g.b, g.x0, "PCG", "DIC", tol=1e-12)
    xc, pc = Ac.solve(c.b, c.x0, "PCG", "DIC", tol=1e-12)
    assert pg["converged"] and pc["converged"]
    # monolithic global and coupled forms agree (the reference's premise)
    assert np.abs(xg - xc).max() / np.abs(xg).max() < 1e-10


def test_directmap_rejects_nonconformal():
    a = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    b = np.array([[0.0, 0, 0], [0.5, 0, 0]])
    with pytest.raises(ValueError, match="not conformal"):
        cases.direct_map(a, b, 1e-3)


def test_ggi_weights_properties(oracle_mod):
    # 3:2 jittered non-conformal faces (the non-conformal GGI case)
    fa = jittered_faces(24, 24, 0.2, 1)
    fb = jittered_faces(16, 24, 0.2, 2)
    (pa, sa, wa), (pb, sb, wb) = oracle_mod.ggi_weights(*fa, *fb)
    # every face covered, weights sum to one (rescaled)
    assert np.allclose(np.add.reduceat(wa, pa[:-1]), 1.0, atol=1e-12)
    assert np.allclose(np.add.reduceat(wb, pb[:-1]), 1.0, atol=1e-12)
    # constants are preserved by the gather
    assert np.allclose(oracle_mod.ggi_apply(pa, sa, wa, np.full(len(pb) - 1, 7.0)), 7.0, atol=1e-12)
    # area conservation: sum_i A_i w_ij = A_j on fully covered patches
    areas_a = np.abs(oracle_mod.face_areas(*fa))
    areas_b = np.abs(oracle_mod.face_areas(*fb))
    acc = np.zeros(len(pb) - 1)
    rows = np.repeat(np.arange(len(pa) - 1), np.diff(pa))
    np.add.at(acc, sa, areas_a[rows] * wa)
    np.testing.assert_allclose(acc, areas_b, rtol=1e-10)
    # a linear field is reproduced to second order at face centres
    cen_a = np.array([fa[1][pa_:pa_ + 4].mean(0) for pa_ in fa[0][:-1]])
    cen_b = np.array([fb[1][p_:p_ + 4].mean(0) for p_ in fb[0][:-1]])
    lin = lambda c: 2.0 * c[:, 0] - 3.0 * c[:, 1]
    err = np.abs(oracle_mod.ggi_apply(pa, sa, wa, lin(cen_b)) - lin(cen_a)).max()
    assert err < 0.2


def test_ggi_conformal_is_identity(oracle_mod):
    fa = jittered_faces(10, 7, 0.2, 5)
    (pa, sa, wa), _ = oracle_mod.ggi_weights(*fa, *fa)
    assert np.array_equal(np.diff(pa), np.ones(70, np.int32))
    assert np.array_equal(sa, np.arange(70))
    np.testing.assert_allclose(wa, 1.0, atol=1e-12)
