"""GPU parity tests: libmrgpu (through the C ABI) against the CPU oracle.

Bars:
* kernel level (Amul, Tmul, sumA, DIC/DILU factor, preconditioner sweeps,
  GGI gather): bit-exact against the oracle's fused mode, which performs the
  same IEEE operations in the same per-cell order;
* solver level (PCG+DIC, PBiCG+DILU, FP64): the same iteration count and
  solution / initial / final residual within 1e-10 relative of the oracle's
  literal (foam-arithmetic) mode; reduction order differs, so not bitwise;
* mixed precision: final foam residual < tolerance and solution error vs the
  FP64 oracle solution stated and bounded.
"""
import numpy as np
import pytest

from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu

REL = 1e-10


def rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


SMALL = {
    "cht": lambda: cases.cht_system(16, 14, 12, 7, seed=1, form="global", k_range=(0.1, 50.0)),
    "chtc": lambda: cases.cht_system(16, 14, 12, 7, seed=1, form="coupled", k_range=(0.1, 50.0)),
    "cd": lambda: cases.convdiff_system(14, 13, 12, seed=2),
}


@pytest.mark.parametrize("name", list(SMALL))
def test_amul_tmul_bitexact(mrg, ctx, oracle_mod, name):
    s = SMALL[name]()
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    x = np.random.default_rng(7).standard_normal(s.n)
    assert np.array_equal(m.amul(x), A.amul(x, fused=True))
    assert np.array_equal(m.amul(x, transpose=True), A.tmul(x, fused=True))
    m.close()


@pytest.mark.parametrize("name", list(SMALL))
def test_residual_normfactor(mrg, ctx, oracle_mod, name):
    s = SMALL[name]()
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    r, nf = m.residual(s.b, s.x0)
    assert abs(nf - A.norm_factor(s.x0, s.b)) <= 1e-12 * nf
    assert abs(r - A.residual(s.b, s.x0)) <= 1e-12 * r
    m.close()


@pytest.mark.parametrize("name", list(SMALL))
def test_factor_and_sweeps_bitexact(mrg, ctx, oracle_mod, name):
    s = SMALL[name]()
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    kind = "DIC" if s.symmetric else "DILU"
    assert np.array_equal(m.factor_diag(kind), A.factor(kind))
    r = np.random.default_rng(8).standard_normal(s.n)
    assert np.array_equal(m.precondition(kind, r), A.precondition(kind, r, fused=True))
    if kind == "DILU":
        assert np.array_equal(m.precondition(kind, r, transpose=True),
                              A.precondition(kind, r, transpose=True, fused=True))
    # level-scheduled GPU sweep == sequential face-ordered sweep, every time
    assert np.array_equal(m.precondition(kind, r), m.precondition(kind, r))
    m.close()


def test_diagonal_and_none_preconditioners(mrg, ctx, oracle_mod):
    s = SMALL["cht"]()
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    r = np.random.default_rng(9).standard_normal(s.n)
    assert np.array_equal(m.precondition("diagonal", r), A.precondition("diagonal", r))
    assert np.array_equal(m.precondition("none", r), r)
    m.close()


def check_solve(mrg, ctx, O, s, solver, pc, tol=1e-8, **kw):
    """GPU solve vs the oracle.

    * vs the GPU-order mirror (same IEEE operations, same reduction tree):
      bit-identical solution, residuals and iteration count;
    * vs foam's sequential-sum arithmetic: same iteration count, solution and
      initial residual within 1e-10 relative, final residual within 1e-10 of
      the initial residual (a converged residual is ~tol x the initial one,
      so summation order alone moves it by ~1e-16/tol relative).
    """
    A = oracle_matrix(O, s)
    xo, po = A.solve(s.b, s.x0, solver, pc, tol=tol, **kw)
    xm, pm = A.solve_mirror(s.b, s.x0, solver, pc, tol=tol, **kw)
    m = gpu_mesh(mrg, ctx, s)
    xg, pg = m.solve(s.b, s.x0, tol=tol, solver=solver, precond=pc, **kw)
    m.close()
    assert np.array_equal(xg, xm), rel_err(xg, xm)
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"])
    if pc == "none":
        # Unpreconditioned CG over hundreds of iterations amplifies the
        # summation-order difference; only the solve tolerance is meaningful.
        assert abs(pg["n_iter"] - po["n_iter"]) <= 3, (pg, po)
        assert rel_err(xg, xo) <= 10 * tol
        return xg, pg, po
    assert pg["n_iter"] == po["n_iter"], (pg, po)
    assert pg["converged"] == po["converged"]
    assert abs(pg["initial_residual"] - po["initial_residual"]) <= REL * po["initial_residual"]
    assert abs(pg["final_residual"] - po["final_residual"]) <= REL * po["initial_residual"]
    assert rel_err(xg, xo) <= REL, rel_err(xg, xo)
    return xg, pg, po


def test_golden_fixtures_bitexact(mrg, ctx, golden_small):
    """Vectors computed on the CPU (x86) and committed are reproduced bit for bit."""
    from conftest import golden_system
    g = golden_small
    for name in ("cht", "chtc", "cd"):
        s = golden_system(g, name)
        m = gpu_mesh(mrg, ctx, s)
        x = g[f"{name}_x"]
        assert np.array_equal(m.amul(x), g[f"{name}_amul_fused"]), name
        assert np.array_equal(m.amul(x, transpose=True), g[f"{name}_tmul_fused"]), name
        kind = "DIC" if s.symmetric else "DILU"
        solver = "PCG" if s.symmetric else "PBiCG"
        assert np.array_equal(m.factor_diag(kind), g[f"{name}_rD"]), name
        assert np.array_equal(m.precondition(kind, x), g[f"{name}_prec_fused"]), name
        xs, p = m.solve(s.b, s.x0, tol=1e-10, solver=solver, precond=kind)
        assert np.array_equal(xs, g[f"{name}_sol_mirror"]), name
        assert [p["initial_residual"], p["final_residual"], p["n_iter"]] == g[f"{name}_perf_mirror"].tolist()
        assert rel_err(xs, g[f"{name}_sol"]) <= REL
        m.close()


def test_pcg_dic_c1_plain_method(mrg, ctx, oracle_mod):
    """C1: fluid 40^3 (k=0.6) over solid 40x40x20 (k=16), PCG+DIC FP64 at 1e-8."""
    s = cases.c1()
    xg, pg, po = check_solve(mrg, ctx, oracle_mod, s, "PCG", "DIC")
    assert pg["converged"] and pg["final_residual"] < 1e-8


def test_pcg_dic_c1_coupled_form(mrg, ctx, oracle_mod):
    s = cases.c1(form="coupled")
    check_solve(mrg, ctx, oracle_mod, s, "PCG", "DIC")


@pytest.mark.parametrize("pc", ["DIC", "diagonal", "none"])
def test_pcg_preconditioners(mrg, ctx, oracle_mod, pc):
    s = SMALL["cht"]()
    check_solve(mrg, ctx, oracle_mod, s, "PCG", pc, tol=1e-9)


def test_pbicg_dilu_permuted_convdiff(mrg, ctx, oracle_mod):
    s = cases.convdiff_system(24, 22, 20, seed=3)
    check_solve(mrg, ctx, oracle_mod, s, "PBiCG", "DILU")


def test_pbicg_dilu_on_symmetric(mrg, ctx, oracle_mod):
    s = SMALL["cht"]()
    check_solve(mrg, ctx, oracle_mod, s, "PBiCG", "DILU")


def test_real_mesh_fixture(mrg, ctx, oracle_mod, fohp):
    for form in ("global", "coupled"):
        s = cases.flow_over_heated_plate(fohp, form=form)
        check_solve(mrg, ctx, oracle_mod, s, "PCG", "DIC", tol=1e-12)


def test_min_max_iter_and_converged_start(mrg, ctx, oracle_mod):
    s = SMALL["cht"]()
    check_solve(mrg, ctx, oracle_mod, s, "PCG", "DIC", tol=1e-30, max_iter=5)
    A = oracle_matrix(oracle_mod, s)
    xs, _ = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-13)
    m = gpu_mesh(mrg, ctx, s)
    x, p = m.solve(s.b, xs, tol=1e-6)
    assert p["n_iter"] == 0 and p["converged"] and np.array_equal(x, xs)
    x, p = m.solve(s.b, xs, tol=1e-6, min_iter=3)
    assert p["n_iter"] == 3
    m.close()


@pytest.mark.parametrize("solver,pc,case", [("PCG", "DIC", "cht"), ("PBiCG", "DILU", "cd")])
def test_mixed_precision(mrg, ctx, oracle_mod, solver, pc, case):
    s = SMALL[case]()
    A = oracle_matrix(oracle_mod, s)
    # FP64 oracle reference: the same method converged far below the target
    xo, po = A.solve(s.b, s.x0, solver, pc, tol=1e-13)
    # the plain FP64 method at the target tolerance, for scale
    xp, pp = A.solve(s.b, s.x0, solver, pc, tol=1e-8)
    plain_err = rel_err(xp, xo)
    m = gpu_mesh(mrg, ctx, s)
    for ordering in ("exact", "colour"):
        x, p = m.solve(s.b, s.x0, tol=1e-8, solver=solver, precond=pc, precision="mixed", ordering=ordering)
        assert p["converged"] and p["final_residual"] < 1e-8, p
        # the reported residual is the true FP64 foam residual of x
        true_r = np.abs(s.b - A.amul(x)).sum() / A.norm_factor(s.x0, s.b)
        assert abs(true_r - p["final_residual"]) < 1e-10
        # error vs the FP64 oracle: no worse than the plain method's own at 1e-8
        err = rel_err(x, xo)
        assert err <= max(1e-8, plain_err), (err, plain_err)
    m.close()


def test_colour_ordering_fp64(mrg, ctx, oracle_mod):
    s = SMALL["cht"]()
    A = oracle_matrix(oracle_mod, s)
    xo, _ = A.solve(s.b, s.x0, "PCG", "DIC", tol=1e-12)
    m = gpu_mesh(mrg, ctx, s)
    assert m.levels("colour") <= 3 < m.levels("exact")
    x, p = m.solve(s.b, s.x0, tol=1e-10, ordering="colour")
    assert p["converged"]
    assert rel_err(x, xo) < 1e-8
    m.close()


def test_ggi_gather_bitexact(mrg, ctx, oracle_mod):
    from test_oracle import jittered_faces
    fa = jittered_faces(24, 24, 0.2, 1)
    fb = jittered_faces(16, 24, 0.2, 2)
    (pa, sa, wa), (pb, sb, wb) = oracle_mod.ggi_weights(*fa, *fb)
    g = mrg.Ggi(ctx, pa, sa, wa, len(pb) - 1)
    src = np.random.default_rng(4).uniform(-1, 1, len(pb) - 1)
    assert np.array_equal(g.apply(src), oracle_mod.ggi_apply(pa, sa, wa, src, fused=True))
    src4 = np.random.default_rng(5).uniform(-1, 1, (len(pb) - 1, 4))
    assert np.array_equal(g.apply(src4.ravel(), ncomp=4), oracle_mod.ggi_apply(pa, sa, wa, src4.ravel(), 4, fused=True))
    g.close()


def test_nonconformal_interface_in_amul(mrg, ctx, oracle_mod):
    """Two regions coupled through a 3:2 GGI interface (general weights)."""
    from test_oracle import jittered_faces
    nx_a, nx_b, ny = 12, 8, 10
    fa = jittered_faces(nx_a, ny, 0.2, 11)
    fb = jittered_faces(nx_b, ny, 0.2, 12)
    (pa, sa, wa), (pb, sb, wb) = oracle_mod.ggi_weights(*fa, *fb)
    na = nx_a * ny * 4
    nb = nx_b * ny * 4
    la, ua, _ = cases.box_faces(nx_a, ny, 4, 0)
    lb, ub, _ = cases.box_faces(nx_b, ny, 4, na)
    n = na + nb
    lower = np.concatenate([la, lb]).astype(np.int32)
    upper = np.concatenate([ua, ub]).astype(np.int32)
    rng = np.random.default_rng(6)
    upc = -rng.uniform(0.5, 2.0, lower.size)
    a_top = np.arange(nx_a * ny) + 3 * nx_a * ny       # A's top layer
    b_bot = na + np.arange(nx_b * ny)                  # B's bottom layer
    cells = np.concatenate([a_top, b_bot]).astype(np.int32)
    ptr = np.concatenate([pa, pa[-1] + pb[1:]]).astype(np.int32)
    src = np.concatenate([b_bot[sa], a_top[sb]]).astype(np.int32)
    w = np.concatenate([wa, wb])
    bou = rng.uniform(0.5, 1.0, cells.size)
    diag = np.full(n, 1.0)
    np.add.at(diag, lower, -upc)
    np.add.at(diag, upper, -upc)
    np.add.at(diag, cells, bou)
    s = cases.LduSystem(n, lower, upper, diag, upc, None, rng.standard_normal(n), np.zeros(n),
                        {"cells": cells, "bou": bou, "int": None, "ptr": ptr, "src": src, "w": w})
    A = oracle_matrix(oracle_mod, s)
    m = gpu_mesh(mrg, ctx, s)
    x = rng.standard_normal(n)
    assert np.array_equal(m.amul(x), A.amul(x, fused=True))
    m.close()
    check_solve(mrg, ctx, oracle_mod, s, "PBiCG", "DILU", tol=1e-10)


def test_invalid_inputs_rejected(mrg, ctx):
    with pytest.raises(mrg.MrgError) as e:
        mrg.Mesh(ctx, 4, np.array([1, 0], np.int32), np.array([0, 2], np.int32))
    assert e.value.code == mrg.MRG_E_INVALID
    with pytest.raises(mrg.MrgError):
        mrg.Mesh(ctx, 4, np.array([0, 0], np.int32), np.array([9, 2], np.int32))
    with pytest.raises(mrg.MrgError, match="upper-triangular"):
        mrg.Mesh(ctx, 4, np.array([1, 0], np.int32), np.array([2, 3], np.int32))


def test_single_cell_and_no_faces(mrg, ctx):
    m = mrg.Mesh(ctx, 1, np.zeros(0, np.int32), np.zeros(0, np.int32))
    m.upload(np.array([4.0]), np.zeros(0))
    x, p = m.solve(np.array([2.0]), np.array([0.0]), tol=1e-12)
    assert x[0] == 0.5 and p["converged"]
    m.close()


def test_nan_coefficients_report_breakdown(mrg, ctx):
    s = SMALL["cht"]()
    diag = s.diag.copy()
    diag[5] = np.nan
    m = mrg.Mesh(ctx, s.n, s.lower, s.upper)
    m.upload(diag, s.upper_c)
    with pytest.raises(mrg.MrgError) as e:
        m.solve(s.b, s.x0, tol=1e-8, max_iter=20)
    assert e.value.code == mrg.MRG_E_BREAKDOWN
    m.close()


def test_hbm_budget_enforced(mrg):
    c = mrg.Context(0, hbm_budget=1 << 20)
    s = cases.cht_system(40, 40, 20, 10, seed=0)
    with pytest.raises(mrg.MrgError) as e:
        m = mrg.Mesh(c, s.n, s.lower, s.upper)
        m.upload(s.diag, s.upper_c)
        m.solve(s.b, s.x0)
    assert e.value.code == mrg.MRG_E_OOM
    c.close()


def test_deterministic_repeat(mrg, ctx):
    s = SMALL["cht"]()
    m = gpu_mesh(mrg, ctx, s)
    x1, p1 = m.solve(s.b, s.x0, tol=1e-9)
    x2, p2 = m.solve(s.b, s.x0, tol=1e-9)
    assert np.array_equal(x1, x2) and p1["n_iter"] == p2["n_iter"]
    m.close()
