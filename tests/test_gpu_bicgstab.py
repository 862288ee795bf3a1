"""BiCGStab on the GPU (MRG_SOLVER_BICGSTAB; foam-extend's "BiCGStab", the
reference tutorials' coupled solver) against the oracle.

Bars, as for PCG / PBiCG:
* exact ordering, FP64: bit-identical to the oracle's GPU-order mirror
  (solution, initial / final residual, iteration count) for DIC / DILU,
  diagonal and no preconditioning, with and without interfaces;
* vs the oracle's foam-order arithmetic: iteration count within one (DIC /
  DILU; 10 % with weaker preconditioning), solution within 10 x the
  tolerance (summation order moves the half-step test);
* colour ordering and mixed precision: converged, the reported residual is
  the true FP64 residual of x, error vs a tight FP64 solve bounded;
* batched and served: bit-identical to the lone solve.
"""
import numpy as np
import pytest

from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


SMALL = {
    "cht": lambda: cases.cht_system(16, 14, 12, 7, seed=1, form="global", k_range=(0.1, 50.0)),
    "chtc": lambda: cases.cht_system(16, 14, 12, 7, seed=1, form="coupled", k_range=(0.1, 50.0)),
    "cd": lambda: cases.convdiff_system(14, 13, 12, seed=2),
}


def check_bs(mrg, ctx, O, s, pc, tol=1e-8, **kw):
    A = oracle_matrix(O, s)
    xm, pm = A.solve_mirror(s.b, s.x0, "BiCGStab", pc, tol=tol, **kw)
    xo, po = A.solve(s.b, s.x0, "BiCGStab", pc, tol=tol, **kw)
    m = gpu_mesh(mrg, ctx, s)
    xg, pg = m.solve(s.b, s.x0, tol=tol, solver="BiCGStab", precond=pc, **kw)
    m.close()
    assert np.array_equal(xg, xm), rel_err(xg, xm)
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"], pg["converged"], pg["singular"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"], pm["converged"], pm["singular"])
    # BiCGStab's irregular residual history makes the count sensitive to the
    # summation order when the preconditioner is weak
    slack = 1 if pc in ("DIC", "DILU") else max(2, po["n_iter"] // 10)
    assert abs(pg["n_iter"] - po["n_iter"]) <= slack, (pg, po)
    if po["converged"]:
        # two residual histories to the same tolerance: the solutions agree to
        # the error that tolerance allows (wider without a factorisation)
        assert rel_err(xg, xo) <= (10 if pc in ("DIC", "DILU") else 100) * tol
    return xg, pg


@pytest.mark.parametrize("name,pc", [("cht", "DIC"), ("cht", "diagonal"), ("cht", "none"), ("chtc", "DIC"),
                                     ("cd", "DILU"), ("cd", "diagonal")])
def test_bicgstab_bitexact_vs_mirror(mrg, ctx, oracle_mod, name, pc):
    s = SMALL[name]()
    xg, pg = check_bs(mrg, ctx, oracle_mod, s, pc, tol=1e-9)
    assert pg["converged"]


def test_bicgstab_c1_coupled_form(mrg, ctx, oracle_mod):
    """C1 in the two-region coupled form: the tutorials' monolithic solve."""
    s = cases.c1(form="coupled")
    xg, pg = check_bs(mrg, ctx, oracle_mod, s, "DIC")
    assert pg["converged"] and pg["final_residual"] < 1e-8


def test_bicgstab_nonconformal_c3_small(mrg, ctx, oracle_mod):
    """Asymmetric convection-diffusion over a 3:2 GGI interface (C3 at 1/4 size)."""
    from c3_case import c3
    s, _ = c3(scale=4, seed=1)
    check_bs(mrg, ctx, oracle_mod, s, "DILU")


def test_bicgstab_iteration_controls(mrg, ctx, oracle_mod):
    s = SMALL["cht"]()
    check_bs(mrg, ctx, oracle_mod, s, "DIC", tol=1e-30, max_iter=5)
    A = oracle_matrix(oracle_mod, s)
    xs, _ = A.solve(s.b, s.x0, "BiCGStab", "DIC", tol=1e-13)
    m = gpu_mesh(mrg, ctx, s)
    x, p = m.solve(s.b, xs, tol=1e-6, solver="BiCGStab")
    assert p["n_iter"] == 0 and p["converged"] and np.array_equal(x, xs)
    x, p = m.solve(s.b, xs, tol=1e-6, min_iter=3, solver="BiCGStab")
    xm, pm = A.solve_mirror(s.b, xs, "BiCGStab", "DIC", tol=1e-6, min_iter=3)
    assert p["n_iter"] == pm["n_iter"] == 3 and np.array_equal(x, xm)
    m.close()


@pytest.mark.parametrize("case,pc", [("cht", "DIC"), ("cd", "DILU"), ("chtc", "DIC")])
def test_bicgstab_colour_and_mixed(mrg, ctx, oracle_mod, case, pc):
    s = SMALL[case]()
    A = oracle_matrix(oracle_mod, s)
    xo, _ = A.solve(s.b, s.x0, "BiCGStab", pc, tol=1e-13)
    xp, _ = A.solve(s.b, s.x0, "BiCGStab", pc, tol=1e-8)
    plain_err = rel_err(xp, xo)
    m = gpu_mesh(mrg, ctx, s)
    for kw in (dict(ordering="colour"), dict(precision="mixed"), dict(precision="mixed", ordering="colour")):
        x, p = m.solve(s.b, s.x0, tol=1e-8, solver="BiCGStab", precond=pc, **kw)
        assert p["converged"] and p["final_residual"] < 1e-8, (kw, p)
        true_r = np.abs(s.b - A.amul(x)).sum() / A.norm_factor(s.x0, s.b)
        assert abs(true_r - p["final_residual"]) < 1e-10, kw
        assert rel_err(x, xo) <= max(1e-8, 2 * plain_err), (kw, rel_err(x, xo), plain_err)
    m.close()


@pytest.mark.parametrize("kw", [dict(), dict(precision="mixed", ordering="colour")])
def test_bicgstab_batch_equals_alone(mrg, ctx, kw):
    sys_ = cases.c4(count=4, seed=7, n_lo=2000, n_hi=40000)
    sys_.append(cases.convdiff_system(15, 12, 11, seed=9))
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    alone = [m.solve(s.b, s.x0, tol=1e-8, solver="BiCGStab", precond="DILU", **kw) for m, s in zip(meshes, sys_)]
    b = mrg.Batch(ctx, meshes, ordering=kw.get("ordering", "exact"))
    xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-8, solver="BiCGStab", precond="DILU",
                        **kw)
    for (xa, pa), xb, pb in zip(alone, xs, perfs):
        assert np.array_equal(xa, xb)
        for k in ("initial_residual", "final_residual", "n_iter", "converged", "n_outer"):
            assert pa[k] == pb[k], (k, pa, pb)
        assert pb["converged"]
    b.close()
    for m in meshes:
        m.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bicgstab_server_equals_alone(mrg, ctx, precision):
    rng = np.random.default_rng(11)
    base = [cases.cht_system(14, 12, 10, 5, seed=1, k_range=(0.1, 50.0)), cases.convdiff_system(13, 12, 11, seed=4),
            cases.cht_system(9, 8, 6, 3, seed=3, k_range=(0.1, 50.0))]
    reqs = [(0, base[0]), (1, base[1]), (2, base[2]), (0, cases.perturb_step(base[0], rng))]
    ordering = "colour" if precision == "mixed" else "exact"
    sym = mrg.controls(tol=1e-8, max_iter=4000, solver="BiCGStab", precond="DIC", precision=precision,
                       ordering=ordering, iters_per_launch=4)
    asym = mrg.controls(tol=1e-8, max_iter=4000, solver="BiCGStab", precond="DILU", precision=precision,
                        ordering=ordering, iters_per_launch=4)
    meshes = [mrg.Mesh(ctx, s.n, s.lower, s.upper) for s in base]
    try:
        ref = []
        for i, s in reqs:
            meshes[i].upload(s.diag, s.upper_c, s.lower_c)
            ref.append(meshes[i].solve(s.b, s.x0, asym if s.lower_c is not None else sym))
        srv = mrg.Server(ctx, sym, asym)
        try:
            ids = [srv.submit(meshes[i], s.b, s.x0, s.diag, s.upper_c, s.lower_c, asym=s.lower_c is not None)
                   for i, s in reqs]
            res = [srv.wait(r, 120000.0) for r in ids]
        finally:
            srv.close()
        for (xa, pa), (xb, pb, _) in zip(ref, res):
            assert np.array_equal(xa, xb)
            assert (pa["final_residual"], pa["n_iter"]) == (pb["final_residual"], pb["n_iter"])
            assert pb["converged"]
    finally:
        for m in meshes:
            m.close()
