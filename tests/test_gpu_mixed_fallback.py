"""Mixed precision: a refinement that stalls finishes in FP64.

When the FP64 outer loop ends without reaching the tolerance (FP32 BiCG
drift, or the refinement-step limit), the solve restarts FP64 Krylov from
the best refined iterate with the solve's own normFactor (PBiCG for a
BiCGStab solve), and reports fallback = 1.  The refinement-step limit max_outer = 1 forces that path
here; the result must converge, its error against a tightly converged FP64
solution must stay within 10x of the plain FP64 method's own at the same
tolerance, and it must be bit-identical alone and inside the server's
continuous batch.
"""
import numpy as np
import pytest

from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["cht", "convdiff", "convdiff_bicgstab"])
def test_stalled_refinement_finishes_in_fp64(mrg, ctx, case):
    if case == "cht":
        s = cases.cht_system(18, 14, 12, 6, seed=5, k_range=(0.1, 50.0))
        kw = dict(solver="PCG", precond="DIC")
    else:
        s = cases.convdiff_system(16, 14, 12, seed=6)
        kw = dict(solver="PBiCG" if case == "convdiff" else "BiCGStab", precond="DILU")
    m = mrg.Mesh(ctx, s.n, s.lower, s.upper)
    m.upload(s.diag, s.upper_c, s.lower_c)
    try:
        xr, _ = m.solve(s.b, s.x0, tol=1e-13, max_iter=20000, precision="fp64", **kw)
        x64, p64 = m.solve(s.b, s.x0, tol=1e-8, max_iter=5000, precision="fp64", ordering="colour", **kw)
        x, p = m.solve(s.b, s.x0, tol=1e-8, max_iter=5000, precision="mixed", ordering="colour", max_outer=1, **kw)
        assert p["fallback"] and p["converged"] and p["final_residual"] < 1e-8
        assert p["n_outer"] == 1
        assert p["initial_residual"] == p64["initial_residual"]
        # error against the tightly converged FP64 solution: within 10x of
        # the plain FP64 method's own at the same residual tolerance
        err = lambda v: np.abs(v - xr).max() / np.abs(xr).max()
        assert err(x) <= max(1e-8, 10.0 * err(x64)), (err(x), err(x64))
        # the reported residual is the true FP64 foam residual of x:
        # sum|b - A x| over the normFactor of the initial guess
        r_x, nf_x = m.residual(s.b, x)
        _, nf_0 = m.residual(s.b, s.x0)
        assert abs(r_x * nf_x / nf_0 - p["final_residual"]) <= 1e-12
        # without the limit the refinement itself converges
        x2, p2 = m.solve(s.b, s.x0, tol=1e-8, max_iter=5000, precision="mixed", ordering="colour", **kw)
        assert not p2["fallback"] and p2["converged"]
    finally:
        m.close()


def test_fallback_in_server_equals_alone(mrg, ctx):
    s1 = cases.cht_system(16, 12, 10, 5, seed=7, k_range=(0.1, 50.0))
    s2 = cases.convdiff_system(14, 12, 10, seed=8)
    m1 = mrg.Mesh(ctx, s1.n, s1.lower, s1.upper)
    m2 = mrg.Mesh(ctx, s2.n, s2.lower, s2.upper)
    kw = dict(tol=1e-8, max_iter=5000, precision="mixed", ordering="colour", max_outer=1, iters_per_launch=4)
    sym = mrg.controls(solver="PCG", precond="DIC", **kw)
    asym = mrg.controls(solver="PBiCG", precond="DILU", **kw)
    try:
        m1.upload(s1.diag, s1.upper_c)
        ref1 = m1.solve(s1.b, s1.x0, sym)
        m2.upload(s2.diag, s2.upper_c, s2.lower_c)
        ref2 = m2.solve(s2.b, s2.x0, asym)
        srv = mrg.Server(ctx, sym, asym)
        try:
            ids = [srv.submit(m1, s1.b, s1.x0, s1.diag, s1.upper_c),
                   srv.submit(m2, s2.b, s2.x0, s2.diag, s2.upper_c, s2.lower_c, asym=True)]
            res = [srv.wait(r, 120000.0) for r in ids]
        finally:
            srv.close()
        for (x_ref, p_ref), (x, p, _) in zip((ref1, ref2), res):
            assert p_ref["fallback"] and p["fallback"]
            assert np.array_equal(x, x_ref)
            for k in ("initial_residual", "final_residual", "n_iter", "n_outer", "converged"):
                assert p[k] == p_ref[k]
    finally:
        m1.close()
        m2.close()
