"""Autotuner: choosing launch shapes never changes a result bit.

mrg_mesh_tune / mrg_batch_tune time the Krylov loop under each candidate
shape (graph of launches or persistent kernel, iterations per launch,
level-sweep chunks per CTA) and keep the fastest; a solve after tuning must
give the same solution, residuals and iteration counts as before it.
"""
import numpy as np
import pytest

from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,ordering", [("fp64", "exact"), ("mixed", "colour"), ("fp64", "colour")])
def test_mesh_tune_keeps_bits(mrg, ctx, precision, ordering):
    s = cases.cht_system(20, 16, 12, 6, seed=3, k_range=(0.1, 50.0))
    m = mrg.Mesh(ctx, s.n, s.lower, s.upper)
    m.upload(s.diag, s.upper_c)
    ctl = mrg.controls(tol=1e-8, max_iter=4000, precision=precision, ordering=ordering)
    d_b, d_x = ctx.to_device(s.b), ctx.to_device(s.x0)
    try:
        x0, p0 = m.solve(s.b, s.x0, ctl)
        t = m.tune(d_b, d_x, ctl)
        assert t["mode"] in (0, 1) and t["iters_per_launch"] in (4, 16) and t["us_per_iter"] > 0
        assert t["candidates"] >= 4
        assert np.array_equal(ctx.from_device(d_x, np.empty(s.n)), s.x0)   # x is not modified
        x1, p1 = m.solve(s.b, s.x0, ctl)
        assert np.array_equal(x0, x1)
        for k in ("initial_residual", "final_residual", "n_iter", "n_outer", "converged"):
            assert p0[k] == p1[k]
    finally:
        ctx.dev_free(d_b)
        ctx.dev_free(d_x)
        m.close()


def test_batch_tune_keeps_bits(mrg, ctx):
    systems = cases.c4(5, seed=4, n_lo=3000, n_hi=20000)
    meshes = []
    for s in systems:
        m = mrg.Mesh(ctx, s.n, s.lower, s.upper)
        m.upload(s.diag, s.upper_c)
        meshes.append(m)
    bt = mrg.Batch(ctx, meshes, "colour")
    ctl = mrg.controls(tol=1e-8, max_iter=4000, precision="mixed", ordering="colour")
    try:
        x0, p0 = bt.solve([s.b for s in systems], [s.x0 for s in systems], ctl)
        d_b = [ctx.to_device(s.b) for s in systems]
        d_x = [ctx.to_device(s.x0) for s in systems]
        t = bt.tune(d_b, d_x, ctl)
        assert t["us_per_iter"] > 0
        x1, p1 = bt.solve([s.b for s in systems], [s.x0 for s in systems], ctl)
        for a, b in zip(x0, x1):
            assert np.array_equal(a, b)
        assert p0 == [dict(p, solve_ms=q["solve_ms"]) for p, q in zip(p1, p0)]
        for a in d_b + d_x:
            ctx.dev_free(a)
    finally:
        bt.close()
        for m in meshes:
            m.close()
