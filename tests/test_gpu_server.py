"""Serving form: continuous batching of solve requests (mrg_server_*).

Each request's result must be the same alone and in the mix: the server runs
it inside a batch whose membership changes while it iterates (requests join
between iteration launches and leave as they converge), and per-system
reductions do not depend on the batch, so the solution, the reported
residuals and the iteration count must equal a lone mrg_solve with the same
controls bit for bit (the stated tolerance is zero).
"""
import time

import numpy as np
import pytest

from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


def _workload(seed=0):
    """(system, asym, steps): 3 symmetric CHT meshes, 2 asymmetric
    convection-diffusion meshes, one mesh recurring over 3 time steps."""
    rng = np.random.default_rng(seed)
    base = [(cases.cht_system(14, 12, 10, 5, seed=1, k_range=(0.1, 50.0)), False),
            (cases.cht_system(22, 18, 14, 7, seed=2, k_range=(0.1, 50.0)), False),
            (cases.cht_system(9, 8, 6, 3, seed=3, k_range=(0.1, 50.0)), False),
            (cases.convdiff_system(13, 12, 11, seed=4), True),
            (cases.convdiff_system(18, 15, 10, seed=5), True)]
    reqs = []
    for i, (s, asym) in enumerate(base):
        steps = 3 if i == 0 else 1
        cur = s
        for k in range(steps):
            reqs.append((i, cur, asym))
            cur = cases.perturb_step(cur, rng)
    return base, reqs


def _controls(mrg, precision):
    ordering = "colour" if precision == "mixed" else "exact"
    sym = mrg.controls(tol=1e-8, max_iter=4000, solver="PCG", precond="DIC", precision=precision,
                       ordering=ordering, iters_per_launch=4)
    asym = mrg.controls(tol=1e-8, max_iter=4000, solver="PBiCG", precond="DILU", precision=precision,
                        ordering=ordering, iters_per_launch=4)
    return sym, asym


def _references(mrg, meshes, reqs, sym, asym):
    out = []
    for i, s, a in reqs:
        m = meshes[i]
        m.upload(s.diag, s.upper_c, s.lower_c)
        out.append(m.solve(s.b, s.x0, asym if a else sym))
    return out


def _run_server(mrg, ctx, meshes, reqs, sym, asym, budget=0, stagger=True):
    srv = mrg.Server(ctx, sym, asym, hbm_budget=budget)
    try:
        ids = []
        for j, (i, s, a) in enumerate(reqs):
            ids.append(srv.submit(meshes[i], s.b, s.x0, s.diag, s.upper_c, s.lower_c, asym=a))
            if stagger and j == 2:
                time.sleep(0.02)   # the rest arrive while the first ones are on the GPU
        res = [srv.wait(r, 120000.0) for r in ids]
        stats = srv.stats()
    finally:
        srv.close()
    return res, stats


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_results_equal_alone(mrg, ctx, precision):
    base, reqs = _workload()
    meshes = [mrg.Mesh(ctx, s.n, s.lower, s.upper) for s, _ in base]
    sym, asym = _controls(mrg, precision)
    try:
        ref = _references(mrg, meshes, reqs, sym, asym)
        res, stats = _run_server(mrg, ctx, meshes, reqs, sym, asym)
    finally:
        for m in meshes:
            m.close()
    assert stats["completed"] == len(reqs)
    assert stats["peak_running"] >= 2          # requests overlapped on the device
    for (x_ref, p_ref), r in zip(ref, res):
        assert r is not None
        x, p, lat = r
        assert lat > 0
        assert p["converged"] and p["final_residual"] < 1e-8
        assert np.array_equal(x, x_ref)
        for k in ("initial_residual", "final_residual", "n_iter", "n_outer", "converged"):
            assert p[k] == p_ref[k], (k, p[k], p_ref[k])


def test_server_hbm_budget_admission(mrg, ctx):
    base, reqs = _workload(seed=1)
    meshes = [mrg.Mesh(ctx, s.n, s.lower, s.upper) for s, _ in base]
    sym, asym = _controls(mrg, "mixed")
    try:
        ref = _references(mrg, meshes, reqs, sym, asym)
        # room for about one working set at a time: requests queue for memory
        budget = 6 * 1024 * 1024
        res, stats = _run_server(mrg, ctx, meshes, reqs, sym, asym, budget=budget, stagger=False)
        assert stats["peak_inflight_bytes"] <= budget
        for (x_ref, _), (x, p, _) in zip(ref, res):
            assert np.array_equal(x, x_ref)
        # a budget below any working set: every request is refused, none runs
        srv = mrg.Server(ctx, sym, asym, hbm_budget=1024)
        try:
            i, s, a = reqs[1]
            rid = srv.submit(meshes[i], s.b, s.x0, s.diag, s.upper_c, s.lower_c, asym=a)
            with pytest.raises(mrg.MrgError) as e:
                srv.wait(rid, 60000.0)
            assert e.value.code == 2
        finally:
            srv.close()
    finally:
        for m in meshes:
            m.close()
