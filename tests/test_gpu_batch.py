"""Batched solves: many independent systems of uneven size in lockstep.

Each member's result must be bit-identical to solving it alone (reductions
are segmented per system, so the batch does not change any sum), and the
batch must agree with the oracle like a single solve does."""
import numpy as np
import pytest

from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


def systems():
    s = cases.c4(count=6, seed=3, n_lo=2000, n_hi=60000)
    s.append(cases.cht_system(12, 10, 9, 4, seed=5, form="coupled", k_range=(0.1, 50.0)))
    return s


@pytest.mark.parametrize("kw", [dict(), dict(ordering="colour"), dict(precision="mixed", ordering="colour"),
                                dict(precision="mixed")])
def test_batch_equals_alone(mrg, ctx, kw):
    sys_ = systems()
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    alone = [m.solve(s.b, s.x0, tol=1e-8, **kw) for m, s in zip(meshes, sys_)]
    b = mrg.Batch(ctx, meshes, ordering=kw.get("ordering", "exact"))
    xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-8, **kw)
    for (xa, pa), xb, pb in zip(alone, xs, perfs):
        assert np.array_equal(xa, xb)
        for k in ("initial_residual", "final_residual", "n_iter", "converged", "n_outer"):
            assert pa[k] == pb[k], (k, pa, pb)
        assert pb["converged"]
    # a second solve of the same batch (resident plans, graphs) repeats it
    xs2, perfs2 = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-8, **kw)
    assert all(np.array_equal(a, c) for a, c in zip(xs, xs2))
    b.close()
    for m in meshes:
        m.close()


@pytest.mark.parametrize("kw", [dict(), dict(precision="mixed", ordering="colour"),
                                dict(solver="BiCGStab", precond="DILU", precision="mixed", ordering="colour")])
def test_compacted_batch_equals_alone(mrg, ctx, kw):
    """Twelve members of very uneven size: once half have converged the rest
    iterate in a compacted sub-batch (and again at a quarter); every result
    must still equal its lone solve bit for bit."""
    sys_ = cases.c4(count=12, seed=11, n_lo=1000, n_hi=80000)
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    alone = [m.solve(s.b, s.x0, tol=1e-8, iters_per_launch=4, **kw) for m, s in zip(meshes, sys_)]
    b = mrg.Batch(ctx, meshes, ordering=kw.get("ordering", "exact"))
    for rep in range(2):   # the second solve reuses the compacted batches' graphs
        xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-8, iters_per_launch=4, **kw)
        for (xa, pa), xb, pb in zip(alone, xs, perfs):
            assert np.array_equal(xa, xb)
            for k in ("initial_residual", "final_residual", "n_iter", "converged", "n_outer"):
                assert pa[k] == pb[k], (k, pa, pb)
    its = [p["n_iter"] for p in perfs]
    assert len(set(its)) > 3   # uneven convergence: the tail runs compacted
    b.close()
    for m in meshes:
        m.close()


def test_batch_against_oracle(mrg, ctx, oracle_mod):
    sys_ = systems()
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    b = mrg.Batch(ctx, meshes)
    xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-9)
    for s, x, p in zip(sys_, xs, perfs):
        A = oracle_matrix(oracle_mod, s)
        xm, pm = A.solve_mirror(s.b, s.x0, "PCG", "DIC", tol=1e-9)
        assert np.array_equal(x, xm)
        assert p["n_iter"] == pm["n_iter"]
    b.close()
    for m in meshes:
        m.close()


def test_batch_pbicg(mrg, ctx, oracle_mod):
    sys_ = [cases.convdiff_system(n, n - 1, n - 2, seed=n) for n in (9, 13, 17)]
    meshes = [gpu_mesh(mrg, ctx, s) for s in sys_]
    b = mrg.Batch(ctx, meshes)
    xs, perfs = b.solve([s.b for s in sys_], [s.x0 for s in sys_], tol=1e-9, solver="PBiCG", precond="DILU")
    for s, x, p in zip(sys_, xs, perfs):
        xm, pm = oracle_matrix(oracle_mod, s).solve_mirror(s.b, s.x0, "PBiCG", "DILU", tol=1e-9)
        assert np.array_equal(x, xm) and p["n_iter"] == pm["n_iter"]
    b.close()
    for m in meshes:
        m.close()


def test_batch_rejects_bad_members(mrg, ctx):
    s = cases.cht_system(6, 6, 6, 3)
    m = gpu_mesh(mrg, ctx, s)
    with pytest.raises(mrg.MrgError):
        mrg.Batch(ctx, [m, m])
    m.close()
