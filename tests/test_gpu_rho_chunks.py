"""rho from the levelled sweeps' per-chunk (r, w) sums (OP_RHO_CH, FP32 PCG
with a colour DIC) on a mesh whose colouring needs more than two levels.

A hex block with one diagonal face per cell column (triangles, so no
two-colouring exists): the forward sweep writes w only at the last level
and the backward sweep at every other level, levels >= 1 of which start
from y and must load r for their chunk sums.  A wrong or missing chunk sum
would not change the FP64-refined answer but would stall the FP32 Krylov
loop, so the test bounds the mixed solve's total inner iterations by the
FP64 solve's in the same colour order, and checks the answer against a
tight FP64 solution.
"""
import numpy as np
import pytest

from multiregionfoam_gb300 import cases
from test_gpu_parity import rel_err

pytestmark = pytest.mark.gpu


def odd_cycle_system(nx, ny, nz, seed=0):
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    lower, upper, _ = cases.box_faces(nx, ny, nz)
    idx = np.arange(n).reshape(nz, ny, nx)
    # diagonal faces (i, j, k) - (i + 1, j + 1, k): triangles with the x and y faces
    dl = idx[:, :-1, :-1].ravel()
    du = idx[:, 1:, 1:].ravel()
    lo = np.concatenate([lower, dl]).astype(np.int64)
    up = np.concatenate([upper, du]).astype(np.int64)
    order = np.lexsort((up, lo))
    lo, up = lo[order].astype(np.int32), up[order].astype(np.int32)
    w = rng.uniform(0.2, 5.0, len(lo))
    diag = np.zeros(n)
    np.add.at(diag, lo, w)
    np.add.at(diag, up, w)
    diag += rng.uniform(0.01, 0.1, n)
    b = rng.uniform(-1.0, 1.0, n)
    return cases.LduSystem(n, lo, up, diag, -w, None, b, np.zeros(n), None, name="odd-cycles")


def test_rho_chunks_on_more_than_two_levels(mrg, ctx):
    s = odd_cycle_system(24, 20, 16, seed=7)
    m = mrg.Mesh(ctx, s.n, s.lower, s.upper)
    m.upload(s.diag, s.upper_c)
    try:
        assert m.levels("colour") > 2
        x64, p64 = m.solve(s.b, s.x0, tol=1e-8, max_iter=5000, solver="PCG", precond="DIC", ordering="colour")
        xt, _ = m.solve(s.b, s.x0, tol=1e-13, max_iter=20000, solver="PCG", precond="DIC")
        xm, pm = m.solve(s.b, s.x0, tol=1e-8, max_iter=5000, solver="PCG", precond="DIC", precision="mixed",
                         ordering="colour")
    finally:
        m.close()
    assert p64["converged"] and pm["converged"] and not pm["fallback"]
    inner = pm.get("inner_iterations", pm["n_iter"])
    assert inner <= 1.5 * p64["n_iter"] + 20, (inner, p64["n_iter"])
    assert rel_err(xm, xt) <= max(1e-8, 10 * rel_err(x64, xt))
