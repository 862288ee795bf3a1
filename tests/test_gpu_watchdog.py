"""The device-wait watchdog, exercised without any GPU fault.

Every wait of a kernel on a value another CTA of the same launch publishes
is bounded.  mrg_ctx_set_watchdog sets the budget (SM cycles) and has a test
hook that leaves one chunk of the exact-order forward sweep unpublished, so
that the waits of the rows depending on it run out.  The solve must then
come back -- quickly, with MRG_E_TIMEOUT -- and the context must stay
usable: the next ordinary solve on it matches the oracle bit for bit (its
GPU-order mirror) and the other forms still work.
"""
import time

import numpy as np
import pytest

from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu

MRG_E_TIMEOUT = 4


def test_unpublished_dependency_times_out_and_context_recovers(mrg, oracle_mod):
    s = cases.cht_system(24, 20, 14, 8, seed=6, form="coupled", k_range=(0.1, 50.0))
    ctx = mrg.Context(0)
    try:
        m = gpu_mesh(mrg, ctx, s)
        assert m.levels("exact") > 2
        ctx.set_watchdog(wait_cycles=2_000_000, unpublished_chunk=0)   # ~1 ms per wait
        t0 = time.perf_counter()
        with pytest.raises(mrg.MrgError) as e:
            m.solve(s.b, s.x0, tol=1e-8, solver="PCG", precond="DIC")
        elapsed = time.perf_counter() - t0
        assert e.value.code == MRG_E_TIMEOUT, e.value
        assert elapsed < 30.0
        # the same context, watchdog back to its default: an ordinary solve
        ctx.set_watchdog(0, -1)
        x, p = m.solve(s.b, s.x0, tol=1e-8, solver="PCG", precond="DIC")
        xm, pm = oracle_matrix(oracle_mod, s).solve_mirror(s.b, s.x0, "PCG", "DIC", tol=1e-8)
        assert np.array_equal(x, xm) and p["n_iter"] == pm["n_iter"] and p["converged"]
        # and the mixed form (levelled sweeps, no dependency waits)
        xmx, pmx = m.solve(s.b, s.x0, tol=1e-8, precision="mixed", ordering="colour")
        assert pmx["converged"] and pmx["final_residual"] < 1e-8
        m.close()
    finally:
        ctx.close()


def test_watchdog_arguments_are_checked(mrg):
    ctx = mrg.Context(0)
    try:
        with pytest.raises(mrg.MrgError):
            ctx.set_watchdog(-1, -1)
        with pytest.raises(mrg.MrgError):
            ctx.set_watchdog(0, -2)
    finally:
        ctx.close()
