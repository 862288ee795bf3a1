"""Parity at the full sizes of the headline and the asymmetric workloads.

Workloads:
* two-region CHT, fluid 128^3 over solid 128x128x64 (3,145,728 cells,
  conductivity log-uniform in [0.1, 50]): plain FP64 PCG + DIC, and the
  mixed form (FP32 PCG + colour DIC inside FP64 refinement);
* the permuted convection-diffusion pair with a 3:2 GGI interface at full
  size (A 96x96x48 + B 64x96x48 = 737,280 cells, 9,216 : 6,144 faces):
  plain FP64 PBiCG + DILU, and the mixed form with BiCGStab and with PBiCG
  inner solves.

Bars, plain FP64 through the C ABI against the CPU oracle:
* bit-identical to the oracle's GPU-order mirror: solution, initial and
  final residual, iteration count;
* against foam's sequential-sum order (the literal mode): the initial
  residual within 1e-10 relative (one Amul and two sums); both converge
  below the tolerance; iteration counts within 1 % (identical on the CHT
  system); the solution at least as accurate as the foam-order one against
  the oracle's FP64 solution converged to 1e-13 (within 1.5x of its error)
  and, on the CHT system, closer to the foam-order solution than that is to
  the converged one.  At these sizes the summation order of the dot
  products alone moves a 1e-8 solve's solution by far more than 1e-10
  (measured on the CPU: CHT foam order vs GPU order 6.3e-9 relative, each
  3.5e-8 from the converged solution; convection-diffusion 609 vs 605
  iterations, foam order 1.2e-5 and GPU order 1.9e-6 from the converged
  solution), so no reduction tree other than foam's own sequential one can
  meet a 1e-10 bar there; the sizes where it is met are in
  test_gpu_parity.py.
Mixed form: the true FP64 residual below the tolerance; max-norm error
against the 1e-13 oracle solution at most 1e-8 (CHT), within 10x of the
plain method's own error (convection-diffusion, cell Peclet up to 10).

The oracle solves (single-threaded C, tens of seconds each at these sizes)
run in spawned processes while the GPU solves run.
"""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

from conftest import gpu_mesh

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REL = 1e-10
MAX_IT = 20000


def _case(name):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    if name == "c2":
        from multiregionfoam_gb300 import cases
        return cases.c2(form="global", seed=0)
    from c3_case import c3
    return c3(scale=1, seed=2)[0]


def _oracle_job(job):
    """One oracle solve in a spawned process: (name, mode, tol) -> (x, perf)."""
    name, solver, pc, tol, mode = job
    s = _case(name)
    import oracle as O
    A = O.OracleMatrix(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.iface)
    if mode == "mirror":
        x, p = A.solve_mirror(s.b, s.x0, solver, pc, tol=tol, max_iter=MAX_IT)
    else:
        x, p = A.solve(s.b, s.x0, solver, pc, tol=tol, max_iter=MAX_IT)
    return (name, mode, tol), (x, p)


JOBS = [("c2", "PCG", "DIC", 1e-8, "literal"), ("c2", "PCG", "DIC", 1e-8, "mirror"),
        ("c2", "PCG", "DIC", 1e-13, "literal"),
        ("c3", "PBiCG", "DILU", 1e-8, "literal"), ("c3", "PBiCG", "DILU", 1e-8, "mirror"),
        ("c3", "PBiCG", "DILU", 1e-13, "literal")]


@pytest.fixture(scope="module")
def oracle_runs(oracle_mod):
    """Start every oracle solve now; the tests collect them when needed."""
    pool = mp.get_context("spawn").Pool(min(len(JOBS), max(1, len(os.sched_getaffinity(0)))))
    pending = pool.map_async(_oracle_job, JOBS)
    cache = {}

    def get(key):
        if not cache:
            cache.update(dict(pending.get(timeout=1800)))
        return cache[key]

    yield get
    pool.terminate()
    pool.join()


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _check_plain(xg, pg, lit, mir, tight, same_iters):
    xo, po = lit
    xm, pm = mir
    xt, pt = tight
    assert pt["converged"]
    # bit-identical to the GPU-order mirror
    assert np.array_equal(xg, xm), rel_err(xg, xm)
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"])
    # foam's sequential-sum order
    assert pg["converged"] and po["converged"]
    assert abs(pg["initial_residual"] - po["initial_residual"]) <= REL * po["initial_residual"]
    if same_iters:
        assert pg["n_iter"] == po["n_iter"], (pg, po)
    else:
        assert abs(pg["n_iter"] - po["n_iter"]) <= max(2, po["n_iter"] // 100), (pg, po)
    foam_err = rel_err(xo, xt)
    assert rel_err(xg, xt) <= 1.5 * foam_err, (rel_err(xg, xt), foam_err)
    if same_iters:
        assert rel_err(xg, xo) <= foam_err, (rel_err(xg, xo), foam_err)
    return foam_err


def test_c2_full_plain_and_mixed_vs_oracle(mrg, ctx, oracle_runs):
    s = _case("c2")
    assert s.n == 3145728
    m = gpu_mesh(mrg, ctx, s)
    try:
        xg, pg = m.solve(s.b, s.x0, tol=1e-8, max_iter=MAX_IT, solver="PCG", precond="DIC")
        xmx, pmx = m.solve(s.b, s.x0, tol=1e-8, max_iter=MAX_IT, solver="PCG", precond="DIC",
                           precision="mixed", ordering="colour")
    finally:
        m.close()
    tight = oracle_runs(("c2", "literal", 1e-13))
    _check_plain(xg, pg, oracle_runs(("c2", "literal", 1e-8)), oracle_runs(("c2", "mirror", 1e-8)), tight,
                 same_iters=True)
    assert pmx["converged"] and pmx["final_residual"] < 1e-8
    assert rel_err(xmx, tight[0]) <= 1e-8, rel_err(xmx, tight[0])


@pytest.mark.parametrize("inner", ["BiCGStab", "PBiCG"])
def test_c3_full_plain_and_mixed_vs_oracle(mrg, ctx, oracle_runs, inner):
    s = _case("c3")
    assert s.n == 737280
    m = gpu_mesh(mrg, ctx, s)
    try:
        xg, pg = m.solve(s.b, s.x0, tol=1e-8, max_iter=MAX_IT, solver="PBiCG", precond="DILU")
        xmx, pmx = m.solve(s.b, s.x0, tol=1e-8, max_iter=MAX_IT, solver=inner, precond="DILU",
                           precision="mixed", ordering="colour")
    finally:
        m.close()
    tight = oracle_runs(("c3", "literal", 1e-13))
    _check_plain(xg, pg, oracle_runs(("c3", "literal", 1e-8)), oracle_runs(("c3", "mirror", 1e-8)), tight,
                 same_iters=False)
    assert pmx["converged"] and pmx["final_residual"] < 1e-8
    # convection-dominated (cell Peclet up to 10): any solution meeting a 1e-8
    # residual is ~1e-6 from the converged one; the mixed form stays within
    # 10x of the plain method's own error
    plain_err = rel_err(xg, tight[0])
    assert rel_err(xmx, tight[0]) <= max(1e-8, 10.0 * plain_err), (rel_err(xmx, tight[0]), plain_err)
