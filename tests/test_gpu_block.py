"""Block-coupled (4 x 4) systems solved through their scalar expansion
(mrg_block_addressing / mrg_block_coeffs) on the GPU:

* FP64, foam order: BiCGStab + DILU and PBiCG + DILU on an asymmetric block
  system, PCG + DIC on a symmetric (SPD) one -- bit-identical to the
  oracle's GPU-order mirror of the same scalar system and within 1e-10 of
  its sequential-sum solve (check_solve);
* the solution's block residual, from the block product itself, is at the
  solve tolerance;
* mixed precision (FP32 inner, colour DIC/DILU) converges to an error no
  worse than ten times the plain method's against a tight FP64 solve.
"""
import numpy as np
import pytest

from multiregionfoam_gb300.cases import block_case
from conftest import gpu_mesh, oracle_matrix
from multiregionfoam_gb300 import cases
from test_gpu_parity import check_solve, rel_err

pytestmark = pytest.mark.gpu


def scalar_system(mrg, c):
    n_s, lo, up, d, uc, lc = mrg.block_system(c["n"], c["lower"], c["upper"], c["bs"], c["D"], c["U"], c["L"])
    sym = c["L"] is None
    return cases.LduSystem(n_s, lo, up, d, uc, None if sym else lc, c["b"].ravel().copy(), c["x0"].ravel().copy(),
                           None, name="block")


def block_residual(bo, c, x):
    r = c["b"] - bo.block_amul(c["n"], c["lower"], c["upper"], c["D"], c["U"], c["L"], x.reshape(c["n"], c["bs"]))
    return np.abs(r).sum() / np.abs(c["b"]).sum()


@pytest.fixture(scope="module")
def bo():
    import block_oracle
    return block_oracle


@pytest.mark.parametrize("solver,bs", [("BiCGStab", 4), ("PBiCG", 4), ("BiCGStab", 2), ("PBiCG", 3)])
def test_block_asym_fp64_matches_oracle(mrg, ctx, oracle_mod, bo, solver, bs):
    c = block_case(10, 8, 6, bs=bs, seed=21 + bs)
    s = scalar_system(mrg, c)
    x, p, _ = check_solve(mrg, ctx, oracle_mod, s, solver, "DILU", tol=1e-9, max_iter=2000)
    assert p["converged"] and block_residual(bo, c, x) < 1e-7


def test_block_sym_fp64_matches_oracle(mrg, ctx, oracle_mod, bo):
    c = block_case(10, 8, 6, bs=4, seed=22, symmetric=True)
    s = scalar_system(mrg, c)
    x, p, _ = check_solve(mrg, ctx, oracle_mod, s, "PCG", "DIC", tol=1e-9, max_iter=2000)
    assert p["converged"] and block_residual(bo, c, x) < 1e-7


@pytest.mark.parametrize("symmetric,solver,pc", [(False, "BiCGStab", "DILU"), (True, "PCG", "DIC")])
def test_block_mixed(mrg, ctx, oracle_mod, bo, symmetric, solver, pc):
    c = block_case(16, 12, 10, bs=4, seed=23, symmetric=symmetric)
    s = scalar_system(mrg, c)
    A = oracle_matrix(oracle_mod, s)
    xo, _ = A.solve(s.b, s.x0, solver, pc, tol=1e-13, max_iter=5000)
    m = gpu_mesh(mrg, ctx, s)
    try:
        xp, pp = m.solve(s.b, s.x0, tol=1e-8, max_iter=3000, solver=solver, precond=pc)
        xm, pm = m.solve(s.b, s.x0, tol=1e-8, max_iter=3000, solver=solver, precond=pc, precision="mixed",
                         ordering="colour")
    finally:
        m.close()
    assert pp["converged"] and pm["converged"] and pm["final_residual"] < 1e-8
    assert rel_err(xm, xo) <= max(1e-8, 10 * rel_err(xp, xo))
    assert block_residual(bo, c, xm) < 1e-6
