"""Block-coupled (4 x 4) systems solved through their scalar expansion
(mrg_block_addressing / mrg_block_coeffs) on the GPU:

* FP64, foam order: BiCGStab + DILU and PBiCG + DILU on an asymmetric block
  system, PCG + DIC on a symmetric (SPD) one -- bit-identical to the
  oracle's GPU-order mirror of the same scalar system and within 1e-10 of
  its sequential-sum solve (check_solve);
* the solution's block residual, from the block product itself, is at the
  solve tolerance;
* mixed precision (FP32 inner, colour DIC/DILU) converges to an error no
  worse than ten times the plain method's against a tight FP64 solve;
* the block preconditioner (MRG_PRECOND_BLOCK, foam-extend's block Cholesky
  on the bs x bs blocks): M^-1 r bit-identical to the oracle's restatement
  (oracle/block_oracle.py) for bs 1..4, symmetric and not, across a
  coefficient change; exact on a block chain; BiCGStab / PCG with it
  converge in no more iterations than with point-wise DILU / DIC.
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


# ---- the block preconditioner (MRG_PRECOND_BLOCK, foam-extend's block Cholesky) ----

def block_mesh(mrg, ctx, c):
    s = scalar_system(mrg, c)
    m = gpu_mesh(mrg, ctx, s)
    m.set_blocks(c["bs"], c["n"], c["lower"], c["upper"])
    return s, m


@pytest.mark.parametrize("bs,symmetric", [(4, False), (4, True), (3, False), (2, True), (1, False)])
def test_block_preconditioner_bitexact(mrg, ctx, bo, bs, symmetric):
    """M^-1 r on the GPU (factor from the scalar coefficients' blocks, forward
    and backward block sweeps) equals the oracle's restatement bit for bit."""
    c = block_case(7, 6, 5, bs=bs, seed=40 + bs, symmetric=symmetric)
    s, m = block_mesh(mrg, ctx, c)
    try:
        dD = bo.block_factor(c["n"], c["lower"], c["upper"], c["D"], c["U"], c["L"])
        for seed in (1, 2):
            r = np.random.default_rng(seed).standard_normal(c["n"] * bs)
            w = m.precondition("block", r)
            wo = bo.block_apply(c["n"], c["lower"], c["upper"], c["D"], c["U"], c["L"], dD, r).ravel()
            assert np.array_equal(w.view(np.uint64), wo.view(np.uint64)), np.abs(w - wo).max()
        # new coefficients: the blocks are gathered and factored again
        c2 = dict(c, D=c["D"] * 1.5)
        s2 = scalar_system(mrg, c2)
        m.upload(s2.diag, s2.upper_c, s2.lower_c)
        dD2 = bo.block_factor(c["n"], c["lower"], c["upper"], c2["D"], c["U"], c["L"])
        w = m.precondition("block", r)
        wo = bo.block_apply(c["n"], c["lower"], c["upper"], c2["D"], c["U"], c["L"], dD2, r).ravel()
        assert np.array_equal(w, wo)
    finally:
        m.close()


def test_block_preconditioner_exact_on_a_block_chain(mrg, ctx, bo):
    """On a chain of cells (block tridiagonal) the incomplete block
    factorisation has no fill-in to drop: M^-1 is A^-1."""
    n, bs = 40, 4
    rng = np.random.default_rng(7)
    lower = np.arange(n - 1, dtype=np.int32)
    upper = lower + 1
    U = rng.uniform(-1, 1, (n - 1, bs, bs))
    L = rng.uniform(-1, 1, (n - 1, bs, bs))
    D = rng.uniform(-0.3, 0.3, (n, bs, bs)) + np.eye(bs) * 12.0
    c = dict(n=n, lower=lower, upper=upper, bs=bs, D=D, U=U, L=L, b=rng.uniform(-1, 1, (n, bs)),
             x0=np.zeros((n, bs)))
    s, m = block_mesh(mrg, ctx, c)
    try:
        w = m.precondition("block", c["b"].ravel())
        r = c["b"] - bo.block_amul(n, lower, upper, D, U, L, w.reshape(n, bs))
        assert np.abs(r).max() < 1e-12 * np.abs(c["b"]).max()
    finally:
        m.close()


@pytest.mark.parametrize("symmetric,solver", [(False, "BiCGStab"), (True, "PCG"), (True, "BiCGStab")])
def test_block_preconditioned_solves(mrg, ctx, oracle_mod, bo, symmetric, solver):
    """BiCGStab / PCG with the block preconditioner converge to the FP64
    solution (block residual from the block product itself), in fewer
    iterations than with point-wise DILU / DIC on the scalar rows."""
    c = block_case(14, 12, 10, bs=4, seed=44, symmetric=symmetric)
    s, m = block_mesh(mrg, ctx, c)
    try:
        xb, pb = m.solve(s.b, s.x0, tol=1e-10, max_iter=2000, solver=solver, precond="block")
        xp, pp = m.solve(s.b, s.x0, tol=1e-10, max_iter=2000, solver=solver,
                         precond="DIC" if symmetric else "DILU")
        xb2, pb2 = m.solve(s.b, s.x0, tol=1e-10, max_iter=2000, solver=solver, precond="block")
    finally:
        m.close()
    assert pb["converged"] and pp["converged"]
    assert pb["n_iter"] <= pp["n_iter"]
    assert np.array_equal(xb, xb2) and pb["n_iter"] == pb2["n_iter"]       # deterministic
    assert block_residual(bo, c, xb) < 1e-8
    A = oracle_matrix(oracle_mod, s)
    xo, _ = A.solve(s.b, s.x0, "BiCGStab", "DILU", tol=1e-14, max_iter=5000)
    assert rel_err(xb, xo) < 1e-7


def test_block_preconditioner_rejects(mrg, ctx):
    c = block_case(5, 4, 3, bs=4, seed=45)
    s = scalar_system(mrg, c)
    m = gpu_mesh(mrg, ctx, s)
    try:
        with pytest.raises(mrg.MrgError, match="block structure"):
            m.solve(s.b, s.x0, solver="BiCGStab", precond="block")
        with pytest.raises(mrg.MrgError, match="expansion"):
            m.set_blocks(4, c["n"] - 1, c["lower"][:-1], c["upper"][:-1])
        m.set_blocks(4, c["n"], c["lower"], c["upper"])
        with pytest.raises(mrg.MrgError, match="PCG or BiCGStab"):
            m.solve(s.b, s.x0, solver="PBiCG", precond="block")
        with pytest.raises(mrg.MrgError, match="FP64"):
            m.solve(s.b, s.x0, solver="BiCGStab", precond="block", precision="mixed", ordering="colour")
    finally:
        m.close()
