"""The foam-extend lduMatrix::solver adapters (gpuPCG, gpuPBiCG, gpuBiCGStab and
their gpuMixed* forms), driven through the run-time selection table exactly as
fvMatrix::solve would, compared with the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu


def write_system(path, s):
    f = s.iface
    ni = 0 if f is None else len(f["cells"])
    nsrc = 0 if f is None else len(f["src"])
    with open(path, "wb") as fh:
        np.array([s.n, s.nf, ni, 0 if s.lower_c is None else 1, nsrc], np.int32).tofile(fh)
        s.lower.astype(np.int32).tofile(fh)
        s.upper.astype(np.int32).tofile(fh)
        for a in (s.diag, s.upper_c) + (() if s.lower_c is None else (s.lower_c,)) + (s.b, s.x0):
            np.asarray(a, np.float64).tofile(fh)
        if ni:
            for k in ("cells", "ptr", "src"):
                f[k].astype(np.int32).tofile(fh)
            f["w"].astype(np.float64).tofile(fh)
            f["bou"].astype(np.float64).tofile(fh)


def run(mrg, tmp_path, s, solver, pc, tol, extra=()):
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf, outf = str(tmp_path / "sys.bin"), str(tmp_path / "x.bin")
    write_system(sysf, s)
    r = subprocess.run([exe, sysf, solver, pc, repr(tol), outf, *extra], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(outf, np.float64), json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("solver", ["gpuPCG", "gpuPBiCG"])
def test_plain_adapter_matches_oracle(mrg, oracle_mod, tmp_path, solver):
    s = cases.c1(form="coupled")
    pc = "DIC" if solver == "gpuPCG" else "DILU"
    x, perf = run(mrg, tmp_path, s, solver, pc, 1e-8)
    xo, po = oracle_matrix(oracle_mod, s).solve(s.b, s.x0, solver[3:], pc, tol=1e-8)
    assert perf["solver"] == solver
    assert perf["n_iter"] == po["n_iter"] and perf["converged"] == 1
    assert abs(perf["initial_residual"] - po["initial_residual"]) <= 1e-10 * po["initial_residual"]
    assert abs(perf["final_residual"] - po["final_residual"]) <= 1e-10 * po["initial_residual"]
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


def test_asymmetric_adapter(mrg, oracle_mod, tmp_path):
    s = cases.convdiff_system(16, 15, 14, seed=7)
    x, perf = run(mrg, tmp_path, s, "gpuPBiCG", "DILU", 1e-9)
    xo, po = oracle_matrix(oracle_mod, s).solve(s.b, s.x0, "PBiCG", "DILU", tol=1e-9)
    assert perf["n_iter"] == po["n_iter"]
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


@pytest.mark.parametrize("solver,case", [("gpuMixedPCG", "cht"), ("gpuMixedPBiCG", "cd")])
def test_mixed_adapter(mrg, oracle_mod, tmp_path, solver, case):
    s = cases.c1(form="coupled") if case == "cht" else cases.convdiff_system(16, 15, 14, seed=7)
    pc = "DIC" if solver == "gpuMixedPCG" else "DILU"
    x, perf = run(mrg, tmp_path, s, solver, pc, 1e-8)
    assert perf["converged"] == 1 and perf["final_residual"] < 1e-8
    A = oracle_matrix(oracle_mod, s)
    assert abs(A.residual(s.b, x) * A.norm_factor(x, s.b) / A.norm_factor(s.x0, s.b) - perf["final_residual"]) \
        < 1e-10


@pytest.mark.parametrize("case", ["cht", "cd"])
def test_bicgstab_adapter(mrg, oracle_mod, tmp_path, case):
    """gpuBiCGStab from both tables (the tutorials' coupled solver) matches the
    oracle's GPU-order mirror bit for bit; gpuMixedBiCGStab converges."""
    s = cases.c1(form="coupled") if case == "cht" else cases.convdiff_system(16, 15, 14, seed=7)
    pc = "DIC" if case == "cht" else "DILU"
    A = oracle_matrix(oracle_mod, s)
    x, perf = run(mrg, tmp_path, s, "gpuBiCGStab", pc, 1e-9)
    xm, pm = A.solve_mirror(s.b, s.x0, "BiCGStab", pc, tol=1e-9)
    assert perf["solver"] == "gpuBiCGStab" and perf["converged"] == 1
    assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)
    if case == "cht":
        # the tutorials' setting: BiCGStab + Cholesky (incomplete Cholesky = DIC here)
        xc, pc_ = run(mrg, tmp_path, s, "gpuBiCGStab", "Cholesky", 1e-9)
        assert np.array_equal(xc, xm) and pc_["n_iter"] == pm["n_iter"]
    x, perf = run(mrg, tmp_path, s, "gpuMixedBiCGStab", pc, 1e-8)
    assert perf["solver"] == "gpuMixedBiCGStab" and perf["converged"] == 1 and perf["final_residual"] < 1e-8
    assert abs(A.residual(s.b, x) * A.norm_factor(x, s.b) / A.norm_factor(s.x0, s.b) - perf["final_residual"]) \
        < 1e-10


def test_biccg_alias(mrg, oracle_mod, tmp_path):
    """gpuBICCG: PBiCG + DILU whatever the preconditioner word says."""
    s = cases.convdiff_system(12, 11, 10, seed=4)
    x, perf = run(mrg, tmp_path, s, "gpuBICCG", "none", 1e-9)
    xm, pm = oracle_matrix(oracle_mod, s).solve_mirror(s.b, s.x0, "PBiCG", "DILU", tol=1e-9)
    assert perf["solver"] == "gpuPBiCG" and perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)


def test_smooth_solver_adapter(mrg, oracle_mod, tmp_path):
    """gpuSmoothSolver (smoother GaussSeidel): the tutorials' fluid U setting."""
    s = cases.convdiff_system(12, 11, 10, seed=9)
    x, perf = run(mrg, tmp_path, s, "gpuSmoothSolver", "none", 1e-8)
    xm, pm = oracle_matrix(oracle_mod, s).smooth(s.b, s.x0, tol=1e-8, mode="mirror")
    assert perf["solver"] == "gpuSmoothSolver" and perf["converged"] == 1
    assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)
    # the fvSolution words smoother / nSweeps
    x, perf = run(mrg, tmp_path, s, "gpuSmoothSolver", "none", 1e-8, ("smoother=DILUGaussSeidel", "nSweeps=2"))
    xm, pm = oracle_matrix(oracle_mod, s).smooth(s.b, s.x0, tol=1e-8, mode="mirror", smoother="DILUGaussSeidel",
                                                 n_sweeps=2)
    assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)


def test_gamg_adapter(mrg, oracle_mod, tmp_path):
    """gpuGAMG with the tutorials' words (smoother GaussSeidel,
    nCellsInCoarsestLevel 10)."""
    import gamg_oracle as G
    s = cases.convdiff_system(12, 11, 10, seed=9)
    x, perf = run(mrg, tmp_path, s, "gpuGAMG", "none", 1e-8, ("smoother=GaussSeidel", "nCellsInCoarsestLevel=10",
                                                              "agglomerator=faceAreaPair", "mergeLevels=1"))
    g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
    xm, pm = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-8, max_iter=5000)
    assert perf["solver"] == "gpuGAMG" and perf["converged"] == 1
    assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)


def test_unknown_solver_is_fatal(mrg, tmp_path):
    s = cases.cht_system(6, 6, 6, 3)
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf = str(tmp_path / "sys.bin")
    write_system(sysf, s)
    r = subprocess.run([exe, sysf, "gpuAMGX", "none", "1e-6", str(tmp_path / "x.bin")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "Unknown symmetric matrix solver gpuAMGX" in r.stdout
