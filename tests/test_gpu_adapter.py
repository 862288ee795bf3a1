"""The foam-extend solver adapters, driven through the run-time selection
tables exactly as foam-extend would, compared with the oracle:

* lduMatrix::solver (gpuPCG, gpuPBiCG, gpuBiCGStab and their gpuMixed*
  forms, gpuBICCG, gpuSmoothSolver, gpuGAMG) as fvMatrix::solve calls it;
* coupledLduSolver (the same names) as coupledFvMatrix::solve calls it for
  the monolithic solve, with the tutorials' Tcoupled dictionary verbatim
  (nested preconditioner dictionary) on two region matrices coupled by one
  regionCouple patch pair.

Interfaces reach the adapter as foam has them: a master and a slave
regionCouple patch (faceCells) with their GGI interpolator (masterAddr /
masterWeights, slaveAddr / slaveWeights over patch faces); the adapter
builds the library's interface description from them."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import oracle_matrix
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu

# ShellAndTubeHeatExchanger/system/solid/fvSolution, the coupled temperature
# solve's entry
TCOUPLED = """
    Tcoupled
    {
        solver           BiCGStab;
        
        preconditioner      
        {                   
            preconditioner  Cholesky;
        }

        tolerance        1e-15;
        relTol           0;

        minIter          0;
        maxIter          200;
    }
"""


def patch_pair(s, n_a):
    """The interface rows of an LDU system as a regionCouple patch pair: the
    first n_a rows are patch A (master), the rest patch B (slave); a row's
    sources (cells on the other side) become faces of the other patch.
    Returns (cellsA, cellsB, (ptr, addr, w) of A from B, (...) of B from A,
    bouA, bouB)."""
    f = s.iface
    cells = np.asarray(f["cells"], np.int64)
    ca, cb = cells[:n_a], cells[n_a:]
    face_of = [{int(c): i for i, c in enumerate(cb)}, {int(c): i for i, c in enumerate(ca)}]
    csr = []
    for side, rows in ((0, range(0, n_a)), (1, range(n_a, len(cells)))):
        ptr, addr, w = [0], [], []
        for r in rows:
            for k in range(f["ptr"][r], f["ptr"][r + 1]):
                addr.append(face_of[side][int(f["src"][k])])
                w.append(f["w"][k])
            ptr.append(len(addr))
        csr.append((np.array(ptr, np.int32), np.array(addr, np.int32), np.array(w, np.float64)))
    bou = np.asarray(f["bou"], np.float64)
    return ca, cb, csr[0], csr[1], bou[:n_a], bou[n_a:]


def _region(fh, n, lower, upper, diag, upper_c, lower_c, b, x0, sf=None):
    np.array([n, len(lower), 0 if lower_c is None else 1], np.int32).tofile(fh)
    np.asarray(lower, np.int32).tofile(fh)
    np.asarray(upper, np.int32).tofile(fh)
    for a in (diag, upper_c) + (() if lower_c is None else (lower_c,)) + (b, x0):
        np.asarray(a, np.float64).tofile(fh)
    # the fvMesh's face area vectors (none: the matrix has bare addressing)
    np.array([0 if sf is None else len(lower)], np.int32).tofile(fh)
    if sf is not None:
        np.ascontiguousarray(sf, np.float64).tofile(fh)


def _patches(fh, ra, rb, pair, off_a=0, off_b=0):
    ca, cb, (pa, aa, wa), (pb, ab, wb), bou_a, bou_b = pair
    np.array([2, ra, rb, len(ca), len(cb)], np.int32).tofile(fh)
    (np.asarray(ca) - off_a).astype(np.int32).tofile(fh)
    (np.asarray(cb) - off_b).astype(np.int32).tofile(fh)
    for p, a, w in ((pa, aa, wa), (pb, ab, wb)):
        p.tofile(fh)
        a.tofile(fh)
        w.tofile(fh)
    bou_a.tofile(fh)
    bou_b.tofile(fh)


def n_iface_a(s):
    """Rows of patch A in a generated system's interface (the first side)."""
    return int(s.meta.get("n_iface", s.meta.get("n_ifa", 0)))


def write_system(path, s, sf=None):
    """One matrix (its interfaces a patch pair inside it); sf: the face area
    vectors of its fvMesh."""
    with open(path, "wb") as fh:
        np.array([1], np.int32).tofile(fh)
        _region(fh, s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, sf)
        if s.iface is None:
            np.array([0], np.int32).tofile(fh)
        else:
            _patches(fh, 0, 0, patch_pair(s, n_iface_a(s)))


def write_regions(path, s, n0):
    """Two region matrices: cells [0, n0) and [n0, n) of a system whose only
    coupling between them is its interface rows (patch A in region 0)."""
    lower, upper = np.asarray(s.lower), np.asarray(s.upper)
    in0 = upper < n0
    assert np.all(lower[~in0] >= n0), "a face joins the regions"
    assert np.all(in0[:-1] >= in0[1:]), "region 0's faces first"
    lc = s.lower_c
    with open(path, "wb") as fh:
        np.array([2], np.int32).tofile(fh)
        for sel, off, lo_c, hi_c in ((in0, 0, 0, n0), (~in0, n0, n0, s.n)):
            _region(fh, hi_c - lo_c, lower[sel] - off, upper[sel] - off, s.diag[lo_c:hi_c], s.upper_c[sel],
                    None if lc is None else lc[sel], s.b[lo_c:hi_c], s.x0[lo_c:hi_c])
        pair = patch_pair(s, n_iface_a(s))
        assert np.all(pair[0] < n0) and np.all(pair[1] >= n0)
        _patches(fh, 0, 1, pair, 0, n0)


def run(mrg, tmp_path, s, solver, pc, tol, extra=(), sf=None):
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf, outf = str(tmp_path / "sys.bin"), str(tmp_path / "x.bin")
    write_system(sysf, s, sf)
    r = subprocess.run([exe, sysf, solver, pc, repr(tol), outf, *extra], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(outf, np.float64), json.loads(r.stdout.strip().splitlines()[-1])


def run_coupled(mrg, tmp_path, s, n0, dict_text, entry="Tcoupled"):
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf, outf, dictf = str(tmp_path / "sys2.bin"), str(tmp_path / "x2.bin"), str(tmp_path / "fvSolution")
    write_regions(sysf, s, n0)
    with open(dictf, "w") as fh:
        fh.write(dict_text)
    r = subprocess.run([exe, "--dict", dictf, entry, sysf, outf], capture_output=True, text=True, timeout=300)
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
    """gpuGAMG with the tutorials' words (smoother GaussSeidel, agglomerator
    faceAreaPair on the fvMesh's Sf, nCellsInCoarsestLevel 10, mergeLevels
    1, scaleCorrection true, nPreSweeps 0, nPostSweeps 0 / 2), and with
    algebraicPair on a matrix without a mesh."""
    import gamg_oracle as G
    s = cases.cht_system(12, 11, 6, 4, seed=9, form="global", k_range=(0.1, 50.0))
    sf = cases.face_area_vectors(s)
    g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, weights=G.face_area_weights(sf))
    for post in (2, 0):
        x, perf = run(mrg, tmp_path, s, "gpuGAMG", "none", 1e-8,
                      ("smoother=GaussSeidel", "nCellsInCoarsestLevel=10", "agglomerator=faceAreaPair",
                       "mergeLevels=1", "cacheAgglomeration=true", "scaleCorrection=true", "nPreSweeps=0",
                       f"nPostSweeps={post}", "nFinestSweeps=2", "directSolveCoarsest=false"), sf=sf)
        xm, pm = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-8,
                         max_iter=5000, n_post=post)
        assert perf["solver"] == "gpuGAMG" and perf["converged"] == 1
        assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)
    t = cases.convdiff_system(12, 11, 10, seed=9)
    x, perf = run(mrg, tmp_path, t, "gpuGAMG", "none", 1e-8, ("agglomerator=algebraicPair",))
    g = G.Gamg(t.n, t.lower, t.upper, t.diag, t.upper_c, t.lower_c)
    xm, pm = g.solve(t.n, t.lower, t.upper, t.diag, t.upper_c, t.lower_c, t.b, t.x0, tol=1e-8, max_iter=5000)
    assert perf["converged"] == 1 and perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)
    # foam's default agglomerator is faceAreaPair: without a mesh it is an error
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    write_system(str(tmp_path / "t.bin"), t)
    r = subprocess.run([exe, str(tmp_path / "t.bin"), "gpuGAMG", "none", "1e-8", str(tmp_path / "o.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "faceAreaPair" in r.stdout


def test_unknown_solver_is_fatal(mrg, tmp_path):
    s = cases.cht_system(6, 6, 6, 3)
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf = str(tmp_path / "sys.bin")
    write_system(sysf, s)
    r = subprocess.run([exe, sysf, "gpuAMGX", "none", "1e-6", str(tmp_path / "x.bin")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "Unknown symmetric matrix solver gpuAMGX" in r.stdout


COUPLED = {
    # conformal CHT: solid below (region 0) and fluid (region 1), DIC
    "cht": lambda: (cases.cht_system(16, 14, 12, 7, seed=1, form="coupled", k_range=(0.1, 50.0)), "DIC"),
    # the non-conformal convection-diffusion pair, 3:2 GGI, DILU
    "c3": lambda: (__import__("c3_case").c3(scale=4, seed=1, permute=False)[0], "DILU"),
}


def _region0_cells(s):
    return int(s.meta["n_solid"]) if "n_solid" in s.meta else int(s.meta["nA"])


@pytest.mark.parametrize("case", list(COUPLED))
def test_coupled_solver_tcoupled_dictionary(mrg, oracle_mod, tmp_path, case):
    """coupledLduSolver::New with the tutorials' Tcoupled entry (BiCGStab,
    nested Cholesky preconditioner, tolerance 1e-15, maxIter 200), mapped to
    gpuBiCGStab: two region matrices and one regionCouple patch pair, solved
    as one system.  Bit-identical to the oracle's GPU-order mirror of the
    coupled form (one LDU with interface rows); within 1e-10 of its foam-order
    solve (at a 1e-15 tolerance the last iterations are rounding-bound, so the
    iteration count may differ from foam order's by a few)."""
    s, pc = COUPLED[case]()
    text = TCOUPLED.replace("BiCGStab;", "gpuBiCGStab;")
    x, perf = run_coupled(mrg, tmp_path, s, _region0_cells(s), text)
    A = oracle_matrix(oracle_mod, s)
    xm, pm = A.solve_mirror(s.b, s.x0, "BiCGStab", pc, tol=1e-15, max_iter=200)
    xo, po = A.solve(s.b, s.x0, "BiCGStab", pc, tol=1e-15, max_iter=200)
    assert perf["solver"] == "gpuBiCGStab"
    assert perf["n_iter"] == pm["n_iter"] and np.array_equal(x, xm)
    assert perf["converged"] == int(pm["converged"])
    assert abs(perf["initial_residual"] - po["initial_residual"]) <= 1e-10 * po["initial_residual"]
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    assert abs(perf["n_iter"] - po["n_iter"]) <= max(3, po["n_iter"] // 10)


def test_coupled_equals_single_matrix_form(mrg, tmp_path):
    """The coupled table's solve of two region matrices gives the bits of the
    lduMatrix::solver table's solve of the same system as one matrix with
    its interface pair inside it (gpuPCG + DIC, and the mixed form)."""
    s = cases.cht_system(12, 10, 8, 6, seed=5, form="coupled", k_range=(0.1, 50.0))
    for solver in ("gpuPCG", "gpuMixedPCG"):
        text = ("Tcoupled { solver %s; preconditioner { preconditioner DIC; } tolerance 1e-9; relTol 0; "
                "maxIter 500; }" % solver)
        xc, pc_ = run_coupled(mrg, tmp_path, s, _region0_cells(s), text)
        xs, ps = run(mrg, tmp_path, s, solver, "DIC", 1e-9, ("maxIter=500",))
        assert np.array_equal(xc, xs) and pc_["n_iter"] == ps["n_iter"], solver


def test_coupled_dictionary_errors(mrg, tmp_path):
    """Unknown coupled solver names are fatal, as foam's table lookup is; a
    preconditioner the library does not have is fatal too."""
    s = cases.cht_system(6, 6, 4, 3, seed=2, form="coupled")
    from multiregionfoam_gb300 import _build
    exe = _build.build_adapter()
    sysf, dictf = str(tmp_path / "s.bin"), str(tmp_path / "fvSolution")
    write_regions(sysf, s, _region0_cells(s))
    for text, msg in (("Tcoupled { solver BiCGStab; }", "Unknown symmetric coupled matrix solver BiCGStab"),
                      ("Tcoupled { solver gpuBiCGStab; preconditioner { preconditioner AMG; } }",
                       "unsupported preconditioner AMG")):
        with open(dictf, "w") as fh:
            fh.write(text)
        r = subprocess.run([exe, "--dict", dictf, "Tcoupled", sysf, str(tmp_path / "x.bin")], capture_output=True,
                           text=True, timeout=60)
        assert r.returncode == 1 and msg in r.stdout, r.stdout
