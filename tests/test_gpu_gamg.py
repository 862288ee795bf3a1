"""GAMG on the GPU (MRG_SOLVER_GAMG; foam's GAMG with the GaussSeidel
smoother, the tutorials' fluid p / T solver) against the oracle's
restatement (oracle/gamg_oracle.py): bit-identical solution, residuals and
V-cycle count in the GPU's order, within the tolerance of foam's order; the
agglomeration is cached from the first matrix (cacheAgglomeration), so a
second solve with drifted coefficients reuses it.  Both agglomerators
(algebraicPair, faceAreaPair from the mesh's face areas), scaleCorrection on
and off, and the tutorials' sweep words (nPostSweeps 0 / 2,
maxPostSweeps, postSweepsLevelMultiplier) are covered."""
import numpy as np
import pytest

import gamg_oracle as G
from conftest import gpu_mesh
from multiregionfoam_gb300 import cases

pytestmark = pytest.mark.gpu

SWEEP_KW = {"n_post_sweeps": "n_post", "n_finest_sweeps": "n_finest", "max_post_sweeps": "max_post",
            "post_sweeps_level_multiplier": "multiplier", "scale_correction": "scale"}


def check(mrg, m, g, s, tol=1e-8, **kw):
    okw = {SWEEP_KW[k]: v for k, v in kw.items() if k in SWEEP_KW}
    xm, pm = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=tol, max_iter=500,
                     mode="mirror", **okw)
    xo, po = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=tol, max_iter=500,
                     mode="literal", **okw)
    xg, pg = m.solve(s.b, s.x0, tol=tol, max_iter=500, solver="GAMG", **kw)
    assert np.array_equal(xg, xm), np.abs(xg - xm).max()
    assert (pg["initial_residual"], pg["final_residual"], pg["n_iter"], pg["converged"]) == \
        (pm["initial_residual"], pm["final_residual"], pm["n_iter"], pm["converged"])
    assert pg["converged"] and abs(pg["n_iter"] - po["n_iter"]) <= 1
    assert np.abs(xg - xo).max() <= 10 * tol * np.abs(xo).max()
    return pg


@pytest.mark.parametrize("name", ["cht", "cd"])
def test_gamg_bitexact_and_cached(mrg, ctx, oracle_mod, name):
    s = (cases.cht_system(14, 12, 10, 6, seed=1, form="global", k_range=(0.1, 50.0)) if name == "cht"
         else cases.convdiff_system(14, 13, 12, seed=2))
    m = gpu_mesh(mrg, ctx, s)
    try:
        g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
        p = check(mrg, m, g, s)
        s2 = cases.perturb_step(s, np.random.default_rng(5))      # the next time step: same agglomeration
        m.upload(s2.diag, s2.upper_c, s2.lower_c)
        check(mrg, m, g, s2)
        check(mrg, m, g, s2, n_post_sweeps=1, n_finest_sweeps=3)
        q = check(mrg, m, g, s2, scale_correction=False)
        assert q["n_iter"] > p["n_iter"]                           # scaling is what makes pairs converge
    finally:
        m.close()


def test_gamg_face_area_pair_and_sweep_words(mrg, ctx, oracle_mod):
    """faceAreaPair (the tutorials' agglomerator) from the mesh's face
    areas; the sweep words of the tutorials' dictionaries."""
    s = cases.cht_system(16, 14, 8, 8, seed=3, form="global", k_range=(0.1, 50.0))
    m = gpu_mesh(mrg, ctx, s)
    try:
        sf = cases.face_area_vectors(s)
        with pytest.raises(mrg.MrgError, match="face area"):
            m.solve(s.b, s.x0, solver="GAMG", agglomerator="faceAreaPair")
        m.set_face_areas(sf)
        g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, weights=G.face_area_weights(sf))
        ga = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c)
        assert any(not np.array_equal(a["agg"], b["agg"]) for a, b in zip(g.levels, ga.levels))
        check(mrg, m, g, s, agglomerator="faceAreaPair")
        check(mrg, m, g, s, agglomerator="faceAreaPair", n_post_sweeps=0)           # ShellAndTube words
        check(mrg, m, g, s, agglomerator="faceAreaPair", max_post_sweeps=2, post_sweeps_level_multiplier=2)
        check(mrg, m, ga, s)                                                          # rebuilt: algebraicPair
    finally:
        m.close()


def test_gamg_coarsest_controls_and_tiny(mrg, ctx, oracle_mod):
    s = cases.convdiff_system(10, 9, 8, seed=4)
    m = gpu_mesh(mrg, ctx, s)
    g = G.Gamg(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, n_coarsest=40)
    assert g.levels[-1]["n"] >= 40
    xg, pg = m.solve(s.b, s.x0, tol=1e-9, max_iter=500, solver="GAMG", n_coarsest_cells=40)
    xm, pm = g.solve(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.b, s.x0, tol=1e-9, max_iter=500)
    assert np.array_equal(xg, xm) and pg["n_iter"] == pm["n_iter"]
    m.close()
    t = cases.convdiff_system(2, 2, 2, seed=3)                   # no level kept: a direct solve
    m = gpu_mesh(mrg, ctx, t)
    g = G.Gamg(t.n, t.lower, t.upper, t.diag, t.upper_c, t.lower_c)
    xg, pg = m.solve(t.b, t.x0, tol=1e-12, solver="GAMG")
    xm, pm = g.solve(t.n, t.lower, t.upper, t.diag, t.upper_c, t.lower_c, t.b, t.x0, tol=1e-12)
    assert np.array_equal(xg, xm) and pg["n_iter"] == pm["n_iter"] == 1
    m.close()


def test_gamg_rejects(mrg, ctx):
    s = cases.cht_system(8, 8, 6, 3, seed=1, form="coupled", k_range=(0.1, 50.0))
    m = gpu_mesh(mrg, ctx, s)
    with pytest.raises(mrg.MrgError, match="interfaces"):
        m.solve(s.b, s.x0, solver="GAMG")
    with pytest.raises(mrg.MrgError, match="FP64"):
        m.solve(s.b, s.x0, solver="GAMG", precision="mixed")
    m.close()
