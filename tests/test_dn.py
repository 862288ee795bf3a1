"""Partitioned Dirichlet-Neumann coupling: oracle restatement (CPU).

The reference's premise (multiRegionFoam tutorials compare monolithic and
partitioned runs) pins the restatement: the DN loop of oracle/dn_oracle.py,
with direct region solves, must converge to the monolithic solution of the
same problem.  Plus known answers of the relaxation models and of
dnaControl::criteriaSatisfied.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from multiregionfoam_gb300 import cases

import dn_oracle as D


def _csr(s):
    n = s.n
    lo = s.lower_c if s.lower_c is not None else s.upper_c
    A = sp.coo_matrix((np.concatenate([s.diag, s.upper_c, lo]),
                       (np.concatenate([np.arange(n), s.lower, s.upper]),
                        np.concatenate([np.arange(n), s.upper, s.lower]))), shape=(n, n)).tocsc()
    return spla.factorized(A)


def _interface(P, model, relax, model_b=None, relax_b=None):
    a, b = P["a"], P["b"]
    t_f, t_s = P["fluid"].x0, P["solid"].x0
    v0 = 0.5 * (t_f[a["face_cells"]] + t_s[b["face_cells"]])
    return D.DnInterface((a["ptr"], a["addr"], a["w"]), (b["ptr"], b["addr"], b["w"]),
                         a["face_cells"], a["delta"], a["k"], a["area"],
                         b["face_cells"], b["delta"], b["k"], b["area"],
                         K=1.0, flux_jump=0.0, model=model, relax=relax,
                         value_a0=v0, grad_b0=np.zeros(len(b["face_cells"])), model_b=model_b, relax_b=relax_b)


def dn_loop(P, model=1, relax=0.75, tol=1e-11, max_corr=60, model_b=None, relax_b=None):
    solve_f, solve_s = _csr(P["fluid"]), _csr(P["solid"])
    I = _interface(P, model, relax, model_b, relax_b)
    t_f, t_s = P["fluid"].x0.copy(), P["solid"].x0.copy()
    hist = []
    for corr in range(1, max_corr + 1):
        I.update_a(t_s)
        t_f = solve_f(I.rhs_a(P["fluid"].b))
        I.update_b(t_f)
        t_s = solve_s(I.rhs_b(P["solid"].b))
        j, f = I.residuals(t_f, t_s)
        hist.append((j, f))
        if D.criteria_satisfied(corr, j, f, tol, tol):
            return t_f, t_s, corr, hist
    return t_f, t_s, max_corr, hist


@pytest.mark.parametrize("model,relax", [(1, 0.75), (0, 1.0), (2, 0.5)])
def test_dn_converges_to_monolithic(model, relax):
    P = cases.partitioned_cht(10, 9, 8, 5, seed=2)
    t_f, t_s, corr, hist = dn_loop(P, model, relax)
    assert corr < 60, hist[-3:]
    mono = P["mono"]
    x = _csr(mono)(mono.b)
    ns = P["solid"].n
    err = max(np.abs(t_s - x[:ns]).max(), np.abs(t_f - x[ns:]).max()) / np.abs(x).max()
    assert err < 1e-9, err


def test_dn_converges_with_cell_conductivities():
    P = cases.partitioned_cht(9, 8, 7, 4, seed=3, k_range=(0.5, 5.0))
    t_f, t_s, corr, hist = dn_loop(P, 1, 0.5, max_corr=200)
    assert corr < 200, hist[-3:]
    mono = P["mono"]
    x = _csr(mono)(mono.b)
    ns = P["solid"].n
    assert max(np.abs(t_s - x[:ns]).max(), np.abs(t_f - x[ns:]).max()) / np.abs(x).max() < 1e-8


def test_relaxation_known_answers():
    # fixed: prev + w (cur - prev)
    r = D.Relaxation(0, 0.5, np.array([1.0, 2.0]))
    assert np.array_equal(r.relax(np.array([3.0, 2.0])), np.array([2.0, 2.0]))
    assert np.array_equal(r.relax(np.array([2.0, 4.0])), np.array([2.0, 3.0]))
    # Aitken: the first two corrector steps use the initial factor; the third
    # uses -w_prev * <r_prev, r - r_prev> / |r - r_prev|^2, |.| clipped to 1
    a = D.Relaxation(1, 0.5, np.array([0.0]))
    a.relax(np.array([2.0]))             # res 2, out 1
    a.relax(np.array([2.0]))             # res 1, out 1.5
    out = a.relax(np.array([1.5 + 0.25]))  # res 0.25: w = 0.5 * 1*(0.25-1)/(0.75^2)... |.|
    w = abs(-0.5 * (1.0 * (0.25 - 1.0)) / ((0.25 - 1.0) ** 2 + D.SMALL))
    assert a.aitken == pytest.approx(min(w, 1.0))
    assert out[0] == pytest.approx(1.5 + a.aitken * 0.25)


def test_iqnils_needs_fewer_coupling_iterations_than_aitken():
    """The tutorials' set-up: the jump (Dirichlet) patch carries the
    acceleration model, the flux patch none (fixed, relax 1)."""
    P = cases.partitioned_cht(9, 8, 7, 4, seed=3, k_range=(0.5, 5.0))
    _, _, corr_aitken, _ = dn_loop(P, 1, 0.75, max_corr=200, model_b=0, relax_b=1.0)
    t_f, t_s, corr_iqn, hist = dn_loop(P, 2, 0.75, max_corr=200, model_b=0, relax_b=1.0)
    assert corr_iqn < corr_aitken, (corr_iqn, corr_aitken)
    mono = P["mono"]
    x = _csr(mono)(mono.b)
    ns = P["solid"].n
    assert max(np.abs(t_s - x[:ns]).max(), np.abs(t_f - x[ns:]).max()) / np.abs(x).max() < 1e-8


@pytest.mark.parametrize("order", ["foam", "gpu"])
def test_iqnils_known_answers(order):
    """On a linear fixed-point map x -> A x + c of dimension m the
    least-squares update is exact once m residual differences are held: the
    IQN-ILS iterates reach the fixed point in m + 3 corrector steps (two to
    set the references, m to collect the columns, one exact step), far
    sooner than relaxation; the first two steps are plain relaxation."""
    rng = np.random.default_rng(1)
    m = 4
    A = 0.6 * rng.uniform(-1.0, 1.0, (m, m)) / m
    c = rng.uniform(-1.0, 1.0, m)
    x_star = np.linalg.solve(np.eye(m) - A, c)
    r = D.Relaxation(2, 0.3, np.zeros(m), order=order)
    x = np.zeros(m)
    out1 = r.relax(A @ x + c)
    assert np.array_equal(out1, 0.3 * (A @ x + c))          # corr 1: prev + relax res
    x = out1
    for k in range(m + 2):
        x = r.relax(A @ x + c)
    assert np.abs(x - x_star).max() < 1e-12
    assert len(r.V) == m + 1 and r.T == [0] * (m + 1)
    # a new time step with couplingReuse 0 drops the old columns, with 1 keeps them
    r.new_time_step()
    r.relax(A @ x + c)
    assert r.V == [] and r.T == []
    k = D.Relaxation(2, 0.3, np.zeros(m), reuse=1, order=order)
    y = np.zeros(m)
    for _ in range(4):
        y = k.relax(A @ y + c)
    k.new_time_step()
    k.relax(A @ y + c)
    assert len(k.V) == 2 and k.T == [0, 0]


def test_iqnils_mode_limit():
    """At most IQN_MODES columns per field: the oldest goes first."""
    r = D.Relaxation(2, 0.5, np.zeros(3))
    rng = np.random.default_rng(2)
    for _ in range(D.IQN_MODES + 6):
        r.relax(rng.uniform(-1.0, 1.0, 3))
    assert len(r.V) == D.IQN_MODES


def test_criteria():
    assert not D.criteria_satisfied(1, 0.0, 0.0, 1e-7, 1e-7)
    assert D.criteria_satisfied(2, 1e-8, 1e-8, 1e-7, 1e-7)
    assert not D.criteria_satisfied(5, 1e-6, 1e-8, 1e-7, 1e-7)
