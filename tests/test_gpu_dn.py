"""Partitioned Dirichlet-Neumann coupling on the device (mrg_dn_*).

1. The device coupling (jump update, flux update, right-hand sides,
   residuals, Aitken factors) follows the oracle restatement
   (oracle/dn_oracle.py) call by call, fed the same region fields; the
   element-wise arithmetic is the same IEEE sequence and only the Aitken
   and residual sums differ in order, so the tolerance is 1e-12 relative.
2. A fully device-resident DN loop -- region solves with the library,
   coupling with mrg_dn_* -- converges to the monolithic solution.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from multiregionfoam_gb300 import cases

import dn_oracle as D

pytestmark = pytest.mark.gpu
REL = 1e-12


def _factor(s):
    n = s.n
    A = sp.coo_matrix((np.concatenate([s.diag, s.upper_c, s.upper_c]),
                       (np.concatenate([np.arange(n), s.lower, s.upper]),
                        np.concatenate([np.arange(n), s.upper, s.lower]))), shape=(n, n)).tocsc()
    return spla.factorized(A)


def _close(a, b, scale=None):
    scale = np.abs(b).max() if scale is None else scale
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= REL * max(scale, 1e-300)


MODELS = {"fixed": 0, "aitken": 1, "IQNILS": 2}


@pytest.mark.parametrize("model,relax,model_b,relax_b", [("aitken", 0.6, None, None), ("fixed", 0.9, None, None),
                                                         ("IQNILS", 0.5, None, None), ("IQNILS", 0.75, "fixed", 1.0)])
def test_dn_kernels_follow_oracle(mrg, ctx, model, relax, model_b, relax_b):
    P = cases.partitioned_cht(9, 8, 7, 4, seed=4, k_range=(0.5, 5.0))
    a, b = P["a"], P["b"]
    fl, so = P["fluid"], P["solid"]
    v0 = 0.5 * (fl.x0[a["face_cells"]] + so.x0[b["face_cells"]])
    g0 = np.zeros(len(b["face_cells"]))
    O = D.DnInterface((a["ptr"], a["addr"], a["w"]), (b["ptr"], b["addr"], b["w"]), a["face_cells"], a["delta"],
                      a["k"], a["area"], b["face_cells"], b["delta"], b["k"], b["area"], K=1.0, flux_jump=0.0,
                      model=MODELS[model], relax=relax, value_a0=v0, grad_b0=g0,
                      order="gpu" if model == "IQNILS" else "foam",
                      model_b=None if model_b is None else MODELS[model_b], relax_b=relax_b)
    G = mrg.DnInterface(ctx, a, b, K=1.0, flux_jump=0.0, relax=relax, model=model, model_b=model_b, relax_b=relax_b)
    G.set_state(v0, g0)
    solve_f, solve_s = _factor(fl), _factor(so)
    t_f, t_s = fl.x0.copy(), so.x0.copy()
    d_tf, d_ts = ctx.to_device(t_f), ctx.to_device(t_s)
    d_b0f, d_b0s = ctx.to_device(fl.b), ctx.to_device(so.b)
    d_bf, d_bs = ctx.dev_alloc(8 * fl.n), ctx.dev_alloc(8 * so.n)
    try:
        for corr in range(1, 9):
            O.update_a(t_s)
            G.update_jump(d_ts)
            bf = O.rhs_a(fl.b)
            G.rhs(0, d_b0f, d_bf)
            va, gb, ai = G.state()
            assert _close(va, O.value_a)
            assert _close(ctx.from_device(d_bf, np.empty(fl.n)), bf)
            t_f = solve_f(bf)
            d_tf_new = ctx.to_device(t_f)
            ctx.dev_free(d_tf)
            d_tf = d_tf_new
            O.update_b(t_f)
            G.update_flux(d_tf)
            bs = O.rhs_b(so.b)
            G.rhs(1, d_b0s, d_bs)
            va, gb, ai = G.state()
            assert _close(gb, O.grad_b, np.abs(O.grad_b).max() + 1e-30)
            assert _close(ctx.from_device(d_bs, np.empty(so.n)), bs)
            if model == "aitken":
                assert abs(ai[0] - O.relax_a.aitken) <= 1e-12 * O.relax_a.aitken
                assert abs(ai[1] - O.relax_b.aitken) <= 1e-12 * O.relax_b.aitken
            if corr == 4:
                # a new time step: IQN-ILS drops the columns older than couplingReuse (0)
                O.new_time_step()
                G.new_time_step()
            t_s = solve_s(bs)
            d_ts_new = ctx.to_device(t_s)
            ctx.dev_free(d_ts)
            d_ts = d_ts_new
            jo, fo = O.residuals(t_f, t_s)
            jg, fg = G.residuals(d_tf, d_ts)
            assert abs(jg - jo) <= 1e-10 * max(jo, 1e-300) + 1e-300
            assert abs(fg - fo) <= 1e-10 * max(fo, 1e-300) + 1e-300
            assert mrg.dn_criteria(corr, jg, fg, 1e-9, 1e-9) == D.criteria_satisfied(corr, jo, fo, 1e-9, 1e-9)
    finally:
        for p in (d_tf, d_ts, d_b0f, d_b0s, d_bf, d_bs):
            ctx.dev_free(p)
        G.close()


_CORR = {}


@pytest.mark.parametrize("model", ["aitken", "IQNILS"])
def test_device_dn_loop_matches_monolithic(mrg, ctx, model):
    """A fully device-resident DN loop converges to the monolithic solution
    -- with the tutorials' set-up: the jump patch accelerated (relax 0.75),
    the flux patch fixed with relax 1 -- IQN-ILS in fewer coupling
    iterations than Aitken."""
    P = cases.partitioned_cht(16, 14, 10, 6, seed=5, k_range=(0.5, 5.0))
    a, b = P["a"], P["b"]
    fl, so, mono = P["fluid"], P["solid"], P["mono"]
    ctl = mrg.controls(tol=1e-13, max_iter=5000, solver="PCG", precond="DIC")
    mf = mrg.Mesh(ctx, fl.n, fl.lower, fl.upper)
    ms = mrg.Mesh(ctx, so.n, so.lower, so.upper)
    mm = mrg.Mesh(ctx, mono.n, mono.lower, mono.upper)
    G = mrg.DnInterface(ctx, a, b, relax=0.75, model=model, model_b="fixed", relax_b=1.0)
    ptrs = []
    try:
        mf.upload(fl.diag, fl.upper_c)
        ms.upload(so.diag, so.upper_c)
        mm.upload(mono.diag, mono.upper_c)
        x_mono, p_mono = mm.solve(mono.b, mono.x0, ctl)
        G.set_state(0.5 * (fl.x0[a["face_cells"]] + so.x0[b["face_cells"]]), np.zeros(len(b["face_cells"])))
        d_tf, d_ts = ctx.to_device(fl.x0), ctx.to_device(so.x0)
        d_b0f, d_b0s = ctx.to_device(fl.b), ctx.to_device(so.b)
        d_bf, d_bs = ctx.dev_alloc(8 * fl.n), ctx.dev_alloc(8 * so.n)
        ptrs = [d_tf, d_ts, d_b0f, d_b0s, d_bf, d_bs]
        done = False
        for corr in range(1, 200):
            G.update_jump(d_ts)
            G.rhs(0, d_b0f, d_bf)
            pf = mf.solve_device(d_bf, d_tf, ctl)
            G.update_flux(d_tf)
            G.rhs(1, d_b0s, d_bs)
            ps = ms.solve_device(d_bs, d_ts, ctl)
            assert pf["converged"] and ps["converged"]
            j, f = G.residuals(d_tf, d_ts)
            if mrg.dn_criteria(corr, j, f, 1e-10, 1e-10):
                done = True
                break
        assert done, (corr, j, f)
        t = np.concatenate([ctx.from_device(d_ts, np.empty(so.n)), ctx.from_device(d_tf, np.empty(fl.n))])
        assert np.abs(t - x_mono).max() <= 1e-8 * np.abs(x_mono).max()
        _CORR[model] = corr
        if model == "IQNILS" and "aitken" in _CORR:
            assert _CORR["IQNILS"] < _CORR["aitken"], _CORR
    finally:
        for p in ptrs:
            ctx.dev_free(p)
        G.close()
        for m in (mf, ms, mm):
            m.close()
