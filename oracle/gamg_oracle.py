"""CPU restatement of the GAMG solver the GPU library implements (test
infrastructure only: tests import it to check the GPU solver,
MRG_SOLVER_GAMG in multiregionfoam_gb300/csrc/gamg.cu).

foam-extend's GAMG (the tutorials' fluid p / T solver, e.g.
tutorials/conjugateHeatTransfer/flowOverHeatedPlate/system/fluid/fvSolution:
GAMG, smoother GaussSeidel, nCellsInCoarsestLevel 10, mergeLevels 1,
cacheAgglomeration true) is external to the reference, so this is the
standard geometric-algebraic multigrid it names, restated with foam's
controls; parity with foam-extend is unpinned.

  agglomeration   pairwise on face weights |upper| + |lower|, cells visited
                  in order: an unpaired cell pairs with its unpaired
                  neighbour of largest weight (the first such face in face
                  order on ties); a cell with no unpaired neighbour joins the
                  group of its neighbour of largest weight (or stays alone);
                  coarse cells numbered as created; levels are added while a
                  level has more than nCellsInCoarsestLevel cells and the
                  last pairing reduced it, computed once from the first
                  matrix (cacheAgglomeration)
  coarse matrix   diag_C = sum of the members' diagonals (ascending cell),
                  then of upper + lower of the faces inside C (ascending
                  face); a coarse face (C < D, sorted) sums its fine faces in
                  face order, a face whose owner lies in D adding lower to
                  the coarse upper and upper to the coarse lower
  V-cycle         corrections start at zero: the finest residual is
                  restricted (sum over members) level by level; the coarsest
                  level is solved directly (dense LU without pivoting); going
                  up, each level's correction is the prolonged coarser one
                  smoothed by nPostSweeps Gauss-Seidel sweeps; the finest x
                  gains the prolonged correction and nFinestSweeps sweeps
  iteration       one V-cycle, then the residual and foam's convergence
                  test; minIter / maxIter as the other solvers
"""
from __future__ import annotations

import numpy as np

import oracle as O


def agglomerate(n, lower, upper, w):
    """(agg, n_coarse) of one level."""
    nf = len(lower)
    start = np.zeros(n + 1, np.int64)
    np.add.at(start, lower + 1, 1)
    np.add.at(start, upper + 1, 1)
    start = np.cumsum(start)
    adj = np.empty(2 * nf, np.int64)
    fill = start[:-1].copy()
    for f in range(nf):                      # faces ascending for every cell
        for c in (lower[f], upper[f]):
            adj[fill[c]] = f
            fill[c] += 1
    agg = np.full(n, -1, np.int64)
    nc = 0
    for c in range(n):
        if agg[c] >= 0:
            continue
        best, bw = -1, -np.inf
        for f in adj[start[c]:start[c + 1]]:
            o = upper[f] if lower[f] == c else lower[f]
            if agg[o] < 0 and w[f] > bw:
                best, bw = o, w[f]
        if best >= 0:
            agg[c] = agg[best] = nc
            nc += 1
            continue
        best, bw = -1, -np.inf
        for f in adj[start[c]:start[c + 1]]:
            o = upper[f] if lower[f] == c else lower[f]
            if w[f] > bw:
                best, bw = o, w[f]
        if best >= 0:
            agg[c] = agg[best]
        else:
            agg[c] = nc
            nc += 1
    return agg, nc


def coarse_addressing(agg, lower, upper):
    """Coarse faces (sorted owner, neighbour) with their fine faces and
    flips, and each coarse cell's interior fine faces."""
    a, b = agg[lower], agg[upper]
    keys = {}
    interior = {}
    for f in range(len(lower)):
        if a[f] == b[f]:
            interior.setdefault(int(a[f]), []).append(f)
        else:
            k = (int(min(a[f], b[f])), int(max(a[f], b[f])))
            keys.setdefault(k, []).append((f, bool(a[f] > b[f])))
    faces = sorted(keys)
    return faces, [keys[k] for k in faces], interior


def coarse_coeffs(level, diag, upper_c, lower_c):
    n_c = level["n"]
    sym = lower_c is None
    lo = upper_c if sym else lower_c
    dc = np.zeros(n_c)
    for C in range(n_c):
        acc = 0.0
        for i in level["members"][C]:
            acc = acc + diag[i]
        for f in level["interior"].get(C, []):
            acc = acc + upper_c[f]
            acc = acc + lo[f]
        dc[C] = acc
    uc = np.zeros(len(level["faces"]))
    lc = np.zeros(len(level["faces"]))
    for F, fl in enumerate(level["face_members"]):
        u = 0.0
        l_ = 0.0
        for f, flip in fl:
            u = u + (lo[f] if flip else upper_c[f])
            l_ = l_ + (upper_c[f] if flip else lo[f])
        uc[F], lc[F] = u, l_
    return dc, uc, (None if sym else lc)


def dense_lu(n, lower, upper, diag, upper_c, lower_c):
    M = np.zeros((n, n))
    lo = upper_c if lower_c is None else lower_c
    for i in range(n):
        M[i, i] = diag[i]
    for f in range(len(lower)):
        M[lower[f], upper[f]] = upper_c[f]
        M[upper[f], lower[f]] = lo[f]
    for k in range(n):
        for i in range(k + 1, n):
            M[i, k] = M[i, k] / M[k, k]
            for j in range(k + 1, n):
                M[i, j] = M[i, j] - M[i, k] * M[k, j]
    return M


def dense_solve(M, b):
    n = len(b)
    y = np.zeros(n)
    for i in range(n):
        acc = b[i]
        for j in range(i):
            acc = acc - M[i, j] * y[j]
        y[i] = acc
    x = np.zeros(n)
    for i in range(n - 1, -1, -1):
        acc = y[i]
        for j in range(i + 1, n):
            acc = acc - M[i, j] * x[j]
        x[i] = acc / M[i, i]
    return x


class Gamg:
    """Hierarchy (cached from the first matrix) and solver."""

    def __init__(self, n, lower, upper, diag, upper_c, lower_c=None, n_coarsest=10, max_levels=50):
        self.levels = []          # level l >= 1: dict n, lower, upper, agg (fine -> coarse), members, ...
        n_l, lo_l, up_l = n, np.asarray(lower, np.int64), np.asarray(upper, np.int64)
        d_l, u_l, l_l = np.asarray(diag, np.float64), np.asarray(upper_c, np.float64), \
            (None if lower_c is None else np.asarray(lower_c, np.float64))
        while n_l > n_coarsest and len(self.levels) + 1 < max_levels:
            w = np.abs(u_l) + np.abs(u_l if l_l is None else l_l)
            agg, nc = agglomerate(n_l, lo_l, up_l, w)
            if nc >= n_l:
                break
            faces, fm, interior = coarse_addressing(agg, lo_l, up_l)
            members = [[] for _ in range(nc)]
            for i in range(n_l):
                members[agg[i]].append(i)
            lvl = {"n": nc, "agg": agg, "members": members, "faces": faces, "face_members": fm,
                   "interior": interior,
                   "lower": np.array([f[0] for f in faces], np.int32),
                   "upper": np.array([f[1] for f in faces], np.int32)}
            d_l, u_l, l_l = coarse_coeffs(lvl, d_l, u_l, l_l)
            self.levels.append(lvl)
            n_l, lo_l, up_l = nc, lvl["lower"].astype(np.int64), lvl["upper"].astype(np.int64)

    def solve(self, n, lower, upper, diag, upper_c, lower_c, b, x0, tol=1e-8, rel_tol=0.0, min_iter=0,
              max_iter=1000, n_post=2, n_finest=2, mode="mirror"):
        A0 = O.OracleMatrix(n, lower, upper, diag, upper_c, lower_c)
        mats, coef = [A0], (np.asarray(diag, np.float64), np.asarray(upper_c, np.float64),
                            None if lower_c is None else np.asarray(lower_c, np.float64))
        for lvl in self.levels:
            coef = coarse_coeffs(lvl, *coef)
            mats.append(O.OracleMatrix(lvl["n"], lvl["lower"], lvl["upper"], *coef))
        L = len(mats)
        top = mats[-1]
        M = dense_lu(top.n, top.lower, top.upper, top.diag, top.upper_c, top.lower_c)
        fused = mode != "literal"
        b = np.asarray(b, np.float64)
        x = np.array(x0, np.float64, copy=True)

        def residual():
            if mode == "mirror":
                return A0.mirror_residual(b, x)
            r = A0.foam_residual(b, x, fused)
            return r, float(np.sum(np.abs(r)))

        nfac = A0.mirror_norm_factor(b, x) if mode == "mirror" else A0.norm_factor(x, b)
        r, s = residual()
        perf = {"initial_residual": s / nfac, "n_iter": 0, "converged": False}
        perf["final_residual"] = perf["initial_residual"]

        def conv():
            res = perf["final_residual"]
            return res < tol or (rel_tol > 1e-20 and res < rel_tol * perf["initial_residual"])

        def restrict(lvl, v):
            out = np.zeros(lvl["n"])
            for C, mem in enumerate(lvl["members"]):
                acc = 0.0
                for i in mem:
                    acc = acc + v[i]
                out[C] = acc
            return out

        perf["converged"] = conv()
        if min_iter > 0 or not perf["converged"]:
            while True:
                src = [None] * L
                v = r
                for l in range(1, L):
                    v = restrict(self.levels[l - 1], v)
                    src[l] = v
                if L == 1:
                    c = dense_solve(M, r)
                    x = x + c
                else:
                    c = dense_solve(M, src[L - 1])
                    for l in range(L - 2, 0, -1):
                        c = np.array(c[self.levels[l]["agg"]], copy=True)   # prolong (copy)
                        for _ in range(n_post):
                            mats[l].gs_sweep(src[l], c, fused)
                    x = x + c[self.levels[0]["agg"]]
                for _ in range(n_finest):
                    mats[0].gs_sweep(b, x, fused)
                r, s = residual()
                perf["final_residual"] = s / nfac
                perf["n_iter"] += 1
                perf["converged"] = conv()
                if not ((perf["n_iter"] < max_iter and not perf["converged"]) or perf["n_iter"] < min_iter):
                    break
        return x, perf
