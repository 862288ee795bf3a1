"""CPU restatement of the GAMG solver the GPU library implements (test
infrastructure only: tests import it to check the GPU solver,
MRG_SOLVER_GAMG in multiregionfoam_gb300/csrc/gamg.cu).

foam-extend's GAMG (the tutorials' fluid p / T solver, e.g.
tutorials/conjugateHeatTransfer/flowOverHeatedPlate/system/fluid/fvSolution:
GAMG, smoother GaussSeidel, agglomerator faceAreaPair, mergeLevels 1,
nCellsInCoarsestLevel 10, cacheAgglomeration true; ShellAndTubeHeat
Exchanger/system/solid/fvSolution adds scaleCorrection true, nPreSweeps 0,
directSolveCoarsest false) is external to the reference.  This restates the
published algorithm of foam's GAMG family (pairGAMGAgglomeration,
GAMGAgglomeration::agglomerateLduAddressing, GAMGSolver's matrix
agglomeration, V-cycle and scale()) with its controls; parity with a
foam-extend build is unpinned.

  face weights    faceAreaPair: |cmptMultiply(Sf / sqrt(|Sf|), (1, 1.01,
                  1.02))| of the finest faces; algebraicPair: |upper| of the
                  finest matrix; a coarser level's weights are its fine
                  faces' weights summed (fine face order)
  pairing         cells in order; a cell's faces are those where it is the
                  upper cell (face order), then those where it is the lower
                  one; an ungrouped cell pairs with the ungrouped neighbour
                  across its face of largest weight (strictly larger wins);
                  with no ungrouped neighbour it joins the group across its
                  face of largest weight; cells left alone become groups of
                  their own after the pass; finally the numbering is
                  reversed (c -> nCoarse - 1 - c)
  levels          a level is kept while it has at least nCellsInCoarsest
                  Level cells (and fewer than its finer level)
  coarse faces    fine faces between two groups, in fine face order, make a
                  face per (owner, neighbour) pair in order of first
                  appearance; faces are numbered by owner, then by that
                  order (not sorted by neighbour)
  coefficients    diag = the members' diagonals summed in fine cell order,
                  then per interior fine face (fine face order) + (upper +
                  lower), symmetric: + 2 upper; coarse upper / lower sum
                  their fine faces in fine face order, swapped for a fine
                  face whose lower cell lies in the coarse upper cell
  V-cycle         the finest residual restricted level by level (sums over
                  members); the coarsest solved directly (dense LU, no
                  pivoting); going up, each level's correction is the
                  prolonged coarser one, scaled (scaleCorrection, on every
                  level but the one below the coarsest), then smoothed by
                  min(nPostSweeps + postSweepsLevelMultiplier * l,
                  maxPostSweeps) Gauss-Seidel sweeps (l = 0 the first
                  coarse level); the finest correction is prolonged, scaled,
                  added to x, then nFinestSweeps sweeps of x
  scale           with Af = A f:  sf = (s . f) / stabilise(Af . f, 1e-300),
                  f = sf f + (s - sf Af) / diag
  iteration       one V-cycle, then the residual and foam's convergence
                  test; minIter / maxIter as the other solvers

Modes: "literal" sums sequentially (a serial foam run), "mirror" repeats
the GPU's arithmetic and reduction order (bit-identical to the GPU)."""
from __future__ import annotations

import numpy as np

import oracle as O

GREAT = 1.0e15
VSMALL = 1.0e-300


def face_area_weights(sf):
    """faceAreaPair weights of the finest faces from their area vectors Sf
    ([nf, 3]): |cmptMultiply(Sf / sqrt(|Sf|), (1, 1.01, 1.02))|."""
    sf = np.asarray(sf, np.float64)
    mag = np.sqrt(sf[:, 0] * sf[:, 0] + sf[:, 1] * sf[:, 1] + sf[:, 2] * sf[:, 2])
    root = np.sqrt(mag)
    x = sf[:, 0] / root * 1.0
    y = sf[:, 1] / root * 1.01
    z = sf[:, 2] / root * 1.02
    return np.sqrt(x * x + y * y + z * z)


def cell_faces(n, lower, upper):
    """Each cell's faces: those where it is the upper cell (face order),
    then those where it is the lower cell (face order)."""
    nf = len(lower)
    cnt = np.zeros(n + 1, np.int64)
    np.add.at(cnt, np.asarray(upper, np.int64) + 1, 1)
    np.add.at(cnt, np.asarray(lower, np.int64) + 1, 1)
    start = np.cumsum(cnt)
    faces = np.empty(2 * nf, np.int64)
    fill = start[:-1].copy()
    for f in range(nf):
        u = upper[f]
        faces[fill[u]] = f
        fill[u] += 1
    for f in range(nf):
        lo = lower[f]
        faces[fill[lo]] = f
        fill[lo] += 1
    return start, faces


def agglomerate(n, lower, upper, w):
    """(agg, n_coarse) of one level: foam's pairwise agglomeration."""
    start, faces = cell_faces(n, lower, upper)
    agg = np.full(n, -1, np.int64)
    nc = 0
    for c in range(n):
        if agg[c] >= 0:
            continue
        match, mw = -1, -GREAT
        for f in faces[start[c]:start[c + 1]]:
            if agg[upper[f]] < 0 and agg[lower[f]] < 0 and w[f] > mw:
                match, mw = f, w[f]
        if match >= 0:
            agg[upper[match]] = nc
            agg[lower[match]] = nc
            nc += 1
            continue
        match, mw = -1, -GREAT
        for f in faces[start[c]:start[c + 1]]:
            if w[f] > mw:
                match, mw = f, w[f]
        if match >= 0:
            agg[c] = max(agg[upper[match]], agg[lower[match]])
    for c in range(n):
        if agg[c] < 0:
            agg[c] = nc
            nc += 1
    return (nc - 1) - agg, nc


def agglomerate_addressing(agg, nc, lower, upper):
    """Coarse (lower, upper) addressing and the face restriction map
    (>= 0: coarse face; < 0: -(coarse cell + 1) for a face inside a cell)."""
    nf = len(lower)
    own_faces = [[] for _ in range(nc)]
    nbr = []
    restrict = np.empty(nf, np.int64)
    for f in range(nf):
        ru, rl = int(agg[upper[f]]), int(agg[lower[f]])
        if ru == rl:
            restrict[f] = -(ru + 1)
            continue
        own, nei = (rl, ru) if ru > rl else (ru, rl)
        for cf in own_faces[own]:
            if nbr[cf] == nei:
                restrict[f] = cf
                break
        else:
            cf = len(nbr)
            nbr.append(nei)
            own_faces[own].append(cf)
            restrict[f] = cf
    fmap = np.empty(len(nbr), np.int64)
    lo_c = np.empty(len(nbr), np.int32)
    up_c = np.empty(len(nbr), np.int32)
    k = 0
    for c in range(nc):
        for cf in own_faces[c]:
            lo_c[k], up_c[k] = c, nbr[cf]
            fmap[cf] = k
            k += 1
    pos = restrict >= 0
    restrict[pos] = fmap[restrict[pos]]
    return lo_c, up_c, restrict


def restrict_faces(restrict, nfc, w):
    out = np.zeros(nfc)
    for f in range(len(restrict)):
        cf = restrict[f]
        if cf >= 0:
            out[cf] = out[cf] + w[f]
    return out


def coarse_coeffs(level, diag, up, lo):
    """Coarse diag / upper / lower (lower None: symmetric)."""
    agg, restrict = level["agg"], level["restrict"]
    cl = level["lower"]
    dc = np.zeros(level["n"])
    for i in range(len(agg)):
        dc[agg[i]] = dc[agg[i]] + diag[i]
    nfc = len(cl)
    uc = np.zeros(nfc)
    lc = None if lo is None else np.zeros(nfc)
    fine_lower = level["fine_lower"]
    for f in range(len(restrict)):
        cf = restrict[f]
        if cf >= 0:
            if lo is None:
                uc[cf] = uc[cf] + up[f]
            elif cl[cf] == agg[fine_lower[f]]:
                uc[cf] = uc[cf] + up[f]
                lc[cf] = lc[cf] + lo[f]
            else:
                uc[cf] = uc[cf] + lo[f]
                lc[cf] = lc[cf] + up[f]
        else:
            C = -1 - cf
            dc[C] = dc[C] + (2.0 * up[f] if lo is None else up[f] + lo[f])
    return dc, uc, lc


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


def stabilise(s, small):
    return s + small if s >= 0 else s - small


class Gamg:
    """Hierarchy (cached from the first matrix) and solver.

    weights: the finest faces' agglomeration weights (face_area_weights for
    faceAreaPair); None: algebraicPair, |upper| of the given matrix."""

    def __init__(self, n, lower, upper, diag, upper_c, lower_c=None, n_coarsest=10, max_levels=50, weights=None):
        self.levels = []   # coarse level l >= 1: n, agg (finer -> this), restrict, lower, upper, members
        n_l = int(n)
        lo_l, up_l = np.asarray(lower, np.int64), np.asarray(upper, np.int64)
        w = np.abs(np.asarray(upper_c, np.float64)) if weights is None else np.asarray(weights, np.float64)
        while len(self.levels) < max_levels - 1:
            agg, nc = agglomerate(n_l, lo_l, up_l, w)
            if nc < n_coarsest or nc >= n_l:
                break
            lo_c, up_c, restrict = agglomerate_addressing(agg, nc, lo_l, up_l)
            members = [[] for _ in range(nc)]
            for i in range(n_l):
                members[agg[i]].append(i)
            self.levels.append({"n": nc, "agg": agg, "restrict": restrict, "lower": lo_c, "upper": up_c,
                                "members": members, "fine_lower": lo_l.copy()})
            w = restrict_faces(restrict, len(lo_c), w)
            n_l, lo_l, up_l = nc, lo_c.astype(np.int64), up_c.astype(np.int64)

    def sweeps(self, leveli, n_post, multiplier, max_post):
        return min(n_post + multiplier * leveli, max_post)

    def solve(self, n, lower, upper, diag, upper_c, lower_c, b, x0, tol=1e-8, rel_tol=0.0, min_iter=0,
              max_iter=1000, n_post=2, n_finest=2, max_post=4, multiplier=1, scale=True, mode="mirror"):
        A0 = O.OracleMatrix(n, lower, upper, diag, upper_c, lower_c)
        mats = [A0]
        coef = (np.asarray(diag, np.float64), np.asarray(upper_c, np.float64),
                None if lower_c is None else np.asarray(lower_c, np.float64))
        for lvl in self.levels:
            coef = coarse_coeffs(lvl, *coef)
            mats.append(O.OracleMatrix(lvl["n"], lvl["lower"], lvl["upper"], *coef))
        if not self.levels:
            # no level kept (the first pairing already falls below
            # nCellsInCoarsestLevel): the matrix itself is the coarsest level
            mats.append(A0)
        top_i = len(mats) - 1
        top = mats[top_i]
        M = dense_lu(top.n, top.lower, top.upper, top.diag, top.upper_c, top.lower_c)
        fused = mode != "literal"
        b = np.asarray(b, np.float64)
        x = np.array(x0, np.float64, copy=True)

        def residual():
            if mode == "mirror":
                return A0.mirror_residual(b, x)
            r = A0.foam_residual(b, x, fused)
            return r, float(np.sum(np.abs(r)))

        def dot(A, u, v):
            if mode == "mirror":
                return A.mirror_dot(u, v)
            acc = 0.0
            for i in range(len(u)):
                acc = acc + u[i] * v[i]
            return acc

        def scaled(A, f, s):
            Af = A.amul(f, fused)
            sf = dot(A, s, f) / stabilise(dot(A, Af, f), VSMALL)
            return sf * f + (s - sf * Af) / A.diag

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
                if not self.levels:
                    x = x + dense_solve(M, r)   # the whole matrix solved directly
                else:
                    src = [None] * (top_i + 1)
                    v = r
                    for l in range(1, top_i + 1):
                        v = restrict(self.levels[l - 1], v)
                        src[l] = v
                    c = dense_solve(M, src[top_i])
                    for l in range(top_i - 1, 0, -1):
                        c = np.array(c[self.levels[l]["agg"]], copy=True)   # prolong (copy)
                        if scale and l < top_i - 1:
                            c = scaled(mats[l], c, src[l])
                        for _ in range(self.sweeps(l - 1, n_post, multiplier, max_post)):
                            mats[l].gs_sweep(src[l], c, fused)
                    corr = np.array(c[self.levels[0]["agg"]], copy=True)
                    if scale:
                        corr = scaled(A0, corr, r)
                    x = x + corr
                for _ in range(n_finest):
                    A0.gs_sweep(b, x, fused)
                r, s = residual()
                perf["final_residual"] = s / nfac
                perf["n_iter"] += 1
                perf["converged"] = conv()
                if not ((perf["n_iter"] < max_iter and not perf["converged"]) or perf["n_iter"] < min_iter):
                    break
        return x, perf
