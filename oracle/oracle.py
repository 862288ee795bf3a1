"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates foam-extend 4.1's LDU solver semantics in plain C
(``ldu_oracle.c``) and GGI overlap weights (``ggi_weights.c``).  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import
this module; the product library never does.

Parity against foam-extend itself is unpinned (foam-extend is a third-party
dependency that is not available); see the header of ``ldu_oracle.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

PC_NONE, PC_DIAG, PC_DIC, PC_DILU = 0, 1, 2, 3
PRECONDITIONERS = {"none": PC_NONE, "diagonal": PC_DIAG, "DIC": PC_DIC, "DILU": PC_DILU}


def build(quiet: bool = True) -> str:
    """Compile liboracle with the committed Makefile; returns the .so path."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "libldu_oracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libldu_oracle.so")
        src = [os.path.join(_HERE, f) for f in ("ldu_oracle.c", "ggi_weights.c")]
        if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in src):
            build()
        L = C.CDLL(path)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        pldu = C.POINTER(_Ldu)
        L.or_amul.argtypes = [pldu, dp, dp, C.c_int]
        L.or_tmul.argtypes = [pldu, dp, dp, C.c_int]
        L.or_sumA.argtypes = [pldu, dp]
        L.or_norm_factor.argtypes = [pldu, dp, dp, dp]
        L.or_norm_factor.restype = C.c_double
        L.or_residual.argtypes = [pldu, dp, dp]
        L.or_residual.restype = C.c_double
        L.or_dic_factor.argtypes = [pldu, dp]
        L.or_dilu_factor.argtypes = [pldu, dp]
        L.or_precondition.argtypes = [pldu, C.c_int, dp, dp, C.c_int, C.c_int]
        for fn in (L.or_pcg, L.or_pbicg, L.or_bicgstab, L.or_solve_mirror):
            fn.argtypes = [pldu, dp, dp, C.c_double, C.c_double, C.c_int, C.c_int,
                           C.c_int, C.c_int, C.POINTER(_Perf)]
        L.or_smooth_gs.argtypes = [pldu, dp, dp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.POINTER(_Perf)]
        L.or_gs_sweep.argtypes = [pldu, dp, dp, C.c_int]
        L.or_foam_residual.argtypes = [pldu, dp, dp, dp, C.c_int]
        L.or_mirror_residual.argtypes = [pldu, dp, dp, dp]
        L.or_mirror_residual.restype = C.c_double
        L.or_mirror_norm_factor.argtypes = [pldu, dp, dp]
        L.or_mirror_norm_factor.restype = C.c_double
        L.or_mirror_dot.argtypes = [pldu, dp, dp]
        L.or_mirror_dot.restype = C.c_double
        L.or_ggi_apply.argtypes = [C.c_int, ip, ip, dp, dp, dp, C.c_int, C.c_int]
        L.gw_overlaps.argtypes = [C.c_int, ip, dp, C.c_int, ip, dp, C.c_double,
                                  C.c_long, ip, ip, dp]
        L.gw_overlaps.restype = C.c_long
        L.gw_face_areas.argtypes = [C.c_int, ip, dp, dp]
        _LIB = L
    return _LIB


class _Ldu(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nf", C.c_int),
        ("lower", C.POINTER(C.c_int32)), ("upper", C.POINTER(C.c_int32)),
        ("diag", C.POINTER(C.c_double)), ("upperc", C.POINTER(C.c_double)),
        ("lowerc", C.POINTER(C.c_double)),
        ("ni", C.c_int),
        ("iface_cells", C.POINTER(C.c_int32)), ("iface_bou", C.POINTER(C.c_double)),
        ("iface_int", C.POINTER(C.c_double)), ("iface_ptr", C.POINTER(C.c_int32)),
        ("iface_src", C.POINTER(C.c_int32)), ("iface_w", C.POINTER(C.c_double)),
    ]


class _Perf(C.Structure):
    _fields_ = [("initial_residual", C.c_double), ("final_residual", C.c_double),
                ("n_iter", C.c_int), ("converged", C.c_int), ("singular", C.c_int)]


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


class OracleMatrix:
    """An LDU matrix (+ flattened interfaces) held for the oracle.

    Arrays follow foam's lduMatrix/lduAddressing conventions: ``lower``/
    ``upper`` are lowerAddr/upperAddr (owner < neighbour, upper-triangular
    face order); ``upper_c``/``lower_c`` the off-diagonal coefficients
    (``lower_c`` None = symmetric).  Interfaces are flattened over patches:
    ``iface_cells`` (faceCells), ``iface_bou``/``iface_int`` (coupleBou/Int
    coefficients) and a CSR (``iface_ptr``, ``iface_src``, ``iface_w``) that
    gives each interface face's neighbour value as a weighted sum of cells.
    """

    def __init__(self, n, lower, upper, diag, upper_c, lower_c=None, iface=None):
        self.n = int(n)
        self.lower = np.ascontiguousarray(lower, dtype=np.int32)
        self.upper = np.ascontiguousarray(upper, dtype=np.int32)
        self.diag = np.ascontiguousarray(diag, dtype=np.float64)
        self.upper_c = np.ascontiguousarray(upper_c, dtype=np.float64)
        self.lower_c = None if lower_c is None else np.ascontiguousarray(lower_c, dtype=np.float64)
        self.iface = None
        if iface is not None and len(iface["cells"]) > 0:
            self.iface = {
                "cells": np.ascontiguousarray(iface["cells"], dtype=np.int32),
                "bou": np.ascontiguousarray(iface["bou"], dtype=np.float64),
                "int": None if iface.get("int") is None else np.ascontiguousarray(iface["int"], dtype=np.float64),
                "ptr": np.ascontiguousarray(iface["ptr"], dtype=np.int32),
                "src": np.ascontiguousarray(iface["src"], dtype=np.int32),
                "w": np.ascontiguousarray(iface["w"], dtype=np.float64),
            }
        s = _Ldu()
        s.n, s.nf = self.n, len(self.lower)
        s.lower, s.upper = _i(self.lower), _i(self.upper)
        s.diag, s.upperc, s.lowerc = _d(self.diag), _d(self.upper_c), _d(self.lower_c)
        if self.iface is None:
            s.ni = 0
        else:
            f = self.iface
            s.ni = len(f["cells"])
            s.iface_cells, s.iface_bou, s.iface_int = _i(f["cells"]), _d(f["bou"]), _d(f["int"])
            s.iface_ptr, s.iface_src, s.iface_w = _i(f["ptr"]), _i(f["src"]), _d(f["w"])
        self._s = s

    # -- products ---------------------------------------------------------
    def amul(self, x, fused=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        lib().or_amul(C.byref(self._s), _d(x), _d(y), int(fused))
        return y

    def tmul(self, x, fused=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        lib().or_tmul(C.byref(self._s), _d(x), _d(y), int(fused))
        return y

    def sumA(self):
        y = np.empty(self.n)
        lib().or_sumA(C.byref(self._s), _d(y))
        return y

    def norm_factor(self, x, b):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        Ax = self.amul(x)
        return lib().or_norm_factor(C.byref(self._s), _d(x), _d(b), _d(Ax))

    def residual(self, b, x):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        return lib().or_residual(C.byref(self._s), _d(b), _d(x))

    def factor(self, kind):
        rD = np.empty(self.n)
        fn = lib().or_dic_factor if kind == "DIC" else lib().or_dilu_factor
        fn(C.byref(self._s), _d(rD))
        return rD

    def precondition(self, kind, r, transpose=False, fused=False):
        r = np.ascontiguousarray(r, dtype=np.float64)
        w = np.empty(self.n)
        lib().or_precondition(C.byref(self._s), PRECONDITIONERS[kind], _d(r), _d(w),
                              int(transpose), int(fused))
        return w

    # -- solvers ----------------------------------------------------------
    def solve(self, b, x0, solver="PCG", precond="DIC", tol=1e-8, rel_tol=0.0,
              min_iter=0, max_iter=1000, fused=False):
        """Foam-semantics solve; returns (x, perf dict)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        p = _Perf()
        fn = {"PCG": lib().or_pcg, "PBiCG": lib().or_pbicg, "BiCGStab": lib().or_bicgstab}[solver]
        fn(C.byref(self._s), _d(b), _d(x), tol, rel_tol, int(min_iter), int(max_iter),
           PRECONDITIONERS[precond], int(fused), C.byref(p))
        return x, {"initial_residual": p.initial_residual, "final_residual": p.final_residual,
                   "n_iter": p.n_iter, "converged": bool(p.converged), "singular": bool(p.singular)}

    SMOOTHERS = {"GaussSeidel": 0, "DIC": 1, "DILU": 2, "DICGaussSeidel": 3, "DILUGaussSeidel": 4}

    # -- building blocks (GAMG restatement) ---------------------------------
    def gs_sweep(self, b, x, fused=True):
        """One Gauss-Seidel sweep of x in place."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        lib().or_gs_sweep(C.byref(self._s), _d(b), _d(x), int(fused))

    def foam_residual(self, b, x, fused=False):
        r = np.empty(self.n)
        lib().or_foam_residual(C.byref(self._s), _d(np.ascontiguousarray(b, np.float64)),
                               _d(np.ascontiguousarray(x, np.float64)), _d(r), int(fused))
        return r

    def mirror_residual(self, b, x):
        """(r = b - A x in the GPU's order, sum|r| in the GPU's tree)."""
        r = np.empty(self.n)
        s = lib().or_mirror_residual(C.byref(self._s), _d(np.ascontiguousarray(b, np.float64)),
                                     _d(np.ascontiguousarray(x, np.float64)), _d(r))
        return r, s

    def mirror_dot(self, a, b):
        """sum a b (fused) in the GPU's reduction order (sliced rows)."""
        return lib().or_mirror_dot(C.byref(self._s), _d(np.ascontiguousarray(a, np.float64)),
                                   _d(np.ascontiguousarray(b, np.float64)))

    def mirror_norm_factor(self, b, x):
        return lib().or_mirror_norm_factor(C.byref(self._s), _d(np.ascontiguousarray(b, np.float64)),
                                           _d(np.ascontiguousarray(x, np.float64)))

    def smooth(self, b, x0, tol=1e-8, rel_tol=0.0, min_iter=0, max_iter=1000, n_sweeps=1, mode="literal",
               smoother="GaussSeidel"):
        """smoothSolver with one of foam's smoothers; mode literal | fused |
        mirror (the GPU's order).  Returns (x, perf dict)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        p = _Perf()
        lib().or_smooth_gs(C.byref(self._s), _d(b), _d(x), tol, rel_tol, int(min_iter), int(max_iter), int(n_sweeps),
                           self.SMOOTHERS[smoother], {"literal": 0, "fused": 1, "mirror": 2}[mode], C.byref(p))
        return x, {"initial_residual": p.initial_residual, "final_residual": p.final_residual,
                   "n_iter": p.n_iter, "converged": bool(p.converged), "singular": bool(p.singular)}

    def solve_mirror(self, b, x0, solver="PCG", precond="DIC", tol=1e-8, rel_tol=0.0,
                     min_iter=0, max_iter=1000):
        """Fused-mode solve that sums in the GPU library's reduction tree.

        Not foam semantics: it exists so the GPU's whole solve can be
        compared bit for bit (see or_solve_mirror in ldu_oracle.c)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        p = _Perf()
        lib().or_solve_mirror(C.byref(self._s), _d(b), _d(x), tol, rel_tol, int(min_iter), int(max_iter),
                              PRECONDITIONERS[precond], {"PCG": 0, "PBiCG": 1, "BiCGStab": 2}[solver],
                              C.byref(p))
        return x, {"initial_residual": p.initial_residual, "final_residual": p.final_residual,
                   "n_iter": p.n_iter, "converged": bool(p.converged), "singular": bool(p.singular)}

    def to_scipy(self):
        import scipy.sparse as sp
        lo = self.upper_c if self.lower_c is None else self.lower_c
        rows = np.concatenate([np.arange(self.n), self.lower, self.upper])
        cols = np.concatenate([np.arange(self.n), self.upper, self.lower])
        vals = np.concatenate([self.diag, self.upper_c, lo])
        A = sp.coo_matrix((vals, (rows, cols)), shape=(self.n, self.n)).tocsr()
        if self.iface is not None:
            f = self.iface
            r, c, v = [], [], []
            for i in range(len(f["cells"])):
                for k in range(f["ptr"][i], f["ptr"][i + 1]):
                    r.append(f["cells"][i]); c.append(f["src"][k]); v.append(-f["bou"][i] * f["w"][k])
            A = A + sp.coo_matrix((v, (r, c)), shape=(self.n, self.n)).tocsr()
        return A


def direct_map(centres_to, centres_from, tol):
    """directMapInterfaceToInterfaceMapping's face map
    (directMapInterfaceToInterfaceMapping.C:147-190): for every face of the
    receiving patch the first face of the other, in face order, whose centre
    is within tol, |c_to - c_from| < tol with mag = sqrt((dx dx + dy dy) +
    dz dz); -1 where there is none.  The reference's N^2 search, literally."""
    ct = np.asarray(centres_to, dtype=np.float64).reshape(-1, 3)
    cf = np.asarray(centres_from, dtype=np.float64).reshape(-1, 3)
    out = np.full(len(ct), -1, np.int64)
    for i, c in enumerate(ct):
        d = c[None, :] - cf
        dist = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        hit = np.flatnonzero(dist < tol)
        if hit.size:
            out[i] = hit[0]
    return out


def ggi_apply(ptr, addr, w, src, ncomp=1, fused=False):
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    addr = np.ascontiguousarray(addr, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    src = np.ascontiguousarray(src, dtype=np.float64)
    ndst = len(ptr) - 1
    dst = np.empty(ndst * ncomp)
    lib().or_ggi_apply(ndst, _i(ptr), _i(addr), _d(w), _d(src), _d(dst), int(ncomp), int(fused))
    return dst if ncomp == 1 else dst.reshape(ndst, ncomp)


def overlaps(fa_ptr, fa_xy, fb_ptr, fb_xy, tol=1e-15):
    """All overlapping (face A, face B, intersection area) triples."""
    fa_ptr = np.ascontiguousarray(fa_ptr, dtype=np.int32)
    fb_ptr = np.ascontiguousarray(fb_ptr, dtype=np.int32)
    fa_xy = np.ascontiguousarray(fa_xy, dtype=np.float64)
    fb_xy = np.ascontiguousarray(fb_xy, dtype=np.float64)
    na, nb = len(fa_ptr) - 1, len(fb_ptr) - 1
    cap = 64 * max(na, nb) + 64
    oa = np.empty(cap, np.int32); ob = np.empty(cap, np.int32); ar = np.empty(cap)
    cnt = lib().gw_overlaps(na, _i(fa_ptr), _d(fa_xy), nb, _i(fb_ptr), _d(fb_xy), tol, cap,
                            _i(oa), _i(ob), _d(ar))
    if cnt < 0:
        raise RuntimeError("overlap capacity exceeded")
    return oa[:cnt].copy(), ob[:cnt].copy(), ar[:cnt].copy()


def face_areas(ptr, xy):
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    out = np.empty(len(ptr) - 1)
    lib().gw_face_areas(len(ptr) - 1, _i(ptr), _d(xy), _d(out))
    return out


def ggi_weights(fa_ptr, fa_xy, fb_ptr, fb_xy, tol=1e-15):
    """GGI weights in both directions (rescaled, uncovered faces empty).

    Returns two CSR triples (ptr, addr, w): ``a_from_b`` gives each A face as
    a weighted sum of B faces (slaveToMaster when A is the master), and
    ``b_from_a`` the reverse (masterToSlave).
    """
    ia, ib, ar = overlaps(fa_ptr, fa_xy, fb_ptr, fb_xy, tol)
    areas_a = np.abs(face_areas(fa_ptr, fa_xy))
    areas_b = np.abs(face_areas(fb_ptr, fb_xy))
    out = []
    for dst, src, adst, ndst in ((ia, ib, areas_a, len(fa_ptr) - 1), (ib, ia, areas_b, len(fb_ptr) - 1)):
        order = np.lexsort((src, dst))
        d, s, a = dst[order], src[order], ar[order]
        w = a / adst[d]
        sums = np.bincount(d, weights=w, minlength=ndst)
        w = w / sums[d]           # rescale so covered faces sum to one
        ptr = np.zeros(ndst + 1, np.int32)
        np.cumsum(np.bincount(d, minlength=ndst), out=ptr[1:])
        out.append((ptr, s.astype(np.int32), w))
    return out[0], out[1]
