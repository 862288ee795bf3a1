"""CPU restatement of the block-to-scalar expansion of block-coupled LDU
systems (test infrastructure only: tests import it to check the library's
mrg_block_addressing / mrg_block_coeffs, multiregionfoam_gb300/csrc/
block.cpp) and the block matrix-vector product it must preserve.

foam-extend's fvBlockMatrix::solve hands a BlockLduMatrix<vectorN> to
BlockLduSolver<Type>::New(...)->solve (filesToReplace/fvBlockMatrix.C:
1360-1388; the pressure-velocity coupled region assembles a
BlockLduMatrix<vector4>, pUCoupledIcoFluid.C:592-617).  Its Amul (foam's LDU
convention, per block face f = (l, u)):

    (A x)_c = D_c x_c + sum_{f: l = c} U_f x_u + sum_{f: u = c} L_f x_l

with bs x bs blocks D_c, U_f, L_f (a symmetric matrix stores no L_f: L_f =
U_f^T).  Written as a scalar LDU system of bs n cells (cell c's component a
is row bs c + a), every nonzero off-diagonal scalar entry (r, s), r < s, is
one face with upper = A[r][s] and lower = A[s][r]; faces in upper-triangular
order (sorted by r, then s).  Built here entry by entry from the dense
coupling pattern, independently of the library's construction.
"""
from __future__ import annotations

import numpy as np


def expand(n, lower, upper, bs, D, U, L=None):
    """(s_lower, s_upper, s_diag, s_upper_c, s_lower_c) of the scalar system."""
    D = np.asarray(D, np.float64).reshape(n, bs, bs)
    U = np.asarray(U, np.float64).reshape(len(lower), bs, bs)
    Lb = np.transpose(U, (0, 2, 1)) if L is None else np.asarray(L, np.float64).reshape(len(lower), bs, bs)
    entries = {}   # (r, s) with r < s -> (upper A[r][s], lower A[s][r])
    for c in range(n):
        for a in range(bs):
            for b in range(a + 1, bs):
                entries[(bs * c + a, bs * c + b)] = (D[c, a, b], D[c, b, a])
    for f in range(len(lower)):
        l, u = int(lower[f]), int(upper[f])
        for a in range(bs):
            for b in range(bs):
                # row l a, column u b: U_f[a][b]; row u b, column l a: L_f[b][a]
                entries[(bs * l + a, bs * u + b)] = (U[f, a, b], Lb[f, b, a])
    keys = sorted(entries)
    s_lower = np.array([k[0] for k in keys], np.int32)
    s_upper = np.array([k[1] for k in keys], np.int32)
    s_uc = np.array([entries[k][0] for k in keys], np.float64)
    s_lc = np.array([entries[k][1] for k in keys], np.float64)
    s_diag = np.array([D[c, a, a] for c in range(n) for a in range(bs)], np.float64)
    return s_lower, s_upper, s_diag, s_uc, s_lc


def block_amul(n, lower, upper, D, U, L, x):
    """A x of the block system (x [n, bs])."""
    bs = x.shape[1]
    D = np.asarray(D, np.float64).reshape(n, bs, bs)
    U = np.asarray(U, np.float64).reshape(len(lower), bs, bs)
    Lb = np.transpose(U, (0, 2, 1)) if L is None else np.asarray(L, np.float64).reshape(len(lower), bs, bs)
    y = np.einsum("cab,cb->ca", D, x)
    np.add.at(y, lower, np.einsum("fab,fb->fa", U, x[upper]))
    np.add.at(y, upper, np.einsum("fab,fb->fa", Lb, x[lower]))
    return y


def scalar_amul(n_s, s_lower, s_upper, s_diag, s_uc, s_lc, x):
    """A x of a scalar LDU system (numpy, any summation order)."""
    y = s_diag * x
    np.add.at(y, s_lower, s_uc * x[s_upper])
    np.add.at(y, s_upper, s_lc * x[s_lower])
    return y


# ---- block preconditioner (MRG_PRECOND_BLOCK) -------------------------------
# foam-extend's block Cholesky preconditioner (BlockCholeskyPrecon) on the
# bs x bs blocks, restated with the library's operation order (the GPU's
# kernels give the same bits): every product sums its terms in index order
# from the first, one rounding per multiply and add; the inverse is
# Gauss-Jordan elimination without pivoting.
#   factor   cells in order: D_c = A_cc - sum over faces f with upper cell c
#            (ascending) of L_f (inv(D_l) U_f); dD_c = inv(D_c)
#   apply    x_c = dD_c r_c; forward, faces ascending: x_u -= dD_u (L_f x_l);
#            backward, faces descending: x_l -= dD_l (U_f x_u)

def _mm(A, B):
    bs = len(A)
    C = [[0.0] * bs for _ in range(bs)]
    for a in range(bs):
        for b in range(bs):
            acc = A[a][0] * B[0][b]
            for k in range(1, bs):
                acc = acc + A[a][k] * B[k][b]
            C[a][b] = acc
    return C


def _mv(A, v):
    bs = len(A)
    out = [0.0] * bs
    for a in range(bs):
        acc = A[a][0] * v[0]
        for k in range(1, bs):
            acc = acc + A[a][k] * v[k]
        out[a] = acc
    return out


def _inv(M):
    bs = len(M)
    M = [list(r) for r in M]
    I = [[1.0 if a == b else 0.0 for b in range(bs)] for a in range(bs)]
    for k in range(bs):
        p = 1.0 / M[k][k]
        for j in range(bs):
            M[k][j] = M[k][j] * p
            I[k][j] = I[k][j] * p
        for i in range(bs):
            if i == k:
                continue
            f = M[i][k]
            for j in range(bs):
                M[i][j] = M[i][j] - f * M[k][j]
                I[i][j] = I[i][j] - f * I[k][j]
    return I


def _blocks(n, lower, upper, D, U, L):
    bs = np.asarray(D).reshape(n, -1).shape[1]
    bs = int(round(bs ** 0.5))
    D = np.asarray(D, np.float64).reshape(n, bs, bs)
    U = np.asarray(U, np.float64).reshape(len(lower), bs, bs)
    Lb = np.transpose(U, (0, 2, 1)) if L is None else np.asarray(L, np.float64).reshape(len(lower), bs, bs)
    return bs, D.tolist(), U.tolist(), Lb.tolist()


def block_factor(n, lower, upper, D, U, L=None):
    """dD [n][bs][bs] (inverses of the factored diagonal blocks)."""
    bs, Dl, Ul, Ll = _blocks(n, lower, upper, D, U, L)
    into = [[] for _ in range(n)]
    for f in range(len(lower)):
        into[int(upper[f])].append(f)
    dD = [None] * n
    for c in range(n):
        M = [list(r) for r in Dl[c]]
        for f in into[c]:            # ascending face order
            P = _mm(Ll[f], _mm(dD[int(lower[f])], Ul[f]))
            M = [[M[a][b] - P[a][b] for b in range(bs)] for a in range(bs)]
        dD[c] = _inv(M)
    return dD


def block_apply(n, lower, upper, D, U, L, dD, r):
    """w = M^-1 r (r [n, bs]) with the factor of block_factor."""
    bs, _, Ul, Ll = _blocks(n, lower, upper, D, U, L)
    r = np.asarray(r, np.float64).reshape(n, bs).tolist()
    into = [[] for _ in range(n)]
    out_ = [[] for _ in range(n)]
    for f in range(len(lower)):
        into[int(upper[f])].append(f)
        out_[int(lower[f])].append(f)
    y = [None] * n
    for c in range(n):
        x = _mv(dD[c], r[c])
        for f in into[c]:
            u = _mv(dD[c], _mv(Ll[f], y[int(lower[f])]))
            x = [x[a] - u[a] for a in range(bs)]
        y[c] = x
    w = [None] * n
    for c in range(n - 1, -1, -1):
        x = list(y[c])
        for f in reversed(out_[c]):   # descending face order
            u = _mv(dD[c], _mv(Ul[f], w[int(upper[f])]))
            x = [x[a] - u[a] for a in range(bs)]
        w[c] = x
    return np.array(w, np.float64)
