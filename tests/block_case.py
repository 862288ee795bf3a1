"""Seeded block-coupled (bs x bs) test systems on a hex block.

Diagonal blocks s I + a small random matrix, face blocks small random
matrices; the diagonal term s is chosen so every scalar row is strictly
diagonally dominant.  symmetric=True: symmetric diagonal blocks and lower
blocks = upper blocks transposed (an SPD matrix).
"""
import numpy as np

from multiregionfoam_gb300 import cases


def block_case(nx, ny, nz, bs=4, seed=0, symmetric=False):
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    lower, upper, _ = cases.box_faces(nx, ny, nz)
    nf = len(lower)
    U = rng.uniform(-1.0, 1.0, (nf, bs, bs))
    L = None if symmetric else rng.uniform(-1.0, 1.0, (nf, bs, bs))
    D = rng.uniform(-0.3, 0.3, (n, bs, bs))
    if symmetric:
        D = 0.5 * (D + np.transpose(D, (0, 2, 1)))
    # row sums of |off-diagonal| per scalar row, plus a margin
    off = np.abs(D).sum(axis=2) - np.abs(np.einsum("caa->ca", D))
    np.add.at(off, lower, np.abs(U).sum(axis=2))
    Lb = np.transpose(U, (0, 2, 1)) if L is None else L
    np.add.at(off, upper, np.abs(Lb).sum(axis=2))
    for a in range(bs):
        D[:, a, a] = off[:, a] * rng.uniform(1.05, 1.3, n) + 0.1
    b = rng.uniform(-1.0, 1.0, (n, bs))
    x0 = np.zeros((n, bs))
    return dict(n=n, lower=lower.astype(np.int32), upper=upper.astype(np.int32), bs=bs, D=D, U=U, L=L, b=b, x0=x0)
