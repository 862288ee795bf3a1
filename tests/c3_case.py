"""The asymmetric, non-conformal configuration (C3) as a test case.

A unit-square column split at z = 1/2: region A is an nA x nA x nz hex block
below, region B an nB x nA x nz block above (x spacing 1.5x A's: a 3:2
face-count ratio across the interface).  Both carry upwind convection-
diffusion with a seeded divergence-free in-plane velocity (stream function
vanishing on the side walls, so there is no flux through them or through
the interface), scaled to a largest cell Peclet number of `pe_max` times a
U(0,1) draw; Dirichlet 0 below A and 1 above B; an implicit source.  The
two regions meet through a GGI interface: the in-plane nodes of both
interface patches are jittered by up to 0.2 h (boundary nodes fixed) and
the weights are the exact polygon overlaps (the oracle's construction,
rescaled as ggiInterfaceToInterfaceMapping.C:62-77 does), with interface
conductance k |overlap| / d.  Cell numbering is randomly permuted and the
faces re-sorted upper-triangular.  Full size (scale 1): A 96x96x48, B
64x96x48 = 737,280 cells, 9,216 : 6,144 interface faces.

Test infrastructure: it uses the oracle's GGI weight construction.
"""
from __future__ import annotations

import numpy as np

from multiregionfoam_gb300 import cases
from test_oracle import jittered_faces


def _block(nx, ny, nz, hx, hy, hz, k, rc, psi, offset):
    """Faces, coefficients and diagonal of one convection-diffusion block."""
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    lo = [idx[:, :, :-1].ravel(), idx[:, :-1, :].ravel(), idx[:-1, :, :].ravel()]
    up = [idx[:, :, 1:].ravel(), idx[:, 1:, :].ravel(), idx[1:, :, :].ravel()]
    xs, ys = np.arange(nx + 1) * hx, np.arange(ny + 1) * hy
    P = psi(xs[None, :], ys[:, None])               # (ny+1, nx+1) at lattice nodes
    # flux through an x-face (node column i, rows j..j+1) and a y-face; w = 0
    fx = (P[1:, :] - P[:-1, :]) * hz                # (ny, nx+1)
    fy = -(P[:, 1:] - P[:, :-1]) * hz               # (ny+1, nx)
    phi = [np.broadcast_to(fx[None, :, 1:-1], (nz, ny, nx - 1)).ravel(),
           np.broadcast_to(fy[None, 1:-1, :], (nz, ny - 1, nx)).ravel(),
           np.zeros(lo[2].size)]
    g = [np.full(lo[0].size, k * hy * hz / hx), np.full(lo[1].size, k * hx * hz / hy),
         np.full(lo[2].size, k * hx * hy / hz)]
    lower, upper = np.concatenate(lo) + offset, np.concatenate(up) + offset
    return lower, upper, np.concatenate(g), np.concatenate(phi), n


def c3(scale: int = 1, seed: int = 0, pe_max: float = 10.0, k: float = 1.0, rc: float = 1.0):
    rng = np.random.default_rng(seed)
    na_xy, nb_x, nz = 96 // scale, 64 // scale, 48 // scale
    hz = 0.5 / nz
    modes = rng.standard_normal((3, 3))

    def psi(x, y):
        s = 0.0
        for p in range(3):
            for q in range(3):
                s = s + modes[p, q] * np.sin(np.pi * (p + 1) * x) * np.sin(np.pi * (q + 1) * y)
        return s

    la, ua, ga, pa_, nA = _block(na_xy, na_xy, nz, 1.0 / na_xy, 1.0 / na_xy, hz, k, rc, psi, 0)
    lb, ub, gb, pb_, nB = _block(nb_x, na_xy, nz, 1.0 / nb_x, 1.0 / na_xy, hz, k, rc, psi, nA)
    n = nA + nB
    lower, upper = np.concatenate([la, lb]), np.concatenate([ua, ub])
    g, phi = np.concatenate([ga, gb]), np.concatenate([pa_, pb_])
    # velocity scale: largest cell Peclet number pe_max, times U(0, 1)
    h_min = min(1.0 / na_xy, hz)
    umax = np.abs(phi).max() / (hz * h_min) if np.abs(phi).max() > 0 else 1.0
    phi = phi * (pe_max * k / rc / (umax * h_min)) * rng.uniform(0.0, 1.0)
    F = rc * phi
    upper_c = -g + np.minimum(F, 0.0)
    lower_c = -g - np.maximum(F, 0.0)
    vol = np.concatenate([np.full(nA, hz / na_xy ** 2), np.full(nB, hz / (nb_x * na_xy))])
    diag = rc * vol
    np.add.at(diag, lower, g + np.maximum(F, 0.0))
    np.add.at(diag, upper, g - np.minimum(F, 0.0))
    t_old = rng.uniform(0.0, 1.0, n)
    b = rc * vol * t_old
    # Dirichlet 0 under A, 1 over B
    a_bot = np.arange(na_xy * na_xy)
    b_top = nA + np.arange(nb_x * na_xy) + (nz - 1) * nb_x * na_xy
    diag[a_bot] += 2.0 * k * (1.0 / na_xy ** 2) / hz
    gtop = 2.0 * k * (1.0 / (nb_x * na_xy)) / hz
    diag[b_top] += gtop
    b[b_top] += gtop
    # GGI interface between A's top layer and B's bottom layer
    import oracle as O
    fa = jittered_faces(na_xy, na_xy, 0.2, seed + 101)
    fb = jittered_faces(nb_x, na_xy, 0.2, seed + 102)
    (pa, sa, wa), (pb, sb, wb) = O.ggi_weights(*fa, *fb)
    area_a, area_b = np.abs(O.face_areas(*fa)), np.abs(O.face_areas(*fb))
    a_top = np.arange(na_xy * na_xy) + (nz - 1) * na_xy * na_xy
    b_bot = nA + np.arange(nb_x * na_xy)
    d = hz                                          # centre-to-centre across the interface
    coef = np.concatenate([k * area_a / d, k * area_b / d])
    cells = np.concatenate([a_top, b_bot])
    np.add.at(diag, cells, coef)
    iface = {"cells": cells.astype(np.int32), "bou": coef, "int": None,
             "ptr": np.concatenate([pa, pa[-1] + pb[1:]]).astype(np.int32),
             "src": np.concatenate([b_bot[sa], a_top[sb]]).astype(np.int32),
             "w": np.concatenate([wa, wb])}
    lo2, up2, upc, loc = cases.upper_triangular(lower, upper, upper_c, lower_c)
    s = cases.LduSystem(n, lo2.astype(np.int32), up2.astype(np.int32), diag, upc, loc, b, t_old, iface,
                        name=f"c3/{scale}", meta=dict(nA=nA, nB=nB, n_ifa=a_top.size, n_ifb=b_bot.size))
    s = cases.random_permute(s, seed + 7)
    ggi = dict(a_from_b=(pa, sa, wa), b_from_a=(pb, sb, wb), n_a=a_top.size, n_b=b_bot.size)
    return s, ggi
