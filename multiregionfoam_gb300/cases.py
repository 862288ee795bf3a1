"""Seeded synthetic coupled-region systems in foam LDU form.

These stand in for the matrices that multiRegionFoam's regions assemble:

* ``conductTemperature::setCoupledEqns`` (src/regions/conductTemperature/
  conductTemperature.C:135-152): ``ddt(rho*cv, T) == laplacian(k, T)``, a
  symmetric matrix, solved with PCG+DIC.
* ``transportTemperature::setCoupledEqns`` (src/regions/transportTemperature/
  transportTemperature.C:129-150): ``rho*cp*(ddt(T) + div(phi, T)) ==
  laplacian(k, T)``, asymmetric (upwind), solved with PBiCG+DILU.
* The monolithic interface conductance of
  monolithicThermalDiffusivityFvPatchScalarField.C:231-243: with uniform
  cells (patch weight 1/2) ``k = kOwn*kNei/(deltaCoeffs*(kOwn+kNei))``
  reduces to the harmonic mean 2*k1*k2/(k1+k2); the face coefficient is
  k*|Sf|*deltaCoeffs.

Every system comes in up to two forms that give the same A x:

* ``global``: one LDU matrix over all regions, the interface faces stored as
  ordinary internal faces (monolithic assembly as in fvBlockMatrix).
* ``coupled``: the region matrices side by side (block diagonal) plus
  interface patches whose contribution enters Amul as
  ``result[faceCells] -= coeffs*interpolate(psi_shadow)``
  (monolithicCouplingFvPatchField.C:381-464) -- the coupledFvMatrix form.

Units: cubic cells of edge h; ``rc`` is rho*c/dt in W/(m^3 K).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class LduSystem:
    """One linear system A x = b in foam LDU storage (+ flattened interfaces)."""
    n: int
    lower: np.ndarray          # lowerAddr (owner), int32 [F]
    upper: np.ndarray          # upperAddr (neighbour), int32 [F]
    diag: np.ndarray           # float64 [n]
    upper_c: np.ndarray        # float64 [F]
    lower_c: np.ndarray | None  # float64 [F] or None (symmetric)
    b: np.ndarray              # float64 [n]
    x0: np.ndarray             # float64 [n] (previous time level = initial guess)
    iface: dict | None = None  # cells, bou, int, ptr, src, w
    name: str = ""
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def nf(self) -> int:
        return int(len(self.lower))

    @property
    def symmetric(self) -> bool:
        return self.lower_c is None


def box_faces(nx: int, ny: int, nz: int, offset: int = 0):
    """Internal faces of a lexicographic (x fastest) hex block.

    Returns (lower, upper, dirn) in upper-triangular order: sorted by owner,
    then neighbour -- the face order foam's lduAddressing requires.
    """
    idx = np.arange(nx * ny * nz, dtype=np.int64).reshape(nz, ny, nx) + offset
    lo = [idx[:, :, :-1].ravel(), idx[:, :-1, :].ravel(), idx[:-1, :, :].ravel()]
    up = [idx[:, :, 1:].ravel(), idx[:, 1:, :].ravel(), idx[1:, :, :].ravel()]
    dr = [np.full(a.size, d, np.int8) for d, a in enumerate(lo)]
    lower = np.concatenate(lo)
    upper = np.concatenate(up)
    dirn = np.concatenate(dr)
    order = np.lexsort((upper, lower))
    return lower[order], upper[order], dirn[order]


def upper_triangular(lower, upper, *payload):
    """Swap (l,u) so l<u and sort faces into upper-triangular order."""
    lower = np.asarray(lower, np.int64)
    upper = np.asarray(upper, np.int64)
    lo = np.minimum(lower, upper)
    hi = np.maximum(lower, upper)
    order = np.lexsort((hi, lo))
    return (lo[order], hi[order]) + tuple(np.asarray(p)[order] for p in payload)


def _harm(a, b):
    return 2.0 * a * b / (a + b)


def cht_system(nx: int, ny: int, nz_fluid: int, nz_solid: int, *, seed: int = 0,
               k_fluid: float = 0.6, k_solid: float = 16.0, k_range=None,
               rc: float = 1.0, t_base: float = 300.0, t_top: float = 350.0,
               form: str = "global", perturb: float = 0.1) -> LduSystem:
    """Two-region conjugate-heat-transfer temperature system.

    Solid block nx*ny*nz_solid at the bottom (Dirichlet t_base on its base),
    fluid block nx*ny*nz_fluid on top (Dirichlet t_top on its lid), sharing a
    conformal nx*ny interface.  Cells: solid first, then fluid, each
    lexicographic.  Conductivity is constant per region, or -- with
    ``k_range=(lo, hi)`` -- log-uniform per cell.  The initial/old field is a
    linear profile plus ``perturb``*N(0,1).
    """
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    ns, nfl = nx * ny * nz_solid, nx * ny * nz_fluid
    n = ns + nfl
    if k_range is None:
        kc = np.concatenate([np.full(ns, k_solid), np.full(nfl, k_fluid)])
    else:
        lo, hi = np.log(k_range[0]), np.log(k_range[1])
        kc = np.exp(rng.uniform(lo, hi, n))
    zc = np.concatenate([
        (np.repeat(np.arange(nz_solid), nx * ny) + 0.5) * h,
        (np.repeat(np.arange(nz_fluid), nx * ny) + 0.5 + nz_solid) * h,
    ])
    ztot = (nz_solid + nz_fluid) * h
    t_old = t_base + (t_top - t_base) * zc / ztot + perturb * rng.standard_normal(n)

    ls, us, _ = box_faces(nx, ny, nz_solid, 0)
    lf, uf, _ = box_faces(nx, ny, nz_fluid, ns)
    s_top = np.arange(nx * ny) + (nz_solid - 1) * nx * ny
    f_bot = np.arange(nx * ny) + ns
    g_int = np.concatenate([_harm(kc[ls], kc[us]), _harm(kc[lf], kc[uf])]) * h
    g_if = _harm(kc[s_top], kc[f_bot]) * h

    diag = np.full(n, rc * h ** 3)
    b = rc * h ** 3 * t_old
    lower = np.concatenate([ls, lf])
    upper = np.concatenate([us, uf])
    np.add.at(diag, lower, g_int)
    np.add.at(diag, upper, g_int)
    diag[s_top] += g_if
    diag[f_bot] += g_if
    s_base = np.arange(nx * ny)
    f_lid = ns + np.arange(nx * ny) + (nz_fluid - 1) * nx * ny
    gb_s = 2.0 * kc[s_base] * h
    gb_f = 2.0 * kc[f_lid] * h
    diag[s_base] += gb_s
    b[s_base] += gb_s * t_base
    diag[f_lid] += gb_f
    b[f_lid] += gb_f * t_top

    ix = np.tile(np.arange(nx), ny * (nz_solid + nz_fluid))
    iy = np.tile(np.repeat(np.arange(ny), nx), nz_solid + nz_fluid)
    centres = np.stack([(ix + 0.5) * h, (iy + 0.5) * h, zc], axis=1)
    meta = dict(nx=nx, ny=ny, nz_fluid=nz_fluid, nz_solid=nz_solid, seed=seed, h=h,
                n_solid=ns, n_fluid=nfl, n_iface=nx * ny, rc=rc, k_cell=kc, centres=centres)
    if form == "global":
        lo2, up2, g2 = upper_triangular(np.concatenate([lower, s_top]),
                                        np.concatenate([upper, f_bot]),
                                        np.concatenate([g_int, g_if]))
        return LduSystem(n, lo2.astype(np.int32), up2.astype(np.int32), diag, -g2, None,
                         b, t_old, None, name="cht-global", meta=meta)
    if form != "coupled":
        raise ValueError(form)
    m = nx * ny
    iface = {
        "cells": np.concatenate([s_top, f_bot]).astype(np.int32),
        "bou": np.concatenate([g_if, g_if]),
        "int": None,
        "ptr": np.arange(2 * m + 1, dtype=np.int32),
        "src": np.concatenate([f_bot, s_top]).astype(np.int32),
        "w": np.ones(2 * m),
    }
    return LduSystem(n, lower.astype(np.int32), upper.astype(np.int32), diag, -g_int, None,
                     b, t_old, iface, name="cht-coupled", meta=meta)


def face_area_vectors(sys: LduSystem) -> np.ndarray:
    """Area vectors Sf ([nf, 3], owner to neighbour) of the internal faces of
    a system on a uniform hex grid of spacing meta["h"] with cell centres
    meta["centres"] (cht_system): (c_upper - c_lower) h."""
    c, h = sys.meta["centres"], sys.meta["h"]
    return (c[sys.upper] - c[sys.lower]) * h


def partitioned_cht(nx: int, ny: int, nz_fluid: int, nz_solid: int, **kw):
    """The two-region CHT problem of cht_system split for partitioned
    Dirichlet-Neumann coupling: region A = fluid (jump / Dirichlet patch on
    its bottom faces), region B = solid (flux / Neumann patch on its top
    faces), conformal face-to-face map.  Returns a dict with the monolithic
    global system, the two region systems (interface faces removed; the
    Dirichlet patch's diagonal term k|Sf|deltaCoeffs = 2 k h added to A),
    and the two patches (faceCells, deltaCoeffs = 2/h, face k = cell k,
    |Sf| = h^2, identity interpolation).  Converged DN coupling reproduces
    the monolithic solution: the harmonic-mean interface conductance of the
    monolithic matrix is what continuity of value and flux gives."""
    mono = cht_system(nx, ny, nz_fluid, nz_solid, form="global", **kw)
    m = mono.meta
    h, ns, n = m["h"], m["n_solid"], mono.n
    kc = m["k_cell"]
    nif = nx * ny
    s_top = np.arange(nif) + (nz_solid - 1) * nif
    f_bot = np.arange(nif) + ns
    lo, up = mono.lower.astype(np.int64), mono.upper.astype(np.int64)
    in_s = up < ns
    in_f = lo >= ns
    iface = ~(in_s | in_f)
    g_if = -mono.upper_c[iface]
    diag = mono.diag.copy()
    np.subtract.at(diag, lo[iface], g_if)
    np.subtract.at(diag, up[iface], g_if)
    fluid_diag = diag[ns:].copy()
    fluid_diag[f_bot - ns] += 2.0 * kc[f_bot] * h
    solid = LduSystem(ns, lo[in_s].astype(np.int32), up[in_s].astype(np.int32), diag[:ns].copy(),
                      mono.upper_c[in_s].copy(), None, mono.b[:ns].copy(), mono.x0[:ns].copy(), None,
                      name="cht-solid")
    fluid = LduSystem(n - ns, (lo[in_f] - ns).astype(np.int32), (up[in_f] - ns).astype(np.int32), fluid_diag,
                      mono.upper_c[in_f].copy(), None, mono.b[ns:].copy(), mono.x0[ns:].copy(), None,
                      name="cht-fluid")
    ident = dict(ptr=np.arange(nif + 1, dtype=np.int32), addr=np.arange(nif, dtype=np.int32), w=np.ones(nif))
    patch_a = dict(n_cells=n - ns, face_cells=(f_bot - ns).astype(np.int32), delta=np.full(nif, 2.0 / h),
                   k=kc[f_bot].copy(), area=np.full(nif, h * h), **ident)
    patch_b = dict(n_cells=ns, face_cells=s_top.astype(np.int32), delta=np.full(nif, 2.0 / h),
                   k=kc[s_top].copy(), area=np.full(nif, h * h), **ident)
    return dict(mono=mono, fluid=fluid, solid=solid, a=patch_a, b=patch_b, s_top=s_top, f_bot=f_bot)


def c1(form="global", seed=0):
    """Plain-method CPU case: fluid 40^3 (k=0.6) over solid 40x40x20 (k=16)."""
    return cht_system(40, 40, 40, 20, seed=seed, form=form)


def c2(form="global", seed=0, scale=1):
    """Plain-vs-mixed GPU case: fluid 128^3 over solid 128x128x64, k log-U[0.1,50].

    ``scale`` divides every dimension (scale=4 gives a 32^3 + 32x32x16 test case).
    """
    s = 128 // scale
    return cht_system(s, s, s, s // 2, seed=seed, k_range=(0.1, 50.0), form=form)


def batch_shapes(count: int, n_lo: int = 8000, n_hi: int = 260000, seed: int = 0):
    """Block dimensions of `count` two-region CHT systems with log-uniform cell
    counts in [n_lo, n_hi] and random aspect ratios (log-U[0.5, 2] per axis);
    the solid is the lower third of each block."""
    rng = np.random.default_rng(seed)
    shapes = []
    for _ in range(count):
        n = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        a = np.exp(rng.uniform(np.log(0.5), np.log(2.0), 3))
        s = (n / a.prod()) ** (1.0 / 3.0)
        nx, ny, nz = (max(2, int(round(v))) for v in a * s)
        nzs = max(1, nz // 3)
        shapes.append((nx, ny, max(1, nz - nzs), nzs))
    return shapes


def c4(count: int = 512, seed: int = 0, n_lo: int = 8000, n_hi: int = 260000):
    """Batched case: independent 2-region CHT systems of uneven size,
    conductivity log-uniform in [0.1, 50] per cell."""
    return [cht_system(nx, ny, nzf, nzs, seed=seed + 1 + i, k_range=(0.1, 50.0))
            for i, (nx, ny, nzf, nzs) in enumerate(batch_shapes(count, n_lo, n_hi, seed))]


def perturb_step(sys: LduSystem, rng, scale: float = 0.05) -> LduSystem:
    """The next time step of a recurring mesh: every off-diagonal coefficient
    and the diagonal's excess over the row's off-diagonal magnitudes are
    multiplied by 1 + scale*N(0,1) (clipped positive), so a diagonally
    dominant matrix stays so; b is perturbed the same way, x0 is kept.  The
    new row sums of off-diagonal magnitudes ride along in meta, so the next
    step does not recompute them."""
    def f(k):
        return np.clip(1.0 + scale * rng.standard_normal(k), 0.2, None)

    def rowsum(up, lo):
        return (np.bincount(sys.lower, np.abs(up), minlength=sys.n) +
                np.bincount(sys.upper, np.abs(lo), minlength=sys.n))

    old = sys.meta.get("abs_rowsum")
    if old is None:
        old = rowsum(sys.upper_c, sys.upper_c if sys.lower_c is None else sys.lower_c)
    excess = sys.diag - old
    up = sys.upper_c * f(sys.nf)
    lo = None if sys.lower_c is None else sys.lower_c * f(sys.nf)
    new = rowsum(up, up if lo is None else lo)
    diag = excess * f(sys.n) + new
    meta = dict(sys.meta)
    meta["abs_rowsum"] = new
    return dataclasses.replace(sys, diag=diag, upper_c=up, lower_c=lo, b=sys.b * f(sys.n), meta=meta)


def c5_meshes(count: int = 100, seed: int = 0, n_lo: int = 10000, n_hi: int = 2000000, asym_frac: float = 0.3):
    """Served case: `count` meshes of log-uniform size in [n_lo, n_hi] cells,
    a fraction `asym_frac` asymmetric convection-diffusion (PBiCG+DILU), the
    rest two-region CHT (PCG+DIC).  Returns [(system, asym)]."""
    return [(c5_mesh(sp), sp[0]) for sp in c5_specs(count, seed, n_lo, n_hi, asym_frac)]


def c5_specs(count: int = 100, seed: int = 0, n_lo: int = 10000, n_hi: int = 2000000, asym_frac: float = 0.3):
    """The served case's meshes as cheap descriptions: [(asym, dims, seed)],
    cells log-uniform in [n_lo, n_hi], random aspect ratios, a fraction
    `asym_frac` asymmetric convection-diffusion.  c5_mesh builds one."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        a = np.exp(rng.uniform(np.log(0.5), np.log(2.0), 3))
        a = a / np.cbrt(a.prod())
        asym = bool(rng.uniform() < asym_frac)
        dims = tuple(max(4, int(round(np.cbrt(n) * a[k]))) for k in range(3))
        out.append((asym, dims, seed + 1 + i))
    return out


def c5_mesh(spec) -> LduSystem:
    """One served mesh from its c5_specs description (time step 0)."""
    asym, (nx, ny, nz), sd = spec
    if asym:
        return convdiff_system(nx, ny, nz, seed=sd)
    nzs = max(2, nz // 3)
    return cht_system(nx, ny, max(2, nz - nzs), nzs, seed=sd, k_range=(0.1, 50.0))


def c5_step(base: LduSystem, mesh: int, step: int, seed: int = 0) -> LduSystem:
    """Time step `step` of served mesh `mesh`: `step` successive 5 %
    perturbations of its step-0 system, each drawn from a generator seeded by
    (seed, mesh, step), so any request can be rebuilt on its own."""
    cur = base
    for k in range(1, step + 1):
        cur = perturb_step(cur, np.random.default_rng((seed, mesh, k)))
    return cur


def jittered_faces(nx, ny, jitter, seed):
    """Quads of a jittered nx*ny lattice on the unit square (boundary nodes
    fixed), counter-clockwise: (vertex pointers, (x, y) vertices)."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.linspace(0, 1, nx + 1), np.linspace(0, 1, ny + 1), indexing="xy")
    hx, hy = 1.0 / nx, 1.0 / ny
    jx = rng.uniform(-jitter, jitter, X.shape) * hx
    jy = rng.uniform(-jitter, jitter, Y.shape) * hy
    jx[:, 0] = jx[:, -1] = 0
    jy[0, :] = jy[-1, :] = 0
    jx[0, :] = jx[-1, :] = 0
    jy[:, 0] = jy[:, -1] = 0
    X, Y = X + jx, Y + jy
    xy = []
    for j in range(ny):
        for i in range(nx):
            for (a, b) in ((j, i), (j, i + 1), (j + 1, i + 1), (j + 1, i)):
                xy.append((X[a, b], Y[a, b]))
    ptr = np.arange(0, 4 * nx * ny + 1, 4, dtype=np.int32)
    return ptr, np.array(xy)


def quad_areas(ptr, xy):
    """|signed area| of quadrilateral faces by the shoelace sum, vertex pair
    by vertex pair (each product and difference rounded on its own)."""
    nf = len(ptr) - 1
    assert np.all(np.diff(ptr) == 4), "quadrilateral faces"
    P = np.asarray(xy, dtype=np.float64).reshape(nf, 4, 2)
    a = np.zeros(nf)
    for i in range(4):
        j = (i + 1) % 4
        a = a + (P[:, i, 0] * P[:, j, 1] - P[:, j, 0] * P[:, i, 1])
    return np.abs(0.5 * a)


def _c3_block(nx, ny, nz, hx, hy, hz, k, psi, offset):
    """Faces, conductances and face fluxes of one convection-diffusion block."""
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


def c3(weights, scale: int = 1, seed: int = 0, pe_max: float = 10.0, k: float = 1.0, rc: float = 1.0,
       permute: bool = True):
    """The asymmetric, non-conformal case.

    A unit-square column split at z = 1/2: region A is an nA x nA x nz hex
    block below, region B an nB x nA x nz block above (x spacing 1.5x A's: a
    3:2 face-count ratio across the interface).  Both carry upwind
    convection-diffusion with a seeded divergence-free in-plane velocity
    (stream function vanishing on the side walls, so there is no flux
    through them or through the interface), scaled to a largest cell Peclet
    number of `pe_max` times a U(0,1) draw; Dirichlet 0 below A and 1 above
    B; an implicit source.  The regions meet through a GGI interface: the
    in-plane nodes of both interface patches are jittered by up to 0.2 h
    (boundary nodes fixed) and ``weights(faces_a, faces_b)`` gives the
    rescaled overlap weights in both directions ((ptr, addr, w) of A from B,
    then of B from A: mrg_ggi_build's, or the oracle's), with interface
    conductance k |face| / d.  Cell numbering is randomly permuted and the
    faces re-sorted upper-triangular (permute=False keeps A's cells, then
    B's, each lexicographic).  Full size (scale 1): A 96x96x48, B
    64x96x48 = 737,280 cells, 9,216 : 6,144 interface faces.  Returns
    (system, ggi) with ggi's CSR triples and patch sizes."""
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

    la, ua, ga, pa_, nA = _c3_block(na_xy, na_xy, nz, 1.0 / na_xy, 1.0 / na_xy, hz, k, psi, 0)
    lb, ub, gb, pb_, nB = _c3_block(nb_x, na_xy, nz, 1.0 / nb_x, 1.0 / na_xy, hz, k, psi, nA)
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
    fa = jittered_faces(na_xy, na_xy, 0.2, seed + 101)
    fb = jittered_faces(nb_x, na_xy, 0.2, seed + 102)
    (pa, sa, wa), (pb, sb, wb) = weights(fa, fb)
    area_a, area_b = quad_areas(*fa), quad_areas(*fb)
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
    lo2, up2, upc, loc = upper_triangular(lower, upper, upper_c, lower_c)
    s = LduSystem(n, lo2.astype(np.int32), up2.astype(np.int32), diag, upc, loc, b, t_old, iface,
                  name=f"c3/{scale}", meta=dict(nA=nA, nB=nB, n_ifa=a_top.size, n_ifb=b_bot.size))
    if permute:
        s = random_permute(s, seed + 7)
    ggi = dict(a_from_b=(pa, sa, wa), b_from_a=(pb, sb, wb), n_a=a_top.size, n_b=b_bot.size)
    return s, ggi


def block_case(nx: int, ny: int, nz: int, bs: int = 4, seed: int = 0, symmetric: bool = False) -> dict:
    """A seeded block-coupled (bs x bs) system on a hex block, in the shape of
    foam-extend's BlockLduMatrix<vectorN>: diagonal blocks s I plus a small
    random matrix, face blocks small random matrices, the diagonal term s
    chosen so every scalar row is strictly diagonally dominant.  symmetric:
    symmetric diagonal blocks and lower blocks = upper blocks transposed (an
    SPD matrix; L None).  Returns n, lower, upper, bs, D [n, bs, bs], U and L
    [F, bs, bs], b [n, bs], x0 (zeros)."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    lower, upper, _ = box_faces(nx, ny, nz)
    nf = len(lower)
    U = rng.uniform(-1.0, 1.0, (nf, bs, bs))
    L = None if symmetric else rng.uniform(-1.0, 1.0, (nf, bs, bs))
    D = rng.uniform(-0.3, 0.3, (n, bs, bs))
    if symmetric:
        D = 0.5 * (D + np.transpose(D, (0, 2, 1)))
    off = np.abs(D).sum(axis=2) - np.abs(np.einsum("caa->ca", D))
    np.add.at(off, lower, np.abs(U).sum(axis=2))
    Lb = np.transpose(U, (0, 2, 1)) if L is None else L
    np.add.at(off, upper, np.abs(Lb).sum(axis=2))
    for a in range(bs):
        D[:, a, a] = off[:, a] * rng.uniform(1.05, 1.3, n) + 0.1
    b = rng.uniform(-1.0, 1.0, (n, bs))
    return dict(n=n, lower=lower.astype(np.int32), upper=upper.astype(np.int32), bs=bs, D=D, U=U, L=L, b=b,
                x0=np.zeros((n, bs)))


def laplace_1d(n: int, dirichlet=(0.0, 1.0), k: float = 1.0):
    """1-D Laplacian with Dirichlet ends: exact solution is linear."""
    lower = np.arange(n - 1, dtype=np.int32)
    upper = lower + 1
    diag = np.full(n, 2.0 * k)
    b = np.zeros(n)
    b[0] += k * 2.0 * dirichlet[0]
    b[-1] += k * 2.0 * dirichlet[1]
    diag[0] += k
    diag[-1] += k
    x_exact = dirichlet[0] + (dirichlet[1] - dirichlet[0]) * (np.arange(n) + 0.5) / n
    return LduSystem(n, lower, upper, diag, np.full(n - 1, -k), None, b, np.zeros(n),
                     name="laplace1d", meta={"x_exact": x_exact})


def random_permute(sys: LduSystem, seed: int) -> LduSystem:
    """Renumber cells by a seeded random permutation, faces re-sorted upper-triangular."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(sys.n)          # new -> old
    inv = np.empty(sys.n, np.int64)
    inv[perm] = np.arange(sys.n)           # old -> new
    l_new, u_new = inv[sys.lower], inv[sys.upper]
    swap = l_new > u_new
    upc = sys.upper_c.copy()
    loc = None if sys.lower_c is None else sys.lower_c.copy()
    if loc is not None:
        upc[swap], loc[swap] = sys.lower_c[swap], sys.upper_c[swap]
    lo2, up2, upc2 = upper_triangular(l_new, u_new, upc)
    loc2 = None
    if loc is not None:
        _, _, loc2 = upper_triangular(l_new, u_new, loc)
    iface = None
    if sys.iface is not None:
        f = sys.iface
        iface = dict(f)
        iface["cells"] = inv[f["cells"]].astype(np.int32)
        iface["src"] = inv[f["src"]].astype(np.int32)
    meta = dict(sys.meta)
    meta["perm"] = perm
    return LduSystem(sys.n, lo2.astype(np.int32), up2.astype(np.int32), sys.diag[perm], upc2,
                     loc2, sys.b[perm], sys.x0[perm], iface, name=sys.name + "-perm", meta=meta)


def convdiff_system(nx: int, ny: int, nz: int, *, seed: int = 0, k: float = 1.0,
                    pe_max: float = 10.0, rc: float = 1.0, permute: bool = True) -> LduSystem:
    """Asymmetric upwind convection-diffusion on a hex block.

    The velocity is the curl of a seeded smooth vector potential, so the face
    fluxes are discretely divergence-free; it is scaled so the largest cell
    Peclet number |U| h / (k/rho c) is ``pe_max``.  Dirichlet 0/1 on the
    z-faces.  With ``permute`` the cell numbering is randomly permuted.
    """
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    n = nx * ny * nz
    lower, upper, dirn = box_faces(nx, ny, nz)
    # Vector potential on cell edges -> face fluxes via discrete curl (divergence-free).
    modes = rng.standard_normal((3, 3, 2))
    def psi_at(x, y, z, comp):
        s = 0.0
        for m in range(3):
            s = s + modes[comp, m, 0] * np.sin(np.pi * (m + 1) * (x + 0.3 * comp)) * \
                np.sin(np.pi * (m + 1) * (y + 0.2 * m)) * np.cos(np.pi * (m + 1) * z) + \
                modes[comp, m, 1] * np.cos(np.pi * (m + 1) * (x + y - 0.1 * comp))
        return s
    # Node-based stream-function on the (nx+1)(ny+1)(nz+1) lattice, 2-D curl per plane pair
    xs = np.arange(nx + 1) * h
    ys = np.arange(ny + 1) * h
    zs = np.arange(nz + 1) * h
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    A = [psi_at(X, Y, Z, c) for c in range(3)]   # potentials at lattice nodes
    # Flux through x-face (i+1/2, j, k): circulation of A around the face's edge loop.
    def edge_avg(Ac, axis):
        sl0 = [slice(None)] * 3
        sl1 = [slice(None)] * 3
        sl0[axis] = slice(0, -1)
        sl1[axis] = slice(1, None)
        return 0.5 * (Ac[tuple(sl0)] + Ac[tuple(sl1)])
    # Edge-integrated potentials: Ax along x-edges, Ay along y-edges, Az along z-edges
    Ex = edge_avg(A[0], 2) * h   # shape (nz+1, ny+1, nx)
    Ey = edge_avg(A[1], 1) * h   # (nz+1, ny, nx+1)
    Ez = edge_avg(A[2], 0) * h   # (nz, ny+1, nx+1)
    # Face fluxes (Stokes): flux_x at face normal +x located at node-plane i
    Fx = (Ez[:, 1:, :] - Ez[:, :-1, :]) - (Ey[1:, :, :] - Ey[:-1, :, :])   # (nz, ny, nx+1)
    Fy = (Ex[1:, :, :] - Ex[:-1, :, :]) - (Ez[:, :, 1:] - Ez[:, :, :-1])   # (nz, ny+1, nx)
    Fz = (Ey[:, :, 1:] - Ey[:, :, :-1]) - (Ex[:, 1:, :] - Ex[:, :-1, :])   # (nz+1, ny, nx)
    # internal face fluxes in box_faces' (unsorted) layout, then sorted like lower/upper
    fl = [Fx[:, :, 1:-1].ravel(), Fy[:, 1:-1, :].ravel(), Fz[1:-1, :, :].ravel()]
    idx = np.arange(n).reshape(nz, ny, nx)
    lo_raw = np.concatenate([idx[:, :, :-1].ravel(), idx[:, :-1, :].ravel(), idx[:-1, :, :].ravel()])
    up_raw = np.concatenate([idx[:, :, 1:].ravel(), idx[:, 1:, :].ravel(), idx[1:, :, :].ravel()])
    phi_raw = np.concatenate(fl)
    order = np.lexsort((up_raw, lo_raw))
    phi = phi_raw[order]
    assert np.array_equal(lo_raw[order], lower) and np.array_equal(up_raw[order], upper)
    umax = np.abs(phi).max() / (h * h)
    alpha = k / rc                     # thermal diffusivity (rho c = rc here)
    scale = pe_max * alpha / (umax * h) if umax > 0 else 0.0
    phi = phi * scale * rng.uniform(0.0, 1.0)  # |U| ~ U(0,1) of the Pe-limited maximum
    # Upwind: flux phi from lower->upper.  a_lu (upper coeff, row l, col u), a_ul (lower coeff)
    g = k * h                          # diffusion conductance k*A/h
    F = rc * phi                       # rho c phi
    upper_c = -g + np.minimum(F, 0.0)
    lower_c = -g - np.maximum(F, 0.0)
    diag = np.full(n, rc * h ** 3)
    np.add.at(diag, lower, g + np.maximum(F, 0.0))
    np.add.at(diag, upper, g - np.minimum(F, 0.0))
    t_old = rng.uniform(0.0, 1.0, n)
    b = rc * h ** 3 * t_old
    bot = np.arange(nx * ny)
    top = n - nx * ny + np.arange(nx * ny)
    gb = 2.0 * k * h
    diag[bot] += gb
    diag[top] += gb
    b[top] += gb * 1.0
    sys = LduSystem(n, lower.astype(np.int32), upper.astype(np.int32), diag, upper_c, lower_c,
                    b, t_old, None, name="convdiff", meta=dict(nx=nx, ny=ny, nz=nz, seed=seed))
    if permute:
        sys = random_permute(sys, seed + 1)
    return sys


def direct_map(centres_a, centres_b, tol):
    """Conformal face map B -> A by face-centre match (|cB - cA| < tol).

    Restates directMapInterfaceToInterfaceMapping::calcZoneAToZoneBFaceMap
    (src/numerics/interfaceToInterfaceMappings/directMapInterfaceToInterfaceMapping/
    directMapInterfaceToInterfaceMapping.C:147-190, tol = relTol*minEdgeLength with
    relTol 1e-3): map[iB] = the first A face within tol, and a face without a
    partner is an error ("interfaces are not conformal").  A uniform hash grid of
    cell size tol replaces the N^2 search; the first match in A order is kept.
    """
    ca = np.asarray(centres_a, float)
    cb = np.asarray(centres_b, float)
    key = lambda c: tuple(np.floor(c / tol).astype(np.int64))
    grid = {}
    for ia, c in enumerate(ca):
        grid.setdefault(key(c), []).append(ia)
    out = np.full(len(cb), -1, np.int64)
    offs = [(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)]
    for ib, c in enumerate(cb):
        k0 = key(c)
        cand = []
        for o in offs:
            cand.extend(grid.get((k0[0] + o[0], k0[1] + o[1], k0[2] + o[2]), ()))
        for ia in sorted(cand):
            if np.linalg.norm(c - ca[ia]) < tol:
                out[ib] = ia
                break
    if (out < 0).any():
        raise ValueError("interfaces are not conformal: directMap found no partner for "
                         f"{int((out < 0).sum())} faces")
    return out


def flow_over_heated_plate(fixture: dict, *, seed: int = 0, k_solid: float = 16.0, k_fluid: float = 0.6,
                           rc: float = 50.0, form: str = "global") -> LduSystem:
    """Temperature system on the reference tutorial's own meshes.

    ``fixture`` holds the LDU addressing of flowOverHeatedPlate's solid (8200
    cells) and fluid (13612 cells) meshes and their 200-face conformal
    regionCouple interface (tests/golden/flowOverHeatedPlate_ldu.npz).  The
    geometry factors are unit (topological Laplacian), conductivities are per
    region, the interface conductance is the harmonic mean; an implicit
    ddt-like diagonal ``rc`` and a seeded source make it well posed.  Solid
    cells come first, then fluid.  The interface pairing is found with
    ``direct_map`` on the face centres, as the reference's directMap does.
    """
    rng = np.random.default_rng(seed)
    ns, nfl = int(fixture["solid_n"]), int(fixture["fluid_n"])
    n = ns + nfl
    ls, us = fixture["solid_lower"].astype(np.int64), fixture["solid_upper"].astype(np.int64)
    lf, uf = fixture["fluid_lower"].astype(np.int64) + ns, fixture["fluid_upper"].astype(np.int64) + ns
    tol = 1e-3 * min(float(fixture["solid_iface_min_edge"]), float(fixture["fluid_iface_min_edge"]))
    m = direct_map(fixture["solid_iface_centres"], fixture["fluid_iface_centres"], tol)  # fluid face -> solid face
    s_cells = fixture["solid_iface_cells"].astype(np.int64)
    f_cells = fixture["fluid_iface_cells"].astype(np.int64) + ns
    s_of_f = s_cells[m]
    g_s, g_f, g_i = k_solid, k_fluid, _harm(k_solid, k_fluid)
    g_int = np.concatenate([np.full(ls.size, g_s), np.full(lf.size, g_f)])
    lower = np.concatenate([ls, lf])
    upper = np.concatenate([us, uf])
    diag = np.full(n, rc)
    np.add.at(diag, lower, g_int)
    np.add.at(diag, upper, g_int)
    np.add.at(diag, s_of_f, g_i)
    np.add.at(diag, f_cells, g_i)
    t_old = 300.0 + 50.0 * rng.uniform(0, 1, n)
    b = rc * t_old + rng.standard_normal(n)
    meta = dict(n_solid=ns, n_fluid=nfl, n_iface=len(f_cells))
    if form == "global":
        lo2, up2, g2 = upper_triangular(np.concatenate([lower, s_of_f]), np.concatenate([upper, f_cells]),
                                        np.concatenate([g_int, np.full(len(f_cells), g_i)]))
        return LduSystem(n, lo2.astype(np.int32), up2.astype(np.int32), diag, -g2, None, b, t_old,
                         name="fohp-global", meta=meta)
    # coupled form: region matrices + the two interface patches (fluid faces order)
    k = len(f_cells)
    iface = {"cells": np.concatenate([s_of_f, f_cells]).astype(np.int32),
             "bou": np.full(2 * k, g_i), "int": None,
             "ptr": np.arange(2 * k + 1, dtype=np.int32),
             "src": np.concatenate([f_cells, s_of_f]).astype(np.int32), "w": np.ones(2 * k)}
    lo2, up2, g2 = upper_triangular(lower, upper, g_int)
    return LduSystem(n, lo2.astype(np.int32), up2.astype(np.int32), diag, -g2, None, b, t_old, iface,
                     name="fohp-coupled", meta=meta)
