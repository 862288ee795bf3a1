"""Synthetic monolithic-interface data for the mono tests (test infrastructure).

Two regions meeting at an interface of planar faces: `conformal` pairs face
i of A with face i of B (identity GGI weights); otherwise the faces are the
jittered 3:2 lattices of the non-conformal case with the oracle's exact
overlap weights.  Some cells carry two interface faces (corner cells), so
the per-cell accumulation of the matrix source is exercised."""
from __future__ import annotations

import numpy as np

from test_oracle import jittered_faces


def side(rng, n_cells, n_faces, h):
    fc = rng.integers(0, n_cells, n_faces).astype(np.int32)
    fc[1::7] = fc[0::7][:len(fc[1::7])]          # repeated cells: several faces per cell
    mld = rng.uniform(0.5, 1.5, n_faces) * h
    return {"n_cells": n_cells, "face_cells": fc, "w": rng.uniform(0.25, 0.75, n_faces), "mld": mld,
            "dc": 1.0 / mld * rng.uniform(0.9, 1.1, n_faces), "sf": rng.uniform(0.5, 1.5, n_faces) * h * h}


def interface(seed=0, conformal=True, oracle_mod=None):
    rng = np.random.default_rng(seed)
    if conformal:
        nfa = nfb = 400
        a, b = side(rng, 900, nfa, 0.05), side(rng, 700, nfb, 0.05)
        ident = (np.arange(nfa + 1, dtype=np.int32), np.arange(nfa, dtype=np.int32), np.ones(nfa))
        a["ptr"], a["addr"], a["wts"] = ident
        b["ptr"], b["addr"], b["wts"] = ident
    else:
        fa = jittered_faces(24, 24, 0.2, seed + 1)
        fb = jittered_faces(16, 24, 0.2, seed + 2)
        (pa, sa, wa), (pb, sb, wb) = oracle_mod.ggi_weights(*fa, *fb)
        a, b = side(rng, 2000, 576, 1 / 24), side(rng, 1500, 384, 1 / 24)
        a["ptr"], a["addr"], a["wts"] = pa, sa, wa
        b["ptr"], b["addr"], b["wts"] = pb, sb, wb
    fields = {
        "T_a": rng.uniform(280.0, 360.0, a["n_cells"]), "T_b": rng.uniform(280.0, 360.0, b["n_cells"]),
        "f_a": rng.uniform(0.5, 20.0, len(a["face_cells"])), "f_b": rng.uniform(0.5, 20.0, len(b["face_cells"])),
        "Qr_a": rng.uniform(-50.0, 50.0, len(a["face_cells"])), "Qr_b": rng.uniform(-50.0, 50.0, len(b["face_cells"])),
        "b_a": rng.uniform(-1.0, 1.0, a["n_cells"]), "b_b": rng.uniform(-1.0, 1.0, b["n_cells"]),
    }
    return a, b, fields
