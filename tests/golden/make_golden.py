"""Generates the committed fixtures under tests/golden/.

1. ``flowOverHeatedPlate_ldu.npz`` -- the LDU addressing of the reference's
   own conjugate-heat-transfer tutorial meshes
   (tutorials/conjugateHeatTransfer/flowOverHeatedPlate/constant/{solid,fluid}/
   polyMesh): owner/neighbour of the internal faces (foam's lowerAddr/
   upperAddr), and for the 200-face regionCouple interface patches ("top" on
   the solid, "interface" on the fluid) their faceCells and face centres.
   Needs the reference tree (read-only) and is run once where that tree
   exists; test runs elsewhere only read the .npz.
2. ``oracle_small.npz`` -- oracle outputs on small seeded systems, so the
   oracle itself is regression-pinned and GPU tests can compare against
   stored vectors.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def _foam_list(path):
    """Parse an ASCII foam list file (labelList / faceList / vectorField)."""
    txt = open(path).read()
    body = txt[txt.index("\n(", txt.index("FoamFile")):]
    # strip header count + outer parentheses
    m = re.search(r"^(\d+)\s*\n\(", txt, re.M)
    count = int(m.group(1))
    inner = txt[m.end():]
    inner = inner[: inner.rindex(")")]
    return count, inner


def read_labels(path):
    n, inner = _foam_list(path)
    a = np.array(inner.split(), dtype=np.int64)
    assert a.size == n, (path, a.size, n)
    return a


def read_points(path):
    n, inner = _foam_list(path)
    v = np.array(re.findall(r"\(([^()]*)\)", inner)[:n], dtype=object)
    return np.array([[float(t) for t in s.split()] for s in v])


def read_faces(path):
    n, inner = _foam_list(path)
    faces = [np.array(s.split(), dtype=np.int64) for s in re.findall(r"\d+\(([^()]*)\)", inner)]
    assert len(faces) == n
    return faces


def read_boundary(path):
    txt = open(path).read()
    out = {}
    for m in re.finditer(r"(\w+)\s*\{([^}]*)\}", txt[txt.index("FoamFile") + 10:]):
        name, body = m.group(1), m.group(2)
        nf = re.search(r"nFaces\s+(\d+);", body)
        sf = re.search(r"startFace\s+(\d+);", body)
        if nf and sf:
            out[name] = (int(nf.group(1)), int(sf.group(1)))
    return out


def mesh_fixture(ref):
    base = os.path.join(ref, "tutorials/conjugateHeatTransfer/flowOverHeatedPlate/constant")
    data = {}
    for region, patch in (("solid", "top"), ("fluid", "interface")):
        pm = os.path.join(base, region, "polyMesh")
        owner = read_labels(os.path.join(pm, "owner"))
        neigh = read_labels(os.path.join(pm, "neighbour"))
        points = read_points(os.path.join(pm, "points"))
        faces = read_faces(os.path.join(pm, "faces"))
        bnd = read_boundary(os.path.join(pm, "boundary"))
        nint = neigh.size
        ncells = int(max(owner.max(), neigh.max()) + 1)
        nfp, start = bnd[patch]
        centres = np.array([points[faces[f]].mean(axis=0) for f in range(start, start + nfp)])
        edges = []
        for f in range(start, start + nfp):
            p = points[faces[f]]
            edges.append(np.linalg.norm(p - np.roll(p, 1, axis=0), axis=1).min())
        data[f"{region}_n"] = np.int64(ncells)
        data[f"{region}_lower"] = owner[:nint].astype(np.int32)
        data[f"{region}_upper"] = neigh.astype(np.int32)
        data[f"{region}_iface_cells"] = owner[start:start + nfp].astype(np.int32)
        data[f"{region}_iface_centres"] = centres
        data[f"{region}_iface_min_edge"] = np.float64(min(edges))
    np.savez_compressed(os.path.join(HERE, "flowOverHeatedPlate_ldu.npz"), **data)
    print("wrote flowOverHeatedPlate_ldu.npz", {k: getattr(v, "shape", v) for k, v in data.items()})


def oracle_fixture():
    import oracle as O
    from multiregionfoam_gb300 import cases
    out = {}
    systems = {
        "cht": cases.cht_system(12, 10, 8, 5, seed=11, form="global"),
        "chtc": cases.cht_system(12, 10, 8, 5, seed=11, form="coupled"),
        "cd": cases.convdiff_system(10, 9, 8, seed=5),
    }
    for name, s in systems.items():
        # inputs are stored too: numpy's exp/log may differ by an ulp across
        # hosts, so tests rebuild the systems from these arrays, not from seeds
        out[f"{name}_n"] = np.int64(s.n)
        out[f"{name}_lower"], out[f"{name}_upper"] = s.lower, s.upper
        out[f"{name}_diag"], out[f"{name}_upper_c"] = s.diag, s.upper_c
        out[f"{name}_b"], out[f"{name}_x0"] = s.b, s.x0
        if s.lower_c is not None:
            out[f"{name}_lower_c"] = s.lower_c
        if s.iface is not None:
            for k in ("cells", "bou", "ptr", "src", "w"):
                out[f"{name}_iface_{k}"] = s.iface[k]
        M = O.OracleMatrix(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.iface)
        rng = np.random.default_rng(99)
        xr = rng.standard_normal(s.n)
        out[f"{name}_x"] = xr
        out[f"{name}_amul"] = M.amul(xr)
        out[f"{name}_tmul"] = M.tmul(xr)
        out[f"{name}_sumA"] = M.sumA()
        kind = "DIC" if s.symmetric else "DILU"
        solver = "PCG" if s.symmetric else "PBiCG"
        out[f"{name}_rD"] = M.factor(kind)
        out[f"{name}_prec"] = M.precondition(kind, xr)
        x, perf = M.solve(s.b, s.x0, solver, kind, tol=1e-10)
        out[f"{name}_sol"] = x
        out[f"{name}_perf"] = np.array([perf["initial_residual"], perf["final_residual"], perf["n_iter"]])
        # GPU-arithmetic mirrors (fused products, GPU reduction tree): the GPU
        # must reproduce these bit for bit from the stored inputs
        out[f"{name}_amul_fused"] = M.amul(xr, fused=True)
        out[f"{name}_tmul_fused"] = M.tmul(xr, fused=True)
        out[f"{name}_prec_fused"] = M.precondition(kind, xr, fused=True)
        xm, pm = M.solve_mirror(s.b, s.x0, solver, kind, tol=1e-10)
        out[f"{name}_sol_mirror"] = xm
        out[f"{name}_perf_mirror"] = np.array([pm["initial_residual"], pm["final_residual"], pm["n_iter"]])
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("wrote oracle_small.npz", len(out), "arrays")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if os.path.isdir(ref):
        mesh_fixture(ref)
    else:
        print("reference tree not found; mesh fixture not regenerated")
    oracle_fixture()
