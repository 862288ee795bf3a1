"""Kernel variants that must not change a bit of any result:

  MRG_SWEEP_PAIRS  FP32 levelled sweeps, two chunks per warp step (default)
                   or one
  MRG_ITERATION    the Krylov iterations as a graph of launches (default) or
                   as phases of one persistent cooperative kernel
                   (=persistent; BiCGStab has no persistent form)
  MRG_SPMV         Amul + (q, p) by the streamed kernel (bulk-copied
                   operands) with one round per step in FP32 and the per-warp
                   staged kernel in FP64 (default); the streamed kernel in
                   both (=stream1); two rounds per step in FP32 (=stream2);
                   the per-warp staged kernel in both (=warp)
  MRG_PART_SWEEPS  exact-order sweeps of one system by the owner-computes
                   kernel, one CTA a part of the cells (default), or by the
                   ticketed sync-free kernel (=0)
  MRG_SF_CTAS      CTAs per SM of the ticketed sync-free sweeps (default 3;
                   =1 here)

Solves with every variant give bit-identical solutions and iteration counts.
The switches are read once per process, so each variant runs in a child
process.  Cases: the coupled CHT system (interfaces) with PCG + DIC, mixed
and FP64 (exact order); the permuted convection-diffusion system with PBiCG
+ DILU (transposed sweeps) and BiCGStab + DILU (the M^-1 p and M^-1 s vector
sets), mixed; the same three in FP64 exact order, and the CHT system mixed
in exact order (FP32 exact sweeps); smoothSolver (Gauss-Seidel) and GAMG
on the global CHT system.  Both systems have more than 64 cells a
part, so their exact sweeps take the owner-computes kernel by default.  A
batch of 24 systems of many sizes (mixed PCG, colour) covers the kernels'
walks over many systems' reduction segments.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from multiregionfoam_gb300 import cases, mrgpu
mrgpu.load()
ctx = mrgpu.Context(0)
out = {}
cht = cases.cht_system(24, 24, 16, 8, seed=3, form="coupled")
cd = cases.convdiff_system(24, 22, 20, seed=4)
chg = cases.cht_system(24, 24, 16, 8, seed=5, form="global")
runs = [
    ("cht", cht, "PCG", "DIC", "mixed", "colour"),
    ("cht64", cht, "PCG", "DIC", "fp64", "exact"),
    ("cht_mixed_exact", cht, "PCG", "DIC", "mixed", "exact"),
    ("cd_pbicg", cd, "PBiCG", "DILU", "mixed", "colour"),
    ("cd_bicgstab", cd, "BiCGStab", "DILU", "mixed", "colour"),
    ("cd_pbicg64", cd, "PBiCG", "DILU", "fp64", "exact"),
    ("cd_bicgstab64", cd, "BiCGStab", "DILU", "fp64", "exact"),
    ("gs", chg, "smoothSolver", "none", "fp64", "exact"),
    ("gamg", chg, "GAMG", "none", "fp64", "exact"),
]
for name, s, solver, pc, prec, ordering in runs:
    m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper, s.iface)
    f = s.iface
    m.upload(s.diag, s.upper_c, s.lower_c, None if f is None else f["bou"], None if f is None else f.get("int"))
    x, p = m.solve(s.b, s.x0, tol=1e-4 if solver == "smoothSolver" else 1e-8, max_iter=3000, solver=solver,
                   precond=pc, precision=prec, ordering=ordering)
    m.close()
    np.save(sys.argv[2] + "_" + name + ".npy", x)
    out[name] = [int(p["n_iter"]), int(p.get("n_outer", 0)), bool(p["converged"])]
# a batch of systems of many sizes (FP32 reduction segments of odd and even
# round counts), mixed PCG + colour DIC
systems = cases.c4(24, seed=6, n_lo=2000, n_hi=40000)
meshes = [mrgpu.Mesh(ctx, s.n, s.lower, s.upper) for s in systems]
for mm, s in zip(meshes, systems):
    mm.upload(s.diag, s.upper_c)
bt = mrgpu.Batch(ctx, meshes, "colour")
xs, ps = bt.solve([s.b for s in systems], [s.x0 for s in systems], tol=1e-8, max_iter=3000, solver="PCG",
                  precond="DIC", precision="mixed", ordering="colour")
bt.close()
np.save(sys.argv[2] + "_batch.npy", np.concatenate(xs))
out["batch"] = [int(sum(p["n_iter"] for p in ps)), 0, all(p["converged"] for p in ps)]
ctx.close()
print(json.dumps(out))
"""


def _run(tmp_path, tag, **switches):
    from multiregionfoam_gb300 import _build
    _build.build()
    env = dict(os.environ, **switches)
    stem = str(tmp_path / tag)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, stem], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return stem, json.loads(r.stdout.strip().splitlines()[-1])


@pytest.fixture(scope="module")
def default_run(tmp_path_factory):
    return _run(tmp_path_factory.mktemp("variants"), "default")


@pytest.mark.parametrize("switch,value", [("MRG_SWEEP_PAIRS", "0"), ("MRG_ITERATION", "persistent"),
                                          ("MRG_SPMV", "warp"), ("MRG_SPMV", "stream1"),
                                          ("MRG_SPMV", "stream2"), ("MRG_PART_SWEEPS", "0"),
                                          ("MRG_SF_CTAS", "1")])
def test_variant_bit_identical(tmp_path, default_run, switch, value):
    s1, p1 = default_run
    s0, p0 = _run(tmp_path, switch, **{switch: value})
    assert p1 == p0
    for name, (_, _, conv) in p1.items():
        assert conv, name
        a, b = np.load(f"{s1}_{name}.npy"), np.load(f"{s0}_{name}.npy")
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), name
