"""The FP32 levelled sweeps' two-chunks-per-warp kernel (MRG_SWEEP_PAIRS,
default on) against the one-chunk kernel: mixed colour-ordered solves give
bit-identical solutions and iteration counts with either.  The switch is
read once per process, so each side runs in a child process.

Cases: the coupled CHT system (interfaces) with PCG + DIC, the permuted
convection-diffusion system with PBiCG + DILU (transposed sweeps) and with
BiCGStab + DILU (the M^-1 p and M^-1 s vector sets).
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
runs = [
    ("cht", cases.cht_system(24, 24, 16, 8, seed=3, form="coupled"), "PCG", "DIC"),
    ("cd_pbicg", cases.convdiff_system(20, 18, 16, seed=4), "PBiCG", "DILU"),
    ("cd_bicgstab", cases.convdiff_system(20, 18, 16, seed=4), "BiCGStab", "DILU"),
]
for name, s, solver, pc in runs:
    m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper, s.iface)
    f = s.iface
    m.upload(s.diag, s.upper_c, s.lower_c, None if f is None else f["bou"], None if f is None else f.get("int"))
    x, p = m.solve(s.b, s.x0, tol=1e-8, max_iter=3000, solver=solver, precond=pc, precision="mixed",
                   ordering="colour")
    m.close()
    np.save(sys.argv[2] + "_" + name + ".npy", x)
    out[name] = [int(p["n_iter"]), int(p.get("n_outer", 0)), bool(p["converged"])]
ctx.close()
print(json.dumps(out))
"""


def _run(tmp_path, pairs):
    from multiregionfoam_gb300 import _build
    _build.build()
    env = dict(os.environ, MRG_SWEEP_PAIRS="1" if pairs else "0")
    stem = str(tmp_path / ("pairs" if pairs else "single"))
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, stem], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return stem, json.loads(r.stdout.strip().splitlines()[-1])


def test_sweep_pairs_bit_identical(tmp_path):
    s1, p1 = _run(tmp_path, True)
    s0, p0 = _run(tmp_path, False)
    assert p1 == p0
    for name, (_, _, conv) in p1.items():
        assert conv, name
        a, b = np.load(f"{s1}_{name}.npy"), np.load(f"{s0}_{name}.npy")
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), name
