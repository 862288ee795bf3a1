"""One solve of a named workload, for profiling the hot-path kernels (a
profiling driver beside the tests; not part of the library).

    python tests/profile_case.py --case c2 --precision mixed
    python tests/profile_case.py --case c2 --precision fp64 --max-iter 6
    python tests/profile_case.py --case gamg64 --solver GAMG --max-iter 2
    python tests/profile_case.py --case cd435 --solver PBiCG --precision fp64 --ordering colour

The case is built and uploaded once and solved once (PCG + DIC at 1e-8;
mixed: colour ordering, fp64: exact foam order), so a kernel profiler sees
every kernel of one solve -- or, with ``--max-iter``, of a few Krylov
iterations after a short prologue.  Prints the solve's performance record.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from multiregionfoam_gb300 import _build, cases, mrgpu  # noqa: E402

CASES = {
    "c1": lambda seed: cases.c1(form="global", seed=seed),
    "c2": lambda seed: cases.c2(form="global", seed=seed),
    "gamg64": lambda seed: cases.cht_system(64, 64, 32, 32, seed=seed, form="global"),
    # a mid-size asymmetric system of the served mix: upwind convection-
    # diffusion on 64 x 68 x 100 cells (435k)
    "cd435": lambda seed: cases.convdiff_system(64, 68, 100, seed=47 + seed),
}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--case", default="c2", choices=sorted(CASES))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solver", default="PCG", choices=["PCG", "PBiCG", "GAMG"],
                    help="GAMG: the tutorials' words (faceAreaPair, GaussSeidel), FP64 exact order; "
                         "PBiCG: with DILU, for the asymmetric cases")
    ap.add_argument("--ordering", default=None, choices=["exact", "colour"],
                    help="default: colour for mixed, exact (foam order) for fp64")
    ap.add_argument("--max-iter", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    _build.build()
    s = CASES[args.case](args.seed)
    ctx = mrgpu.Context(0)
    m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper)
    m.upload(s.diag, s.upper_c, s.lower_c)
    if args.solver == "GAMG":
        m.set_face_areas(cases.face_area_vectors(s))
        _, perf = m.solve(s.b, s.x0, tol=1e-8, solver="GAMG", agglomerator="faceAreaPair", max_iter=args.max_iter)
    else:
        ordering = args.ordering or ("colour" if args.precision == "mixed" else "exact")
        pc = "DILU" if args.solver == "PBiCG" else "DIC"
        _, perf = m.solve(s.b, s.x0, tol=1e-8, precision=args.precision, ordering=ordering, solver=args.solver,
                          precond=pc, max_iter=args.max_iter, iters_per_launch=2 if args.max_iter < 100 else 16)
    print(json.dumps({"case": args.case, "n": s.n, "precision": args.precision, **perf}), flush=True)
    m.close()
    ctx.close()


if __name__ == "__main__":
    main()
